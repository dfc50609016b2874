// CPU restatement of the reference XPBD cloth substep -- TEST INFRASTRUCTURE ONLY.
//
// This library is the correctness oracle and the timed CPU baseline.  It is
// loaded only by tests/, by __graft_entry__.smoke() and by bench.py's CPU
// baseline leg; the product path (the CUDA library) never calls it.
//
// Parity status: the reference (Python + Taichi 1.7.1) runs here only through
// a numpy stand-in for the Taichi API (serial loops, IEEE float32); its outputs
// are committed as golden vectors (tests/golden/reference_vectors.npz) and this
// library matches them bit for bit on classification, distances, Morton codes,
// the cell BVH and the substep kernels, and to float32 rounding on contact
// gradients, positions and velocities (contact records equal).  Each function
// below restates the reference file:line it follows; known-answer tests and
// brute-force checks in tests/ cover the rest.
//
// Numeric conventions shared with the CUDA kernels (documented, not taken from
// the reference, whose Taichi build uses float atomics and fast math):
//   * IEEE float32, no FMA contraction (compile with -ffp-contract=off),
//     correctly rounded sqrt and division;
//   * spring/bending accumulation in ascending constraint index per vertex
//     (= a serial execution of the reference loop);
//   * contact corrections accumulated in 64-bit fixed point with 40 fractional
//     bits (order independent, so the serial and parallel orders agree);
//   * float -> int conversions truncate toward zero and saturate; NaN -> 0.
//
// nthreads > 1 runs the loops with OpenMP the way the reference's Taichi
// ti.cpu backend would: parallel loops, float atomics for the spring
// accumulation (so the spring result is then order dependent) -- used only for
// timing.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#define API extern "C" __attribute__((visibility("default")))

namespace {

struct V3 {
    float x, y, z;
};
inline V3 v3(const float* p) { return V3{p[0], p[1], p[2]}; }
inline V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 scale(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
inline V3 neg(V3 a) { return V3{-a.x, -a.y, -a.z}; }
inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 vmin(V3 a, V3 b) { return V3{std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)}; }
inline V3 vmax(V3 a, V3 b) { return V3{std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)}; }

// float -> int32, truncation toward zero, saturating, NaN -> 0
inline int32_t f2i_sat(float f) {
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f <= -2147483648.0f) return INT32_MIN;
    return (int32_t)f;
}

// contact fixed point: 40 fractional bits, saturating at +-2^62
constexpr double kFixScale = 1099511627776.0;        // 2^40
constexpr double kFixInv = 1.0 / 1099511627776.0;    // 2^-40
constexpr double kFixMax = 4611686018427387904.0;    // 2^62
inline int64_t to_fix(float c, int* bad) {
    double d = (double)c * kFixScale;
    if (d != d) { *bad = 1; return 0; }
    if (d >= kFixMax) { *bad = 1; return (int64_t)4611686018427387904LL; }
    if (d <= -kFixMax) { *bad = 1; return -(int64_t)4611686018427387904LL; }
    return (int64_t)std::nearbyint(d);
}
inline float from_fix(int64_t a) { return (float)((double)a * kFixInv); }

inline void atomic_addf(float* p, float v, bool par) {
    if (par) {
#pragma omp atomic
        *p += v;
    } else {
        *p += v;
    }
}

int set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    return nthreads > 1;
#else
    (void)nthreads;
    return 0;
#endif
}

}  // namespace

// ---------------------------------------------------------------------------
// cloth state kernels  (framework/physics/XPBD.py)
// ---------------------------------------------------------------------------

// XPBD.py:116-118 compute_y: y = x + fixed*v*dt + g*dt*dt ; y.w = x.w
API int or_predict(int V, const float* x4, const float* v4, const float* fixed, float* y4,
                   float dt, float gx, float gy, float gz, int nthreads) {
    int par = set_threads(nthreads);
    const float g[3] = {gx, gy, gz};
#pragma omp parallel for if (par)
    for (int i = 0; i < V; ++i) {
        for (int k = 0; k < 3; ++k)
            y4[4 * i + k] = (x4[4 * i + k] + (fixed[i] * v4[4 * i + k]) * dt) + (g[k] * dt) * dt;
        y4[4 * i + 3] = x4[4 * i + 3];
    }
    return 0;
}

// XPBD.py:141-184 solve_spring_constraints_x + XPBD.py:384-387 update_dx, with
// XPBD.py:345-348 init_variables in front.  Springs read y; bending pairs read x
// as in the reference (XPBD.py:169) when bend_on_y == 0, or the current y when
// bend_on_y == 1 (iterated Jacobi: every sweep evaluates all constraints on the
// current iterate).  k_spring / k_bend are the two "compliance" arguments
// (stiffness * dt^2) already assigned to their constraint types.
// dx3 (3V floats) and nc (V floats) are scratch.
API int or_spring_sweep(int V, int E, int B, const float* x4, float* y4, const float* fixed,
                        const float* m_inv, const int* edges, const float* l0, const int* bend,
                        const float* bend_l0, float k_spring, float k_bend, int bend_on_y, float* dx3, float* nc,
                        int nthreads) {
    int par = set_threads(nthreads);
    std::memset(dx3, 0, sizeof(float) * 3 * (size_t)V);
    std::memset(nc, 0, sizeof(float) * (size_t)V);
#pragma omp parallel for if (par)
    for (int i = 0; i < E + B; ++i) {
        int v0, v1;
        float rest, k;
        const float* P;
        if (i < E) {
            v0 = edges[2 * i];
            v1 = edges[2 * i + 1];
            rest = l0[i];
            k = k_spring;
            P = y4;
        } else {
            int b = i - E;
            v0 = bend[2 * b];
            v1 = bend[2 * b + 1];
            rest = bend_l0[b];
            k = k_bend;
            P = bend_on_y ? y4 : x4;
        }
        V3 x10 = sub(v3(P + 4 * v0), v3(P + 4 * v1));
        float lij = std::sqrt(dot(x10, x10));
        float C = lij - rest;
        float inv = 1.0f / lij;
        V3 n = scale(inv, x10);
        float w0 = fixed[v0] * m_inv[v0];
        float w1 = fixed[v1] * m_inv[v1];
        float schur = (w0 + w1) * dot(n, n);
        float ld = (k * C) / (k * schur + 1.0f);
        float a0 = w0 * ld, a1 = w1 * ld;
        atomic_addf(&dx3[3 * v0 + 0], -(a0 * n.x), par);
        atomic_addf(&dx3[3 * v0 + 1], -(a0 * n.y), par);
        atomic_addf(&dx3[3 * v0 + 2], -(a0 * n.z), par);
        atomic_addf(&dx3[3 * v1 + 0], a1 * n.x, par);
        atomic_addf(&dx3[3 * v1 + 1], a1 * n.y, par);
        atomic_addf(&dx3[3 * v1 + 2], a1 * n.z, par);
        atomic_addf(&nc[v0], 1.0f, par);
        atomic_addf(&nc[v1], 1.0f, par);
    }
#pragma omp parallel for if (par)
    for (int v = 0; v < V; ++v) {
        if (nc[v] > 0.0f) {
            for (int k = 0; k < 3; ++k) y4[4 * v + k] = y4[4 * v + k] + fixed[v] * (dx3[3 * v + k] / nc[v]);
        }
    }
    return 0;
}

// The same sweep as a per-vertex gather over the vertex-centric CSR (adjacency
// entries in ascending constraint index: springs, then bending pairs), for
// multithreaded runs that must equal the serial one bit for bit.  A vertex
// meets its constraints in the order the serial loop above does, and from the
// second endpoint the difference P[v] - P[u] is the exact negation of the
// scatter's x10, so lij, C, schur (w0 + w1 commutes) and ld are the same bits
// and -(w_self * ld * n_self) is the scattered term bit for bit.  ynew is
// scratch of 4 V floats.
API int or_spring_sweep_gather(int V, const float* x4, float* y4, const float* fixed, const float* m_inv,
                               const int32_t* ptr, const int32_t* adj, float k_spring, float k_bend, int bend_on_y,
                               float* ynew, int nthreads) {
    int par = set_threads(nthreads);
#pragma omp parallel for if (par) schedule(static, 256)
    for (int v = 0; v < V; ++v) {
        float d0 = 0.0f, d1 = 0.0f, d2 = 0.0f, cnt = 0.0f;
        const float wv = fixed[v] * m_inv[v];
        for (int e = ptr[v]; e < ptr[v + 1]; ++e) {
            const uint32_t w = (uint32_t)adj[2 * e];
            const int u = (int)(w & 0x7fffffffu);
            const bool bending = (w >> 31) != 0;
            float rest;
            std::memcpy(&rest, &adj[2 * e + 1], 4);
            const float k = bending ? k_bend : k_spring;
            const float* P = (bending && !bend_on_y) ? x4 : y4;
            V3 x = sub(v3(P + 4 * v), v3(P + 4 * u));
            float lij = std::sqrt(dot(x, x));
            float C = lij - rest;
            float inv = 1.0f / lij;
            V3 n = scale(inv, x);
            float wu = fixed[u] * m_inv[u];
            // the scatter evaluates (w0 + w1) with w0 of the constraint's first vertex
            float schur = (wv + wu) * dot(n, n);
            float ld = (k * C) / (k * schur + 1.0f);
            float a = wv * ld;
            d0 = d0 + -(a * n.x);
            d1 = d1 + -(a * n.y);
            d2 = d2 + -(a * n.z);
            cnt = cnt + 1.0f;
        }
        float* o = ynew + 4 * (size_t)v;
        const float* yi = y4 + 4 * (size_t)v;
        o[0] = yi[0]; o[1] = yi[1]; o[2] = yi[2]; o[3] = yi[3];
        if (cnt > 0.0f) {
            o[0] = yi[0] + fixed[v] * (d0 / cnt);
            o[1] = yi[1] + fixed[v] * (d1 / cnt);
            o[2] = yi[2] + fixed[v] * (d2 / cnt);
        }
    }
    std::memcpy(y4, ynew, sizeof(float) * 4 * (size_t)V);
    return 0;
}

// XPBD.py:341-343 compute_velocity then XPBD.py:333-337 update_x
API int or_velocity_update(int V, float* x4, const float* y4, float* v4, const float* fixed,
                           float damping, float dt, int nthreads) {
    int par = set_threads(nthreads);
    float s0 = 1.0f - damping;
#pragma omp parallel for if (par)
    for (int i = 0; i < V; ++i) {
        float s = s0 * fixed[i];
        for (int k = 0; k < 3; ++k) {
            float vel = (s * (y4[4 * i + k] - x4[4 * i + k])) / dt;
            v4[4 * i + k] = vel;
            x4[4 * i + k] = x4[4 * i + k] + dt * vel;
        }
    }
    return 0;
}

// meshTaichiWrapper.py:351-365 computeAABB_faces on a position array P (x4 layout)
API int or_face_aabbs(int F, const float* P4, const int* faces, float padding, float* mn4, float* mx4) {
    for (int f = 0; f < F; ++f) {
        V3 a = v3(P4 + 4 * faces[3 * f]), b = v3(P4 + 4 * faces[3 * f + 1]), c = v3(P4 + 4 * faces[3 * f + 2]);
        V3 lo = vmin(vmin(a, b), c), hi = vmax(vmax(a, b), c);
        mn4[4 * f + 0] = lo.x - padding; mn4[4 * f + 1] = lo.y - padding; mn4[4 * f + 2] = lo.z - padding; mn4[4 * f + 3] = 0.f;
        mx4[4 * f + 0] = hi.x + padding; mx4[4 * f + 1] = hi.y + padding; mx4[4 * f + 2] = hi.z + padding; mx4[4 * f + 3] = 0.f;
    }
    return 0;
}

// meshTaichiWrapper.py:335-347 computeAABB -> out6 = (min xyz, max xyz)
API int or_scene_aabb(int V, const float* P4, float padding, float* out6) {
    V3 lo{1e5f, 1e5f, 1e5f}, hi{-1e5f, -1e5f, -1e5f};
    for (int i = 0; i < V; ++i) {
        V3 p = v3(P4 + 4 * i);
        lo = vmin(lo, p);
        hi = vmax(hi, p);
    }
    out6[0] = lo.x - padding; out6[1] = lo.y - padding; out6[2] = lo.z - padding;
    out6[3] = hi.x + padding; out6[4] = hi.y + padding; out6[5] = hi.z + padding;
    return 0;
}

// ---------------------------------------------------------------------------
// Morton codes, radix sort, Karras hierarchy  (framework/collision/lbvh_cell.py)
// ---------------------------------------------------------------------------
namespace {
// lbvh_cell.py:87-92
inline uint64_t expand_bits(uint64_t v) {
    v = (v | (v << 16)) & 0x030000FFull;
    v = (v | (v << 8)) & 0x0300F00Full;
    v = (v | (v << 4)) & 0x030C30C3ull;
    v = (v | (v << 2)) & 0x09249249ull;
    return v;
}
inline float clampf(float v, float lo, float hi) { return std::min(std::max(v, lo), hi); }
// lbvh_cell.py:95-102 (input already normalised and clamped to [0,1])
inline int32_t morton3d(float x, float y, float z) {
    x = clampf(x * 1024.0f, 0.0f, 1023.0f);
    y = clampf(y * 1024.0f, 0.0f, 1023.0f);
    z = clampf(z * 1024.0f, 0.0f, 1023.0f);
    uint64_t xx = expand_bits((uint64_t)x), yy = expand_bits((uint64_t)y), zz = expand_bits((uint64_t)z);
    return (int32_t)(uint32_t)(xx | (yy << 1) | (zz << 2));
}
// lbvh_cell.py:139-148: normalise a point by the box, clamp, encode
inline int32_t morton_of(V3 p, V3 lo, V3 hi) {
    float x = (p.x - lo.x) / (hi.x - lo.x);
    float y = (p.y - lo.y) / (hi.y - lo.y);
    float z = (p.z - lo.z) / (hi.z - lo.z);
    return morton3d(clampf(x, 0.f, 1.f), clampf(y, 0.f, 1.f), clampf(z, 0.f, 1.f));
}
inline int clz32(uint32_t v) { return v == 0 ? 32 : __builtin_clz(v); }
}  // namespace

API int or_morton3d(int n, const float* xyz, int32_t* codes) {
    for (int i = 0; i < n; ++i) codes[i] = morton3d(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    return 0;
}

// Face-centre Morton codes for the face-level LBVH, following the intended form
// lbvh_cell.py:196-232: centre = 0.5*(aabb_max + aabb_min), normalised by the
// scene box, clamped, encoded.  ids[i] = i.
API int or_face_morton(int F, const float* mn4, const float* mx4, const float* box6, int32_t* codes, int32_t* ids) {
    V3 lo{box6[0], box6[1], box6[2]}, hi{box6[3], box6[4], box6[5]};
    for (int f = 0; f < F; ++f) {
        V3 c = scale(0.5f, add(v3(mx4 + 4 * f), v3(mn4 + 4 * f)));
        codes[f] = morton_of(c, lo, hi);
        ids[f] = f;
    }
    return 0;
}

// lbvh_cell.py:525-562: LSD radix sort, 6-bit digits, atomic histogram,
// inclusive scan, serialized back-to-front scatter.  Sorts (keys, vals) in place
// over the low `bits` key bits (keys treated as unsigned).
API int or_radix_sort(int n, uint32_t* keys, int32_t* vals, int bits) {
    const int BPP = 6, R = 1 << BPP;
    int passes = (bits + BPP - 1) / BPP;
    std::vector<uint32_t> k2(n);
    std::vector<int32_t> v2(n);
    for (int p = 0; p < passes; ++p) {
        int ps[R] = {0};
        for (int i = 0; i < n; ++i) ps[(keys[i] >> (p * BPP)) & (R - 1)] += 1;
        for (int d = 1; d < R; ++d) ps[d] += ps[d - 1];
        for (int i = 0; i < n; ++i) {
            int I = n - 1 - i;
            int d = (keys[I] >> (p * BPP)) & (R - 1);
            int idx = ps[d] - 1;
            k2[idx] = keys[I];
            v2[idx] = vals[I];
            ps[d] -= 1;
        }
        std::memcpy(keys, k2.data(), sizeof(uint32_t) * n);
        std::memcpy(vals, v2.data(), sizeof(int32_t) * n);
    }
    return 0;
}

namespace {
// lbvh_cell.py:256-264 delta.  tie==1 adds the index tie-break of Karras 2012
// (equal codes compare by index), which the reference does not have.
inline int kdelta(int i, int j, int n, const int32_t* c, int tie) {
    if (j > n - 1 || j < 0) return -1;
    uint32_t x = (uint32_t)(c[i] ^ c[j]);
    if (x == 0) return tie ? 32 + clz32((uint32_t)(i ^ j)) : 32;
    return clz32(x);
}
// lbvh_cell.py:273-298 find_split
inline int find_split(int l, int r, const int32_t* c, int n, int tie) {
    int32_t first = c[l], last = c[r];
    if (first == last && !tie) return (l + r) / 2;
    int common = kdelta(l, r, n, c, tie);
    int split = l, step = r - l;
    while (step > 1) {
        step = (step + 1) / 2;
        int ns = split + step;
        if (ns < r) {
            if (kdelta(l, ns, n, c, tie) > common) split = ns;
        }
    }
    return split;
}
// lbvh_cell.py:302-336 determine_range (note the exponential step l_max <<= 2)
inline void determine_range(int i, int n, const int32_t* c, int tie, int* start, int* end) {
    int dl = kdelta(i, i - 1, n, c, tie), dr = kdelta(i, i + 1, n, c, tie);
    int d = 1, dmin = dl;
    if (dr < dl) { d = -1; dmin = dr; }
    int64_t lmax = 2;
    while (lmax < (int64_t)4 * n) {
        int64_t j = i + lmax * d;
        if (j < INT32_MIN || j > INT32_MAX) break;
        if (kdelta(i, (int)j, n, c, tie) > dmin) lmax <<= 2; else break;
    }
    int64_t l = 0, t = lmax / 2;
    while (t > 0) {
        int64_t j = i + (l + t) * d;
        int dd = -1;
        if (j >= 0 && j < n) dd = kdelta(i, (int)j, n, c, tie);
        if (dd > dmin) l += t;
        t /= 2;
    }
    *start = i; *end = (int)(i + l * d);
    if (d == -1) { *start = (int)(i + l * d); *end = i; }
}
}  // namespace

// lbvh_cell.py:384-430 assign_internal_nodes_Karras12(_cells).  Writes, for
// internal node i in [0, n-1): child_a, child_b, range_l, range_r; parent[] for
// all 2n-1 nodes is written in node order (the last writer wins, as a serial run
// of the reference would leave it); parent[0] = -1 here.
API int or_karras(int n, const int32_t* codes, int tie, int32_t* child_a, int32_t* child_b,
                  int32_t* range_l, int32_t* range_r, int32_t* parent) {
    for (int i = 0; i < 2 * n - 1; ++i) parent[i] = -1;
    for (int i = 0; i < n - 1; ++i) {
        int s, e;
        determine_range(i, n, codes, tie, &s, &e);
        int split = find_split(s, e, codes, n, tie);
        int left = split;
        if (split == s) left += n - 1;
        int right = split + 1;
        if (right == e) right += n - 1;
        child_a[i] = left; child_b[i] = right;
        range_l[i] = s; range_r[i] = e;
        parent[left] = i; parent[right] = i;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Cell-grid LBVH (LBVH_CELL, lbvh_cell.py:16-714)
// Node arrays cover 2n-1 nodes: internal 0..n-2, leaves n-1..2n-2.
// ---------------------------------------------------------------------------
namespace {
constexpr int GR = 32;
constexpr int NC = GR * GR * GR;
inline V3 cell_size_of(const float* box6) {
    return V3{(box6[3] - box6[0]) / (float)GR, (box6[4] - box6[1]) / (float)GR, (box6[5] - box6[2]) / (float)GR};
}
inline V3 cell_center(int i, V3 cs, V3 lo) {
    int x0 = i / (GR * GR), y0 = (i % (GR * GR)) / GR, z0 = i % GR;
    V3 p{cs.x * (float)x0 + 0.5f * cs.x, cs.y * (float)y0 + 0.5f * cs.y, cs.z * (float)z0 + 0.5f * cs.z};
    return add(p, lo);
}
// lbvh_cell.py:565-574 (truncating float->int cast, then x*1024 + y*32 + z in
// wrapping int32 arithmetic)
inline int32_t flat_cell(V3 pos, V3 cs, V3 org) {
    int32_t ix = f2i_sat((pos.x - org.x) / cs.x);
    int32_t iy = f2i_sat((pos.y - org.y) / cs.y);
    int32_t iz = f2i_sat((pos.z - org.z) / cs.z);
    uint32_t r = (uint32_t)ix * (uint32_t)(GR * GR) + (uint32_t)iy * (uint32_t)GR + (uint32_t)iz;
    return (int32_t)r;
}
inline bool overlap(V3 a0, V3 a1, V3 b0, V3 b1) {
    return a0.x <= b1.x && a1.x >= b0.x && a0.y <= b1.y && a1.y >= b0.y && a0.z <= b1.z && a1.z >= b0.z;
}
}  // namespace

// LBVH_CELL.__init__ (lbvh_cell.py:78-80): cell Morton codes over the box
// (0,0,0)-(1e3,1e3,1e3), 6-bit radix sort, Karras build.  Outputs the sorted
// codes and ids and the internal-node topology.
API int or_cell_bvh_init(int32_t* sorted_codes, int32_t* sorted_ids, int32_t* child_a, int32_t* child_b,
                         int32_t* range_l, int32_t* range_r, int32_t* parent) {
    float box[6] = {0.f, 0.f, 0.f, 1e3f, 1e3f, 1e3f};
    V3 lo{0.f, 0.f, 0.f}, hi{1e3f, 1e3f, 1e3f};
    V3 cs = cell_size_of(box);
    std::vector<uint32_t> k(NC);
    for (int i = 0; i < NC; ++i) {
        V3 p = cell_center(i, cs, lo);
        k[i] = (uint32_t)morton_of(p, lo, hi);
        sorted_ids[i] = i;
    }
    or_radix_sort(NC, k.data(), sorted_ids, 30);
    for (int i = 0; i < NC; ++i) sorted_codes[i] = (int32_t)k[i];
    return or_karras(NC, sorted_codes, 0, child_a, child_b, range_l, range_r, parent);
}

// LBVH_CELL.build (lbvh_cell.py:637-653) for one mesh whose face AABBs are given.
// In:  topology from or_cell_bvh_init; face AABBs mn4/mx4 (F); box6 = scene AABB.
// Out: sorted_face_ids[F], prefix[NC] (inclusive), node num_faces/aabb for 2n-1
//      nodes (nmin4/nmax4 float4 each), cell_size3.
// Faces whose centre cell coordinate falls outside [0,32) are clamped into the
// grid (the reference would index out of bounds there).
API int or_cell_bvh_build(int F, const float* mn4, const float* mx4, const float* box6, const int32_t* child_a,
                          const int32_t* child_b, const int32_t* parent, int32_t* sorted_face_ids, int32_t* prefix,
                          int32_t* num_faces, float* nmin4, float* nmax4, float* cell_size3) {
    V3 lo{box6[0], box6[1], box6[2]};
    V3 cs = cell_size_of(box6);
    cell_size3[0] = cs.x; cell_size3[1] = cs.y; cell_size3[2] = cs.z;
    std::vector<int32_t> fcell(F);
    std::fill(prefix, prefix + NC, 0);
    for (int f = 0; f < F; ++f) {  // assign_face_cell_ids :577-586
        V3 c = scale(0.5f, add(v3(mn4 + 4 * f), v3(mx4 + 4 * f)));
        int ix = std::min(std::max(f2i_sat((c.x - lo.x) / cs.x), 0), GR - 1);
        int iy = std::min(std::max(f2i_sat((c.y - lo.y) / cs.y), 0), GR - 1);
        int iz = std::min(std::max(f2i_sat((c.z - lo.z) / cs.z), 0), GR - 1);
        int cell = ix * GR * GR + iy * GR + iz;
        fcell[f] = cell;
        prefix[cell] += 1;
    }
    for (int i = 1; i < NC; ++i) prefix[i] += prefix[i - 1];  // PrefixSumExecutor (inclusive)
    std::vector<int32_t> tmp(prefix, prefix + NC);
    for (int fid = 0; fid < F; ++fid) {  // counting_sort_cells :589-598, serial order
        int I = F - 1 - fid;
        int idx = --tmp[fcell[I]];
        sorted_face_ids[idx] = I;
    }
    const int N = 2 * NC - 1;
    std::vector<int32_t> visited(N, 0);
    std::fill(num_faces, num_faces + N, 0);
    for (int i = 0; i < NC; ++i) {  // assign_leaf_cell_nodes :602-634
        int leaf = i + NC - 1;
        int rl = i == 0 ? 0 : prefix[i - 1];
        int rr = prefix[i] - 1;
        int size = rr - rl + 1;
        V3 c = cell_center(i, cs, lo);
        V3 a = c, b = c;
        num_faces[leaf] = size;
        for (int j = 0; j < size; ++j) {
            int fid = sorted_face_ids[j + rl];
            a = vmin(a, v3(mn4 + 4 * fid));
            b = vmax(b, v3(mx4 + 4 * fid));
        }
        nmin4[4 * leaf] = a.x; nmin4[4 * leaf + 1] = a.y; nmin4[4 * leaf + 2] = a.z;
        std::memcpy(nmin4 + 4 * leaf + 3, &size, 4);  // node layout: min.w = face count (int bits)
        nmax4[4 * leaf] = b.x; nmax4[4 * leaf + 1] = b.y; nmax4[4 * leaf + 2] = b.z; nmax4[4 * leaf + 3] = 0.f;
        visited[parent[leaf]] += 1;
    }
    for (;;) {  // compute_bvh_aabbs_cells :481-522
        int cnt = 0;
        for (int i = 0; i < NC - 1; ++i) {
            if (visited[i] != 2) continue;
            int l = child_a[i], r = child_b[i];
            V3 min0 = v3(nmin4 + 4 * l), min1 = v3(nmin4 + 4 * r), max0 = v3(nmax4 + 4 * l), max1 = v3(nmax4 + 4 * r);
            num_faces[i] = num_faces[l] + num_faces[r];
            V3 a, b;
            if (num_faces[l] > 0 && num_faces[r] > 0) { a = vmin(min0, min1); b = vmax(max0, max1); }
            else if (num_faces[l] > 0) { a = min0; b = max0; }
            else if (num_faces[r] > 0) { a = min1; b = max1; }
            else { a = scale(0.25f, add(add(add(min0, max0), min1), max1)); b = a; }
            nmin4[4 * i] = a.x; nmin4[4 * i + 1] = a.y; nmin4[4 * i + 2] = a.z;
            std::memcpy(nmin4 + 4 * i + 3, &num_faces[i], 4);
            nmax4[4 * i] = b.x; nmax4[4 * i + 1] = b.y; nmax4[4 * i + 2] = b.z; nmax4[4 * i + 3] = 0.f;
            int p = parent[i];
            visited[i] += 1;
            if (p >= 0) visited[p] += 1;
            cnt += 1;
        }
        if (cnt == 0) break;
    }
    return 0;
}

// traverse_cell_bvh_single (lbvh_cell.py:662-714) for Q queries with AABBs
// qmin4/qmax4.  Candidates go to cand[q*cap + j] for j < cap; num[q] counts all
// overlaps (num > cap marks a truncated list).  Stack depth 64; a push beyond it
// sets *status |= 2 and drops the node.
API int or_cell_bvh_traverse(int Q, const float* qmin4, const float* qmax4, const float* cell_size3,
                             const float* origin3, const int32_t* child_a, const int32_t* child_b,
                             const int32_t* num_faces, const float* nmin4, const float* nmax4,
                             const int32_t* prefix, const int32_t* sorted_face_ids, const float* fmn4,
                             const float* fmx4, int cap, int32_t* cand, int32_t* num, int32_t* status) {
    V3 cs{cell_size3[0], cell_size3[1], cell_size3[2]}, org{origin3[0], origin3[1], origin3[2]};
    for (int q = 0; q < Q; ++q) {
        V3 a = v3(qmin4 + 4 * q), b = v3(qmax4 + 4 * q);
        num[q] = 0;
        V3 pos = scale(0.5f, add(a, b));
        int32_t cid = flat_cell(pos, cs, org);
        if (cid > NC - 1) continue;
        int stack[64];
        int sc = 0;
        stack[sc++] = 0;
        long long pops = 0;
        while (sc > 0) {
            if (++pops > 2LL * NC) { *status |= 2; break; }
            int idx = stack[--sc];
            if (num_faces[idx] <= 0) continue;
            if (!overlap(a, b, v3(nmin4 + 4 * idx), v3(nmax4 + 4 * idx))) continue;
            if (idx >= NC - 1) {
                int i = idx - (NC - 1);
                int rl = i == 0 ? 0 : prefix[i - 1];
                int size = prefix[i] - rl;
                for (int j = 0; j < size; ++j) {
                    int fid = sorted_face_ids[j + rl];
                    if (overlap(a, b, v3(fmn4 + 4 * fid), v3(fmx4 + 4 * fid))) {
                        if (num[q] < cap) cand[(size_t)q * cap + num[q]] = fid;
                        num[q] += 1;
                    }
                }
            } else {
                int l = child_a[idx], r = child_b[idx];
                if (num_faces[l] > 0) { if (sc < 64) stack[sc++] = l; else *status |= 2; }
                if (num_faces[r] > 0) { if (sc < 64) stack[sc++] = r; else *status |= 2; }
            }
        }
        if (num[q] > cap) *status |= 1;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Face-level LBVH (standalone broad phase)
// ---------------------------------------------------------------------------
// Leaves hold one face each (leaf n-1+j = sorted face j); refit with the
// compute_cell_node_aabbs rules (lbvh_cell.py:491-522), every leaf holding one
// face, so each internal box is the union of its children.  Bottom-up by
// repeated passes like the reference; nodes never reached stay untouched.
API int or_face_bvh_refit(int n, const int32_t* sorted_ids, const float* fmn4, const float* fmx4,
                          const int32_t* child_a, const int32_t* child_b, const int32_t* parent, float* nmin4,
                          float* nmax4) {
    const int N = 2 * n - 1;
    std::vector<int32_t> visited(N, 0);
    for (int j = 0; j < n; ++j) {
        int leaf = n - 1 + j, f = sorted_ids[j];
        std::memcpy(nmin4 + 4 * leaf, fmn4 + 4 * f, 16);
        std::memcpy(nmax4 + 4 * leaf, fmx4 + 4 * f, 16);
        if (parent[leaf] >= 0) visited[parent[leaf]] += 1;
    }
    for (;;) {
        int cnt = 0;
        for (int i = 0; i < n - 1; ++i) {
            if (visited[i] != 2) continue;
            int l = child_a[i], r = child_b[i];
            V3 a = vmin(v3(nmin4 + 4 * l), v3(nmin4 + 4 * r)), b = vmax(v3(nmax4 + 4 * l), v3(nmax4 + 4 * r));
            nmin4[4 * i] = a.x; nmin4[4 * i + 1] = a.y; nmin4[4 * i + 2] = a.z; nmin4[4 * i + 3] = 0.f;
            nmax4[4 * i] = b.x; nmax4[4 * i + 1] = b.y; nmax4[4 * i + 2] = b.z; nmax4[4 * i + 3] = 0.f;
            visited[i] += 1;
            if (parent[i] >= 0) visited[parent[i]] += 1;
            cnt += 1;
        }
        if (cnt == 0) break;
    }
    return 0;
}

// Stack traversal of the face-level LBVH (same visiting order as
// traverse_cell_bvh_single: pop, test, push child_a then child_b).
API int or_face_bvh_traverse(int n, int Q, const float* qmin4, const float* qmax4, const int32_t* child_a,
                             const int32_t* child_b, const int32_t* sorted_ids, const float* nmin4,
                             const float* nmax4, int cap, int32_t* cand, int32_t* num, int32_t* status) {
    for (int q = 0; q < Q; ++q) {
        V3 a = v3(qmin4 + 4 * q), b = v3(qmax4 + 4 * q);
        num[q] = 0;
        int stack[64];
        int sc = 0;
        stack[sc++] = 0;
        if (n == 1) stack[0] = 0;
        long long pops = 0;
        while (sc > 0) {
            if (++pops > 2LL * n) { *status |= 2; break; }
            int idx = stack[--sc];
            if (!overlap(a, b, v3(nmin4 + 4 * idx), v3(nmax4 + 4 * idx))) continue;
            if (idx >= n - 1) {
                int fid = sorted_ids[idx - (n - 1)];
                if (num[q] < cap) cand[(size_t)q * cap + num[q]] = fid;
                num[q] += 1;
            } else {
                int l = child_a[idx], r = child_b[idx];
                if (sc < 64) stack[sc++] = l; else *status |= 2;
                if (sc < 64) stack[sc++] = r; else *status |= 2;
            }
        }
        if (num[q] > cap) *status |= 1;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Narrow phase  (framework/collision/distance.py,
//                framework/physics/collision_constraints_x.py)
// ---------------------------------------------------------------------------
namespace {
// distance.py:5-47 d_type_PT: region of the closest feature of triangle
// (v1,v2,v3) to v0, via three 2x2 solves A^{-1} b with
// A^{-1} = (1/det) [[a11, -a01], [-a10, a00]].
inline void solve2(float a00, float a01, float a10, float a11, float b0, float b1, float* p0, float* p1) {
    float det = a00 * a11 - a01 * a10;
    float id = 1.0f / det;
    float m00 = id * a11, m01 = id * (-a01), m10 = id * (-a10), m11 = id * a00;
    *p0 = m00 * b0 + m01 * b1;
    *p1 = m10 * b0 + m11 * b1;
}
int d_type_PT(V3 v0, V3 v1, V3 v2, V3 v3) {
    V3 v12 = sub(v2, v1), v13 = sub(v3, v1);
    V3 n = cross(v12, v13);
    V3 v13n = cross(v12, n);
    V3 v10 = sub(v0, v1);
    float p00, p01;
    solve2(dot(v12, v12), dot(v12, v13n), dot(v13n, v12), dot(v13n, v13n), dot(v12, v10), dot(v13n, v10), &p00, &p01);
    if (p00 > 0.0f && p00 < 1.0f && p01 >= 0.0f) return 3;
    V3 v32 = sub(v3, v2), v32n = cross(v32, n), v20 = sub(v0, v2);
    float p10, p11;
    solve2(dot(v32, v32), dot(v32, v32n), dot(v32n, v32), dot(v32n, v32n), dot(v32, v20), dot(v32n, v20), &p10, &p11);
    if (p10 > 0.0f && p10 < 1.0f && p11 >= 0.0f) return 4;
    V3 v31 = sub(v1, v3), v31n = cross(v31, n), v30 = sub(v0, v3);
    float p20, p21;
    solve2(dot(v31, v31), dot(v31, v31n), dot(v31n, v31), dot(v31n, v31n), dot(v31, v30), dot(v31n, v30), &p20, &p21);
    if (p20 > 0.0f && p20 < 1.0f && p21 >= 0.0f) return 5;
    if (p00 <= 0.0f && p20 >= 1.0f) return 0;
    if (p10 <= 0.0f && p00 >= 1.0f) return 1;
    if (p20 <= 0.0f && p10 >= 1.0f) return 2;
    return 6;
}
// squared distances, distance.py:102-116
inline float d_PP(V3 a, V3 b) { V3 d = sub(a, b); return dot(d, d); }
inline float d_PE(V3 p, V3 e0, V3 e1) {
    V3 c = cross(sub(e0, p), sub(e1, p));
    V3 e = sub(e1, e0);
    return dot(c, c) / dot(e, e);
}
inline float d_PT(V3 p, V3 t0, V3 t1, V3 t2) {
    V3 b = cross(sub(t1, t0), sub(t2, t0));
    float s = dot(sub(p, t0), b);
    return s * s / dot(b, b);
}
// Gradients of the squared distances (the quantities of distance.py g_PP :127,
// g_PE :145-184, g_PT :413-459), written from the closed-form derivatives:
//  PP: d=|a-b|^2                      g_a = 2(a-b), g_b = -g_a
//  PE: c=(e0-p)x(e1-p), L=|e1-e0|^2, d=c.c/L
//      g_e0 = (2 (e1-p)xc + 2 d (e1-e0)) / L
//      g_e1 = (2 cx(e0-p) - 2 d (e1-e0)) / L,   g_p = -(g_e0 + g_e1)
//  PT: n=(t1-t0)x(t2-t0), r=p-t0, s=r.n, N=n.n, d=s^2/N
//      g_p  = 2 s n / N
//      g_t1 = (2 s (t2-t0)xr - 2 d (t2-t0)xn) / N
//      g_t2 = (2 s rx(t1-t0) - 2 d nx(t1-t0)) / N,   g_t0 = -(g_p + g_t1 + g_t2)
inline void g_PP(V3 a, V3 b, V3* ga, V3* gb) {
    V3 d = sub(a, b);
    *ga = scale(2.0f, d);
    *gb = neg(*ga);
}
inline void g_PE(V3 p, V3 e0, V3 e1, V3* gp, V3* g0, V3* g1) {
    V3 a = sub(e0, p), b = sub(e1, p);
    V3 c = cross(a, b);
    V3 e = sub(e1, e0);
    float L = dot(e, e);
    float iL = 1.0f / L;
    float d = dot(c, c) * iL;
    V3 bc = cross(b, c), ca = cross(c, a);
    float td = 2.0f * d;
    V3 t0 = add(scale(2.0f, bc), scale(td, e));
    V3 t1 = sub(scale(2.0f, ca), scale(td, e));
    *g0 = scale(iL, t0);
    *g1 = scale(iL, t1);
    *gp = neg(add(*g0, *g1));
}
inline void g_PT(V3 p, V3 t0, V3 t1, V3 t2, V3* gp, V3* g0, V3* g1, V3* g2) {
    V3 u = sub(t1, t0), w = sub(t2, t0);
    V3 n = cross(u, w);
    V3 r = sub(p, t0);
    float s = dot(r, n);
    float N = dot(n, n);
    float iN = 1.0f / N;
    float d = (s * s) * iN;
    float ts = 2.0f * s, td = 2.0f * d;
    *gp = scale(ts * iN, n);
    V3 a1 = sub(scale(ts, cross(w, r)), scale(td, cross(w, n)));
    V3 a2 = sub(scale(ts, cross(r, u)), scale(td, cross(n, u)));
    *g1 = scale(iN, a1);
    *g2 = scale(iN, a2);
    *g0 = neg(add(add(*gp, *g1), *g2));
}

// Evaluate the point-triangle distance by region.  g[0] is the point's gradient,
// g[1..3] the triangle vertices' (zero where the feature excludes the vertex).
inline float pt_distance(int dtype, V3 x0, V3 x1, V3 x2, V3 x3, V3 g[4], bool want_grad, float dflt) {
    float d = dflt;
    switch (dtype) {
        case 0: d = d_PP(x0, x1); if (want_grad) g_PP(x0, x1, &g[0], &g[1]); break;
        case 1: d = d_PP(x0, x2); if (want_grad) g_PP(x0, x2, &g[0], &g[2]); break;
        case 2: d = d_PP(x0, x3); if (want_grad) g_PP(x0, x3, &g[0], &g[3]); break;
        case 3: d = d_PE(x0, x1, x2); if (want_grad) g_PE(x0, x1, x2, &g[0], &g[1], &g[2]); break;
        case 4: d = d_PE(x0, x2, x3); if (want_grad) g_PE(x0, x2, x3, &g[0], &g[2], &g[3]); break;
        case 5: d = d_PE(x0, x1, x3); if (want_grad) g_PE(x0, x1, x3, &g[0], &g[1], &g[3]); break;
        case 6: d = d_PT(x0, x1, x2, x3); if (want_grad) g_PT(x0, x1, x2, x3, &g[0], &g[1], &g[2], &g[3]); break;
        default: break;
    }
    return d;
}
// vertex mask per region: which of (x0..x3) the feature involves
inline int region_mask(int dtype) {
    static const int m[7] = {0x3, 0x5, 0x9, 0x7, 0xD, 0xB, 0xF};
    return (dtype >= 0 && dtype < 7) ? m[dtype] : 0;
}

struct Acc {
    int64_t* dx;  // 3 per vertex
    int32_t* nc;
    int* bad;
    bool par;
    void add(int v, float a, V3 g) {
        int64_t c0 = to_fix(a * g.x, bad), c1 = to_fix(a * g.y, bad), c2 = to_fix(a * g.z, bad);
        if (par) {
#pragma omp atomic
            dx[3 * v] += c0;
#pragma omp atomic
            dx[3 * v + 1] += c1;
#pragma omp atomic
            dx[3 * v + 2] += c2;
#pragma omp atomic
            nc[v] += 1;
        } else {
            dx[3 * v] += c0; dx[3 * v + 1] += c1; dx[3 * v + 2] += c2; nc[v] += 1;
        }
    }
};

struct Pairs {  // optional pair records: pair[(q*cap+j)*2 + {0,1}] = (face, dtype)
    int32_t* pair;
    float* g;       // (q*cap+j)*16 : 4 gradients as float4
    float* schur;
    int32_t* num;
    int cap;
    void rec(int q, int face, int dtype, const V3 gg[4], float s) {
        if (!num) return;
        int j = num[q];
        if (j >= cap) return;
        size_t o = (size_t)q * cap + j;
        pair[2 * o] = face; pair[2 * o + 1] = dtype;
        for (int k = 0; k < 4; ++k) { g[16 * o + 4 * k] = gg[k].x; g[16 * o + 4 * k + 1] = gg[k].y; g[16 * o + 4 * k + 2] = gg[k].z; g[16 * o + 4 * k + 3] = 0.f; }
        schur[o] = s;
        num[q] = j + 1;
    }
};
}  // namespace

// solve_collision_constraints_x (XPBD.py:237-264) -> __vt_st / __vt_dy / __tv_st
// (collision_constraints_x.py:6-310) with fixed-point accumulation, then
// update_dx (XPBD.py:384-387) on the dynamic mesh (y4).
//   dynamic mesh: y4 (positions; .w unused here), fixed, m_inv, faces_dy
//   static mesh:  xs4 (positions), faces_st
//   candidates:   vt_st (Vd x cap), vt_dy (Vd x cap), tv_st (Vs x cap), counts
// Optional pair records (pass NULL to skip): three blocks, same layout.
// cull_d2 > 0: a pair whose point-to-triangle-box squared distance, or whose
// separating-axis bound (sat_far below), exceeds cull_d2 is skipped before
// classification (the CUDA pair-list sweep's cull; every region's distance is
// at least both, so with cull_d2 above dHat the skipped pair would add
// nothing).  0 classifies every pair.
static float box_d2(V3 p, V3 t0, V3 t1, V3 t2) {
    float ex = std::fmax(std::fmax(std::fmin(std::fmin(t0.x, t1.x), t2.x) - p.x, p.x - std::fmax(std::fmax(t0.x, t1.x), t2.x)), 0.0f);
    float ey = std::fmax(std::fmax(std::fmin(std::fmin(t0.y, t1.y), t2.y) - p.y, p.y - std::fmax(std::fmax(t0.y, t1.y), t2.y)), 0.0f);
    float ez = std::fmax(std::fmax(std::fmin(std::fmin(t0.z, t1.z), t2.z) - p.z, p.z - std::fmax(std::fmax(t0.z, t1.z), t2.z)), 0.0f);
    return (ex * ex + ey * ey) + ez * ez;
}

// Both cull stages skip only pairs of triangles on which d_type_PT's 2x2
// solves stay far inside float32's normal range (determinant about
// |e|^4 |n|^2): |n|^2 min|e|^4 > 1e-30 and |n|^2 max|e|^4 < 1e30.  On tinier
// or degenerate triangles the classification turns arbitrary (a far point can
// get the plane region and a spurious contact, which the reference applies).
static bool classifiable(V3 a, V3 b, V3 c) {
    V3 e0 = sub(b, a), e1 = sub(c, b), e2 = sub(a, c);
    V3 n = cross(e0, sub(c, a));
    float nn = dot(n, n);
    float l0 = dot(e0, e0), l1 = dot(e1, e1), l2 = dot(e2, e2);
    float lo = std::fmin(std::fmin(l0, l1), l2), hi = std::fmax(std::fmax(l0, l1), l2);
    return (nn * lo) * lo > 1e-30f && (nn * hi) * hi < 1e30f;
}

// Second cull stage of the CUDA pair-list sweep, mirrored so that the
// oracle's cull mode skips the same pairs: a separating-axis lower bound on
// dist(p, T) along the face normal n = (b-a) x (c-a) and the in-plane edge
// normals e x n, made safe against rounding (each projection errs by less
// than 2.4e-7 max|v - p|_1 |m|_1; 1e-6 of that is subtracted and a 1e-5
// relative margin asked for; axes with |m|^2 <= 1e-30 are not used).  Every
// region's distance is at least dist(p, T), so with cull_d2 above dHat a pair
// it removes would add nothing.
static float l1n(V3 a) { return (std::fabs(a.x) + std::fabs(a.y)) + std::fabs(a.z); }

static bool far_along(V3 m, V3 da, V3 db, V3 dc, float l1, float cull_d2) {
    float mm = dot(m, m);
    float sa = dot(da, m), sb = dot(db, m), sc = dot(dc, m);
    float gap = std::fmax(std::fmin(std::fmin(sa, sb), sc), -std::fmax(std::fmax(sa, sb), sc)) - 1e-6f * (l1 * l1n(m));
    return mm > 1e-30f && gap > 0.0f && gap * gap > (cull_d2 * mm) * 1.00001f;
}

static bool sat_far(V3 p, V3 a, V3 b, V3 c, float cull_d2) {
    V3 da = sub(a, p), db = sub(b, p), dc = sub(c, p);
    float l1 = std::fmax(std::fmax(l1n(da), l1n(db)), l1n(dc));
    V3 eab = sub(db, da), ebc = sub(dc, db), eca = sub(da, dc);
    V3 n = cross(eab, sub(dc, da));
    return far_along(n, da, db, dc, l1, cull_d2) || far_along(cross(eab, n), da, db, dc, l1, cull_d2) ||
           far_along(cross(ebc, n), da, db, dc, l1, cull_d2) || far_along(cross(eca, n), da, db, dc, l1, cull_d2);
}

static bool culled(float cull_d2, V3 p, V3 a, V3 b, V3 c) {
    return cull_d2 > 0.0f && classifiable(a, b, c) && (box_d2(p, a, b, c) > cull_d2 || sat_far(p, a, b, c, cull_d2));
}

// The two cull stages over n quadruples (12 floats each): out[i] = 1 box,
// 2 separating axes, 0 kept.
API int or_contact_cull(int n, const float* p12, float cull_d2, int32_t* out) {
    for (int i = 0; i < n; ++i) {
        const float* q = p12 + 12 * (size_t)i;
        V3 p = v3(q), a = v3(q + 3), b = v3(q + 6), c = v3(q + 9);
        out[i] = !classifiable(a, b, c) ? 0 : box_d2(p, a, b, c) > cull_d2 ? 1 : sat_far(p, a, b, c, cull_d2) ? 2 : 0;
    }
    return 0;
}

// accumulate != 0: dx_fix / nc already hold this iteration's edge-edge terms
// (or_edge_edge_sweep) and are added to instead of cleared.
API int or_collision_sweep(int Vd, int Vs, const int32_t* faces_dy, const int32_t* faces_st, float* y4,
                           const float* xs4, const float* fixed, const float* m_inv, float dHat, float compliance,
                           float cull_d2, int cap, const int32_t* vt_st_c, const int32_t* vt_st_n, const int32_t* vt_dy_c,
                           const int32_t* vt_dy_n, const int32_t* tv_st_c, const int32_t* tv_st_n,
                           int64_t* dx_fix, int32_t* nc, int32_t* pair, float* pair_g, float* pair_schur,
                           int32_t* pair_num, int32_t* status, int nthreads, int accumulate) {
    int par = set_threads(nthreads);
    if (!accumulate) {
        std::memset(dx_fix, 0, sizeof(int64_t) * 3 * (size_t)Vd);
        std::memset(nc, 0, sizeof(int32_t) * (size_t)Vd);
    }
    int bad = 0;
    Acc acc{dx_fix, nc, &bad, par != 0};
    Pairs P[3];
    for (int s = 0; s < 3; ++s) {
        size_t qoff = s == 2 ? 2 * (size_t)Vd : s * (size_t)Vd;
        P[s].cap = cap;
        P[s].num = pair_num ? pair_num + qoff : nullptr;
        P[s].pair = pair ? pair + 2 * qoff * cap : nullptr;
        P[s].g = pair_g ? pair_g + 16 * qoff * cap : nullptr;
        P[s].schur = pair_schur ? pair_schur + qoff * cap : nullptr;
    }
    if (pair_num) std::memset(pair_num, 0, sizeof(int32_t) * (2 * (size_t)Vd + Vs));
    const int total = 2 * Vd + Vs;
#pragma omp parallel for if (par) schedule(dynamic, 64)
    for (int i = 0; i < total; ++i) {
        if (i < Vd) {  // __vt_st: dynamic vertex (y) vs static triangle (x)
            int vid = i;
            int n = std::min(vt_st_n[vid], cap);
            for (int j = 0; j < n; ++j) {
                int fs = vt_st_c[(size_t)vid * cap + j];
                V3 x0 = v3(y4 + 4 * vid);
                V3 x1 = v3(xs4 + 4 * faces_st[3 * fs]), x2 = v3(xs4 + 4 * faces_st[3 * fs + 1]), x3 = v3(xs4 + 4 * faces_st[3 * fs + 2]);
                if (culled(cull_d2, x0, x1, x2, x3)) continue;
                V3 g[4] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                int dt = d_type_PT(x0, x1, x2, x3);
                float d = pt_distance(dt, x0, x1, x2, x3, g, true, dHat);
                if (d < dHat) {
                    float schur = m_inv[vid] * dot(g[0], g[0]);
                    float ld = (compliance * (dHat - d)) / (compliance * schur + 1.0f);
                    acc.add(vid, m_inv[vid] * ld, g[0]);  // no `fixed` factor (collision_constraints_x.py:58)
                    P[0].rec(vid, fs, dt, g, schur);
                }
            }
        } else if (i < 2 * Vd) {  // __vt_dy: self collision, incident faces skipped (XPBD.py:121-127)
            int vid = i - Vd;
            int n = std::min(vt_dy_n[vid], cap);
            for (int j = 0; j < n; ++j) {
                int fd = vt_dy_c[(size_t)vid * cap + j];
                int a = faces_dy[3 * fd], b = faces_dy[3 * fd + 1], c = faces_dy[3 * fd + 2];
                if (a == vid || b == vid || c == vid) continue;
                int vv[4] = {vid, a, b, c};
                V3 x[4] = {v3(y4 + 4 * vid), v3(y4 + 4 * a), v3(y4 + 4 * b), v3(y4 + 4 * c)};
                if (culled(cull_d2, x[0], x[1], x[2], x[3])) continue;
                V3 g[4] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                int dt = d_type_PT(x[0], x[1], x[2], x[3]);
                float d = pt_distance(dt, x[0], x[1], x[2], x[3], g, false, dHat);
                float schur = 0.0f;
                if (d < dHat) {
                    pt_distance(dt, x[0], x[1], x[2], x[3], g, true, dHat);
                    int m = region_mask(dt);
                    float s = 0.0f;
                    bool first = true;
                    for (int k = 0; k < 4; ++k) {
                        if (!(m & (1 << k))) continue;
                        float t = (fixed[vv[k]] * m_inv[vv[k]]) * dot(g[k], g[k]);
                        s = first ? t : s + t;
                        first = false;
                    }
                    schur = s + 1e-4f;
                    float ld = (dHat - d) / schur;
                    for (int k = 0; k < 4; ++k) {
                        if (!(m & (1 << k))) continue;
                        // dtype 0 applies m_inv without `fixed` (collision_constraints_x.py:199-200)
                        float w = dt == 0 ? m_inv[vv[k]] : fixed[vv[k]] * m_inv[vv[k]];
                        acc.add(vv[k], w * ld, g[k]);
                    }
                }
                P[1].rec(vid, fd, dt, g, schur);
            }
        } else {  // __tv_st: static vertex (x) vs dynamic triangle (y)
            int vis = i - 2 * Vd;
            int n = std::min(tv_st_n[vis], cap);
            for (int j = 0; j < n; ++j) {
                int fd = tv_st_c[(size_t)vis * cap + j];
                int vv[4] = {-1, faces_dy[3 * fd], faces_dy[3 * fd + 1], faces_dy[3 * fd + 2]};
                V3 x[4] = {v3(xs4 + 4 * vis), v3(y4 + 4 * vv[1]), v3(y4 + 4 * vv[2]), v3(y4 + 4 * vv[3])};
                if (culled(cull_d2, x[0], x[1], x[2], x[3])) continue;
                V3 g[4] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                int dt = d_type_PT(x[0], x[1], x[2], x[3]);
                float d = pt_distance(dt, x[0], x[1], x[2], x[3], g, false, dHat);
                float schur = 0.0f;
                if (d < dHat) {
                    pt_distance(dt, x[0], x[1], x[2], x[3], g, true, dHat);
                    int m = region_mask(dt) & ~1;
                    float s = 0.0f;
                    bool first = true;
                    for (int k = 1; k < 4; ++k) {
                        if (!(m & (1 << k))) continue;
                        float t = (fixed[vv[k]] * m_inv[vv[k]]) * dot(g[k], g[k]);
                        s = first ? t : s + t;
                        first = false;
                    }
                    schur = s;
                    float ld = (compliance * (dHat - d)) / (compliance * schur + 1.0f);
                    for (int k = 1; k < 4; ++k) {
                        if (!(m & (1 << k))) continue;
                        acc.add(vv[k], (fixed[vv[k]] * m_inv[vv[k]]) * ld, g[k]);
                    }
                }
                P[2].rec(vis, fd, dt, g, schur);
            }
        }
    }
    // update_dx on the dynamic mesh
#pragma omp parallel for if (par)
    for (int v = 0; v < Vd; ++v) {
        if (nc[v] > 0) {
            float c = (float)nc[v];
            for (int k = 0; k < 3; ++k) y4[4 * v + k] = y4[4 * v + k] + fixed[v] * (from_fix(dx_fix[3 * v + k]) / c);
        }
    }
    if (bad && status) *status |= 4;
    return 0;
}

// ---------------------------------------------------------------------------
// Edge-edge narrow phase: __ee_st / __ee_dy (collision_constraints_x.py:313-588)
// as the commented-out callers would run them (XPBD.py:217-232 broad phase on
// edge boxes, :266-281 narrow phase over the three edges of every candidate
// face, vertex-sharing pairs skipped for ee_dy).  Only the interior-interior
// case (dtype 8) with |x01 x x23| > 1e-3 projects; the other cases are
// commented out in the reference.
// ---------------------------------------------------------------------------
// d_type_EE (distance.py:50-99)
int d_type_EE(V3 v0, V3 v1, V3 v2, V3 v3) {
    const V3 u = sub(v1, v0), v = sub(v3, v2), w = sub(v0, v2);
    const float a = dot(u, u), b = dot(u, v), c = dot(v, v), d = dot(u, w), e = dot(v, w);
    const float D = a * c - b * b;
    float tD = D, tN = 0.0f;
    int dc = 8;
    const float sN = b * e - c * d;
    if (sN <= 0.0f) {
        tN = e;
        tD = c;
        dc = 2;
    } else if (sN >= D) {
        tN = e + b;
        tD = c;
        dc = 5;
    } else {
        tN = a * e - b * d;
        const V3 uv = cross(u, v);
        if (tN > 0.0f && tN < tD && (dot(uv, w) < 1e-4f || dot(uv, uv) < 1.0e-20f * a * c)) {
            if (sN < D / 2.0f) {
                tN = e;
                tD = c;
                dc = 2;
            } else {
                tN = e + b;
                tD = c;
                dc = 5;
            }
        }
    }
    if (tN <= 0.0f) {
        if (-d <= 0.0f) dc = 0;
        else if (-d >= a) dc = 3;
        else dc = 6;
    } else if (tN >= tD) {
        if (-d + b <= 0.0f) dc = 1;
        else if (-d + b >= a) dc = 4;
        else dc = 7;
    }
    return dc;
}
// d_EE (distance.py:119-124): squared distance between the two lines
inline float d_EE(V3 x0, V3 x1, V3 x2, V3 x3) {
    const V3 b = cross(sub(x1, x0), sub(x3, x2));
    const float aTb = dot(sub(x2, x0), b);
    return aTb * aTb / dot(b, b);
}
// Closed-form gradient of d_EE: u = x1-x0, v = x3-x2, r = x2-x0, n = u x v,
// s = r.n, N = n.n, d = s^2/N;
//   g0 = (-2s (n + v x r) + 2d v x n)/N,  g1 = (2s v x r - 2d v x n)/N,
//   g2 = (2s (n - r x u) + 2d n x u)/N,   g3 = (2s r x u - 2d n x u)/N.
inline void g_EE(V3 x0, V3 x1, V3 x2, V3 x3, V3 g[4]) {
    const V3 u = sub(x1, x0), v = sub(x3, x2), r = sub(x2, x0);
    const V3 n = cross(u, v);
    const float s = dot(r, n);
    const float N = dot(n, n);
    const float iN = 1.0f / N;
    const float d = (s * s) * iN;
    const float ts = 2.0f * s, td = 2.0f * d;
    const V3 vr = cross(v, r), ru = cross(r, u), vn = cross(v, n), nu = cross(n, u);
    g[0] = scale(iN, add(scale(-ts, add(n, vr)), scale(td, vn)));
    g[1] = scale(iN, sub(scale(ts, vr), scale(td, vn)));
    g[2] = scale(iN, add(scale(ts, sub(n, ru)), scale(td, nu)));
    g[3] = scale(iN, sub(scale(ts, ru), scale(td, nu)));
}
// One edge pair: dtype, and for dtype 8 with |x01 x x23| > 1e-3 the squared
// distance and (when it is below dHat) its gradient; d = dHat otherwise.
inline float ee_pair(V3 x0, V3 x1, V3 x2, V3 x3, float dHat, int* dtype, V3 g[4]) {
    const int dt = d_type_EE(x0, x1, x2, x3);
    *dtype = dt;
    float d = dHat;
    if (dt == 8) {
        const V3 c = cross(sub(x0, x1), sub(x2, x3));
        if (std::sqrt(dot(c, c)) > 1e-3f) {
            d = d_EE(x0, x1, x2, x3);
            if (d < dHat) g_EE(x0, x1, x2, x3, g);
        }
    }
    return d;
}

// Classification and distance of n point quadruples (12 floats each): the
// kernel-level check of every branch.
API int or_edge_edge_classify(int n, const float* p12, float dHat, int32_t* dtype, float* d, float* g12) {
    for (int i = 0; i < n; ++i) {
        const float* p = p12 + 12 * (size_t)i;
        V3 g[4] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        d[i] = ee_pair(v3(p), v3(p + 3), v3(p + 6), v3(p + 9), dHat, dtype + i, g);
        for (int k = 0; k < 4; ++k) {
            g12[12 * (size_t)i + 3 * k] = g[k].x;
            g12[12 * (size_t)i + 3 * k + 1] = g[k].y;
            g12[12 * (size_t)i + 3 * k + 2] = g[k].z;
        }
    }
    return 0;
}

// Edge-edge terms of one iteration, added to dx_fix / nc (no update_dx: the
// vertex-triangle sweep follows with accumulate = 1 and applies both).
//   dynamic edges (Ed): edges_dy, face_edges_dy[3 F_dy], positions y4
//   static mesh: edges_st, face_edges_st, xs4 (NULL: no ee_st)
//   candidates (faces): ee_st (Ed x cap) on the static BVH, ee_dy on the
//   dynamic one.  Records (optional): ee_st block then ee_dy block of Ed
//   queries, (partner edge, dtype), 4 gradients, schur; records past cap are
//   dropped.
API int or_edge_edge_sweep(int Ed, const int32_t* edges_dy, const int32_t* edges_st, const int32_t* face_edges_dy,
                           const int32_t* face_edges_st, const float* y4, const float* xs4, const float* fixed,
                           const float* m_inv, float dHat, float compliance, int cap, const int32_t* ee_st_c,
                           const int32_t* ee_st_n, const int32_t* ee_dy_c, const int32_t* ee_dy_n, int64_t* dx_fix,
                           int32_t* nc, int32_t* pair, float* pair_g, float* pair_schur, int32_t* pair_num,
                           int32_t* status, int nthreads) {
    int par = set_threads(nthreads);
    int bad = 0;
    Acc acc{dx_fix, nc, &bad, par != 0};
    Pairs P[2];
    for (int s = 0; s < 2; ++s) {
        size_t qoff = s * (size_t)Ed;
        P[s].cap = cap;
        P[s].num = pair_num ? pair_num + qoff : nullptr;
        P[s].pair = pair ? pair + 2 * qoff * cap : nullptr;
        P[s].g = pair_g ? pair_g + 16 * qoff * cap : nullptr;
        P[s].schur = pair_schur ? pair_schur + qoff * cap : nullptr;
    }
    if (pair_num) std::memset(pair_num, 0, sizeof(int32_t) * 2 * (size_t)Ed);
#pragma omp parallel for if (par) schedule(dynamic, 64)
    for (int i = 0; i < 2 * Ed; ++i) {
        const bool st = i < Ed;
        const int e = st ? i : i - Ed;
        if (st && !ee_st_c) continue;
        const int v0 = edges_dy[2 * e], v1 = edges_dy[2 * e + 1];
        const int n = std::min(st ? ee_st_n[e] : ee_dy_n[e], cap);
        for (int j = 0; j < n; ++j) {
            const int f = st ? ee_st_c[(size_t)e * cap + j] : ee_dy_c[(size_t)e * cap + j];
            for (int k = 0; k < 3; ++k) {
                const int e2 = st ? face_edges_st[3 * f + k] : face_edges_dy[3 * f + k];
                const int v2 = st ? edges_st[2 * e2] : edges_dy[2 * e2];
                const int v3i = st ? edges_st[2 * e2 + 1] : edges_dy[2 * e2 + 1];
                if (!st && (v0 == v2 || v0 == v3i || v1 == v2 || v1 == v3i)) continue;  // share_vertex (XPBD.py:130-136)
                const V3 x0 = v3(y4 + 4 * v0), x1 = v3(y4 + 4 * v1);
                const V3 x2 = st ? v3(xs4 + 4 * v2) : v3(y4 + 4 * v2), x3 = st ? v3(xs4 + 4 * v3i) : v3(y4 + 4 * v3i);
                V3 g[4] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                int dt;
                const float d = ee_pair(x0, x1, x2, x3, dHat, &dt, g);
                float schur = 0.0f;
                if (d < dHat) {
                    const float w0 = fixed[v0] * m_inv[v0], w1 = fixed[v1] * m_inv[v1];
                    if (st) {
                        schur = w0 * dot(g[0], g[0]) + w1 * dot(g[1], g[1]);
                    } else {
                        const float w2 = fixed[v2] * m_inv[v2], w3 = fixed[v3i] * m_inv[v3i];
                        schur = ((w0 * dot(g[0], g[0]) + w1 * dot(g[1], g[1])) + w2 * dot(g[2], g[2])) +
                                w3 * dot(g[3], g[3]);
                    }
                    const float ld = (compliance * (dHat - d)) / (compliance * schur + 1.0f);
                    acc.add(v0, w0 * ld, g[0]);
                    acc.add(v1, w1 * ld, g[1]);
                    if (!st) {
                        acc.add(v2, (fixed[v2] * m_inv[v2]) * ld, g[2]);
                        acc.add(v3i, (fixed[v3i] * m_inv[v3i]) * ld, g[3]);
                    }
                    P[st ? 0 : 1].rec(e, e2, dt, g, schur);
                }
            }
        }
    }
    if (bad && status) *status |= 4;
    return 0;
}

// Constraint residual of the CUDA library (sx_constraint_residual and the
// checked sweep), in its exact summation order: C = |p_self - p_other| - l0 in
// float per adjacency entry (vertex-centric CSR: entry word = neighbour with
// bit 31 set for bending pairs, rest length bits), per-vertex float sums in
// entry order, 32-vertex warp xor trees, 256-vertex block values
// ((w0+w1)+(w2+w3))+((w4+w5)+(w6+w7)) converted to double, then the FP64
// finish: 16384 strided thread sums, 32-lane xor trees, 8-warp pair trees and
// 64 block values in index order.  out3 = {S, n, sqrt(S/n)}.
API int or_residual(int V, const float* p4, const int32_t* ptr, const int32_t* adj, double* out3) {
    const int nb = V > 0 ? (V + 255) / 256 : 1;
    std::vector<double> partial(nb, 0.0);
    for (int blk = 0; blk < nb; ++blk) {
        float w[8];
        for (int wi = 0; wi < 8; ++wi) {
            float a[32];
            for (int l = 0; l < 32; ++l) {
                const int v = blk * 256 + wi * 32 + l;
                float c2 = 0.0f;
                if (v < V) {
                    const float* ps = p4 + 4 * (size_t)v;
                    for (int k = ptr[v]; k < ptr[v + 1]; ++k) {
                        const int nbv = adj[2 * k] & 0x7fffffff;
                        float rest;
                        std::memcpy(&rest, adj + 2 * k + 1, 4);
                        const float* o = p4 + 4 * (size_t)nbv;
                        const float ex = ps[0] - o[0], ey = ps[1] - o[1], ez = ps[2] - o[2];
                        const float C = std::sqrt((ex * ex + ey * ey) + ez * ez) - rest;
                        c2 = c2 + C * C;
                    }
                }
                a[l] = c2;
            }
            for (int o = 16; o > 0; o >>= 1) {
                float t[32];
                for (int l = 0; l < 32; ++l) t[l] = a[l] + a[l ^ o];
                std::memcpy(a, t, sizeof(a));
            }
            w[wi] = a[0];
        }
        partial[blk] = (double)(((w[0] + w[1]) + (w[2] + w[3])) + ((w[4] + w[5]) + (w[6] + w[7])));
    }
    const int RB = 64, RT = 256;
    std::vector<double> part2(RB);
    for (int b = 0; b < RB; ++b) {
        double ws[8];
        for (int wi = 0; wi < 8; ++wi) {
            double a[32];
            for (int l = 0; l < 32; ++l) {
                double acc = 0.0;
                for (int i = b * RT + wi * 32 + l; i < nb; i += RB * RT) acc += partial[i];
                a[l] = acc;
            }
            for (int o = 16; o > 0; o >>= 1) {
                double t[32];
                for (int l = 0; l < 32; ++l) t[l] = a[l] + a[l ^ o];
                std::memcpy(a, t, sizeof(a));
            }
            ws[wi] = a[0];
        }
        part2[b] = ((ws[0] + ws[1]) + (ws[2] + ws[3])) + ((ws[4] + ws[5]) + (ws[6] + ws[7]));
    }
    double S = 0.0;
    for (int b = 0; b < RB; ++b) S += part2[b];
    const double n = V > 0 ? (double)ptr[V] : 0.0;
    out3[0] = S;
    out3[1] = n;
    out3[2] = n > 0.0 ? std::sqrt(S / n) : 0.0;
    return 0;
}

// Features of the learned warm start (the CUDA library's warm_features_kernel;
// no counterpart in the reference): per vertex, from the predicted positions
// y4, start-of-substep positions x4, previous solve correction c4, fixed flags,
// the vertex-centric constraint CSR and L = mean spring rest length, 24 FP32
// values clamped to [-16, 16], rounded to BF16 (round to nearest even) and
// padded with 8 zeros.  Same expressions, same order.
static uint16_t bf16_rne(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

API int or_warm_features(int V, const float* x4, const float* y4, const float* c4, const float* fixed,
                         const int32_t* ptr, const int32_t* adj, const float* Lref, float gx, float gy, float gz,
                         float dt, uint16_t* feat) {
    for (int v = 0; v < V; ++v) {
        const float* ps = y4 + 4 * (size_t)v;
        const float* xs = x4 + 4 * (size_t)v;
        const float* cp = c4 + 4 * (size_t)v;
        const float inv = 1.0f / Lref[v];
        float sx = 0.0f, sy = 0.0f, sz = 0.0f, bx = 0.0f, by = 0.0f, bz = 0.0f;
        float sa = 0.0f, ba = 0.0f, smax = 0.0f, smin = 0.0f;
        int ns = 0, nb = 0;
        for (int k = ptr[v]; k < ptr[v + 1]; ++k) {
            const int32_t w = adj[2 * k];
            float rest;
            std::memcpy(&rest, adj + 2 * k + 1, 4);
            const float* o = y4 + 4 * (size_t)(w & 0x7fffffff);
            const float ex = ps[0] - o[0], ey = ps[1] - o[1], ez = ps[2] - o[2];
            const float l = std::sqrt((ex * ex + ey * ey) + ez * ez);
            const float C = l - rest;
            const float il = l > 0.0f ? 1.0f / l : 0.0f;
            const float cx = C * (il * ex), cy = C * (il * ey), cz = C * (il * ez);
            const float r = rest > 0.0f ? C / rest : 0.0f;
            if (w < 0) {
                bx = bx + cx; by = by + cy; bz = bz + cz;
                ba = ba + std::fabs(r);
                ++nb;
            } else {
                sx = sx + cx; sy = sy + cy; sz = sz + cz;
                sa = sa + std::fabs(r);
                smax = ns ? std::fmax(smax, r) : r;
                smin = ns ? std::fmin(smin, r) : r;
                ++ns;
            }
        }
        const float fs = (float)ns, fb = (float)nb;
        float f[24];
        f[0] = ns ? -((sx / fs) * inv) : 0.0f;
        f[1] = ns ? -((sy / fs) * inv) : 0.0f;
        f[2] = ns ? -((sz / fs) * inv) : 0.0f;
        f[3] = nb ? -((bx / fb) * inv) : 0.0f;
        f[4] = nb ? -((by / fb) * inv) : 0.0f;
        f[5] = nb ? -((bz / fb) * inv) : 0.0f;
        f[6] = ns ? sa / fs : 0.0f;
        f[7] = smax;
        f[8] = smin;
        f[9] = nb ? ba / fb : 0.0f;
        const float dx = ps[0] - xs[0], dy = ps[1] - xs[1], dz = ps[2] - xs[2];
        f[10] = dx * inv;
        f[11] = dy * inv;
        f[12] = dz * inv;
        f[13] = cp[0] * inv;
        f[14] = cp[1] * inv;
        f[15] = cp[2] * inv;
        f[16] = fixed[v];
        f[17] = fs / 6.0f;
        f[18] = fb / 6.0f;
        f[19] = std::sqrt((cp[0] * cp[0] + cp[1] * cp[1]) + cp[2] * cp[2]) * inv;
        f[20] = std::sqrt((dx * dx + dy * dy) + dz * dz) * inv;
        f[21] = ((gx * dt) * dt) * inv;
        f[22] = ((gy * dt) * dt) * inv;
        f[23] = ((gz * dt) * dt) * inv;
        uint16_t* out = feat + 32 * (size_t)v;
        for (int i = 0; i < 24; ++i) out[i] = bf16_rne(std::fmin(std::fmax(f[i], -16.0f), 16.0f));
        for (int i = 24; i < 32; ++i) out[i] = 0;
    }
    return 0;
}

// solve_sewing_constraints_x (XPBD.py:425-441) + update_dx, gathered per sewn
// vertex over its partners in ascending pair index (the CUDA sewing sweep's
// order); coincident pairs add nothing.  Updates y4 in place.
API int or_sewing_step(int n_sewn, const int32_t* sewn, const int32_t* sptr, const int32_t* partner, float* y4,
                       const float* fixed, float k) {
    std::vector<float> out(4 * (size_t)n_sewn);
    for (int i = 0; i < n_sewn; ++i) {
        const float* ps = y4 + 4 * (size_t)sewn[i];
        float dx = 0.0f, dy = 0.0f, dz = 0.0f;
        for (int j = sptr[i]; j < sptr[i + 1]; ++j) {
            const float* o = y4 + 4 * (size_t)partner[j];
            const float ex = ps[0] - o[0], ey = ps[1] - o[1], ez = ps[2] - o[2];
            const float C = std::sqrt((ex * ex + ey * ey) + ez * ez);
            if (C > 0.0f) {
                const float inv = 1.0f / C;
                const float nx = inv * ex, ny = inv * ey, nz = inv * ez;
                const float ld = (k * C) / (k * (ps[3] + o[3]) + 1.0f);
                const float a0 = ps[3] * ld;
                dx = dx - a0 * nx;
                dy = dy - a0 * ny;
                dz = dz - a0 * nz;
            }
        }
        float* r = out.data() + 4 * (size_t)i;
        r[0] = ps[0]; r[1] = ps[1]; r[2] = ps[2]; r[3] = ps[3];
        const float nc = (float)(sptr[i + 1] - sptr[i]);
        if (nc > 0.0f) {
            const float f = fixed[sewn[i]];
            r[0] = ps[0] + f * (dx / nc);
            r[1] = ps[1] + f * (dy / nc);
            r[2] = ps[2] + f * (dz / nc);
        }
    }
    for (int i = 0; i < n_sewn; ++i) std::memcpy(y4 + 4 * (size_t)sewn[i], out.data() + 4 * (size_t)i, 16);
    return 0;
}

// solve_constraints_v (XPBD.py:374-381, :398-404) over the pair records:
// collision_constraints_v.py __vt_st (:6-133), __tv_st (:137-330) and __vt_dy
// (:334-570), branch by branch in the reference's own expression order
// (scalar products evaluated left to right: f*m*ld*g = ((f*m)*ld)*g,
// f*m*g*ld = ((f*m)*g)*ld), each `dv += ...` with its `nc += 1`, fixed-point
// accumulation, then update_dv.  Quirks kept: __vt_st region 3 scales the
// normal impulse by the static mesh's m_inv at the dynamic vertex's id (0 past
// the static mesh), region 5 reverses the tangent; __tv_st's Cv uses g3 for v2;
// __vt_dy region 1 scales v2's tangential impulse by m_inv of v1.
namespace {
struct VelAcc {
    int64_t* dv;
    int32_t* nc;
    int* bad;
    void add(int v, V3 d) {
        dv[3 * v] += to_fix(d.x, bad);
        dv[3 * v + 1] += to_fix(d.y, bad);
        dv[3 * v + 2] += to_fix(d.z, bad);
        nc[v] += 1;
    }
};
inline V3 load3(const float* p) { return V3{p[0], p[1], p[2]}; }
inline V3 mulv(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
inline float norm3(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 divs(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
inline V3 wsum2(float a, V3 p, float b, V3 q) { return V3{a * p.x + b * q.x, a * p.y + b * q.y, a * p.z + b * q.z}; }
inline V3 wsum3(float a, V3 p, float b, V3 q, float c, V3 r) {
    return V3{(a * p.x + b * q.x) + c * r.x, (a * p.y + b * q.y) + c * r.y, (a * p.z + b * q.z) + c * r.z};
}
inline float mu_eff(float mu, float Cv, float cTan) { return mu * std::fabs(Cv) > cTan ? 1.0f : mu; }

void or_vt_st_v(VelAcc& A, int v0, int v1, int v2, int v3, int dtype, const V3* g, float schur, float mu,
                const float* v4, const float* vs4, const float* m_inv, const float* m_inv_st, int Vs) {
    V3 u0 = load3(v4 + 4 * v0), s1 = load3(vs4 + 4 * v1), s2 = load3(vs4 + 4 * v2), s3 = load3(vs4 + 4 * v3);
    float Cv = ((dot(g[0], u0) + dot(g[1], s1)) + dot(g[2], s2)) + dot(g[3], s3);
    if (!(Cv < 0.0f) || dtype < 0 || dtype > 6) return;
    float ld_v = -Cv / schur;
    float m0 = m_inv[v0];
    float mn = dtype == 3 ? (v0 < Vs ? m_inv_st[v0] : 0.0f) : m0;
    A.add(v0, scale(mn * ld_v, g[0]));
    V3 vTan0 = add(u0, scale(m0 * ld_v, g[0]));
    V3 g0Tan;
    if (dtype == 0) g0Tan = sub(s1, vTan0);
    else if (dtype == 1) g0Tan = sub(s2, vTan0);
    else if (dtype == 2) g0Tan = sub(s3, vTan0);
    else if (dtype == 3) { float a = norm3(g[1]), b = norm3(g[2]); g0Tan = sub(divs(wsum2(a, s1, b, s2), a + b), vTan0); }
    else if (dtype == 4) { float a = norm3(g[2]), b = norm3(g[3]); g0Tan = sub(divs(wsum2(a, s2, b, s3), a + b), vTan0); }
    else if (dtype == 5) { float a = norm3(g[1]), b = norm3(g[3]); g0Tan = sub(vTan0, divs(wsum2(a, s1, b, s3), a + b)); }
    else {
        float a = norm3(g[1]), b = norm3(g[2]), c = norm3(g[3]);
        g0Tan = sub(divs(wsum3(a, s1, b, s2, c, s3), (a + b) + c), vTan0);
    }
    float cTan = 0.5f * dot(g0Tan, g0Tan);
    float sT = m0 * dot(g0Tan, g0Tan) + 1e-4f;
    float ldTan = cTan / sT;
    V3 dvTan = scale(m0 * ldTan, g0Tan);
    A.add(v0, scale(mu_eff(mu, Cv, cTan), dvTan));
}

void or_tv_st_v(VelAcc& A, int v0, int v1, int v2, int v3, int dtype, const V3* g, float schur, float mu,
                const float* v4, const float* vs4, const float* fixed, const float* m_inv) {
    V3 w0 = load3(vs4 + 4 * v0), u1 = load3(v4 + 4 * v1), u2 = load3(v4 + 4 * v2), u3 = load3(v4 + 4 * v3);
    float Cv = ((dot(g[0], w0) + dot(g[1], u1)) + dot(g[3], u2)) + dot(g[3], u3);
    if (!(Cv < 0.0f) || dtype < 0 || dtype > 6) return;
    float ld_v = -Cv / schur;
    int vid[3] = {v1, v2, v3};
    V3 uu[3] = {u1, u2, u3};
    auto impulse = [&](int k) {  // dv[vk] += f m ld g_k ; returns vTan_k = v_k + f m g_k ld
        float fm = fixed[vid[k]] * m_inv[vid[k]];
        A.add(vid[k], scale(fm * ld_v, g[k + 1]));
        return add(uu[k], mulv(scale(fm, g[k + 1]), ld_v));
    };
    if (dtype <= 2) {
        int k = dtype;
        V3 vT = impulse(k);
        V3 gT = sub(w0, vT);
        float cTan = 0.5f * dot(gT, gT);
        float sT = m_inv[vid[k]] * dot(gT, gT) + 1e-4f;
        float ldTan = cTan / sT;
        V3 dvT = scale(m_inv[vid[k]] * ldTan, gT);
        A.add(vid[k], scale(mu_eff(mu, Cv, cTan), dvT));
    } else if (dtype <= 5) {
        int i = dtype == 4 ? 1 : 0, j = dtype == 3 ? 1 : 2;
        V3 vTi = impulse(i), vTj = impulse(j);
        float a = norm3(g[i + 1]), b = norm3(g[j + 1]);
        float ab = a + b;
        V3 p = divs(wsum2(a, vTi, b, vTj), dtype == 3 ? (a + b) : ab);
        V3 d = sub(w0, p);
        V3 giT = scale(a / ab, d), gjT = scale(b / ab, d);
        float cTan = 0.5f * dot(d, d);
        float sT = (m_inv[vid[i]] * dot(giT, giT) + m_inv[vid[j]] * dot(gjT, gjT)) + 1e-4f;
        float ldTan = cTan / sT;
        V3 dvi = scale(m_inv[vid[i]] * ldTan, giT), dvj = scale(m_inv[vid[j]] * ldTan, gjT);
        float me = mu_eff(mu, Cv, cTan);
        A.add(vid[i], scale(me, dvi));
        A.add(vid[j], scale(me, dvj));
    } else {
        V3 vT1 = impulse(0), vT2 = impulse(1), vT3 = impulse(2);
        float a = norm3(g[1]), b = norm3(g[2]), c = norm3(g[3]);
        float abc = (a + b) + c;
        V3 p = divs(wsum3(a, vT1, b, vT2, c, vT3), abc);
        V3 d = sub(w0, p);
        V3 g1T = scale(a / abc, d), g2T = scale(b / abc, d), g3T = scale(c / abc, d);
        float cTan = 0.5f * dot(d, d);
        float sT = ((m_inv[v1] * dot(g1T, g1T) + m_inv[v2] * dot(g2T, g2T)) + m_inv[v3] * dot(g3T, g3T)) + 1e-4f;
        float ldTan = cTan / sT;
        float me = mu_eff(mu, Cv, cTan);
        A.add(v1, scale(me, scale(m_inv[v1] * ldTan, g1T)));
        A.add(v2, scale(me, scale(m_inv[v2] * ldTan, g2T)));
        A.add(v3, scale(me, scale(m_inv[v3] * ldTan, g3T)));
    }
}

void or_vt_dy_v(VelAcc& A, const int* vv, int dtype, const V3* g, float schur, float mu, const float* v4,
                const float* fixed, const float* m_inv) {
    V3 u[4];
    for (int k = 0; k < 4; ++k) u[k] = load3(v4 + 4 * vv[k]);
    float Cv = ((dot(g[0], u[0]) + dot(g[1], u[1])) + dot(g[2], u[2])) + dot(g[3], u[3]);
    if (!(Cv < 0.0f) || dtype < 0 || dtype > 6) return;
    float ld_v = -Cv / schur;
    auto impulse = [&](int k) {  // dv[vk] += f m g_k ld ; returns vTan_k = v_k + f m g_k ld
        float fm = fixed[vv[k]] * m_inv[vv[k]];
        A.add(vv[k], mulv(scale(fm, g[k]), ld_v));
        return add(u[k], mulv(scale(fm, g[k]), ld_v));
    };
    if (dtype <= 2) {
        int k = dtype + 1;
        V3 vT0 = impulse(0), vTk = impulse(k);
        V3 g0T = neg(sub(vT0, vTk)), gkT = sub(vT0, vTk);
        float cTan = 0.5f * (dot(gkT, gkT) + dot(g0T, g0T));
        float sT = (m_inv[vv[0]] * dot(g0T, g0T) + m_inv[vv[k]] * dot(gkT, gkT)) + 1e-4f;
        float ldTan = cTan / sT;
        V3 dv0 = scale(m_inv[vv[0]] * ldTan, g0T);
        V3 dvk = scale(m_inv[dtype == 1 ? vv[1] : vv[k]] * ldTan, gkT);
        float me = mu_eff(mu, Cv, cTan);
        A.add(vv[0], scale(me, dv0));
        A.add(vv[k], scale(me, dvk));
    } else if (dtype <= 5) {
        int i = dtype == 4 ? 2 : 1, j = dtype == 3 ? 2 : 3;
        V3 vT0 = impulse(0), vTi = impulse(i), vTj = impulse(j);
        float a = norm3(g[i]), b = norm3(g[j]);
        float ab = a + b;
        V3 p = divs(wsum2(a, vTi, b, vTj), ab);
        V3 g0T = sub(p, vT0);
        V3 giT = scale(-(a / ab), g0T), gjT = scale(-(b / ab), g0T);
        float cTan = 0.5f * ((dot(g0T, g0T) + dot(giT, giT)) + dot(gjT, gjT));
        float sT = ((m_inv[vv[0]] * dot(g0T, g0T) + m_inv[vv[i]] * dot(giT, giT)) + m_inv[vv[j]] * dot(gjT, gjT)) +
                   1e-4f;
        float ldTan = cTan / sT;
        float me = mu_eff(mu, Cv, cTan);
        A.add(vv[0], scale(me, scale(m_inv[vv[0]] * ldTan, g0T)));
        A.add(vv[i], scale(me, scale(m_inv[vv[i]] * ldTan, giT)));
        A.add(vv[j], scale(me, scale(m_inv[vv[j]] * ldTan, gjT)));
    } else {
        V3 vT0 = impulse(0), vT1 = impulse(1), vT2 = impulse(2), vT3 = impulse(3);
        float a = norm3(g[1]), b = norm3(g[2]), c = norm3(g[3]);
        float abc = (a + b) + c;
        V3 p = divs(wsum3(a, vT1, b, vT2, c, vT3), abc);
        V3 g0T = sub(p, vT0);
        V3 g1T = scale(-(a / abc), g0T), g2T = scale(-(b / abc), g0T), g3T = scale(-(c / abc), g0T);
        float cTan = 0.5f * (((dot(g0T, g0T) + dot(g1T, g1T)) + dot(g2T, g2T)) + dot(g3T, g3T));
        float sT = (((m_inv[vv[0]] * dot(g0T, g0T) + m_inv[vv[1]] * dot(g1T, g1T)) + m_inv[vv[2]] * dot(g2T, g2T)) +
                    m_inv[vv[3]] * dot(g3T, g3T)) + 1e-4f;
        float ldTan = cTan / sT;
        float me = mu_eff(mu, Cv, cTan);
        A.add(vv[0], scale(me, scale(m_inv[vv[0]] * ldTan, g0T)));
        A.add(vv[1], scale(me, scale(m_inv[vv[1]] * ldTan, g1T)));
        A.add(vv[2], scale(me, scale(m_inv[vv[2]] * ldTan, g2T)));
        A.add(vv[3], scale(me, scale(m_inv[vv[3]] * ldTan, g3T)));
    }
}
}  // namespace

API int or_velocity_contacts(int Vd, int Vs, const int32_t* faces_dy, const int32_t* faces_st, int cap,
                             const int32_t* pair, const float* pair_g, const float* pair_schur,
                             const int32_t* pair_num, float* v4, const float* vs4, const float* fixed,
                             const float* m_inv, const float* m_inv_st, float mu, int32_t* status) {
    std::vector<int64_t> dv(3 * (size_t)Vd, 0);
    std::vector<int32_t> nc((size_t)Vd, 0);
    int bad = 0;
    VelAcc A{dv.data(), nc.data(), &bad};
    for (int q = 0; q < 2 * Vd + Vs; ++q) {
        int n = std::min(pair_num[q], cap);
        for (int j = 0; j < n; ++j) {
            size_t o = (size_t)q * cap + j;
            int face = pair[2 * o], dtype = pair[2 * o + 1];
            V3 g[4];
            for (int k = 0; k < 4; ++k) g[k] = v3(pair_g + 16 * o + 4 * k);
            float sc = pair_schur[o];
            if (q < Vd) {
                or_vt_st_v(A, q, faces_st[3 * face], faces_st[3 * face + 1], faces_st[3 * face + 2], dtype, g, sc, mu,
                           v4, vs4, m_inv, m_inv_st, Vs);
            } else if (q < 2 * Vd) {
                int vv[4] = {q - Vd, faces_dy[3 * face], faces_dy[3 * face + 1], faces_dy[3 * face + 2]};
                or_vt_dy_v(A, vv, dtype, g, sc, mu, v4, fixed, m_inv);
            } else {
                or_tv_st_v(A, q - 2 * Vd, faces_dy[3 * face], faces_dy[3 * face + 1], faces_dy[3 * face + 2], dtype, g,
                           sc, mu, v4, vs4, fixed, m_inv);
            }
        }
    }
    for (int v = 0; v < Vd; ++v) {  // update_dv (XPBD.py:398-404)
        if (nc[v] > 0 && m_inv[v] > 0.0f) {
            float c = (float)nc[v];
            for (int k = 0; k < 3; ++k) v4[4 * v + k] = v4[4 * v + k] + fixed[v] * (from_fix(dv[3 * v + k]) / c);
        }
    }
    if (bad && status) *status |= 4;
    return 0;
}

// The region classifier, distance and gradient for one point-triangle query
// (used by tests: known-answer and finite-difference checks).
API int or_point_triangle(const float* p12, float* d_out, float* g12) {
    V3 x0 = v3(p12), x1 = v3(p12 + 3), x2 = v3(p12 + 6), x3 = v3(p12 + 9);
    V3 g[4] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    int dt = d_type_PT(x0, x1, x2, x3);
    *d_out = pt_distance(dt, x0, x1, x2, x3, g, true, 0.0f);
    for (int k = 0; k < 4; ++k) { g12[3 * k] = g[k].x; g12[3 * k + 1] = g[k].y; g12[3 * k + 2] = g[k].z; }
    return dt;
}

// or_point_triangle over n quadruples (12 floats each): dtype[n], d[n], g12[12 n]
API int or_point_triangles(int n, const float* p12, int32_t* dtype, float* d, float* g12) {
    for (int i = 0; i < n; ++i) dtype[i] = or_point_triangle(p12 + 12 * (size_t)i, d + i, g12 + 12 * (size_t)i);
    return 0;
}

// ---------------------------------------------------------------------------
// Graph colouring (framework/utilities/graph_coloring.py)
// ---------------------------------------------------------------------------
// initAdjEdges (:112-129) + colorEdgesGreedy (:131-149): sequential first-fit in
// edge-id order; two edges are adjacent when they share a vertex; the colour is
// argmax of the 0/1 availability vector over max_colors entries (all forbidden
// -> colour 0).  colorCountingSort (:172-201): stable counting sort, back to
// front; prefix[c] = start offset of colour c (E for colours past the last).
API int or_color_edges(int V, int E, const int32_t* edges, int max_colors, int32_t* color, int32_t* sorted_edges,
                       int32_t* prefix) {
    std::vector<std::vector<int>> inc(V);
    for (int e = 0; e < E; ++e) { inc[edges[2 * e]].push_back(e); inc[edges[2 * e + 1]].push_back(e); }
    for (int e = 0; e < E; ++e) color[e] = -1;
    std::vector<char> avail(max_colors);
    for (int e = 0; e < E; ++e) {
        std::fill(avail.begin(), avail.end(), 1);
        for (int s = 0; s < 2; ++s)
            for (int o : inc[edges[2 * e + s]])
                if (o != e && color[o] != -1) avail[color[o]] = 0;
        int c = 0;
        for (int k = 0; k < max_colors; ++k) if (avail[k]) { c = k; break; }
        color[e] = c;
    }
    std::fill(prefix, prefix + max_colors, 0);
    for (int e = 0; e < E; ++e) prefix[color[e]] += 1;
    for (int i = 1; i < max_colors; ++i) prefix[i] += prefix[i - 1];
    for (int i = E - 1; i >= 0; --i) {
        int c = color[i];
        prefix[c] -= 1;
        sorted_edges[prefix[c]] = i;
    }
    return 0;
}

// Colour-ordered Gauss-Seidel sweep (the consumer the reference's colouring is
// for, README.md:20-22; its solver has only the Jacobi sweep): serially over
// colours and, within a colour, over cons in order.  cons[i] = {v0, v1 | bit 31
// for a bending pair, bits(l0), id}.  The projection is the stretch step of
// XPBD.py:141-164 evaluated on the current positions, applied at once to both
// endpoints: y0 -= (w0*ld)*n, y1 += (w1*ld)*n with w = y4[.].w.
API int or_gs_sweep(int n_colors, const int32_t* colour_start, const int32_t* cons, float* y4, float k_spring,
                    float k_bend) {
    for (int c = 0; c < n_colors; ++c) {
        for (int i = colour_start[c]; i < colour_start[c + 1]; ++i) {
            const int32_t* q = cons + 4 * (size_t)i;
            const int v0 = q[0];
            const int v1 = (int)((uint32_t)q[1] & 0x7fffffffu);
            const float k = q[1] < 0 ? k_bend : k_spring;
            float rest;
            std::memcpy(&rest, &q[2], 4);
            float* p0 = y4 + 4 * (size_t)v0;
            float* p1 = y4 + 4 * (size_t)v1;
            V3 x10 = sub(v3(p0), v3(p1));
            float lij = std::sqrt(dot(x10, x10));
            float C = lij - rest;
            float inv = 1.0f / lij;
            V3 n = scale(inv, x10);
            float schur = (p0[3] + p1[3]) * dot(n, n);
            float ld = (k * C) / (k * schur + 1.0f);
            V3 a = sub(v3(p0), scale(p0[3] * ld, n));
            V3 b = add(v3(p1), scale(p1[3] * ld, n));
            p0[0] = a.x; p0[1] = a.y; p0[2] = a.z;
            p1[0] = b.x; p1[1] = b.y; p1[2] = b.z;
        }
    }
    return 0;
}

API int or_version(void) { return 1; }
