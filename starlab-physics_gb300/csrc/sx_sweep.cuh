// One vertex of the Jacobi spring / bending sweep (XPBD.py:141-184 +
// :384-387), shared by the grid-wide sweep kernel and the persistent batched
// substep kernel so that both evaluate the same expressions in the same order.
//
// For a constraint (v0, v1) the reference computes x10 = p0 - p1,
// n = x10 * (1/|x10|), ld = k*C/(k*(w0+w1)*(n.n) + 1) and scatters
// dx0 -= (w0*ld)*n, dx1 += (w1*ld)*n with float atomics.  From v1's side
// p1 - p0 = -x10 exactly, so n flips sign exactly and
// dx1 - (w1*ld)*(-n) == dx1 + (w1*ld)*n bit for bit: every vertex evaluates
// dx -= (w_self*ld) * normalize(p_self - p_other) over its incident constraints
// in ascending constraint index, which equals a serial run of the reference.
//
// G: entries whose loads are issued together.  BY: bending pairs on y (the
// bend_y argument is then ignored).  FAST: fused multiply-adds, the hardware
// reciprocal square root, a fast divide and n.n taken as 1 (within float
// rounding of the exact form, not bit-identical).  CHECK: also sum C^2 into
// *c2.  YLDG: y is read through the read-only path (it does not change during
// the launch); kernels that write y themselves read it with plain loads.
#pragma once
#include "sx_common.cuh"

namespace sx {

template <bool YLDG>
__device__ __forceinline__ float4 load_y(const float4* p) {
    if (YLDG) return __ldg(p);
    return *p;
}

// Entry sources: entry k of vertex v's list as the adjacency word
// (neighbour | bit 31 for a bending pair, bits(rest length)).
struct AdjInt2 {  // the CSR of int2 entries
    const int2* __restrict__ adj;
    __device__ __forceinline__ int2 operator()(int, int k) const { return __ldg(adj + k); }
};
// The same entries read with the streaming (evict-first) cache policy: each
// entry is read once per sweep, so on a batch larger than L2 the positions,
// which neighbouring vertices gather again, keep their L2 lines.
struct AdjInt2Stream {
    const int2* __restrict__ adj;
    __device__ __forceinline__ int2 operator()(int, int k) const { return __ldcs(adj + k); }
};
// The packed CSR: nbr16[k] = neighbour - v, rest32[k] = bits(rest length) with
// bit 31 set for a bending pair (6 bytes per entry instead of 8), read from a
// shared-memory copy of the block's range [a0, a0 + n) when staged, else from
// global memory.
struct AdjPacked {
    const short* nbr;
    const unsigned* rest;
    int a0;
    __device__ __forceinline__ int2 operator()(int v, int k) const {
        const unsigned r = rest[k - a0];
        return make_int2((v + (int)nbr[k - a0]) | (int)(r & 0x80000000u), (int)(r & 0x7fffffffu));
    }
};

// The packed CSR read from global memory through the read-only path.
struct AdjPackedGlobal {
    const short* __restrict__ nbr;
    const unsigned* __restrict__ rest;
    __device__ __forceinline__ int2 operator()(int v, int k) const {
        const unsigned r = __ldg(rest + k);
        return make_int2((v + (int)__ldg(nbr + k)) | (int)(r & 0x80000000u), (int)(r & 0x7fffffffu));
    }
};

template <int G, bool BY, bool FAST, bool CHECK, bool YLDG, typename Src>
__device__ __forceinline__ float4 sweep_vertex_src(int v, const float4* __restrict__ x4, const float4* yin,
                                                   const float* __restrict__ fixed, int b, int e, const Src& src,
                                                   float ks, float kb, int bend_y, float* c2) {
    const float4 ps = load_y<YLDG>(yin + v), xs = __ldg(x4 + v);
    float dx = 0.0f, dy = 0.0f, dz = 0.0f;
    for (int k0 = b; k0 < e; k0 += G) {
        int2 a[G];
        float4 o[G];
#pragma unroll
        for (int g = 0; g < G; ++g) a[g] = k0 + g < e ? src(v, k0 + g) : make_int2(0, 0);
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const bool use_x = !BY && a[g].x < 0 && !bend_y;
            const int u = a[g].x & 0x7fffffff;
            o[g] = k0 + g < e ? (use_x ? __ldg(x4 + u) : load_y<YLDG>(yin + u)) : ps;
        }
#pragma unroll
        for (int g = 0; g < G; ++g) {
            if (k0 + g >= e) break;
            const bool bend = a[g].x < 0;
            const float rest = __int_as_float(a[g].y);
            const bool use_x = !BY && bend && !bend_y;
            const float4 self = use_x ? xs : ps;
            const float kk = bend ? kb : ks;
            const float ex = self.x - o[g].x, ey = self.y - o[g].y, ez = self.z - o[g].z;
            if (FAST) {
                const float d2 = __fmaf_rn(ex, ex, __fmaf_rn(ey, ey, ez * ez));
                const float inv = rsqrtf(d2);
                const float C = d2 * inv - rest;
                if (CHECK) *c2 = __fmaf_rn(C, C, *c2);
                const float ld = __fdividef(kk * C, __fmaf_rn(kk, self.w + o[g].w, 1.0f));
                const float a0 = (self.w * ld) * inv;  // times the unnormalised difference
                dx = __fmaf_rn(-a0, ex, dx);
                dy = __fmaf_rn(-a0, ey, dy);
                dz = __fmaf_rn(-a0, ez, dz);
            } else {
                const float lij = sqrtf((ex * ex + ey * ey) + ez * ez);
                const float C = lij - rest;
                if (CHECK) *c2 = *c2 + C * C;
                const float inv = 1.0f / lij;
                const float nx = inv * ex, ny = inv * ey, nz = inv * ez;
                const float schur = (self.w + o[g].w) * ((nx * nx + ny * ny) + nz * nz);
                const float ld = (kk * C) / (kk * schur + 1.0f);
                const float a0 = self.w * ld;
                dx = dx - a0 * nx;
                dy = dy - a0 * ny;
                dz = dz - a0 * nz;
            }
        }
    }
    float4 out = ps;
    const float nc = (float)(e - b);
    if (nc > 0.0f) {
        const float f = fixed[v];
        if (FAST) {
            const float fs = __fdividef(f, nc);
            out.x = __fmaf_rn(fs, dx, ps.x);
            out.y = __fmaf_rn(fs, dy, ps.y);
            out.z = __fmaf_rn(fs, dz, ps.z);
        } else {
            out.x = ps.x + f * (dx / nc);
            out.y = ps.y + f * (dy / nc);
            out.z = ps.z + f * (dz / nc);
        }
    }
    return out;
}

// The same vertex evaluated by L consecutive lanes of a warp (L = 2, 4 or 8).
// Lane j of the group evaluates entries b + j, b + j + L, ... (G of them per
// batch, loads issued together), and the group then adds the terms in
// ascending entry order, each lane receiving every term through shuffles, so
// each lane holds exactly the sums of sweep_vertex_src (same operations, same
// order).  A mesh with few vertices per SM keeps L times more loads in flight.
// Every lane of the warp must call it (a lane past the last vertex passes
// valid == false and b == e); the trip count is the warp's largest.
template <int L, int G, bool BY, bool FAST, bool YLDG>
__device__ __forceinline__ float4 sweep_vertex_lanes(int v, bool valid, const float4* __restrict__ x4,
                                                     const float4* yin, const float* __restrict__ fixed, int b, int e,
                                                     const int2* __restrict__ adj, float ks, float kb, int bend_y) {
    static_assert(L == 2 || L == 4 || L == 8, "lanes per vertex: 2, 4 or 8");
    const int sub = threadIdx.x & (L - 1);
    const float4 ps = valid ? load_y<YLDG>(yin + v) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 xs = valid && e > b ? __ldg(x4 + v) : ps;
    float dx = 0.0f, dy = 0.0f, dz = 0.0f;
    constexpr int SPAN = G * L;
    const int steps = __reduce_max_sync(0xffffffffu, (e - b + SPAN - 1) / SPAN);
    for (int st = 0; st < steps; ++st) {
        const int k0 = b + st * SPAN;
        int2 a[G];
        float4 o[G];
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const int k = k0 + g * L + sub;
            a[g] = k < e ? __ldg(adj + k) : make_int2(0, 0);
        }
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const int k = k0 + g * L + sub;
            const bool use_x = !BY && a[g].x < 0 && !bend_y;
            const int u = a[g].x & 0x7fffffff;
            o[g] = k < e ? (use_x ? __ldg(x4 + u) : load_y<YLDG>(yin + u)) : ps;
        }
        // per entry: exact form (a0 nx, a0 ny, a0 nz); fast form (a0, ex, ey, ez)
        float t0[G], t1[G], t2[G], t3[G];
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const bool bend = a[g].x < 0;
            const float rest = __int_as_float(a[g].y);
            const bool use_x = !BY && bend && !bend_y;
            const float4 self = use_x ? xs : ps;
            const float kk = bend ? kb : ks;
            const float ex = self.x - o[g].x, ey = self.y - o[g].y, ez = self.z - o[g].z;
            if (FAST) {
                const float d2 = __fmaf_rn(ex, ex, __fmaf_rn(ey, ey, ez * ez));
                const float inv = rsqrtf(d2);
                const float C = d2 * inv - rest;
                const float ld = __fdividef(kk * C, __fmaf_rn(kk, self.w + o[g].w, 1.0f));
                t0[g] = (self.w * ld) * inv;
                t1[g] = ex;
                t2[g] = ey;
                t3[g] = ez;
            } else {
                const float lij = sqrtf((ex * ex + ey * ey) + ez * ez);
                const float C = lij - rest;
                const float inv = 1.0f / lij;
                const float nx = inv * ex, ny = inv * ey, nz = inv * ez;
                const float schur = (self.w + o[g].w) * ((nx * nx + ny * ny) + nz * nz);
                const float ld = (kk * C) / (kk * schur + 1.0f);
                const float a0 = self.w * ld;
                t0[g] = a0 * nx;
                t1[g] = a0 * ny;
                t2[g] = a0 * nz;
                t3[g] = 0.0f;
            }
        }
#pragma unroll
        for (int g = 0; g < G; ++g) {
#pragma unroll
            for (int j = 0; j < L; ++j) {
                const int k = k0 + g * L + j;  // the same for every lane of the group
                const float q0 = __shfl_sync(0xffffffffu, t0[g], j, L);
                const float q1 = __shfl_sync(0xffffffffu, t1[g], j, L);
                const float q2 = __shfl_sync(0xffffffffu, t2[g], j, L);
                if (FAST) {
                    const float q3 = __shfl_sync(0xffffffffu, t3[g], j, L);
                    if (k < e) {
                        dx = __fmaf_rn(-q0, q1, dx);
                        dy = __fmaf_rn(-q0, q2, dy);
                        dz = __fmaf_rn(-q0, q3, dz);
                    }
                } else if (k < e) {
                    dx = dx - q0;
                    dy = dy - q1;
                    dz = dz - q2;
                }
            }
        }
    }
    float4 out = ps;
    const float nc = (float)(e - b);
    if (nc > 0.0f) {
        const float f = fixed[v];
        if (FAST) {
            const float fs = __fdividef(f, nc);
            out.x = __fmaf_rn(fs, dx, ps.x);
            out.y = __fmaf_rn(fs, dy, ps.y);
            out.z = __fmaf_rn(fs, dz, ps.z);
        } else {
            out.x = ps.x + f * (dx / nc);
            out.y = ps.y + f * (dy / nc);
            out.z = ps.z + f * (dz / nc);
        }
    }
    return out;
}

template <int G, bool BY, bool FAST, bool CHECK, bool YLDG>
__device__ __forceinline__ float4 sweep_vertex(int v, const float4* __restrict__ x4, const float4* yin,
                                               const float* __restrict__ fixed, const int* __restrict__ ptr,
                                               const int2* __restrict__ adj, float ks, float kb, int bend_y,
                                               float* c2) {
    return sweep_vertex_src<G, BY, FAST, CHECK, YLDG>(v, x4, yin, fixed, __ldg(ptr + v), __ldg(ptr + v + 1),
                                                      AdjInt2{adj}, ks, kb, bend_y, c2);
}

}  // namespace sx
