// Cloth state kernels: predict, Jacobi spring/bending sweep, velocity + position
// update, face AABBs and scene AABB.  Reference: framework/physics/XPBD.py and
// framework/meshio/meshTaichiWrapper.py.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "sx_common.cuh"
#include "sx_sweep.cuh"

namespace sx {

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

static int g_pdl = 1;
static thread_local int g_pdl_suspend = 0;  // > 0 while a device-side loop body is recorded
bool pdl_enabled() { return g_pdl != 0 && g_pdl_suspend == 0; }
}  // namespace sx
extern "C" int sx_set_programmatic_launch(int enable) {
    const int prev = sx::g_pdl;
    sx::g_pdl = enable ? 1 : 0;
    return prev;
}
namespace sx {

int resident_blocks_of(const void* kernel, int block) {
    static std::mutex mu;
    static const void* keys[64];
    static int vals[64];
    static int n = 0;
    std::lock_guard<std::mutex> lock(mu);
    for (int i = 0; i < n; ++i)
        if (keys[i] == kernel) return vals[i];
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess || per_sm < 1)
        return 1024;
    if (n < 64) {
        keys[n] = kernel;
        vals[n] = sms * per_sm;
        ++n;
    }
    return sms * per_sm;
}

void set_error(const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

int cuda_status(cudaError_t e, const char* what) {
    set_error("%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
    return SX_ERR_CUDA;
}

int check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e, what);
    return SX_OK;
}

// ---------------------------------------------------------------------------
// compute_y (XPBD.py:116-118)
// ---------------------------------------------------------------------------
__global__ void predict_kernel(int V, const float4* __restrict__ x4, const float4* __restrict__ v4,
                               const float* __restrict__ fixed, float4* __restrict__ y4, float dt, float gx,
                               float gy, float gz) {
    pdl_entry();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    float4 x = x4[i], v = v4[i];
    float f = fixed[i];
    float4 y;
    y.x = (x.x + (f * v.x) * dt) + (gx * dt) * dt;
    y.y = (x.y + (f * v.y) * dt) + (gy * dt) * dt;
    y.z = (x.z + (f * v.z) * dt) + (gz * dt) * dt;
    y.w = x.w;
    y4[i] = y;
}

// ---------------------------------------------------------------------------
// One Jacobi sweep (XPBD.py:141-184 + :384-387), gathered per vertex
// (sweep_vertex, sx_sweep.cuh, states why the gather equals a serial run of
// the reference's scatter).
// ---------------------------------------------------------------------------
constexpr int SW_BLOCK = 256;  // one vertex per thread
inline int sweep_blocks(int n_verts) { return grid_for(n_verts, SW_BLOCK); }

// ---------------------------------------------------------------------------
// Residual reduction shared by the checked sweep and sx_constraint_residual.
// Each thread holds its vertex's float sum of C^2 over its entries in
// ascending order; the warp value is the xor tree over its 32 vertices (IEEE
// addition is commutative, so every lane ends with the same value), the block
// value ((w0 + w1) + (w2 + w3)) + ((w4 + w5) + (w6 + w7)) over the 8 warps,
// all in float; the block values are then summed in FP64 by
// residual_finish_kernel.  The CPU oracle reproduces this order exactly.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void block_residual_partial(float c2, double* __restrict__ partial, int tile) {
    __shared__ float wsum[SW_BLOCK / 32];
    float w = c2;
    for (int o = 16; o > 0; o >>= 1) w = w + __shfl_xor_sync(0xffffffffu, w, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = w;
    __syncthreads();
    if (threadIdx.x == 0)
        partial[tile] =
            (double)(((wsum[0] + wsum[1]) + (wsum[2] + wsum[3])) + ((wsum[4] + wsum[5]) + (wsum[6] + wsum[7])));
    __syncthreads();  // wsum is reused by the block's next tile
}

// Kernels over vertex tiles of SW_BLOCK: a block walks tiles blockIdx.x,
// blockIdx.x + gridDim.x, ...  Per-tile results (residual partials) do not
// depend on the grid size.  Gated launches (whose iteration may be skipped by
// the convergence control) cap the grid at one resident wave (tile_grid), so a
// skipped launch costs one short wave; other launches give every tile a block.
template <typename K>
inline int tile_grid(K kernel, int n_verts) {
    const int tiles = sweep_blocks(n_verts);
    const int cap = resident_blocks(kernel, SW_BLOCK);
    return tiles < cap ? tiles : cap;
}

// One vertex per thread.  Entries are taken two at a time with both adjacency
// loads and then both neighbour loads issued before the arithmetic, which keeps
// several independent gathers in flight per thread.
// G: entries whose loads are issued together; BLOCK: threads (= vertices) per
// tile.  Every (G, BLOCK) gives the same result; the residual partials of
// CHECK assume BLOCK == SW_BLOCK.
// BY: bending pairs evaluated on y, fixed at compile time (the bend_y
// argument is then ignored), which drops the per-entry x/y selection.
// FAST: the same constraint projection with fused multiply-adds, the
// hardware reciprocal square root for the length and normal, a fast divide
// for the multiplier, and n.n taken as 1 (n is a unit vector up to rounding):
// fewer instructions per entry, results within float rounding of the exact
// form but not bit-identical to it; validated against the oracle at the
// position and residual tolerance of the substep instead.
// STREAM: adjacency entries read with the evict-first policy (AdjInt2Stream).
template <bool CHECK, int G = 2, int BLOCK = SW_BLOCK, bool BY = false, bool FAST = false, bool STREAM = false>
__global__ void __launch_bounds__(BLOCK) jacobi_sweep_kernel(int V, const float4* __restrict__ x4,
                                                                const float4* __restrict__ yin,
                                                                float4* __restrict__ yout,
                                                                const float* __restrict__ fixed,
                                                                const int* __restrict__ ptr,
                                                                const int2* __restrict__ adj, float ks, float kb,
                                                                int bend_y, const int* conv, int iter,
                                                                double* __restrict__ partial) {
    pdl_entry();
    if (iteration_skipped(conv, iter)) return;  // grid-uniform
    static_assert(!CHECK || BLOCK == SW_BLOCK, "residual partials are per SW_BLOCK tile");
    const int ntiles = (V + BLOCK - 1) / BLOCK;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int v = tile * BLOCK + threadIdx.x;
    float c2 = 0.0f;  // sum of C^2 over this vertex's entries (CHECK)
    if (v < V) {
        if (STREAM)
            yout[v] = sweep_vertex_src<G, BY, FAST, CHECK, true>(v, x4, yin, fixed, __ldg(ptr + v), __ldg(ptr + v + 1),
                                                                 AdjInt2Stream{adj}, ks, kb, bend_y, &c2);
        else
            yout[v] = sweep_vertex<G, BY, FAST, CHECK, true>(v, x4, yin, fixed, ptr, adj, ks, kb, bend_y, &c2);
    }
    if (CHECK) block_residual_partial(c2, partial, tile);
    }
}

// L lanes per vertex (sweep_vertex_lanes): for meshes whose vertices alone
// leave the SMs short of warps (65 536 vertices are 13 warps per SM), L times
// the threads and a shorter chain of dependent loads per thread; the same
// sums in the same order, so bit-identical to jacobi_sweep_kernel.
template <int L, int G, int BLOCK, bool BY = false, bool FAST = false>
__global__ void __launch_bounds__(BLOCK) jacobi_sweep_lanes_kernel(int V, const float4* __restrict__ x4,
                                                                      const float4* __restrict__ yin,
                                                                      float4* __restrict__ yout,
                                                                      const float* __restrict__ fixed,
                                                                      const int* __restrict__ ptr,
                                                                      const int2* __restrict__ adj, float ks,
                                                                      float kb, int bend_y, const int* conv, int iter,
                                                                      double* __restrict__ partial) {
    pdl_entry();
    if (iteration_skipped(conv, iter)) return;  // grid-uniform
    const long long t = (long long)blockIdx.x * BLOCK + threadIdx.x;
    const int v = (int)(t / L);
    const bool valid = v < V;
    int b = 0, e = 0;
    if (valid) {
        b = __ldg(ptr + v);
        e = __ldg(ptr + v + 1);
    }
    const float4 out = sweep_vertex_lanes<L, G, BY, FAST, true>(v, valid, x4, yin, fixed, b, e, adj, ks, kb, bend_y);
    if (valid && (threadIdx.x & (L - 1)) == 0) yout[v] = out;
}

// ---------------------------------------------------------------------------
// Sewing (solve_sewing_constraints_x, XPBD.py:425-441, + update_dx): zero-rest
// distance constraints between vertex pairs, C = |y_b - y_a|,
// n = normalize(y_a - y_b), schur = f_a w_a + f_b w_b, ld = k C / (k schur + 1),
// dx_a -= f_a w_a ld n, dx_b += f_b w_b ld n.  Gathered per sewn vertex over its
// partners in ascending pair index (from b's side n flips sign exactly), then
// y += fixed dx / nc.  Coincident vertices (C = 0) contribute nothing, where
// the reference's normalize would give NaN.  The reference's call is
// commented out (XPBD.py:371-372); here it runs after the contact update of
// every Jacobi iteration, where that comment places it.
// ---------------------------------------------------------------------------
__global__ void sewing_gather_kernel(int n_sewn, const int* __restrict__ sewn, const int* __restrict__ sptr,
                                     const int* __restrict__ partner, const float4* __restrict__ y4,
                                     const float* __restrict__ fixed, float k, float4* __restrict__ out) {
    pdl_entry();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_sewn) return;
    const int v = sewn[i];
    const float4 ps = y4[v];
    float dx = 0.0f, dy = 0.0f, dz = 0.0f;
    const int b = sptr[i], e = sptr[i + 1];
    for (int j = b; j < e; ++j) {
        const float4 o = y4[partner[j]];
        const float ex = ps.x - o.x, ey = ps.y - o.y, ez = ps.z - o.z;
        const float C = sqrtf((ex * ex + ey * ey) + ez * ez);
        if (C > 0.0f) {
            const float inv = 1.0f / C;
            const float nx = inv * ex, ny = inv * ey, nz = inv * ez;
            const float ld = (k * C) / (k * (ps.w + o.w) + 1.0f);
            const float a0 = ps.w * ld;
            dx = dx - a0 * nx;
            dy = dy - a0 * ny;
            dz = dz - a0 * nz;
        }
    }
    float4 r = ps;
    const float nc = (float)(e - b);
    if (nc > 0.0f) {
        const float f = fixed[v];
        r.x = ps.x + f * (dx / nc);
        r.y = ps.y + f * (dy / nc);
        r.z = ps.z + f * (dz / nc);
    }
    out[i] = r;
}

__global__ void sewing_scatter_kernel(int n_sewn, const int* __restrict__ sewn, const float4* __restrict__ out,
                                      float4* __restrict__ y4) {
    pdl_entry();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_sewn) y4[sewn[i]] = out[i];
}

// ---------------------------------------------------------------------------
// compute_velocity + update_x (XPBD.py:341-343, :333-337)
// ---------------------------------------------------------------------------
__global__ void velocity_update_kernel(int V, float4* __restrict__ x4, const float4* __restrict__ y4,
                                       float4* __restrict__ v4, const float* __restrict__ fixed, float damping,
                                       float dt) {
    pdl_entry();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    float4 x = x4[i], y = y4[i];
    float s = (1.0f - damping) * fixed[i];
    float4 v;
    v.x = (s * (y.x - x.x)) / dt;
    v.y = (s * (y.y - x.y)) / dt;
    v.z = (s * (y.z - x.z)) / dt;
    v.w = 0.0f;
    v4[i] = v;
    x.x = x.x + dt * v.x;
    x.y = x.y + dt * v.y;
    x.z = x.z + dt * v.z;
    x4[i] = x;
}

// compute_velocity alone (XPBD.py:341-343) and update_x alone (:333-337), for
// substeps with the velocity-level contact pass between them; the same
// arithmetic as velocity_update_kernel.
__global__ void compute_velocity_kernel(int V, const float4* __restrict__ x4, const float4* __restrict__ y4,
                                        float4* __restrict__ v4, const float* __restrict__ fixed, float damping,
                                        float dt) {
    pdl_entry();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    float4 x = x4[i], y = y4[i];
    float s = (1.0f - damping) * fixed[i];
    v4[i] = make_float4((s * (y.x - x.x)) / dt, (s * (y.y - x.y)) / dt, (s * (y.z - x.z)) / dt, 0.0f);
}

__global__ void update_x_kernel(int V, float4* __restrict__ x4, const float4* __restrict__ v4, float dt) {
    pdl_entry();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    float4 x = x4[i], v = v4[i];
    x.x = x.x + dt * v.x;
    x.y = x.y + dt * v.y;
    x.z = x.z + dt * v.z;
    x4[i] = x;
}

// ---------------------------------------------------------------------------
// computeAABB_faces (meshTaichiWrapper.py:351-365)
// ---------------------------------------------------------------------------
// cmn4/cmx4 (optional): the union of the padded boxes of faces 32c .. 32c+31
// (chunk c), for broad phases that test chunks before faces
__global__ void face_aabb_kernel(int F, const float4* __restrict__ p4, const int* __restrict__ faces, float pad,
                                 float4* __restrict__ mn4, float4* __restrict__ mx4, float4* __restrict__ cmn4,
                                 float4* __restrict__ cmx4) {
    pdl_entry();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    V3 lo{INFINITY, INFINITY, INFINITY}, hi{-INFINITY, -INFINITY, -INFINITY};
    if (f < F) {
        const V3 a = mk(p4[faces[3 * f]]), b = mk(p4[faces[3 * f + 1]]), c = mk(p4[faces[3 * f + 2]]);
        const V3 l = vmin(vmin(a, b), c), h = vmax(vmax(a, b), c);
        lo = V3{l.x - pad, l.y - pad, l.z - pad};
        hi = V3{h.x + pad, h.y + pad, h.z + pad};
        mn4[f] = make_float4(lo.x, lo.y, lo.z, 0.0f);
        mx4[f] = make_float4(hi.x, hi.y, hi.z, 0.0f);
    }
    if (cmn4 != nullptr) {  // block size is a multiple of 32: warp w of the grid is chunk w
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo = vmin(lo, V3{__shfl_xor_sync(0xffffffffu, lo.x, o), __shfl_xor_sync(0xffffffffu, lo.y, o),
                             __shfl_xor_sync(0xffffffffu, lo.z, o)});
            hi = vmax(hi, V3{__shfl_xor_sync(0xffffffffu, hi.x, o), __shfl_xor_sync(0xffffffffu, hi.y, o),
                             __shfl_xor_sync(0xffffffffu, hi.z, o)});
        }
        const int chunk = f >> 5;
        if ((threadIdx.x & 31) == 0 && 32 * chunk < F) {
            cmn4[chunk] = make_float4(lo.x, lo.y, lo.z, 0.0f);
            cmx4[chunk] = make_float4(hi.x, hi.y, hi.z, 0.0f);
        }
    }
}

// ---------------------------------------------------------------------------
// computeAABB (meshTaichiWrapper.py:335-347).  Min/max are exact, so an atomic
// reduction on order-preserving integer images of the floats is deterministic.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned f2ord(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__global__ void scene_aabb_init(unsigned* box) {
    pdl_entry();
    int t = threadIdx.x;
    if (t < 3) box[t] = f2ord(1e5f);
    else if (t < 6) box[t] = f2ord(-1e5f);
}

// Per block: four loads in flight per thread, warp shuffles, then the block's
// warps combine in shared memory and one thread issues the six atomics (min
// and max are exact, so the order does not matter).
__global__ void __launch_bounds__(256) scene_aabb_reduce(int V, const float4* __restrict__ p4, unsigned* box) {
    pdl_entry();
    float lo[3] = {1e5f, 1e5f, 1e5f}, hi[3] = {-1e5f, -1e5f, -1e5f};
    const int stride = gridDim.x * blockDim.x;
    auto take = [&](float4 p) {
        lo[0] = fminf(lo[0], p.x); lo[1] = fminf(lo[1], p.y); lo[2] = fminf(lo[2], p.z);
        hi[0] = fmaxf(hi[0], p.x); hi[1] = fmaxf(hi[1], p.y); hi[2] = fmaxf(hi[2], p.z);
    };
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < V; i += 4 * stride) {
        const float4 a = p4[i], b = p4[i + stride], c = p4[i + 2 * stride], d = p4[i + 3 * stride];
        take(a);
        take(b);
        take(c);
        take(d);
    }
    for (; i < V; i += stride) take(p4[i]);
    for (int o = 16; o > 0; o >>= 1) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    }
    __shared__ float red[8][6];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; ++k) {
            red[w][k] = lo[k];
            red[w][3 + k] = hi[k];
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        float v = red[0][k];
        for (int j = 1; j < (int)(blockDim.x >> 5); ++j) v = k < 3 ? fminf(v, red[j][k]) : fmaxf(v, red[j][k]);
        if (k < 3) atomicMin(box + k, f2ord(v));
        else atomicMax(box + k, f2ord(v));
    }
}

__global__ void scene_aabb_finish(unsigned* box, float pad) {
    pdl_entry();
    int t = threadIdx.x;
    if (t < 6) {
        float v = ord2f(box[t]);
        reinterpret_cast<float*>(box)[t] = t < 3 ? v - pad : v + pad;
    }
}

}  // namespace sx

using namespace sx;

extern "C" int sx_version(void) { return 1; }
extern "C" const char* sx_last_error(void) { return g_last_error.c_str(); }
extern "C" long long sx_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" int sx_predict(const float* x4, const float* v4, const float* fixed, float* y4, int n_verts, float dt,
                          float gx, float gy, float gz, void* stream) {
    SX_REQUIRE(n_verts >= 0, "sx_predict: n_verts < 0");
    if (n_verts == 0) return SX_OK;
    SX_REQUIRE(x4 && v4 && fixed && y4, "sx_predict: null pointer");
    launch(predict_kernel, grid_for(n_verts, 256), 256, 0, as_stream(stream), 
        n_verts, (const float4*)x4, (const float4*)v4, fixed, (float4*)y4, dt, gx, gy, gz);
    return check_launch("predict_kernel");
}

extern "C" int sx_jacobi_sweep(const float* x4, const float* y_in4, float* y_out4, const float* fixed,
                               const int* adj_ptr, const int* adj, int n_verts, float k_spring, float k_bend,
                               int bend_on_y, void* stream) {
    SX_REQUIRE(n_verts >= 0, "sx_jacobi_sweep: n_verts < 0");
    if (n_verts == 0) return SX_OK;
    SX_REQUIRE(x4 && y_in4 && y_out4 && fixed && adj_ptr && adj, "sx_jacobi_sweep: null pointer");
    SX_REQUIRE(y_in4 != y_out4, "sx_jacobi_sweep: y_in4 and y_out4 must not alias");
    launch(bend_on_y ? jacobi_sweep_kernel<false, 2, SW_BLOCK, true> : jacobi_sweep_kernel<false>, sweep_blocks(n_verts),
           SW_BLOCK, 0, as_stream(stream), n_verts, (const float4*)x4, (const float4*)y_in4, (float4*)y_out4, fixed,
           adj_ptr, (const int2*)adj, k_spring, k_bend, bend_on_y ? 1 : 0, (const int*)nullptr, 0, (double*)nullptr);
    return check_launch("jacobi_sweep_kernel");
}

// Launch configurations of the sweep for the autotuner: entries per load
// batch, threads per block, lanes per vertex, and whether the adjacency is
// read with the streaming cache policy.  All give bit-identical results.
namespace sx {
using SweepKernel = void (*)(int, const float4*, const float4*, float4*, const float*, const int*, const int2*, float,
                            float, int, const int*, int, double*);
struct SweepVariant {
    int g, block, lanes, stream;
    SweepKernel kern, kern_y;  // bending on x or y chosen at run time / bending on y
    SweepKernel fast, fast_y;  // the FAST arithmetic
};
#define SX_SWEEP_VARIANT(G, B)                                                                                  \
    {G, B, 1, 0, jacobi_sweep_kernel<false, G, B>, jacobi_sweep_kernel<false, G, B, true>,                     \
     jacobi_sweep_kernel<false, G, B, false, true>, jacobi_sweep_kernel<false, G, B, true, true>}
#define SX_SWEEP_LANES(L, G, B)                                                                                 \
    {G, B, L, 0, jacobi_sweep_lanes_kernel<L, G, B>, jacobi_sweep_lanes_kernel<L, G, B, true>,                 \
     jacobi_sweep_lanes_kernel<L, G, B, false, true>, jacobi_sweep_lanes_kernel<L, G, B, true, true>}
#define SX_SWEEP_STREAM(G, B)                                                                                   \
    {G, B, 1, 1, jacobi_sweep_kernel<false, G, B, false, false, true>,                                         \
     jacobi_sweep_kernel<false, G, B, true, false, true>, jacobi_sweep_kernel<false, G, B, false, true, true>,   \
     jacobi_sweep_kernel<false, G, B, true, true, true>}
static const SweepVariant kSweepVariants[] = {
    SX_SWEEP_VARIANT(2, 256), SX_SWEEP_VARIANT(1, 256), SX_SWEEP_VARIANT(4, 256), SX_SWEEP_VARIANT(2, 128),
    SX_SWEEP_VARIANT(2, 512), SX_SWEEP_VARIANT(4, 128), SX_SWEEP_VARIANT(1, 128), SX_SWEEP_VARIANT(3, 256),
    SX_SWEEP_LANES(2, 2, 256), SX_SWEEP_LANES(2, 3, 256), SX_SWEEP_LANES(4, 1, 256), SX_SWEEP_LANES(4, 2, 256),
    SX_SWEEP_LANES(4, 3, 256), SX_SWEEP_LANES(8, 1, 256), SX_SWEEP_LANES(8, 2, 256),
    SX_SWEEP_STREAM(2, 128), SX_SWEEP_STREAM(3, 256), SX_SWEEP_STREAM(2, 256),
};
#undef SX_SWEEP_VARIANT
#undef SX_SWEEP_LANES
#undef SX_SWEEP_STREAM
constexpr int kNumSweepVariants = sizeof(kSweepVariants) / sizeof(kSweepVariants[0]);
}  // namespace sx

extern "C" int sx_jacobi_sweep_variants(void) { return kNumSweepVariants; }

extern "C" int sx_jacobi_sweep_variant_info(int variant, int* g, int* block) {
    SX_REQUIRE(variant >= 0 && variant < kNumSweepVariants && g && block, "sx_jacobi_sweep_variant_info: bad variant");
    *g = kSweepVariants[variant].g;
    *block = kSweepVariants[variant].block;
    return SX_OK;
}

extern "C" int sx_jacobi_sweep_variant_form(int variant, int* lanes, int* streaming) {
    SX_REQUIRE(variant >= 0 && variant < kNumSweepVariants && lanes && streaming,
               "sx_jacobi_sweep_variant_form: bad variant");
    *lanes = kSweepVariants[variant].lanes;
    *streaming = kSweepVariants[variant].stream;
    return SX_OK;
}

extern "C" int sx_jacobi_sweep_v(const float* x4, const float* y_in4, float* y_out4, const float* fixed,
                                 const int* adj_ptr, const int* adj, int n_verts, float k_spring, float k_bend,
                                 int bend_on_y, int variant, void* stream) {
    return sx_jacobi_sweep_mode(x4, y_in4, y_out4, fixed, adj_ptr, adj, n_verts, k_spring, k_bend, bend_on_y, variant,
                                0, stream);
}

extern "C" int sx_jacobi_sweep_mode(const float* x4, const float* y_in4, float* y_out4, const float* fixed,
                                    const int* adj_ptr, const int* adj, int n_verts, float k_spring, float k_bend,
                                    int bend_on_y, int variant, int fast, void* stream) {
    SX_REQUIRE(n_verts >= 0, "sx_jacobi_sweep_v: n_verts < 0");
    SX_REQUIRE(variant >= 0 && variant < kNumSweepVariants, "sx_jacobi_sweep_v: bad variant");
    if (n_verts == 0) return SX_OK;
    SX_REQUIRE(x4 && y_in4 && y_out4 && fixed && adj_ptr && adj, "sx_jacobi_sweep_v: null pointer");
    SX_REQUIRE(y_in4 != y_out4, "sx_jacobi_sweep_v: y_in4 and y_out4 must not alias");
    const SweepVariant& sv = kSweepVariants[variant];
    const SweepKernel k = fast ? (bend_on_y ? sv.fast_y : sv.fast) : (bend_on_y ? sv.kern_y : sv.kern);
    launch(k, grid_for((long long)n_verts * sv.lanes, sv.block), sv.block, 0, as_stream(stream), n_verts, (const float4*)x4,
           (const float4*)y_in4, (float4*)y_out4, fixed, adj_ptr, (const int2*)adj, k_spring, k_bend,
           bend_on_y ? 1 : 0, (const int*)nullptr, 0, (double*)nullptr);
    return check_launch("jacobi_sweep_kernel");
}

// ---------------------------------------------------------------------------
// The sweep over the packed CSR (6 bytes per entry: int16 neighbour offset,
// rest-length bits with the bending flag in bit 31), with the block's range of
// entries staged in shared memory.  A block of BLOCK vertices reads the
// entries [ptr[v0], ptr[v0 + BLOCK]) widened to 16-byte boundaries with
// coalesced 16-byte streaming loads (L2 evict-first, so that the positions,
// which neighbouring blocks gather again, stay in L2), then every thread walks
// its own entries in shared memory.  A block whose range exceeds CAP entries
// reads its entries from global memory instead.  The projection is the same
// code as the int2 sweep (sweep_vertex_src), so results are bit-identical.
namespace sx {
constexpr int kStagedCap = 4096;  // entries per block: 16 KB rest bits + 8 KB offsets

template <int BLOCK, bool BY, bool FAST>
__global__ void __launch_bounds__(BLOCK) jacobi_sweep_staged_kernel(int V, const float4* __restrict__ x4,
                                                                       const float4* __restrict__ yin,
                                                                       float4* __restrict__ yout,
                                                                       const float* __restrict__ fixed,
                                                                       const int* __restrict__ ptr,
                                                                       const short* __restrict__ nbr16,
                                                                       const unsigned* __restrict__ rest32,
                                                                       float ks, float kb, int bend_y) {
    __shared__ __align__(16) unsigned s_rest[kStagedCap];
    __shared__ __align__(16) short s_nbr[kStagedCap];
    pdl_entry();
    const int ntiles = (V + BLOCK - 1) / BLOCK;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int v0 = tile * BLOCK;
        const int v1 = min(v0 + BLOCK, V);
        const int e0 = __ldg(ptr + v0), e1 = __ldg(ptr + v1);
        const int a0 = e0 & ~7, a1 = (e1 + 7) & ~7;  // 8 entries = 16 B of offsets, 32 B of rest bits
        const bool staged = a1 - a0 <= kStagedCap;
        if (staged) {
            const uint4* gr = reinterpret_cast<const uint4*>(rest32 + a0);
            const uint4* gn = reinterpret_cast<const uint4*>(nbr16 + a0);
            uint4* sr = reinterpret_cast<uint4*>(s_rest);
            uint4* sn = reinterpret_cast<uint4*>(s_nbr);
            const int nr = (a1 - a0) >> 2, nn = (a1 - a0) >> 3;
            for (int i = threadIdx.x; i < nr; i += BLOCK) sr[i] = __ldcs(gr + i);
            for (int i = threadIdx.x; i < nn; i += BLOCK) sn[i] = __ldcs(gn + i);
        }
        __syncthreads();
        const int v = v0 + threadIdx.x;
        if (v < V) {
            const int b = __ldg(ptr + v), e = __ldg(ptr + v + 1);
            float c2 = 0.0f;
            yout[v] = staged ? sweep_vertex_src<2, BY, FAST, false, true>(v, x4, yin, fixed, b, e,
                                                                          AdjPacked{s_nbr, s_rest, a0}, ks, kb,
                                                                          bend_y, &c2)
                             : sweep_vertex_src<2, BY, FAST, false, true>(v, x4, yin, fixed, b, e,
                                                                          AdjPacked{nbr16, rest32, 0}, ks, kb,
                                                                          bend_y, &c2);
        }
        __syncthreads();
    }
}

// The packed adjacency read straight from global memory, one vertex per
// thread, G entries' loads issued together: 6 bytes per entry (two loads)
// instead of the int2 entry's 8 and none of the staging's barriers.  Same
// projection code, so bit-identical.
template <int G, int BLOCK, bool BY, bool FAST>
__global__ void __launch_bounds__(BLOCK) jacobi_sweep_packed_kernel(int V, const float4* __restrict__ x4,
                                                                       const float4* __restrict__ yin,
                                                                       float4* __restrict__ yout,
                                                                       const float* __restrict__ fixed,
                                                                       const int* __restrict__ ptr,
                                                                       const short* __restrict__ nbr16,
                                                                       const unsigned* __restrict__ rest32,
                                                                       float ks, float kb, int bend_y) {
    pdl_entry();
    const int v = blockIdx.x * BLOCK + threadIdx.x;
    if (v >= V) return;
    float c2 = 0.0f;
    yout[v] = sweep_vertex_src<G, BY, FAST, false, true>(v, x4, yin, fixed, __ldg(ptr + v), __ldg(ptr + v + 1),
                                                         AdjPackedGlobal{nbr16, rest32}, ks, kb, bend_y, &c2);
}

// Forms of the packed sweep: 0 staged (sx_jacobi_sweep_packed), then the
// direct kernel in several (entries per load batch, threads per block).
using PackedKernel = void (*)(int, const float4*, const float4*, float4*, const float*, const int*, const short*,
                              const unsigned*, float, float, int);
struct PackedForm {
    int g, block;
    PackedKernel kern, kern_y, fast, fast_y;
};
#define SX_PACKED_FORM(G, B)                                                                                    \
    {G, B, jacobi_sweep_packed_kernel<G, B, false, false>, jacobi_sweep_packed_kernel<G, B, true, false>,       \
     jacobi_sweep_packed_kernel<G, B, false, true>, jacobi_sweep_packed_kernel<G, B, true, true>}
static const PackedForm kPackedForms[] = {
    {0, SW_BLOCK, nullptr, nullptr, nullptr, nullptr},  // staged: sx_jacobi_sweep_packed
    SX_PACKED_FORM(4, 256), SX_PACKED_FORM(2, 256), SX_PACKED_FORM(6, 256), SX_PACKED_FORM(4, 128),
    SX_PACKED_FORM(3, 512),
};
#undef SX_PACKED_FORM
constexpr int kNumPackedForms = sizeof(kPackedForms) / sizeof(kPackedForms[0]);
}  // namespace sx

extern "C" int sx_jacobi_sweep_packed(const float* x4, const float* y_in4, float* y_out4, const float* fixed,
                                      const int* adj_ptr, const short* nbr16, const unsigned* rest32, int n_verts,
                                      float k_spring, float k_bend, int bend_on_y, int fast, void* stream) {
    SX_REQUIRE(n_verts >= 0, "sx_jacobi_sweep_packed: n_verts < 0");
    if (n_verts == 0) return SX_OK;
    SX_REQUIRE(x4 && y_in4 && y_out4 && fixed && adj_ptr && nbr16 && rest32, "sx_jacobi_sweep_packed: null pointer");
    SX_REQUIRE(y_in4 != y_out4, "sx_jacobi_sweep_packed: y_in4 and y_out4 must not alias");
    SX_REQUIRE(((uintptr_t)nbr16 & 15) == 0 && ((uintptr_t)rest32 & 15) == 0,
               "sx_jacobi_sweep_packed: nbr16 and rest32 must be 16-byte aligned");
    using K = void (*)(int, const float4*, const float4*, float4*, const float*, const int*, const short*,
                       const unsigned*, float, float, int);
    const K k = fast ? (bend_on_y ? jacobi_sweep_staged_kernel<SW_BLOCK, true, true>
                                  : jacobi_sweep_staged_kernel<SW_BLOCK, false, true>)
                     : (bend_on_y ? jacobi_sweep_staged_kernel<SW_BLOCK, true, false>
                                  : jacobi_sweep_staged_kernel<SW_BLOCK, false, false>);
    launch(k, sweep_blocks(n_verts), SW_BLOCK, 0, as_stream(stream), n_verts, (const float4*)x4,
           (const float4*)y_in4, (float4*)y_out4, fixed, adj_ptr, nbr16, rest32, k_spring, k_bend,
           bend_on_y ? 1 : 0);
    return check_launch("jacobi_sweep_staged_kernel");
}

extern "C" int sx_jacobi_sweep_packed_v(const float* x4, const float* y_in4, float* y_out4, const float* fixed,
                                        const int* adj_ptr, const short* nbr16, const unsigned* rest32, int n_verts,
                                        float k_spring, float k_bend, int bend_on_y, int form, int fast,
                                        void* stream) {
    SX_REQUIRE(form >= 0 && form < kNumPackedForms, "sx_jacobi_sweep_packed_v: bad form");
    if (form == 0)
        return sx_jacobi_sweep_packed(x4, y_in4, y_out4, fixed, adj_ptr, nbr16, rest32, n_verts, k_spring, k_bend,
                                      bend_on_y, fast, stream);
    SX_REQUIRE(n_verts >= 0, "sx_jacobi_sweep_packed_v: n_verts < 0");
    if (n_verts == 0) return SX_OK;
    SX_REQUIRE(x4 && y_in4 && y_out4 && fixed && adj_ptr && nbr16 && rest32, "sx_jacobi_sweep_packed_v: null pointer");
    SX_REQUIRE(y_in4 != y_out4, "sx_jacobi_sweep_packed_v: y_in4 and y_out4 must not alias");
    const PackedForm& pf = kPackedForms[form];
    const PackedKernel k = fast ? (bend_on_y ? pf.fast_y : pf.fast) : (bend_on_y ? pf.kern_y : pf.kern);
    launch(k, grid_for(n_verts, pf.block), pf.block, 0, as_stream(stream), n_verts, (const float4*)x4,
           (const float4*)y_in4, (float4*)y_out4, fixed, adj_ptr, nbr16, rest32, k_spring, k_bend, bend_on_y ? 1 : 0);
    return check_launch("jacobi_sweep_packed_kernel");
}

extern "C" int sx_jacobi_sweep_packed_forms(void) { return kNumPackedForms; }

extern "C" int sx_sewing_sweep(float* y4, const float* fixed, int n_sewn, const int* sewn, const int* sptr,
                               const int* partner, float k, float* scratch4, void* stream) {
    SX_REQUIRE(n_sewn >= 0, "sx_sewing_sweep: n_sewn < 0");
    if (n_sewn == 0) return SX_OK;
    SX_REQUIRE(y4 && fixed && sewn && sptr && partner && scratch4, "sx_sewing_sweep: null pointer");
    cudaStream_t s = as_stream(stream);
    launch(sewing_gather_kernel, grid_for(n_sewn, 256), 256, 0, s, n_sewn, sewn, sptr, partner, (const float4*)y4,
           fixed, k, (float4*)scratch4);
    int rc = check_launch("sewing_gather_kernel");
    if (rc) return rc;
    launch(sewing_scatter_kernel, grid_for(n_sewn, 256), 256, 0, s, n_sewn, sewn, (const float4*)scratch4,
           (float4*)y4);
    return check_launch("sewing_scatter_kernel");
}

extern "C" int sx_velocity_update(float* x4, const float* y4, float* v4, const float* fixed, int n_verts,
                                  float damping, float dt, void* stream) {
    SX_REQUIRE(n_verts >= 0, "sx_velocity_update: n_verts < 0");
    if (n_verts == 0) return SX_OK;
    SX_REQUIRE(x4 && y4 && v4 && fixed, "sx_velocity_update: null pointer");
    launch(velocity_update_kernel, grid_for(n_verts, 256), 256, 0, as_stream(stream), 
        n_verts, (float4*)x4, (const float4*)y4, (float4*)v4, fixed, damping, dt);
    return check_launch("velocity_update_kernel");
}

extern "C" int sx_compute_velocity(const float* x4, const float* y4, float* v4, const float* fixed, int n_verts,
                                   float damping, float dt, void* stream) {
    SX_REQUIRE(n_verts >= 0, "sx_compute_velocity: n_verts < 0");
    if (n_verts == 0) return SX_OK;
    SX_REQUIRE(x4 && y4 && v4 && fixed, "sx_compute_velocity: null pointer");
    launch(compute_velocity_kernel, grid_for(n_verts, 256), 256, 0, as_stream(stream), n_verts, (const float4*)x4,
           (const float4*)y4, (float4*)v4, fixed, damping, dt);
    return check_launch("compute_velocity_kernel");
}

extern "C" int sx_update_x(float* x4, const float* v4, int n_verts, float dt, void* stream) {
    SX_REQUIRE(n_verts >= 0, "sx_update_x: n_verts < 0");
    if (n_verts == 0) return SX_OK;
    SX_REQUIRE(x4 && v4, "sx_update_x: null pointer");
    launch(update_x_kernel, grid_for(n_verts, 256), 256, 0, as_stream(stream), n_verts, (float4*)x4,
           (const float4*)v4, dt);
    return check_launch("update_x_kernel");
}

extern "C" int sx_face_aabbs(const float* p4, const int* faces, int n_faces, float padding, float* aabb_min4,
                             float* aabb_max4, void* stream) {
    SX_REQUIRE(n_faces >= 0, "sx_face_aabbs: n_faces < 0");
    if (n_faces == 0) return SX_OK;
    SX_REQUIRE(p4 && faces && aabb_min4 && aabb_max4, "sx_face_aabbs: null pointer");
    launch(face_aabb_kernel, grid_for(n_faces, 256), 256, 0, as_stream(stream), n_faces, (const float4*)p4, faces,
           padding, (float4*)aabb_min4, (float4*)aabb_max4, (float4*)nullptr, (float4*)nullptr);
    return check_launch("face_aabb_kernel");
}

extern "C" int sx_face_aabbs_chunked(const float* p4, const int* faces, int n_faces, float padding, float* aabb_min4,
                                     float* aabb_max4, float* chunk_min4, float* chunk_max4, void* stream) {
    SX_REQUIRE(n_faces >= 0, "sx_face_aabbs_chunked: n_faces < 0");
    if (n_faces == 0) return SX_OK;
    SX_REQUIRE(p4 && faces && aabb_min4 && aabb_max4 && chunk_min4 && chunk_max4,
               "sx_face_aabbs_chunked: null pointer");
    launch(face_aabb_kernel, grid_for(n_faces, 256), 256, 0, as_stream(stream), n_faces, (const float4*)p4, faces,
           padding, (float4*)aabb_min4, (float4*)aabb_max4, (float4*)chunk_min4, (float4*)chunk_max4);
    return check_launch("face_aabb_kernel");
}

extern "C" int sx_scene_aabb(const float* p4, int n_verts, float padding, float* box6, void* stream) {
    SX_REQUIRE(n_verts >= 0, "sx_scene_aabb: n_verts < 0");
    SX_REQUIRE(box6 && (p4 || n_verts == 0), "sx_scene_aabb: null pointer");
    cudaStream_t s = as_stream(stream);
    unsigned* box = reinterpret_cast<unsigned*>(box6);
    launch(scene_aabb_init, 1, 32, 0, s, box);
    if (n_verts > 0) {
        int g = grid_for(n_verts, 256);
        const int cap = resident_blocks(scene_aabb_reduce, 256);
        if (g > cap) g = cap;
        launch(scene_aabb_reduce, g, 256, 0, s, n_verts, (const float4*)p4, box);
    }
    launch(scene_aabb_finish, 1, 32, 0, s, box, padding);
    return check_launch("scene_aabb");
}

// ---------------------------------------------------------------------------
// Constraint residual.  The reference defines none (XPBD.py:350-369 runs a
// fixed number of sweeps).  Here it is sqrt(sum C^2 / n) over all adjacency
// entries -- every spring and bending pair counted from both endpoints, so the
// mean equals the per-constraint mean -- with C = |p_self - p_other| - l0 in
// float exactly as the sweep evaluates it, per-vertex and per-block sums in
// float (block_residual_partial) and the sum over blocks in FP64.  The checked
// sweep produces the same value for its input positions.
// ---------------------------------------------------------------------------
namespace sx {
constexpr int RF_BLOCKS = 64, RF_THREADS = 256;

__global__ void __launch_bounds__(SW_BLOCK) residual_partial_kernel(int V, const float4* __restrict__ p4,
                                                                 const int* __restrict__ ptr,
                                                                 const int2* __restrict__ adj,
                                                                 double* __restrict__ partial) {
    pdl_entry();
    const int ntiles = (V + SW_BLOCK - 1) / SW_BLOCK;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int v = tile * SW_BLOCK + threadIdx.x;
        float c2 = 0.0f;
        if (v < V) {
            const float4 ps = __ldg(p4 + v);
            const int e = __ldg(ptr + v + 1);
            for (int k = __ldg(ptr + v); k < e; ++k) {
                const int2 a = __ldg(adj + k);
                const float4 o = __ldg(p4 + (a.x & 0x7fffffff));
                const float ex = ps.x - o.x, ey = ps.y - o.y, ez = ps.z - o.z;
                const float C = sqrtf((ex * ex + ey * ey) + ez * ez) - __int_as_float(a.y);
                c2 = c2 + C * C;
            }
        }
        block_residual_partial(c2, partial, tile);
    }
}

// Sums the block values in FP64 (fixed order: strided per thread, xor tree per
// warp, warps in pairs, then the RF_BLOCKS block values in index order by the
// last block to finish).  With conv != nullptr it also records a check:
// conv[2] += 1 and, if the residual is at or below the threshold (tol, or
// tol times the residual ref3 over the same constraints) and no stop
// iteration is set, conv[0] = iter, conv[3] += iter, conv[4] += 1.
__global__ void __launch_bounds__(RF_THREADS) residual_finish_kernel(int nb, const double* __restrict__ partial,
                                                                     double* part2, int* counter,
                                                                     const int* __restrict__ ptr, int V,
                                                                     double* out3, int* conv, int iter,
                                                                     double tol2, const double* ref3,
                                                                     unsigned long long loop, int n_iter) {
    pdl_entry();
    if (iteration_skipped(conv, iter)) return;
    __shared__ double wsum[RF_THREADS / 32];
    __shared__ bool last;
    double acc = 0.0;
    for (int i = blockIdx.x * RF_THREADS + threadIdx.x; i < nb; i += RF_BLOCKS * RF_THREADS) acc += partial[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        part2[blockIdx.x] = ((wsum[0] + wsum[1]) + (wsum[2] + wsum[3])) + ((wsum[4] + wsum[5]) + (wsum[6] + wsum[7]));
        __threadfence();
        last = atomicAdd(counter, 1) == RF_BLOCKS - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    const volatile double* p2 = part2;
    double S = 0.0;
    for (int i = 0; i < RF_BLOCKS; ++i) S += p2[i];
    const double n = V > 0 ? (double)ptr[V] : 0.0;
    out3[0] = S;
    out3[1] = n;
    out3[2] = n > 0.0 ? sqrt(S / n) : 0.0;
    *counter = 0;
    if (conv != nullptr) {
        // inside a device-side loop the iteration of this check is conv[5]
        const int j = loop ? conv[5] : iter;
        conv[2] += 1;
        bool done = false;
        // absolute: rms <= tol; relative to a reference residual ref3: rms <= tol * rms(ref)
        if (conv[0] < 0 && S <= tol2 * (ref3 != nullptr ? ref3[0] : n)) {
            conv[0] = j;
            conv[3] += j;
            conv[4] += 1;
            done = true;
        }
        if (loop) {
            const int next = j + conv[6];
            conv[5] = next;
            cudaGraphSetConditional((cudaGraphConditionalHandle)loop, (done || next >= n_iter) ? 0u : 1u);
        }
    }
}

__global__ void convergence_begin_kernel(int* conv, int check_every, int reset_totals) {
    pdl_entry();
    if (threadIdx.x != 0) return;
    conv[0] = -1;
    conv[2] = 0;
    conv[5] = check_every;  // the first check
    conv[6] = check_every;
    if (reset_totals) {
        conv[3] = 0;
        conv[4] = 0;
    }
}

}  // namespace sx

// partial[sweep_blocks] + part2[RF_BLOCKS] (doubles), then the block counter
extern "C" size_t sx_residual_workspace_bytes(int n_verts) {
    return sizeof(double) * ((size_t)sweep_blocks(n_verts > 0 ? n_verts : 1) + RF_BLOCKS) + 16;
}

static int residual_finish(int n_verts, const int* adj_ptr, void* ws, double* out3, int* conv, int iter, double tol,
                           const double* ref3, unsigned long long loop, int n_iter, cudaStream_t s) {
    const int nb = sweep_blocks(n_verts > 0 ? n_verts : 1);
    double* partial = (double*)ws;
    double* part2 = partial + nb;
    int* counter = (int*)(part2 + RF_BLOCKS);
    launch(residual_finish_kernel, RF_BLOCKS, RF_THREADS, 0, s, nb, (const double*)partial, part2, counter, adj_ptr,
           n_verts, out3, conv, iter, tol * tol, ref3, loop, n_iter);
    return check_launch("residual_finish_kernel");
}

extern "C" int sx_constraint_residual(const float* p4, const int* adj_ptr, const int* adj, int n_verts, double* out3,
                                      void* ws, size_t ws_bytes, void* stream) {
    SX_REQUIRE(n_verts >= 0, "sx_constraint_residual: n_verts < 0");
    SX_REQUIRE(out3 && ws && (n_verts == 0 || (p4 && adj_ptr && adj)), "sx_constraint_residual: null pointer");
    SX_REQUIRE(ws_bytes >= sx_residual_workspace_bytes(n_verts), "sx_constraint_residual: workspace too small");
    cudaStream_t s = as_stream(stream);
    const int nb = sweep_blocks(n_verts > 0 ? n_verts : 1);
    if (n_verts == 0) {
        SX_CUDA(cudaMemsetAsync(ws, 0, sizeof(double) * nb, s));
    } else {
        launch(residual_partial_kernel, tile_grid(residual_partial_kernel, n_verts), SW_BLOCK, 0, s, n_verts,
               (const float4*)p4, adj_ptr,
               (const int2*)adj, (double*)ws);
        int rc = check_launch("residual_partial_kernel");
        if (rc) return rc;
    }
    return residual_finish(n_verts, adj_ptr, ws, out3, nullptr, 0, 0.0, nullptr, 0ull, 0, s);
}

// ---------------------------------------------------------------------------
// System energy in FP64 (no counterpart in the reference): kinetic
// 1/2 sum m |v|^2 and gravitational -sum m (g . x) over vertices with mass
// (m = 1 / m_inv, m_inv > 0), and elastic 1/2 sum k C^2 over the springs and
// bending pairs (C = |p_a - p_b| - l0, every constraint seen from both
// endpoints, so the entries carry 1/4 each; k the spring or the bending
// stiffness).  Every term is evaluated in double from the float positions;
// per-block sums in a fixed order (thread, xor tree over the warp, warps in
// index order), then the blocks in index order by one block: deterministic.
// ---------------------------------------------------------------------------
namespace sx {
constexpr int EN_BLOCK = 256;

__global__ void __launch_bounds__(EN_BLOCK) energy_partial_kernel(int V, const float4* __restrict__ x4,
                                                               const float4* __restrict__ v4,
                                                               const float* __restrict__ m_inv,
                                                               const int* __restrict__ ptr,
                                                               const int2* __restrict__ adj, double ks, double kb,
                                                               double gx, double gy, double gz,
                                                               double* __restrict__ partial) {
    pdl_entry();
    __shared__ double wsum[3][EN_BLOCK / 32];
    const int v = blockIdx.x * EN_BLOCK + threadIdx.x;
    double ek = 0.0, eg = 0.0, ee = 0.0;
    if (v < V) {
        const float4 p = x4[v];
        const float mi = m_inv[v];
        if (mi > 0.0f) {
            const double m = 1.0 / (double)mi;
            const float4 u = v4[v];
            ek = 0.5 * m * (((double)u.x * u.x + (double)u.y * u.y) + (double)u.z * u.z);
            eg = -m * ((gx * p.x + gy * p.y) + gz * p.z);
        }
        for (int k = ptr[v]; k < ptr[v + 1]; ++k) {
            const int2 a = adj[k];
            const float4 o = x4[a.x & 0x7fffffff];
            const double ex = (double)p.x - o.x, ey = (double)p.y - o.y, ez = (double)p.z - o.z;
            const double C = sqrt((ex * ex + ey * ey) + ez * ez) - (double)__int_as_float(a.y);
            ee += 0.25 * (a.x < 0 ? kb : ks) * C * C;
        }
    }
    double t[3] = {ek, eg, ee};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        double w = t[q];
        for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
        if ((threadIdx.x & 31) == 0) wsum[q][threadIdx.x >> 5] = w;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double a = 0.0;
        for (int w = 0; w < EN_BLOCK / 32; ++w) a += wsum[threadIdx.x][w];
        partial[3 * (size_t)blockIdx.x + threadIdx.x] = a;
    }
}

__global__ void energy_finish_kernel(int nb, const double* __restrict__ partial, double* out3) {
    pdl_entry();
    if (threadIdx.x >= 3) return;
    double a = 0.0;
    for (int b = 0; b < nb; ++b) a += partial[3 * (size_t)b + threadIdx.x];
    out3[threadIdx.x] = a;
}
}  // namespace sx

extern "C" size_t sx_energy_workspace_bytes(int n_verts) {
    return (size_t)3 * sizeof(double) * (size_t)grid_for(n_verts > 0 ? n_verts : 1, EN_BLOCK);
}

extern "C" int sx_system_energy(const float* x4, const float* v4, const float* m_inv, const int* adj_ptr,
                                const int* adj, int n_verts, float k_spring, float k_bend, float gx, float gy,
                                float gz, double* out3, void* ws, size_t ws_bytes, void* stream) {
    SX_REQUIRE(n_verts >= 0, "sx_system_energy: n_verts < 0");
    SX_REQUIRE(out3 && ws && (n_verts == 0 || (x4 && v4 && m_inv && adj_ptr && adj)),
               "sx_system_energy: null pointer");
    SX_REQUIRE(ws_bytes >= sx_energy_workspace_bytes(n_verts), "sx_system_energy: workspace too small");
    cudaStream_t s = as_stream(stream);
    if (n_verts == 0) {
        SX_CUDA(cudaMemsetAsync(out3, 0, 3 * sizeof(double), s));
        return SX_OK;
    }
    const int nb = grid_for(n_verts, EN_BLOCK);
    launch(energy_partial_kernel, nb, EN_BLOCK, 0, s, n_verts, (const float4*)x4, (const float4*)v4, m_inv, adj_ptr,
           (const int2*)adj, (double)k_spring, (double)k_bend, (double)gx, (double)gy, (double)gz, (double*)ws);
    launch(energy_finish_kernel, 1, 32, 0, s, nb, (const double*)ws, out3);
    return check_launch("energy_finish_kernel");
}

extern "C" int sx_convergence_begin(int* conv, int check_every, int reset_totals, void* stream) {
    SX_REQUIRE(conv, "sx_convergence_begin: null pointer");
    SX_REQUIRE(check_every >= 2 && check_every % 2 == 0, "sx_convergence_begin: check_every must be even and >= 2");
    launch(convergence_begin_kernel, 1, 32, 0, as_stream(stream), conv, check_every, reset_totals);
    return check_launch("convergence_begin_kernel");
}

extern "C" int sx_jacobi_sweep_checked(const float* x4, const float* y_in4, float* y_out4, const float* fixed,
                                       const int* adj_ptr, const int* adj, int n_verts, float k_spring,
                                       float k_bend, int iter, int check, double tol, const double* ref3,
                                       int* conv, double* res3, void* ws, size_t ws_bytes,
                                       unsigned long long loop, int n_iter, void* stream) {
    return sx_jacobi_sweep_checked_mode(x4, y_in4, y_out4, fixed, adj_ptr, adj, n_verts, k_spring, k_bend, iter,
                                        check, tol, ref3, conv, res3, ws, ws_bytes, loop, n_iter, 0, stream);
}

extern "C" int sx_jacobi_sweep_checked_mode(const float* x4, const float* y_in4, float* y_out4, const float* fixed,
                                            const int* adj_ptr, const int* adj, int n_verts, float k_spring,
                                            float k_bend, int iter, int check, double tol, const double* ref3,
                                            int* conv, double* res3, void* ws, size_t ws_bytes,
                                            unsigned long long loop, int n_iter, int fast, void* stream) {
    SX_REQUIRE(n_verts > 0, "sx_jacobi_sweep_checked: n_verts must be positive");
    SX_REQUIRE(x4 && y_in4 && y_out4 && fixed && adj_ptr && adj && conv, "sx_jacobi_sweep_checked: null pointer");
    SX_REQUIRE(y_in4 != y_out4, "sx_jacobi_sweep_checked: y_in4 and y_out4 must not alias");
    SX_REQUIRE(iter >= 0, "sx_jacobi_sweep_checked: iter < 0");
    SX_REQUIRE(!check || (iter % 2 == 0 && res3 && ws && ws_bytes >= sx_residual_workspace_bytes(n_verts) && tol >= 0.0),
               "sx_jacobi_sweep_checked: a check needs an even iter, res3, a residual workspace and tol >= 0");
    SX_REQUIRE(!loop || check, "sx_jacobi_sweep_checked: a loop handle goes with the check of the loop body");
    cudaStream_t s = as_stream(stream);
    // inside a device-side loop the kernels are not gated (the loop stops instead)
    const int* gate = loop ? nullptr : (const int*)conv;
    const int nb = sweep_blocks(n_verts);
    if (check) {
        const auto kc = fast ? jacobi_sweep_kernel<true, 2, SW_BLOCK, true, true>
                             : jacobi_sweep_kernel<true, 2, SW_BLOCK, true>;
        launch(kc, gate ? tile_grid(kc, n_verts) : sweep_blocks(n_verts), SW_BLOCK, 0, s, n_verts,
               (const float4*)x4, (const float4*)y_in4, (float4*)y_out4, fixed, adj_ptr, (const int2*)adj, k_spring,
               k_bend, 1, gate, iter, (double*)ws);
        int rc = check_launch("jacobi_sweep_kernel");
        if (rc) return rc;
        return residual_finish(n_verts, adj_ptr, ws, res3, conv, iter, tol, ref3, loop, n_iter, s);
    }
    const auto kp = fast ? jacobi_sweep_kernel<false, 2, SW_BLOCK, true, true>
                         : jacobi_sweep_kernel<false, 2, SW_BLOCK, true>;
    launch(kp, gate ? tile_grid(kp, n_verts) : sweep_blocks(n_verts), SW_BLOCK, 0, s, n_verts,
           (const float4*)x4, (const float4*)y_in4, (float4*)y_out4, fixed, adj_ptr, (const int2*)adj, k_spring,
           k_bend, 1, gate, iter, (double*)nullptr);
    return check_launch("jacobi_sweep_kernel");
}

// ---------------------------------------------------------------------------
// Device-side iteration loop for CUDA graphs.  While `stream` is being
// captured, sx_loop_begin adds a conditional WHILE node after the work
// captured so far and starts capturing its body on `body_stream`; the caller
// then issues one block of iterations on body_stream, whose checked sweep
// passes *handle_out (it sets the loop condition: 0 once converged or at the
// iteration cap), and sx_loop_end closes the body and makes the rest of the
// capture on `stream` follow the loop.  The condition starts at 1 on every
// launch of the graph.
// ---------------------------------------------------------------------------
namespace sx {
struct LoopCtx {
    cudaStream_t main, body;
    cudaGraphNode_t node;
};
}  // namespace sx

extern "C" int sx_loop_begin(void* stream, void* body_stream, unsigned long long* handle_out, void** ctx_out) {
    SX_REQUIRE(handle_out && ctx_out && body_stream, "sx_loop_begin: null pointer");
    cudaStream_t s = as_stream(stream), bs = as_stream(body_stream);
    SX_REQUIRE(s != bs, "sx_loop_begin: the body needs its own stream");
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    SX_CUDA(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd));
    SX_REQUIRE(st == cudaStreamCaptureStatusActive, "sx_loop_begin: the stream is not being captured");
    cudaGraphConditionalHandle h;
    SX_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    SX_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
    SX_CUDA(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    SX_CUDA(cudaStreamBeginCaptureToGraph(bs, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeRelaxed));
    *handle_out = (unsigned long long)h;
    *ctx_out = new LoopCtx{s, bs, node};
    ++g_pdl_suspend;  // the body's kernels are plain launches
    return SX_OK;
}

extern "C" int sx_loop_end(void* ctx) {
    SX_REQUIRE(ctx, "sx_loop_end: null context");
    LoopCtx* c = (LoopCtx*)ctx;
    cudaGraph_t body = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->body, &body);
    delete c;
    if (g_pdl_suspend > 0) --g_pdl_suspend;
    if (e != cudaSuccess) return cuda_status(e, "sx_loop_end");
    return SX_OK;
}
