// Cloth state kernels: predict, Jacobi spring/bending sweep, velocity + position
// update, face AABBs and scene AABB.  Reference: framework/physics/XPBD.py and
// framework/meshio/meshTaichiWrapper.py.
#include <atomic>
#include <cstdarg>
#include <cstdio>

#include "sx_common.cuh"

namespace sx {

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

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
// One Jacobi sweep (XPBD.py:141-184 + :384-387), gathered per vertex.
//
// For a constraint (v0, v1) the reference computes x10 = p0 - p1,
// n = x10 * (1/|x10|), ld = k*C/(k*(w0+w1)*(n.n) + 1) and scatters
// dx0 -= (w0*ld)*n, dx1 += (w1*ld)*n with float atomics.  From v1's side
// p1 - p0 = -x10 exactly, so n flips sign exactly and
// dx1 - (w1*ld)*(-n) == dx1 + (w1*ld)*n bit for bit: every vertex evaluates
// dx -= (w_self*ld) * normalize(p_self - p_other) over its incident constraints
// in ascending constraint index, which equals a serial run of the reference.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) jacobi_sweep_kernel(int V, const float4* __restrict__ x4,
                                                           const float4* __restrict__ yin,
                                                           float4* __restrict__ yout,
                                                           const float* __restrict__ fixed,
                                                           const int* __restrict__ ptr,
                                                           const int2* __restrict__ adj, float ks, float kb,
                                                           int bend_y) {
    // Four lanes per vertex: in round r lane j evaluates entry b + 4r + j, then
    // every lane of the quad adds the four terms in ascending entry order
    // (shuffles), so the sum is the serial one while the loads, square roots and
    // divisions run four-wide.
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int j = gt & 3;
    const int v = gt >> 2;
    const bool valid = v < V;
    float4 ps = make_float4(0.f, 0.f, 0.f, 0.f), xs = ps;
    int b = 0, e = 0;
    if (valid) {
        ps = __ldg(yin + v);
        xs = __ldg(x4 + v);
        b = __ldg(ptr + v);
        e = __ldg(ptr + v + 1);
    }
    const int rounds = (e - b + 3) >> 2;
    int rmax = rounds;
    for (int o = 4; o < 32; o <<= 1) rmax = max(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    const int qbase = lane & ~3;
    float dx = 0.0f, dy = 0.0f, dz = 0.0f;
    for (int r = 0; r < rmax; ++r) {
        const int k = b + 4 * r + j;
        float tx = 0.0f, ty = 0.0f, tz = 0.0f;
        if (k < e) {
            const int2 a = __ldg(adj + k);
            const bool bend = a.x < 0;
            const int nb = a.x & 0x7fffffff;
            const float rest = __int_as_float(a.y);
            const bool use_x = bend && !bend_y;
            const float4 self = use_x ? xs : ps;
            const float4 other = __ldg((use_x ? x4 : yin) + nb);
            const float kk = bend ? kb : ks;
            const float ex = self.x - other.x, ey = self.y - other.y, ez = self.z - other.z;
            const float lij = sqrtf((ex * ex + ey * ey) + ez * ez);
            const float C = lij - rest;
            const float inv = 1.0f / lij;
            const float nx = inv * ex, ny = inv * ey, nz = inv * ez;
            const float schur = (self.w + other.w) * ((nx * nx + ny * ny) + nz * nz);
            const float ld = (kk * C) / (kk * schur + 1.0f);
            const float a0 = self.w * ld;
            tx = a0 * nx;
            ty = a0 * ny;
            tz = a0 * nz;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const float sx_ = __shfl_sync(0xffffffffu, tx, qbase + u);
            const float sy_ = __shfl_sync(0xffffffffu, ty, qbase + u);
            const float sz_ = __shfl_sync(0xffffffffu, tz, qbase + u);
            if (b + 4 * r + u < e) {
                dx = dx - sx_;
                dy = dy - sy_;
                dz = dz - sz_;
            }
        }
    }
    if (!valid || j != 0) return;
    float4 out = ps;
    const float nc = (float)(e - b);
    if (nc > 0.0f) {
        const float f = fixed[v];
        out.x = ps.x + f * (dx / nc);
        out.y = ps.y + f * (dy / nc);
        out.z = ps.z + f * (dz / nc);
    }
    yout[v] = out;
}

// ---------------------------------------------------------------------------
// compute_velocity + update_x (XPBD.py:341-343, :333-337)
// ---------------------------------------------------------------------------
__global__ void velocity_update_kernel(int V, float4* __restrict__ x4, const float4* __restrict__ y4,
                                       float4* __restrict__ v4, const float* __restrict__ fixed, float damping,
                                       float dt) {
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

// ---------------------------------------------------------------------------
// computeAABB_faces (meshTaichiWrapper.py:351-365)
// ---------------------------------------------------------------------------
__global__ void face_aabb_kernel(int F, const float4* __restrict__ p4, const int* __restrict__ faces, float pad,
                                 float4* __restrict__ mn4, float4* __restrict__ mx4) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    V3 a = mk(p4[faces[3 * f]]), b = mk(p4[faces[3 * f + 1]]), c = mk(p4[faces[3 * f + 2]]);
    V3 lo = vmin(vmin(a, b), c), hi = vmax(vmax(a, b), c);
    mn4[f] = make_float4(lo.x - pad, lo.y - pad, lo.z - pad, 0.0f);
    mx4[f] = make_float4(hi.x + pad, hi.y + pad, hi.z + pad, 0.0f);
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
    int t = threadIdx.x;
    if (t < 3) box[t] = f2ord(1e5f);
    else if (t < 6) box[t] = f2ord(-1e5f);
}

__global__ void scene_aabb_reduce(int V, const float4* __restrict__ p4, unsigned* box) {
    float lo[3] = {1e5f, 1e5f, 1e5f}, hi[3] = {-1e5f, -1e5f, -1e5f};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x) {
        float4 p = p4[i];
        lo[0] = fminf(lo[0], p.x); lo[1] = fminf(lo[1], p.y); lo[2] = fminf(lo[2], p.z);
        hi[0] = fmaxf(hi[0], p.x); hi[1] = fmaxf(hi[1], p.y); hi[2] = fmaxf(hi[2], p.z);
    }
    for (int o = 16; o > 0; o >>= 1) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; ++k) {
            atomicMin(box + k, f2ord(lo[k]));
            atomicMax(box + 3 + k, f2ord(hi[k]));
        }
    }
}

__global__ void scene_aabb_finish(unsigned* box, float pad) {
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
    launch(jacobi_sweep_kernel, grid_for(4LL * n_verts, 128), 128, 0, as_stream(stream), 
        n_verts, (const float4*)x4, (const float4*)y_in4, (float4*)y_out4, fixed, adj_ptr, (const int2*)adj,
        k_spring, k_bend, bend_on_y ? 1 : 0);
    return check_launch("jacobi_sweep_kernel");
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

extern "C" int sx_face_aabbs(const float* p4, const int* faces, int n_faces, float padding, float* aabb_min4,
                             float* aabb_max4, void* stream) {
    SX_REQUIRE(n_faces >= 0, "sx_face_aabbs: n_faces < 0");
    if (n_faces == 0) return SX_OK;
    SX_REQUIRE(p4 && faces && aabb_min4 && aabb_max4, "sx_face_aabbs: null pointer");
    launch(face_aabb_kernel, grid_for(n_faces, 256), 256, 0, as_stream(stream), 
        n_faces, (const float4*)p4, faces, padding, (float4*)aabb_min4, (float4*)aabb_max4);
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
        if (g > 1024) g = 1024;
        launch(scene_aabb_reduce, g, 256, 0, s, n_verts, (const float4*)p4, box);
    }
    launch(scene_aabb_finish, 1, 32, 0, s, box, padding);
    return check_launch("scene_aabb");
}

// ---------------------------------------------------------------------------
// Constraint residual.  The reference defines none (XPBD.py:350-369 runs a
// fixed number of sweeps); here it is the RMS of C = |p0 - p1| - l0 over the
// springs and bending pairs, evaluated in FP64 from the float positions.  Each
// constraint is counted at its lower-numbered endpoint; block sums are combined
// in a fixed order, so the value is deterministic.
// ---------------------------------------------------------------------------
namespace sx {
constexpr int RES_BLOCK = 256;

__global__ void __launch_bounds__(RES_BLOCK) residual_partial_kernel(int V, const float4* __restrict__ p4,
                                                                     const int* __restrict__ ptr,
                                                                     const int2* __restrict__ adj,
                                                                     double* __restrict__ partial) {
    __shared__ double red[RES_BLOCK];
    __shared__ double cnt[RES_BLOCK];
    const int v = blockIdx.x * RES_BLOCK + threadIdx.x;
    double s = 0.0, c = 0.0;
    if (v < V) {
        const float4 pv = p4[v];
        for (int k = ptr[v]; k < ptr[v + 1]; ++k) {
            const int2 a = adj[k];
            const int nb = a.x & 0x7fffffff;
            if (nb <= v) continue;
            const float4 pn = p4[nb];
            const double dx = (double)pv.x - (double)pn.x, dy = (double)pv.y - (double)pn.y,
                         dz = (double)pv.z - (double)pn.z;
            const double C = sqrt(dx * dx + dy * dy + dz * dz) - (double)__int_as_float(a.y);
            s += C * C;
            c += 1.0;
        }
    }
    red[threadIdx.x] = s;
    cnt[threadIdx.x] = c;
    __syncthreads();
    for (int o = RES_BLOCK / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            red[threadIdx.x] += red[threadIdx.x + o];
            cnt[threadIdx.x] += cnt[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = red[0];
        partial[2 * blockIdx.x + 1] = cnt[0];
    }
}

__global__ void residual_final_kernel(int nb, const double* __restrict__ partial, double* out) {
    if (threadIdx.x != 0) return;
    double s = 0.0, c = 0.0;
    for (int i = 0; i < nb; ++i) {
        s += partial[2 * i];
        c += partial[2 * i + 1];
    }
    out[0] = s;
    out[1] = c;
    out[2] = c > 0.0 ? sqrt(s / c) : 0.0;
}
}  // namespace sx

extern "C" size_t sx_residual_workspace_bytes(int n_verts) {
    return (size_t)2 * sizeof(double) * (size_t)grid_for(n_verts > 0 ? n_verts : 1, RES_BLOCK);
}

extern "C" int sx_constraint_residual(const float* p4, const int* adj_ptr, const int* adj, int n_verts, double* out3,
                                      void* ws, size_t ws_bytes, void* stream) {
    SX_REQUIRE(n_verts >= 0, "sx_constraint_residual: n_verts < 0");
    SX_REQUIRE(out3 && ws && (n_verts == 0 || (p4 && adj_ptr && adj)), "sx_constraint_residual: null pointer");
    SX_REQUIRE(ws_bytes >= sx_residual_workspace_bytes(n_verts), "sx_constraint_residual: workspace too small");
    cudaStream_t s = as_stream(stream);
    const int nb = grid_for(n_verts > 0 ? n_verts : 1, RES_BLOCK);
    launch(residual_partial_kernel, nb, RES_BLOCK, 0, s, n_verts, (const float4*)p4, adj_ptr, (const int2*)adj,
           (double*)ws);
    launch(residual_final_kernel, 1, 32, 0, s, nb, (const double*)ws, out3);
    return check_launch("constraint_residual");
}
