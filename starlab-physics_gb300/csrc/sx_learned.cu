// Learned warm start for the Jacobi solve (no counterpart in the reference,
// whose substep starts every solve from the predicted positions y,
// XPBD.py:116-118).  A per-vertex MLP 24 -> 64 -> 64 -> 3 (SiLU) maps local
// features of the predicted state to a position correction in units of the
// vertex's mean spring rest length; the solve then starts from
// y + fixed * L * correction.
//
//   features : sx_warm_features     (vertex gather, FP32, stored as BF16[V][32])
//   inference: sx_mlp_forward       (BF16 tensor-core mma, FP32 accumulate,
//                                    activations kept in registers)
//   training : sx_mlp_train_step    (forward + backward data path per 16-row
//                                    tile, weight gradients as dZ^T H products
//                                    on tensor cores, deterministic reduction,
//                                    Adam on FP32 master weights)
//
// Parameter blob (FP32 master, 6792 floats): W1[64][32] | b1[64] | W2[64][64]
// | b2[64] | W3[8][64] | b3[8]; W1's columns 24..31 and W3's rows 3..7 are
// zero.  The BF16 copy holds W1 | W2 | W3 in the same layout.
#include <cuda_bf16.h>

#include "sx_common.cuh"

namespace sx {

constexpr int kFeat = 32;   // 24 features + 8 zero columns
constexpr int kHid = 64;
constexpr int kOut = 8;     // 3 used
constexpr int oW1 = 0, ob1 = oW1 + kHid * kFeat, oW2 = ob1 + kHid, ob2 = oW2 + kHid * kHid, oW3 = ob2 + kHid,
              ob3 = oW3 + kOut * kHid, kParams = ob3 + kOut;
constexpr int kW16 = kHid * kFeat + kHid * kHid + kOut * kHid;  // BF16 weights
constexpr int qW1 = 0, qW2 = kHid * kFeat, qW3 = qW2 + kHid * kHid;

__device__ __forceinline__ unsigned short f2bf(float f) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(f));
}
__device__ __forceinline__ float bf2f(unsigned short u) { return __bfloat162float(__ushort_as_bfloat16(u)); }
__device__ __forceinline__ unsigned pack_bf2(float lo, float hi) {
    return (unsigned)f2bf(lo) | ((unsigned)f2bf(hi) << 16);
}

// D += A(16x16, row) * B(16x8, col), BF16 inputs, FP32 accumulate.
__device__ __forceinline__ void mma16816(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void ldsm_x4_trans(unsigned (&r)[4], const void* p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.0f / (1.0f + expf(-z));
    return s + z * (s * (1.0f - s));
}

// ---------------------------------------------------------------------------
// Features (24, then 8 zeros), from the predicted positions y4, the start of
// substep positions x4, the previous substep's solve correction c4 and the
// constraint adjacency.  L = mean spring rest length at the vertex (Lref).
//   0-2  -(mean over springs of C n) / L        3-5  same over bending pairs
//   6    mean |C|/l0 springs   7 max C/l0   8 min C/l0   9 mean |C|/l0 bending
//   10-12 (y - x)/L            13-15 c/L    16 fixed   17 springs/6  18 bends/6
//   19   |c|/L                 20 |y - x|/L             21-23 g dt^2 / L
// each clamped to [-16, 16] and rounded to BF16.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) warm_features_kernel(int V, const float4* __restrict__ x4,
                                                            const float4* __restrict__ y4,
                                                            const float4* __restrict__ c4,
                                                            const float* __restrict__ fixed,
                                                            const int* __restrict__ ptr,
                                                            const int2* __restrict__ adj,
                                                            const float* __restrict__ Lref, float gx, float gy,
                                                            float gz, float dt, unsigned short* __restrict__ feat,
                                                            float4* __restrict__ ypred) {
    pdl_entry();
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const float4 ps = y4[v], xs = x4[v], cp = c4[v];
    if (ypred) ypred[v] = ps;
    const float inv = 1.0f / Lref[v];
    float sx = 0.0f, sy = 0.0f, sz = 0.0f, bx = 0.0f, by = 0.0f, bz = 0.0f;
    float sa = 0.0f, ba = 0.0f, smax = 0.0f, smin = 0.0f;
    int ns = 0, nb = 0;
    const int e = ptr[v + 1];
    for (int k = ptr[v]; k < e; ++k) {
        const int2 a = adj[k];
        const float4 o = y4[a.x & 0x7fffffff];
        const float rest = __int_as_float(a.y);
        const float ex = ps.x - o.x, ey = ps.y - o.y, ez = ps.z - o.z;
        const float l = sqrtf((ex * ex + ey * ey) + ez * ez);
        const float C = l - rest;
        const float il = l > 0.0f ? 1.0f / l : 0.0f;
        const float cx = C * (il * ex), cy = C * (il * ey), cz = C * (il * ez);
        const float r = rest > 0.0f ? C / rest : 0.0f;
        if (a.x < 0) {
            bx = bx + cx; by = by + cy; bz = bz + cz;
            ba = ba + fabsf(r);
            ++nb;
        } else {
            sx = sx + cx; sy = sy + cy; sz = sz + cz;
            sa = sa + fabsf(r);
            smax = ns ? fmaxf(smax, r) : r;
            smin = ns ? fminf(smin, r) : r;
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
    const float dx = ps.x - xs.x, dy = ps.y - xs.y, dz = ps.z - xs.z;
    f[10] = dx * inv;
    f[11] = dy * inv;
    f[12] = dz * inv;
    f[13] = cp.x * inv;
    f[14] = cp.y * inv;
    f[15] = cp.z * inv;
    f[16] = fixed[v];
    f[17] = fs / 6.0f;
    f[18] = fb / 6.0f;
    f[19] = sqrtf((cp.x * cp.x + cp.y * cp.y) + cp.z * cp.z) * inv;
    f[20] = sqrtf((dx * dx + dy * dy) + dz * dz) * inv;
    f[21] = ((gx * dt) * dt) * inv;
    f[22] = ((gy * dt) * dt) * inv;
    f[23] = ((gz * dt) * dt) * inv;
    unsigned* out = reinterpret_cast<unsigned*>(feat + (size_t)v * kFeat);
#pragma unroll
    for (int i = 0; i < 12; ++i)
        out[i] = pack_bf2(fminf(fmaxf(f[2 * i], -16.0f), 16.0f), fminf(fmaxf(f[2 * i + 1], -16.0f), 16.0f));
#pragma unroll
    for (int i = 12; i < 16; ++i) out[i] = 0u;
}

// y = y_pred + fixed * (L * d) for the first three outputs d of the MLP.
__global__ void warm_apply_kernel(int V, const float4* __restrict__ ypred, const float* __restrict__ out4,
                                  const float* __restrict__ fixed, const float* __restrict__ Lref,
                                  float4* __restrict__ y4) {
    pdl_entry();
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const float4 p = ypred[v];
    const float f = fixed[v], L = Lref[v];
    float4 y = p;
    y.x = p.x + f * (L * out4[4 * v]);
    y.y = p.y + f * (L * out4[4 * v + 1]);
    y.z = p.z + f * (L * out4[4 * v + 2]);
    y4[v] = y;
}

// After the solve: c = y - y_pred (the next substep's feature 13-15) and the
// training target (c / L, fixed) as float4.
__global__ void warm_record_kernel(int V, const float4* __restrict__ y4, const float4* __restrict__ ypred,
                                   const float* __restrict__ fixed, const float* __restrict__ Lref,
                                   float4* __restrict__ c4, float4* __restrict__ target4) {
    pdl_entry();
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const float4 y = y4[v], p = ypred[v];
    const float4 c = make_float4(y.x - p.x, y.y - p.y, y.z - p.z, 0.0f);
    c4[v] = c;
    if (target4) {
        const float inv = 1.0f / Lref[v];
        target4[v] = make_float4(c.x * inv, c.y * inv, c.z * inv, fixed[v]);
    }
}

// If the warm start raised the residual (res_warm[2] > res_cold[2]), restore
// the cold start y = y_pred; flag[0] counts fallbacks, flag[1] warm starts.
__global__ void warm_select_kernel(int V, const double* __restrict__ res_warm, const double* __restrict__ res_cold,
                                   const float4* __restrict__ ypred, float4* __restrict__ y4, int* flag) {
    pdl_entry();
    const bool cold = res_warm[2] > res_cold[2];
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v == 0) {
        if (cold) flag[0] += 1;
        else flag[1] += 1;
    }
    if (cold && v < V) y4[v] = ypred[v];
}

// ---------------------------------------------------------------------------
// MLP tiles.  A warp owns 16 rows.  Shared weights (BF16, rows padded so that
// the fragment loads are bank-conflict free):
//   W1s[64][40] (n, k), W2s[64][72] (n, k), W3s[8][72] (n, k),
//   W2t[64][72] (k, n) and W3t[64][24] (k, n) for the backward data path.
// ---------------------------------------------------------------------------
constexpr int S1 = 40, S2 = 72, S3 = 72, S2T = 72, S3T = 24;

struct MlpSmem {
    unsigned short W1[kHid * S1];
    unsigned short W2[kHid * S2];
    unsigned short W3[kOut * S3];
    float b1[kHid], b2[kHid], b3[kOut];
};
struct MlpSmemT {
    unsigned short W2t[kHid * S2T];
    unsigned short W3t[kHid * S3T];
};

__device__ void stage_weights(MlpSmem& s, const unsigned short* __restrict__ w16, const float* __restrict__ p32) {
    for (int i = threadIdx.x; i < kHid * kFeat; i += blockDim.x) s.W1[(i / kFeat) * S1 + i % kFeat] = w16[qW1 + i];
    for (int i = threadIdx.x; i < kHid * kHid; i += blockDim.x) s.W2[(i / kHid) * S2 + i % kHid] = w16[qW2 + i];
    for (int i = threadIdx.x; i < kOut * kHid; i += blockDim.x) s.W3[(i / kHid) * S3 + i % kHid] = w16[qW3 + i];
    for (int i = threadIdx.x; i < kHid; i += blockDim.x) {
        s.b1[i] = p32[ob1 + i];
        s.b2[i] = p32[ob2 + i];
    }
    if (threadIdx.x < kOut) s.b3[threadIdx.x] = p32[ob3 + threadIdx.x];
}

__device__ void stage_weights_t(MlpSmemT& t, const unsigned short* __restrict__ w16) {
    // W2t[k = in][n = out] = W2[n][k]; W3t[k = hidden][n = out] = W3[n][k]
    for (int i = threadIdx.x; i < kHid * kHid; i += blockDim.x) t.W2t[(i % kHid) * S2T + i / kHid] = w16[qW2 + i];
    for (int i = threadIdx.x; i < kHid * S3T; i += blockDim.x) {
        const int k = i / S3T, n = i % S3T;
        t.W3t[i] = n < kOut ? w16[qW3 + n * kHid + k] : (unsigned short)0;
    }
}

__device__ __forceinline__ unsigned lds32(const unsigned short* p) { return *reinterpret_cast<const unsigned*>(p); }

// Forward of one 16-row tile.  X rows: feature row of tile row r is
// xrow(r) (or -1 for padding rows).  Outputs Z1, Z2 (pre-activations, C
// layout) and O (C layout, 8 columns).
struct Frag64 {
    float c[8][4];
};

__device__ __forceinline__ void tile_forward(const MlpSmem& s, const unsigned (&ax)[2][4], Frag64& z1, Frag64& z2,
                                             float (&o)[4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float b0 = s.b1[8 * j + 2 * tig], b1v = s.b1[8 * j + 2 * tig + 1];
        z1.c[j][0] = b0; z1.c[j][1] = b1v; z1.c[j][2] = b0; z1.c[j][3] = b1v;
    }
#pragma unroll
    for (int ks = 0; ks < 2; ++ks)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const unsigned short* w = s.W1 + (8 * j + g) * S1 + 16 * ks + 2 * tig;
            mma16816(z1.c[j], ax[ks], lds32(w), lds32(w + 8));
        }
    unsigned ah[4][4];
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
        ah[ks][0] = pack_bf2(silu(z1.c[2 * ks][0]), silu(z1.c[2 * ks][1]));
        ah[ks][1] = pack_bf2(silu(z1.c[2 * ks][2]), silu(z1.c[2 * ks][3]));
        ah[ks][2] = pack_bf2(silu(z1.c[2 * ks + 1][0]), silu(z1.c[2 * ks + 1][1]));
        ah[ks][3] = pack_bf2(silu(z1.c[2 * ks + 1][2]), silu(z1.c[2 * ks + 1][3]));
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float b0 = s.b2[8 * j + 2 * tig], b1v = s.b2[8 * j + 2 * tig + 1];
        z2.c[j][0] = b0; z2.c[j][1] = b1v; z2.c[j][2] = b0; z2.c[j][3] = b1v;
    }
#pragma unroll
    for (int ks = 0; ks < 4; ++ks)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const unsigned short* w = s.W2 + (8 * j + g) * S2 + 16 * ks + 2 * tig;
            mma16816(z2.c[j], ah[ks], lds32(w), lds32(w + 8));
        }
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
        ah[ks][0] = pack_bf2(silu(z2.c[2 * ks][0]), silu(z2.c[2 * ks][1]));
        ah[ks][1] = pack_bf2(silu(z2.c[2 * ks][2]), silu(z2.c[2 * ks][3]));
        ah[ks][2] = pack_bf2(silu(z2.c[2 * ks + 1][0]), silu(z2.c[2 * ks + 1][1]));
        ah[ks][3] = pack_bf2(silu(z2.c[2 * ks + 1][2]), silu(z2.c[2 * ks + 1][3]));
    }
    o[0] = s.b3[2 * tig]; o[1] = s.b3[2 * tig + 1]; o[2] = o[0]; o[3] = o[1];
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
        const unsigned short* w = s.W3 + g * S3 + 16 * ks + 2 * tig;
        mma16816(o, ah[ks], lds32(w), lds32(w + 8));
    }
}

// A fragments of a 16-row tile of BF16 features (rows r0+g, r0+g+8).
__device__ __forceinline__ void load_x_frag(const unsigned short* __restrict__ feat, int ra, int rb,
                                            unsigned (&ax)[2][4]) {
    const int tig = threadIdx.x & 3;
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        const int c = 16 * ks + 2 * tig;
        ax[ks][0] = ra >= 0 ? *reinterpret_cast<const unsigned*>(feat + (size_t)ra * kFeat + c) : 0u;
        ax[ks][1] = rb >= 0 ? *reinterpret_cast<const unsigned*>(feat + (size_t)rb * kFeat + c) : 0u;
        ax[ks][2] = ra >= 0 ? *reinterpret_cast<const unsigned*>(feat + (size_t)ra * kFeat + c + 8) : 0u;
        ax[ks][3] = rb >= 0 ? *reinterpret_cast<const unsigned*>(feat + (size_t)rb * kFeat + c + 8) : 0u;
    }
}

constexpr int MLP_BLOCK = 128;

__global__ void __launch_bounds__(MLP_BLOCK) mlp_forward_kernel(int V, const unsigned short* __restrict__ feat,
                                                                const unsigned short* __restrict__ w16,
                                                                const float* __restrict__ p32,
                                                                float* __restrict__ out4) {
    pdl_entry();
    __shared__ MlpSmem s;
    stage_weights(s, w16, p32);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int r0 = warp * 16; r0 < V; r0 += nwarps * 16) {
        const int ra = r0 + g < V ? r0 + g : -1, rb = r0 + g + 8 < V ? r0 + g + 8 : -1;
        unsigned ax[2][4];
        load_x_frag(feat, ra, rb, ax);
        Frag64 z1, z2;
        float o[4];
        tile_forward(s, ax, z1, z2, o);
        if (tig < 2) {
            if (ra >= 0) *reinterpret_cast<float2*>(out4 + 4 * (size_t)ra + 2 * tig) = make_float2(o[0], o[1]);
            if (rb >= 0) *reinterpret_cast<float2*>(out4 + 4 * (size_t)rb + 2 * tig) = make_float2(o[2], o[3]);
        }
    }
}

// ---------------------------------------------------------------------------
// Inference on the 5th-generation tensor cores (tcgen05).  One CTA of 256
// threads takes 128 rows at a time (M = 128; two threads per row, one per
// half of the 64 hidden columns): the rows' features, the hidden
// activations and the three weight matrices sit in shared memory in the
// canonical no-swizzle K-major layout (8 x 16-byte core matrices; LBO = 128 B
// between core matrices along K, SBO = (K / 8) x 128 B between 8-row groups);
// thread 0 issues tcgen05.mma (kind::f16, BF16 x BF16 -> FP32) into tensor
// memory, whose completion tcgen05.commit signals on an mbarrier; each warp
// then reads its 32 rows of the accumulator with tcgen05.ld, adds the bias,
// applies SiLU, and writes the next layer's BF16 operand.  Layer 3 is N = 16
// (W3's 8 rows and 8 zero rows); 128 tensor-memory columns per CTA (D1 at 0,
// D2 at 64, D3 at 0 once D1 is read).  Every wait is bounded (1 s of global time);
// a wait that gives up sets SX_STATUS_WAIT_TIMEOUT, waits once more (bounded)
// for the MMAs in flight, frees the tensor memory and ends the kernel.
// ---------------------------------------------------------------------------
constexpr int TC_ROWS = 128;
constexpr int TC_THREADS = 256;  // warp w reads tensor-memory lanes 32 (w % 4).., columns half w / 4
constexpr int TC_TMEM_COLS = 128;  // D1 at column 0, D2 at 64, D3 at 0 (D1 is read by then)
constexpr int TC_PAD_SMEM = 12 * 1024;  // with the 39.5 KB static: 4 CTAs per SM fit, 5 do not

struct TcSmem {
    alignas(128) unsigned short A1[TC_ROWS * kFeat];
    alignas(128) unsigned short A2[TC_ROWS * kHid];
    alignas(128) unsigned short B1[kHid * kFeat];
    alignas(128) unsigned short B2[kHid * kHid];
    alignas(128) unsigned short B3[16 * kHid];
    float b1[kHid], b2[kHid], b3[16];
    alignas(8) unsigned long long bar;
    unsigned tmem_base;
};

// element (r, k) of a K-major operand with K columns, canonical layout
__device__ __forceinline__ int canon(int r, int k, int K) {
    return ((r >> 3) * (K >> 3) + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
// shared-memory matrix descriptor: start, LBO, SBO (16-byte units), version 1, no swizzle
__device__ __forceinline__ unsigned long long umma_sdesc(unsigned saddr, unsigned lbo, unsigned sbo) {
    return (unsigned long long)((saddr >> 4) & 0x3FFFu) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
           ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor, kind::f16: D F32, A and B BF16, both K-major
__host__ __device__ constexpr unsigned umma_idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void umma_bf16(unsigned d_tmem, unsigned long long a, unsigned long long b, unsigned idesc,
                                          unsigned accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accum)
        : "memory");
}
__device__ __forceinline__ void umma_commit(unsigned bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned bar, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0u;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ bool mbar_wait_bounded(unsigned bar, unsigned parity) {
    const unsigned long long t0 = global_ns();
    while (!mbar_test(bar, parity))
        if (global_ns() - t0 > 1000000000ull) return false;
    return true;
}
__device__ __forceinline__ void tmem_ld32(unsigned taddr, unsigned (&r)[32]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr)
                 : "memory");
}
__device__ __forceinline__ void tmem_ld16(unsigned taddr, unsigned (&r)[16]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// SiLU through the hardware tanh: z * sigmoid(z) = h + h * tanh(h) with
// h = z / 2, one special-function instruction instead of an exponential and a
// reciprocal (the epilogue's special-function unit was its limit).  The
// tensor-core path's hidden activations are rounded to BF16, far coarser than
// tanh.approx's error.
__device__ __forceinline__ float tanh_hw(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float silu_fast(float z) {
    const float h = 0.5f * z;
    return __fmaf_rn(h, tanh_hw(h), h);
}

// 32 accumulator columns of this thread's row (at taddr) + bias -> SiLU ->
// BF16 columns [c0, c0 + 32) of row `row` of A2
__device__ __forceinline__ void tc_hidden_half(unsigned taddr, const float* bias, unsigned short* A2, int row, int c0) {
    unsigned r[32];
    tmem_ld32(taddr, r);
    tmem_wait_ld();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        uint4 v;
        unsigned* pv = reinterpret_cast<unsigned*>(&v);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int c = 8 * q + 2 * e;
            pv[e] = pack_bf2(silu_fast(__uint_as_float(r[c]) + bias[c0 + c]),
                             silu_fast(__uint_as_float(r[c + 1]) + bias[c0 + c + 1]));
        }
        *reinterpret_cast<uint4*>(A2 + canon(row, c0 + 8 * q, kHid)) = v;
    }
}

__global__ void __launch_bounds__(TC_THREADS, 1) mlp_forward_tc_kernel(int V, const unsigned short* __restrict__ feat,
                                                                    const unsigned short* __restrict__ w16,
                                                                    const float* __restrict__ p32,
                                                                    float* __restrict__ out4, int* status) {
    pdl_entry();
    __shared__ TcSmem s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int quad = warp & 3, half = warp >> 2;
    const int trow = 32 * quad + lane;  // this thread's row within a tile
    for (int i = tid; i < kHid * kFeat; i += TC_THREADS) s.B1[canon(i / kFeat, i % kFeat, kFeat)] = w16[qW1 + i];
    for (int i = tid; i < kHid * kHid; i += TC_THREADS) s.B2[canon(i / kHid, i % kHid, kHid)] = w16[qW2 + i];
    for (int i = tid; i < 16 * kHid; i += TC_THREADS) {
        const int n = i / kHid, k = i % kHid;
        s.B3[canon(n, k, kHid)] = n < kOut ? w16[qW3 + n * kHid + k] : (unsigned short)0;
    }
    for (int i = tid; i < kHid; i += TC_THREADS) {
        s.b1[i] = p32[ob1 + i];
        s.b2[i] = p32[ob2 + i];
    }
    if (tid < 16) s.b3[tid] = tid < kOut ? p32[ob3 + tid] : 0.0f;
    const unsigned bar = smem_u32(&s.bar);
    if (tid == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s.tmem_base)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tbase = s.tmem_base;
    const unsigned lane_row = (unsigned)(32 * quad) << 16;  // this warp's 32 tensor-memory lanes
    const unsigned long long dB1 = umma_sdesc(smem_u32(s.B1), 128, 512);
    const unsigned long long dB2 = umma_sdesc(smem_u32(s.B2), 128, 1024);
    const unsigned long long dB3 = umma_sdesc(smem_u32(s.B3), 128, 1024);
    const unsigned long long dA1 = umma_sdesc(smem_u32(s.A1), 128, 512);
    const unsigned long long dA2 = umma_sdesc(smem_u32(s.A2), 128, 1024);
    constexpr unsigned id64 = umma_idesc_bf16(TC_ROWS, kHid), id16 = umma_idesc_bf16(TC_ROWS, 16);
    unsigned phase = 0;
    bool ok = true;
    const int ntiles = (V + TC_ROWS - 1) / TC_ROWS;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int row = tile * TC_ROWS + trow;
        // layer 1: features (BF16, 32 columns; half a row per thread) -> A1
        uint4 f[2];
#pragma unroll
        for (int j = 0; j < 2; ++j)
            f[j] = row < V ? __ldg(reinterpret_cast<const uint4*>(feat + (size_t)row * kFeat) + 2 * half + j)
                           : make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int j = 0; j < 2; ++j) *reinterpret_cast<uint4*>(s.A1 + canon(trow, 16 * half + 8 * j, kFeat)) = f[j];
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int ks = 0; ks < kFeat / 16; ++ks) umma_bf16(tbase, dA1 + 16 * ks, dB1 + 16 * ks, id64, ks);
            umma_commit(bar);
        }
        ok = __syncthreads_and(mbar_wait_bounded(bar, phase));
        if (!ok) break;
        phase ^= 1u;
        tc_fence_after();
        tc_hidden_half(tbase + lane_row + 32 * half, s.b1, s.A2, trow, 32 * half);
        // layer 2
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int ks = 0; ks < kHid / 16; ++ks) umma_bf16(tbase + 64, dA2 + 16 * ks, dB2 + 16 * ks, id64, ks);
            umma_commit(bar);
        }
        ok = __syncthreads_and(mbar_wait_bounded(bar, phase));
        if (!ok) break;
        phase ^= 1u;
        tc_fence_after();
        tc_hidden_half(tbase + lane_row + 64 + 32 * half, s.b2, s.A2, trow, 32 * half);  // layer 2 is done with A2
        // layer 3 (N = 16)
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int ks = 0; ks < kHid / 16; ++ks) umma_bf16(tbase, dA2 + 16 * ks, dB3 + 16 * ks, id16, ks);
            umma_commit(bar);
        }
        ok = __syncthreads_and(mbar_wait_bounded(bar, phase));
        if (!ok) break;
        phase ^= 1u;
        tc_fence_after();
        unsigned r[16];
        tmem_ld16(tbase + lane_row, r);
        tmem_wait_ld();
        if (half == 0 && row < V)
            *reinterpret_cast<float4*>(out4 + 4 * (size_t)row) =
                make_float4(__uint_as_float(r[0]) + s.b3[0], __uint_as_float(r[1]) + s.b3[1],
                            __uint_as_float(r[2]) + s.b3[2], __uint_as_float(r[3]) + s.b3[3]);
        tc_fence_before();
        __syncthreads();  // every row read before the next tile's MMAs reuse the accumulators
    }
    if (!ok) {
        if (tid == 0) atomicOr(status, SX_STATUS_WAIT_TIMEOUT);
        mbar_wait_bounded(bar, phase);  // the MMAs in flight, once more within the bound
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(TC_TMEM_COLS)
                     : "memory");
}

// ---------------------------------------------------------------------------
// Training, part 1: forward + backward data path of a minibatch.  Rows are
// idx[i] into the sample arrays (feat, target4 = (t, mask)).  Loss =
// sum over rows and the 3 outputs of mask * (o - t)^2 / n_valid.  Writes per
// row: H1, H2, dZ1, dZ2 (BF16, 64 each) and dO (BF16, 16, columns 3..15 zero),
// and per warp: partial loss and bias gradients (FP32, in row order within the
// warp, then summed over lanes in a fixed tree).
// ---------------------------------------------------------------------------
struct TrainBuf {
    unsigned short* h1;
    unsigned short* h2;
    unsigned short* dz1;
    unsigned short* dz2;
    unsigned short* dout;  // [M][16]
    float* wpart;          // [nwarps][1 + 64 + 64 + 8]: loss, db1, db2, db3
};
constexpr int kWpart = 1 + kHid + kHid + kOut;

__device__ __forceinline__ void store_c_bf16(unsigned short* base, int ra, int rb, int ld, int col,
                                             const float (&c)[4]) {
    if (ra >= 0) *reinterpret_cast<unsigned*>(base + (size_t)ra * ld + col) = pack_bf2(c[0], c[1]);
    if (rb >= 0) *reinterpret_cast<unsigned*>(base + (size_t)rb * ld + col) = pack_bf2(c[2], c[3]);
}

// sum over the 8 row groups g of a C-fragment column pair (lanes with equal tig)
__device__ __forceinline__ float colsum(float v) {
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 8);
    v += __shfl_xor_sync(0xffffffffu, v, 16);
    return v;
}

__global__ void __launch_bounds__(MLP_BLOCK) mlp_train_fwd_bwd_kernel(int M, const int* __restrict__ idx,
                                                                      const unsigned short* __restrict__ feat,
                                                                      const float4* __restrict__ target4,
                                                                      float inv_valid,
                                                                      const unsigned short* __restrict__ w16,
                                                                      const float* __restrict__ p32, TrainBuf tb) {
    pdl_entry();
    __shared__ MlpSmem s;
    __shared__ MlpSmemT st;
    stage_weights(s, w16, p32);
    stage_weights_t(st, w16);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    float loss = 0.0f, db1[8][2], db2[8][2], db3[2];
#pragma unroll
    for (int j = 0; j < 8; ++j) db1[j][0] = db1[j][1] = db2[j][0] = db2[j][1] = 0.0f;
    db3[0] = db3[1] = 0.0f;
    for (int r0 = warp * 16; r0 < M; r0 += nwarps * 16) {
        const int ra = r0 + g < M ? r0 + g : -1, rb = r0 + g + 8 < M ? r0 + g + 8 : -1;
        const int sa = ra >= 0 ? idx[ra] : -1, sb = rb >= 0 ? idx[rb] : -1;
        unsigned ax[2][4];
        load_x_frag(feat, sa, sb, ax);
        Frag64 z1, z2;
        float o[4];
        tile_forward(s, ax, z1, z2, o);
        // dO (C layout: rows g, g+8; columns 2tig, 2tig+1)
        float d[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (tig < 2) {
            const float4 ta = sa >= 0 ? target4[sa] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 tb4 = sb >= 0 ? target4[sb] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float tta[4] = {ta.x, ta.y, ta.z, 0.0f}, ttb[4] = {tb4.x, tb4.y, tb4.z, 0.0f};
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int col = 2 * tig + u;
                if (col < 3) {
                    const float ea = ta.w * (o[u] - tta[col]), eb = tb4.w * (o[2 + u] - ttb[col]);
                    loss = loss + (ea * (o[u] - tta[col]) + eb * (o[2 + u] - ttb[col]));
                    d[u] = (2.0f * inv_valid) * ea;
                    d[2 + u] = (2.0f * inv_valid) * eb;
                }
            }
        }
        // dH2 = dO W3 (K = 16, columns 8..15 of dO are zero)
        unsigned ad[4] = {pack_bf2(d[0], d[1]), pack_bf2(d[2], d[3]), 0u, 0u};
        Frag64 dz;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            dz.c[j][0] = dz.c[j][1] = dz.c[j][2] = dz.c[j][3] = 0.0f;
            const unsigned short* w = st.W3t + (8 * j + g) * S3T + 2 * tig;
            mma16816(dz.c[j], ad, lds32(w), lds32(w + 8));
        }
        // dZ2 = dH2 * silu'(Z2); H2 = silu(Z2); H1 = silu(Z1)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            float h[4], h1[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                dz.c[j][u] = dz.c[j][u] * silu_grad(z2.c[j][u]);
                h[u] = silu(z2.c[j][u]);
                h1[u] = silu(z1.c[j][u]);
            }
            store_c_bf16(tb.h2, ra, rb, kHid, 8 * j + 2 * tig, h);
            store_c_bf16(tb.h1, ra, rb, kHid, 8 * j + 2 * tig, h1);
            store_c_bf16(tb.dz2, ra, rb, kHid, 8 * j + 2 * tig, dz.c[j]);
            db2[j][0] += dz.c[j][0] + dz.c[j][2];
            db2[j][1] += dz.c[j][1] + dz.c[j][3];
        }
        store_c_bf16(tb.dout, ra, rb, 16, 2 * tig, d);
        if (ra >= 0) *reinterpret_cast<unsigned*>(tb.dout + (size_t)ra * 16 + 8 + 2 * tig) = 0u;
        if (rb >= 0) *reinterpret_cast<unsigned*>(tb.dout + (size_t)rb * 16 + 8 + 2 * tig) = 0u;
        db3[0] += d[0] + d[2];
        db3[1] += d[1] + d[3];
        // dH1 = dZ2 W2, dZ1 = dH1 * silu'(Z1)
        unsigned az[4][4];
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            az[ks][0] = pack_bf2(dz.c[2 * ks][0], dz.c[2 * ks][1]);
            az[ks][1] = pack_bf2(dz.c[2 * ks][2], dz.c[2 * ks][3]);
            az[ks][2] = pack_bf2(dz.c[2 * ks + 1][0], dz.c[2 * ks + 1][1]);
            az[ks][3] = pack_bf2(dz.c[2 * ks + 1][2], dz.c[2 * ks + 1][3]);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                const unsigned short* w = st.W2t + (8 * j + g) * S2T + 16 * ks + 2 * tig;
                mma16816(c, az[ks], lds32(w), lds32(w + 8));
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) c[u] = c[u] * silu_grad(z1.c[j][u]);
            store_c_bf16(tb.dz1, ra, rb, kHid, 8 * j + 2 * tig, c);
            db1[j][0] += c[0] + c[2];
            db1[j][1] += c[1] + c[3];
        }
    }
    // per-warp partials: loss and bias gradients, summed over the row groups
    float* wp = tb.wpart + (size_t)warp * kWpart;
    float l = loss;
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if (lane == 0) wp[0] = l;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float a0 = colsum(db1[j][0]), a1 = colsum(db1[j][1]);
        const float c0 = colsum(db2[j][0]), c1 = colsum(db2[j][1]);
        if (g == 0) {
            wp[1 + 8 * j + 2 * tig] = a0;
            wp[1 + 8 * j + 2 * tig + 1] = a1;
            wp[1 + kHid + 8 * j + 2 * tig] = c0;
            wp[1 + kHid + 8 * j + 2 * tig + 1] = c1;
        }
    }
    const float e0 = colsum(db3[0]), e1 = colsum(db3[1]);
    if (g == 0) {
        wp[1 + 2 * kHid + 2 * tig] = e0;
        wp[1 + 2 * kHid + 2 * tig + 1] = e1;
    }
}

// ---------------------------------------------------------------------------
// Training, part 2: weight gradients dW1 = dZ1^T X, dW2 = dZ2^T H1,
// dW3 = dO^T H2 over this block's rows (64-row tiles staged in shared memory,
// A = dZ^T and B = H fragments by ldmatrix.trans), one partial per block.
// Warp w owns output rows 16w..16w+15 of dW1 and dW2 and columns 16w..16w+15
// of dW3.
// ---------------------------------------------------------------------------
constexpr int WG_ROWS = 64, SL = 72;  // tile rows; padded row stride (BF16)
constexpr int kWgrad = kHid * kFeat + kHid * kHid + kOut * kHid;

__global__ void __launch_bounds__(MLP_BLOCK) mlp_wgrad_kernel(int M, int rows_per_block,
                                                              const int* __restrict__ idx,
                                                              const unsigned short* __restrict__ feat,
                                                              TrainBuf tb, float* __restrict__ bpart) {
    pdl_entry();
    __shared__ __align__(16) unsigned short X[WG_ROWS * SL], H1[WG_ROWS * SL], H2[WG_ROWS * SL],
        D1[WG_ROWS * SL], D2[WG_ROWS * SL], DO[WG_ROWS * SL];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, g = lane >> 2, tig = lane & 3;
    const int q = lane >> 3, r8 = lane & 7;
    float a1[4][4], a2[8][4], a3[2][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) a2[j][0] = a2[j][1] = a2[j][2] = a2[j][3] = 0.0f;
#pragma unroll
    for (int j = 0; j < 4; ++j) a1[j][0] = a1[j][1] = a1[j][2] = a1[j][3] = 0.0f;
#pragma unroll
    for (int j = 0; j < 2; ++j) a3[j][0] = a3[j][1] = a3[j][2] = a3[j][3] = 0.0f;
    const int rbeg = blockIdx.x * rows_per_block, rend = min(M, rbeg + rows_per_block);
    for (int t0 = rbeg; t0 < rend; t0 += WG_ROWS) {
        __syncthreads();
        // stage 64 rows (zero past the end): 8 BF16 = 16 bytes per copy
        for (int i = threadIdx.x; i < WG_ROWS * 8; i += blockDim.x) {
            const int r = i >> 3, c8 = (i & 7) * 8, row = t0 + r;
            const bool ok = row < rend;
            const uint4 z = make_uint4(0u, 0u, 0u, 0u);
            *reinterpret_cast<uint4*>(H1 + r * SL + c8) = ok ? *reinterpret_cast<const uint4*>(tb.h1 + (size_t)row * kHid + c8) : z;
            *reinterpret_cast<uint4*>(H2 + r * SL + c8) = ok ? *reinterpret_cast<const uint4*>(tb.h2 + (size_t)row * kHid + c8) : z;
            *reinterpret_cast<uint4*>(D1 + r * SL + c8) = ok ? *reinterpret_cast<const uint4*>(tb.dz1 + (size_t)row * kHid + c8) : z;
            *reinterpret_cast<uint4*>(D2 + r * SL + c8) = ok ? *reinterpret_cast<const uint4*>(tb.dz2 + (size_t)row * kHid + c8) : z;
            if (c8 < kFeat)
                *reinterpret_cast<uint4*>(X + r * SL + c8) =
                    ok ? *reinterpret_cast<const uint4*>(feat + (size_t)idx[row] * kFeat + c8) : z;
            if (c8 < 16)
                *reinterpret_cast<uint4*>(DO + r * SL + c8) = ok ? *reinterpret_cast<const uint4*>(tb.dout + (size_t)row * 16 + c8) : z;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < WG_ROWS / 16; ++ks) {
            const int m0 = 16 * ks;
            // A = D^T rows o0 = 16w .. 16w+15 (matrices: (m0,o0) (m0,o0+8) (m0+8,o0) (m0+8,o0+8))
            const int am = m0 + (q >> 1) * 8 + r8, ao = 16 * w + (q & 1) * 8;
            unsigned A2[4], A1[4];
            ldsm_x4_trans(A2, D2 + am * SL + ao);
            ldsm_x4_trans(A1, D1 + am * SL + ao);
            // B fragments for two n-tiles per load: matrices (m0,n0) (m0+8,n0) (m0,n0+8) (m0+8,n0+8)
            const int bm = m0 + (q & 1) * 8 + r8, bn = (q >> 1) * 8;
#pragma unroll
            for (int jp = 0; jp < 4; ++jp) {
                unsigned B[4];
                ldsm_x4_trans(B, H1 + bm * SL + 16 * jp + bn);
                mma16816(a2[2 * jp], A2, B[0], B[1]);
                mma16816(a2[2 * jp + 1], A2, B[2], B[3]);
            }
#pragma unroll
            for (int jp = 0; jp < 2; ++jp) {
                unsigned B[4];
                ldsm_x4_trans(B, X + bm * SL + 16 * jp + bn);
                mma16816(a1[2 * jp], A1, B[0], B[1]);
                mma16816(a1[2 * jp + 1], A1, B[2], B[3]);
            }
            // dW3: A = dO^T (16 rows, 8 used), B = H2 columns 16w .. 16w+15
            unsigned A3[4], B3[4];
            ldsm_x4_trans(A3, DO + am * SL + (q & 1) * 8);
            ldsm_x4_trans(B3, H2 + bm * SL + 16 * w + bn);
            mma16816(a3[0], A3, B3[0], B3[1]);
            mma16816(a3[1], A3, B3[2], B3[3]);
        }
    }
    // write this block's partial (C layout: rows g, g+8; columns 2tig, 2tig+1)
    float* bp = bpart + (size_t)blockIdx.x * kWgrad;
    const int o_lo = 16 * w + g, o_hi = o_lo + 8;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int c = 8 * j + 2 * tig;
        bp[o_lo * kFeat + c] = a1[j][0];
        bp[o_lo * kFeat + c + 1] = a1[j][1];
        bp[o_hi * kFeat + c] = a1[j][2];
        bp[o_hi * kFeat + c + 1] = a1[j][3];
    }
    float* bp2 = bp + kHid * kFeat;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int c = 8 * j + 2 * tig;
        bp2[o_lo * kHid + c] = a2[j][0];
        bp2[o_lo * kHid + c + 1] = a2[j][1];
        bp2[o_hi * kHid + c] = a2[j][2];
        bp2[o_hi * kHid + c + 1] = a2[j][3];
    }
    float* bp3 = bp2 + kHid * kHid;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const int c = 16 * w + 8 * j + 2 * tig;
        if (g < kOut) {
            bp3[g * kHid + c] = a3[j][0];
            bp3[g * kHid + c + 1] = a3[j][1];
        }
    }
}

// ---------------------------------------------------------------------------
// Training, part 3: sum the block and warp partials in a fixed order into
// grad; stats[0] = loss (sum over the warps' partials).
// Part 4: Adam on the FP32 master weights, refreshing the BF16 copy.
// Structurally zero parameters (W1 columns >= 24, W3/b3 rows >= 3) stay zero.
// ---------------------------------------------------------------------------
constexpr int RD_GROUPS = 16;  // partial groups per parameter column in mlp_reduce_kernel

// Block = 32 parameter columns x RD_GROUPS groups: group y sums partials
// y, y + RD_GROUPS, ... of its column (coalesced across the columns), then
// the groups are added in order -- a fixed order, so the sums are
// deterministic.  Column -1 is the loss.
__global__ void __launch_bounds__(32 * RD_GROUPS) mlp_reduce_kernel(int nblocks, const float* __restrict__ bpart,
                                                                   int nwarps, const float* __restrict__ wpart,
                                                                   float* __restrict__ grad,
                                                                   float* __restrict__ stats) {
    pdl_entry();
    __shared__ float part[RD_GROUPS][33];
    const int tx = threadIdx.x & 31, gy = threadIdx.x >> 5;
    const int i = blockIdx.x * 32 + tx - 1;
    const float* base = wpart;
    size_t stride = kWpart;
    int count = 0;
    if (i == -1) {
        count = nwarps;
    } else if (i < ob1) {
        base = bpart + (i - oW1), stride = kWgrad, count = nblocks;
    } else if (i < oW2) {
        base = wpart + 1 + (i - ob1), count = nwarps;
    } else if (i < ob2) {
        base = bpart + kHid * kFeat + (i - oW2), stride = kWgrad, count = nblocks;
    } else if (i < oW3) {
        base = wpart + 1 + kHid + (i - ob2), count = nwarps;
    } else if (i < ob3) {
        base = bpart + kHid * kFeat + kHid * kHid + (i - oW3), stride = kWgrad, count = nblocks;
    } else if (i < kParams) {
        base = wpart + 1 + 2 * kHid + (i - ob3), count = nwarps;
    }
    float sum = 0.0f;
    for (int k = gy; k < count; k += RD_GROUPS) sum += base[(size_t)k * stride];
    part[gy][tx] = sum;
    __syncthreads();
    if (gy == 0 && i < kParams) {
        float t = part[0][tx];
        for (int y = 1; y < RD_GROUPS; ++y) t += part[y][tx];
        if (i < 0)
            stats[0] = t;
        else
            grad[i] = t;
    }
}

__device__ __forceinline__ bool structural_zero(int i) {
    return (i < ob1 && (i % kFeat) >= 24) || (i >= oW3 && i < ob3 && (i - oW3) / kHid >= 3) || (i >= ob3 && i - ob3 >= 3);
}

__global__ void mlp_adam_kernel(const float* __restrict__ grad, float* __restrict__ p32, float* __restrict__ m1,
                                float* __restrict__ m2, unsigned short* __restrict__ w16, float lr, float beta1,
                                float beta2, float eps, float bc1, float bc2) {
    pdl_entry();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    float p = p32[i];
    if (structural_zero(i)) {
        p = 0.0f;
        m1[i] = 0.0f;
        m2[i] = 0.0f;
    } else {
        const float gsum = grad[i];
        const float a = beta1 * m1[i] + (1.0f - beta1) * gsum;
        const float b = beta2 * m2[i] + (1.0f - beta2) * (gsum * gsum);
        m1[i] = a;
        m2[i] = b;
        p = p - lr * ((a / bc1) / (sqrtf(b / bc2) + eps));
    }
    p32[i] = p;
    if (i < ob1) w16[qW1 + (i - oW1)] = f2bf(p);
    else if (i >= oW2 && i < ob2) w16[qW2 + (i - oW2)] = f2bf(p);
    else if (i >= oW3 && i < ob3) w16[qW3 + (i - oW3)] = f2bf(p);
}

__global__ void mlp_sync_bf16_kernel(const float* __restrict__ p32, unsigned short* __restrict__ w16) {
    pdl_entry();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    if (i < ob1) w16[qW1 + (i - oW1)] = f2bf(p32[i]);
    else if (i >= oW2 && i < ob2) w16[qW2 + (i - oW2)] = f2bf(p32[i]);
    else if (i >= oW3 && i < ob3) w16[qW3 + (i - oW3)] = f2bf(p32[i]);
}

}  // namespace sx

using namespace sx;

extern "C" int sx_mlp_param_count(void) { return kParams; }
extern "C" int sx_mlp_bf16_count(void) { return kW16; }

extern "C" int sx_warm_features(const float* x4, const float* y4, const float* c4, const float* fixed,
                                const int* adj_ptr, const int* adj, const float* Lref, int n_verts, float gx, float gy,
                                float gz, float dt, void* feat, float* y_pred4, void* stream) {
    SX_REQUIRE(n_verts >= 0, "sx_warm_features: n_verts < 0");
    if (n_verts == 0) return SX_OK;
    SX_REQUIRE(x4 && y4 && c4 && fixed && adj_ptr && adj && Lref && feat, "sx_warm_features: null pointer");
    launch(warm_features_kernel, grid_for(n_verts, 256), 256, 0, as_stream(stream), n_verts, (const float4*)x4,
           (const float4*)y4, (const float4*)c4, fixed, adj_ptr, (const int2*)adj, Lref, gx, gy, gz, dt,
           (unsigned short*)feat, (float4*)y_pred4);
    return check_launch("warm_features_kernel");
}

extern "C" int sx_warm_apply(const float* y_pred4, const float* out4, const float* fixed, const float* Lref,
                             int n_verts, float* y4, void* stream) {
    SX_REQUIRE(n_verts >= 0, "sx_warm_apply: n_verts < 0");
    if (n_verts == 0) return SX_OK;
    SX_REQUIRE(y_pred4 && out4 && fixed && Lref && y4, "sx_warm_apply: null pointer");
    launch(warm_apply_kernel, grid_for(n_verts, 256), 256, 0, as_stream(stream), n_verts, (const float4*)y_pred4,
           out4, fixed, Lref, (float4*)y4);
    return check_launch("warm_apply_kernel");
}

extern "C" int sx_warm_record(const float* y4, const float* y_pred4, const float* fixed, const float* Lref,
                              int n_verts, float* c4, float* target4, void* stream) {
    SX_REQUIRE(n_verts >= 0, "sx_warm_record: n_verts < 0");
    if (n_verts == 0) return SX_OK;
    SX_REQUIRE(y4 && y_pred4 && fixed && Lref && c4, "sx_warm_record: null pointer");
    launch(warm_record_kernel, grid_for(n_verts, 256), 256, 0, as_stream(stream), n_verts, (const float4*)y4,
           (const float4*)y_pred4, fixed, Lref, (float4*)c4, (float4*)target4);
    return check_launch("warm_record_kernel");
}

extern "C" int sx_warm_select(const double* res_warm3, const double* res_cold3, const float* y_pred4, float* y4,
                              int n_verts, int* flags2, void* stream) {
    SX_REQUIRE(n_verts > 0, "sx_warm_select: n_verts must be positive");
    SX_REQUIRE(res_warm3 && res_cold3 && y_pred4 && y4 && flags2, "sx_warm_select: null pointer");
    launch(warm_select_kernel, grid_for(n_verts, 256), 256, 0, as_stream(stream), n_verts, res_warm3, res_cold3,
           (const float4*)y_pred4, (float4*)y4, flags2);
    return check_launch("warm_select_kernel");
}

extern "C" int sx_mlp_forward_tc(const void* feat, int n_rows, const void* w16, const float* p32, float* out4,
                                 int* status, void* stream) {
    SX_REQUIRE(n_rows >= 0, "sx_mlp_forward_tc: n_rows < 0");
    if (n_rows == 0) return SX_OK;
    SX_REQUIRE(feat && w16 && p32 && out4 && status, "sx_mlp_forward_tc: null pointer");
    const int tiles = (n_rows + TC_ROWS - 1) / TC_ROWS;
    int dev = 0, sms = 0;
    SX_CUDA(cudaGetDevice(&dev));
    SX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // four CTAs per SM share the SM's 512 tensor-memory columns; unused dynamic
    // shared memory keeps a fifth from becoming resident and waiting in
    // tcgen05.alloc for a column range
    static bool attr = false;
    if (!attr) {
        SX_CUDA(cudaFuncSetAttribute(mlp_forward_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_PAD_SMEM));
        attr = true;
    }
    const int blocks = tiles < 4 * sms ? tiles : 4 * sms;
    launch(mlp_forward_tc_kernel, blocks, TC_THREADS, TC_PAD_SMEM, as_stream(stream), n_rows,
           (const unsigned short*)feat, (const unsigned short*)w16, p32, out4, status);
    return check_launch("mlp_forward_tc_kernel");
}

extern "C" int sx_mlp_forward(const void* feat, int n_rows, const void* w16, const float* p32, float* out4,
                              void* stream) {
    SX_REQUIRE(n_rows >= 0, "sx_mlp_forward: n_rows < 0");
    if (n_rows == 0) return SX_OK;
    SX_REQUIRE(feat && w16 && p32 && out4, "sx_mlp_forward: null pointer");
    const int tiles = (n_rows + 15) / 16;
    int blocks = (tiles + MLP_BLOCK / 32 - 1) / (MLP_BLOCK / 32);
    if (blocks > 152 * 16) blocks = 152 * 16;
    launch(mlp_forward_kernel, blocks, MLP_BLOCK, 0, as_stream(stream), n_rows, (const unsigned short*)feat,
           (const unsigned short*)w16, p32, out4);
    return check_launch("mlp_forward_kernel");
}

// Training workspace: per row 4x64 + 16 BF16, per warp kWpart floats, per
// weight-gradient block kWgrad floats, then the gradient (kParams floats).
static void train_shape(int M, int* fb_blocks, int* nwarps, int* wg_blocks, int* rows_per_block) {
    const int tiles = (M + 15) / 16;
    int b = (tiles + MLP_BLOCK / 32 - 1) / (MLP_BLOCK / 32);
    if (b > 152 * 8) b = 152 * 8;
    *fb_blocks = b;
    *nwarps = b * (MLP_BLOCK / 32);
    // about two blocks per SM, whole 64-row tiles each
    const int rpb = ((M + 152 * 2 - 1) / (152 * 2) + WG_ROWS - 1) / WG_ROWS * WG_ROWS;
    const int wg = (M + rpb - 1) / rpb;
    *wg_blocks = wg;
    *rows_per_block = rpb;
}

struct TrainWs {
    TrainBuf tb;
    float* bpart;
    float* grad;
    int fb, nw, wg, rpb;
};

static TrainWs train_ws(void* ws, int n_rows) {
    TrainWs w;
    train_shape(n_rows, &w.fb, &w.nw, &w.wg, &w.rpb);
    char* p = (char*)ws;
    const size_t rows = (size_t)n_rows;
    w.tb.h1 = (unsigned short*)p;
    w.tb.h2 = w.tb.h1 + rows * kHid;
    w.tb.dz1 = w.tb.h2 + rows * kHid;
    w.tb.dz2 = w.tb.dz1 + rows * kHid;
    w.tb.dout = w.tb.dz2 + rows * kHid;
    w.tb.wpart = (float*)(p + rows * (4 * kHid + 16) * 2);
    w.bpart = w.tb.wpart + (size_t)w.nw * kWpart;
    w.grad = w.bpart + (size_t)w.wg * kWgrad;
    return w;
}

extern "C" size_t sx_mlp_train_workspace_bytes(int max_rows) {
    int fb, nw, wg, rpb;
    const int M = max_rows > 0 ? max_rows : 1;
    train_shape(M, &fb, &nw, &wg, &rpb);
    return (size_t)M * (4 * kHid + 16) * 2 + (size_t)nw * kWpart * 4 + (size_t)wg * kWgrad * 4 +
           (size_t)kParams * 4 + 256;
}

static int mlp_grad_launches(const TrainWs& w, const void* feat, const float* target4, const int* idx, int n_rows,
                             int n_valid, const void* w16, const float* p32, float* grad, float* stats,
                             cudaStream_t s) {
    launch(mlp_train_fwd_bwd_kernel, w.fb, MLP_BLOCK, 0, s, n_rows, idx, (const unsigned short*)feat,
           (const float4*)target4, 1.0f / (float)n_valid, (const unsigned short*)w16, p32, w.tb);
    int rc = check_launch("mlp_train_fwd_bwd_kernel");
    if (rc) return rc;
    launch(mlp_wgrad_kernel, w.wg, MLP_BLOCK, 0, s, n_rows, w.rpb, idx, (const unsigned short*)feat, w.tb, w.bpart);
    rc = check_launch("mlp_wgrad_kernel");
    if (rc) return rc;
    launch(mlp_reduce_kernel, (kParams + 1 + 31) / 32, 32 * RD_GROUPS, 0, s, w.wg, (const float*)w.bpart, w.nw,
           (const float*)w.tb.wpart, grad, stats);
    return check_launch("mlp_reduce_kernel");
}

extern "C" int sx_mlp_gradients(const void* feat, const float* target4, const int* idx, int n_rows, int n_valid,
                                const void* w16, const float* p32, float* grad, float* stats, void* ws,
                                size_t ws_bytes, void* stream) {
    SX_REQUIRE(n_rows > 0 && n_valid > 0, "sx_mlp_gradients: bad sizes");
    SX_REQUIRE(feat && target4 && idx && w16 && p32 && grad && stats && ws, "sx_mlp_gradients: null pointer");
    SX_REQUIRE(ws_bytes >= sx_mlp_train_workspace_bytes(n_rows), "sx_mlp_gradients: workspace too small");
    const TrainWs w = train_ws(ws, n_rows);
    return mlp_grad_launches(w, feat, target4, idx, n_rows, n_valid, w16, p32, grad, stats, as_stream(stream));
}

extern "C" int sx_mlp_train_step(const void* feat, const float* target4, const int* idx, int n_rows, int n_valid,
                                 void* w16, float* p32, float* adam_m, float* adam_v, float lr, float beta1,
                                 float beta2, float eps, int step, float* stats, void* ws, size_t ws_bytes,
                                 void* stream) {
    SX_REQUIRE(n_rows > 0 && n_valid > 0 && step >= 1, "sx_mlp_train_step: bad sizes");
    SX_REQUIRE(feat && target4 && idx && w16 && p32 && adam_m && adam_v && stats && ws,
               "sx_mlp_train_step: null pointer");
    SX_REQUIRE(ws_bytes >= sx_mlp_train_workspace_bytes(n_rows), "sx_mlp_train_step: workspace too small");
    const TrainWs w = train_ws(ws, n_rows);
    cudaStream_t s = as_stream(stream);
    int rc = mlp_grad_launches(w, feat, target4, idx, n_rows, n_valid, w16, p32, w.grad, stats, s);
    if (rc) return rc;
    const float bc1 = 1.0f - powf(beta1, (float)step), bc2 = 1.0f - powf(beta2, (float)step);
    launch(mlp_adam_kernel, grid_for(kParams, 256), 256, 0, s, (const float*)w.grad, p32, adam_m, adam_v,
           (unsigned short*)w16, lr, beta1, beta2, eps, bc1, bc2);
    return check_launch("mlp_adam_kernel");
}

extern "C" int sx_mlp_sync_bf16(const float* p32, void* w16, void* stream) {
    SX_REQUIRE(p32 && w16, "sx_mlp_sync_bf16: null pointer");
    launch(mlp_sync_bf16_kernel, grid_for(kParams, 256), 256, 0, as_stream(stream), p32, (unsigned short*)w16);
    return check_launch("mlp_sync_bf16_kernel");
}
