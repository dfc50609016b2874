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

template <int G, bool BY, bool FAST, bool CHECK, bool YLDG>
__device__ __forceinline__ float4 sweep_vertex(int v, const float4* __restrict__ x4, const float4* yin,
                                               const float* __restrict__ fixed, const int* __restrict__ ptr,
                                               const int2* __restrict__ adj, float ks, float kb, int bend_y,
                                               float* c2) {
    return sweep_vertex_src<G, BY, FAST, CHECK, YLDG>(v, x4, yin, fixed, __ldg(ptr + v), __ldg(ptr + v + 1),
                                                      AdjInt2{adj}, ks, kb, bend_y, c2);
}

}  // namespace sx
