// Colour-ordered Gauss-Seidel sweep over the stretch springs and bending pairs.
//
// The reference colours its constraint graph (framework/utilities/
// graph_coloring.py:131-201) for a parallel Gauss-Seidel solver that it marks
// as work in progress (README.md:20-22); its XPBD solver only runs the Jacobi
// sweep (XPBD.py:141-184, :384-387).  This file is that consumer: the springs
// and bending pairs are coloured together as one edge list (two constraints
// conflict when they share a vertex), stored in colour order, and each colour
// is one launch in which every thread projects one constraint and writes both
// endpoints in place -- no two constraints of a colour share a vertex, so the
// launch has no races and its result does not depend on thread order.
//
// Per constraint (v0, v1) the projection is the reference's stretch step
// evaluated on the current positions: x10 = y0 - y1, lij = |x10|, C = lij - l0,
// n = x10 * (1/lij), schur = (w0 + w1) * (n.n), ld = k*C / (k*schur + 1),
// y0 -= (w0*ld)*n and y1 += (w1*ld)*n with w = fixed * m_inv (the .w of y4).
// Unlike the Jacobi update (XPBD.py:384-387) the correction is applied at once,
// not averaged over the vertex's constraint count.
#include "sx_common.cuh"

namespace sx {

__global__ void __launch_bounds__(256) gs_color_kernel(float4* y, const int4* __restrict__ cons, int begin, int end,
                                                       float k_spring, float k_bend) {
    pdl_entry();
    const int i = begin + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= end) return;
    const int4 c = __ldg(cons + i);
    const int v0 = c.x, v1 = c.y & 0x7fffffff;
    const float k = c.y < 0 ? k_bend : k_spring;
    const float rest = __int_as_float(c.z);
    const float4 p0 = y[v0], p1 = y[v1];
    const V3 x10 = sub(mk(p0), mk(p1));
    const float lij = sqrtf(dot(x10, x10));
    const float C = lij - rest;
    const float inv = 1.0f / lij;
    const V3 n = scale(inv, x10);
    const float schur = (p0.w + p1.w) * dot(n, n);
    const float ld = (k * C) / (k * schur + 1.0f);
    const V3 q0 = sub(mk(p0), scale(p0.w * ld, n));
    const V3 q1 = add(mk(p1), scale(p1.w * ld, n));
    y[v0] = make_float4(q0.x, q0.y, q0.z, p0.w);
    y[v1] = make_float4(q1.x, q1.y, q1.z, p1.w);
}

__global__ void gs_pack_kernel(int E, int B, const int* __restrict__ edges, const float* __restrict__ l0,
                               const int* __restrict__ bend, const float* __restrict__ bend_l0,
                               const int* __restrict__ sorted, int4* cons, int* bad) {
    pdl_entry();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= E + B) return;
    const int id = sorted[i];
    if (id < 0 || id >= E + B) {
        atomicOr(bad, 1);
        cons[i] = make_int4(0, 0, 0, 0);
        return;
    }
    if (id < E)
        cons[i] = make_int4(edges[2 * id], edges[2 * id + 1], __float_as_int(l0[id]), id);
    else
        cons[i] = make_int4(bend[2 * (id - E)], bend[2 * (id - E) + 1] | (int)0x80000000,
                            __float_as_int(bend_l0[id - E]), id);
}

}  // namespace sx

using namespace sx;

extern "C" int sx_gs_pack(const int* edges, const float* l0, int E, const int* bend, const float* bend_l0, int B,
                          const int* sorted, int* cons, int* bad, void* stream) {
    SX_REQUIRE(E >= 0 && B >= 0, "sx_gs_pack: negative count");
    SX_REQUIRE(E + B == 0 || (sorted && cons && bad), "sx_gs_pack: null pointer");
    SX_REQUIRE(E == 0 || (edges && l0), "sx_gs_pack: null edge arrays");
    SX_REQUIRE(B == 0 || (bend && bend_l0), "sx_gs_pack: null bending arrays");
    if (E + B == 0) return SX_OK;
    launch(gs_pack_kernel, dim3(grid_for(E + B, 256)), dim3(256), 0, as_stream(stream), E, B, edges, l0, bend,
           bend_l0, sorted, reinterpret_cast<int4*>(cons), bad);
    return check_launch("gs_pack_kernel");
}

extern "C" int sx_gs_sweep(float* y4, const int* cons, const int* colour_start, int n_colors, float k_spring,
                           float k_bend, void* stream) {
    SX_REQUIRE(n_colors >= 0, "sx_gs_sweep: negative colour count");
    SX_REQUIRE(n_colors == 0 || (y4 && cons && colour_start), "sx_gs_sweep: null pointer");
    for (int c = 0; c < n_colors; ++c)
        SX_REQUIRE(colour_start[c] >= 0 && colour_start[c + 1] >= colour_start[c],
                   "sx_gs_sweep: colour_start must be non-decreasing from 0");
    cudaStream_t s = as_stream(stream);
    for (int c = 0; c < n_colors; ++c) {
        const int b = colour_start[c], e = colour_start[c + 1];
        if (e == b) continue;
        launch(gs_color_kernel, dim3(grid_for(e - b, 256)), dim3(256), 0, s, reinterpret_cast<float4*>(y4),
               reinterpret_cast<const int4*>(cons), b, e, k_spring, k_bend);
    }
    return check_launch("gs_color_kernel");
}
