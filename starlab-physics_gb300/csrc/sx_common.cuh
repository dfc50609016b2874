// Shared device helpers for the starxpbd CUDA library (sm_103a).
//
// Numerics: the library is compiled with -fmad=false, -prec-div=true and
// -prec-sqrt=true, so every float expression below is evaluated as written in
// IEEE float32 (no FMA contraction, correctly rounded '/' and sqrtf).  Vector
// helpers fix the evaluation order: dot = (x*x' + y*y') + z*z'.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/starxpbd.h"

namespace sx {

// ---- error plumbing ---------------------------------------------------------
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* what);
inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }
int check_launch(const char* what);

#define SX_REQUIRE(cond, ...)              \
    do {                                   \
        if (!(cond)) {                     \
            ::sx::set_error(__VA_ARGS__);  \
            return SX_ERR_ARG;             \
        }                                  \
    } while (0)

#define SX_CUDA(call)                                                 \
    do {                                                              \
        cudaError_t _e = (call);                                      \
        if (_e != cudaSuccess) return ::sx::cuda_status(_e, #call);   \
    } while (0)

inline int grid_for(long long n, int block) {
    long long g = (n + block - 1) / block;
    return (int)(g < 1 ? 1 : g);
}

// Blocks of `kernel` (block threads, no dynamic shared memory) that the
// current device keeps resident at once: SMs x active blocks per SM.  Queried
// once per kernel (keyed by its address) and cached.
int resident_blocks_of(const void* kernel, int block);
template <typename K>
inline int resident_blocks(K kernel, int block) {
    return resident_blocks_of(reinterpret_cast<const void*>(kernel), block);
}

// Every kernel launch of the library goes through launch(), which counts it
// (sx_kernel_launches() reports the running total for benchmarks) and, unless
// switched off, makes it a programmatic dependent launch: the kernel may be
// scheduled while the previous kernel on the stream is still finishing.
// Every kernel of the library therefore starts with pdl_entry(), whose
// griddepcontrol.wait returns once the previous grid has completed and its
// writes are visible (before the kernel touches any memory), and whose
// launch_dependents lets the kernel's own successor be scheduled early.
// Launches recorded into the body of a device-side loop (sx_loop_begin ..
// sx_loop_end) are plain launches.
void note_launch();
bool pdl_enabled();
template <typename... KArgs, typename... A>
inline void launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A... args) {
    if (!pdl_enabled()) {
        kernel<<<grid, block, smem, s>>>(args...);
    } else {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = grid;
        cfg.blockDim = block;
        cfg.dynamicSmemBytes = smem;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
    }
    note_launch();
}
__device__ __forceinline__ void pdl_entry() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ---- float3 arithmetic with fixed evaluation order ----------------------------
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 mk(float4 a) { return V3{a.x, a.y, a.z}; }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 scale(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3 neg(V3 a) { return V3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ V3 vmin(V3 a, V3 b) { return V3{fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)}; }
__device__ __forceinline__ V3 vmax(V3 a, V3 b) { return V3{fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)}; }
__device__ __forceinline__ bool overlap(V3 a0, V3 a1, V3 b0, V3 b1) {
    return a0.x <= b1.x && a1.x >= b0.x && a0.y <= b1.y && a1.y >= b0.y && a0.z <= b1.z && a1.z >= b0.z;
}

// float -> int32: truncate toward zero, saturate, NaN -> 0 (cvt.rzi.s32.f32)
__device__ __forceinline__ int f2i_sat(float f) { return __float2int_rz(f); }

// ---- contact accumulation in 64-bit fixed point (40 fractional bits) -----------
constexpr double kFixScale = 1099511627776.0;      // 2^40
constexpr double kFixInv = 1.0 / 1099511627776.0;  // 2^-40
constexpr double kFixMax = 4611686018427387904.0;  // 2^62
__device__ __forceinline__ long long to_fix(float c, int* bad) {
    double d = (double)c * kFixScale;
    if (d != d) { *bad = 1; return 0; }
    if (d >= kFixMax) { *bad = 1; return 4611686018427387904LL; }
    if (d <= -kFixMax) { *bad = 1; return -4611686018427387904LL; }
    return __double2ll_rn(d);
}
__device__ __forceinline__ float from_fix(long long a) { return __double2float_rn(__ll2double_rn(a) * kFixInv); }

// In-place scan (exclusive or inclusive) of n uint32 on one block (sx_lbvh.cu).
int scan_u32(unsigned* data, int n, int inclusive, cudaStream_t s);

// ---- cell grid ----------------------------------------------------------------
constexpr int kGridRes = 32;
constexpr int kNumCells = kGridRes * kGridRes * kGridRes;
// grid descriptor of a cell-BVH build: 8 floats (cell size xyz, max leaf
// overhang xyz, 2 unused) then 1024 occupancy words (bit z of word x*32 + y:
// cell (x, y, z) holds faces)
constexpr int kGridHeader = 8;
constexpr int kGridWords = kGridHeader + kGridRes * kGridRes;

// ---- convergence control -------------------------------------------------------
// conv[0] = stop iteration of the current substep: -1 while it has not
// converged, else the iteration j (a multiple of the check interval
// conv[6], which is even) whose checked sweep found the residual of its input
// at or below the tolerance.  Iterations j .. j + conv[6] - 1 still run (the
// block of an even number of sweeps keeps the y ping-pong in step); every
// kernel of a later iteration returns at once.  conv == nullptr: nothing is
// skipped.
__device__ __forceinline__ bool iteration_skipped(const int* conv, int iter) {
    if (conv == nullptr) return false;
    const volatile int* c = conv;
    const int stop = c[0];
    return stop >= 0 && iter >= stop + c[6];
}

}  // namespace sx
