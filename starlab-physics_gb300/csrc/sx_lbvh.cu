// LBVH broad phase: Morton codes, stable LSD radix sort, Karras 2012 hierarchy,
// single-launch bottom-up refit and stack traversal, for the reference's 32^3
// cell-grid BVH (framework/collision/lbvh_cell.py, class LBVH_CELL) and for a
// face-level LBVH over triangle soups.
#include <cuda/atomic>
#include <mutex>

#include "sx_common.cuh"

namespace sx {

// ---------------------------------------------------------------------------
// Morton codes (lbvh_cell.py:87-102, :139-148)
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long expand_bits(unsigned long long v) {
    v = (v | (v << 16)) & 0x030000FFull;
    v = (v | (v << 8)) & 0x0300F00Full;
    v = (v | (v << 4)) & 0x030C30C3ull;
    v = (v | (v << 2)) & 0x09249249ull;
    return v;
}
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
__device__ __forceinline__ unsigned morton3d(float x, float y, float z) {
    x = clampf(x * 1024.0f, 0.0f, 1023.0f);
    y = clampf(y * 1024.0f, 0.0f, 1023.0f);
    z = clampf(z * 1024.0f, 0.0f, 1023.0f);
    unsigned long long xx = expand_bits((unsigned long long)x), yy = expand_bits((unsigned long long)y),
                       zz = expand_bits((unsigned long long)z);
    return (unsigned)(xx | (yy << 1) | (zz << 2));
}
__device__ __forceinline__ unsigned morton_of(V3 p, V3 lo, V3 hi) {
    float x = (p.x - lo.x) / (hi.x - lo.x);
    float y = (p.y - lo.y) / (hi.y - lo.y);
    float z = (p.z - lo.z) / (hi.z - lo.z);
    return morton3d(clampf(x, 0.f, 1.f), clampf(y, 0.f, 1.f), clampf(z, 0.f, 1.f));
}

__device__ __forceinline__ V3 cell_size_of(const float* box6) {
    return V3{(box6[3] - box6[0]) / (float)kGridRes, (box6[4] - box6[1]) / (float)kGridRes,
              (box6[5] - box6[2]) / (float)kGridRes};
}
// assign_cell_centers (lbvh_cell.py:105-120)
__device__ __forceinline__ V3 cell_center(int i, V3 cs, V3 lo) {
    int x0 = i / (kGridRes * kGridRes), y0 = (i % (kGridRes * kGridRes)) / kGridRes, z0 = i % kGridRes;
    V3 p{cs.x * (float)x0 + 0.5f * cs.x, cs.y * (float)y0 + 0.5f * cs.y, cs.z * (float)z0 + 0.5f * cs.z};
    return add(p, lo);
}

__global__ void cell_morton_kernel(unsigned* codes, int* ids) {
    pdl_entry();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kNumCells) return;
    const float box[6] = {0.f, 0.f, 0.f, 1e3f, 1e3f, 1e3f};
    V3 lo{0.f, 0.f, 0.f}, hi{1e3f, 1e3f, 1e3f};
    V3 cs = cell_size_of(box);
    codes[i] = morton_of(cell_center(i, cs, lo), lo, hi);
    ids[i] = i;
}

__global__ void face_morton_kernel(int F, const float4* __restrict__ mn4, const float4* __restrict__ mx4,
                                   const float* __restrict__ box6, unsigned* codes, int* ids) {
    pdl_entry();
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    V3 lo{box6[0], box6[1], box6[2]}, hi{box6[3], box6[4], box6[5]};
    V3 c = scale(0.5f, add(mk(mx4[f]), mk(mn4[f])));
    codes[f] = morton_of(c, lo, hi);
    ids[f] = f;
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits.
//   upsweep : per-tile digit histogram -> hist[digit * nblocks + block]
//   scan    : one block per digit scans its column (exclusive over the tiles,
//             in tile order) and writes the digit's total
//   scatter : each tile takes its digit bases (exclusive scan of the 256
//             totals + its column offset); each warp owns a contiguous 256-key
//             slice of the tile and ranks its keys within their digit in input
//             order (__match_any_sync, warp-private counters), so the order is
//             stable with three block barriers per tile.
// ---------------------------------------------------------------------------
constexpr int RS_BLOCK = 256;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_BLOCK * RS_ITEMS;
constexpr int RS_WARPS = RS_BLOCK / 32;

__global__ void __launch_bounds__(RS_BLOCK) rs_upsweep(const unsigned* __restrict__ keys, int n, int shift,
                                                       unsigned dmask, unsigned* __restrict__ hist, int nblocks) {
    pdl_entry();
    __shared__ unsigned cnt[256];
    const int tid = threadIdx.x;
    cnt[tid] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * RS_TILE;
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        long long idx = base + r * RS_BLOCK + tid;
        if (idx < n) atomicAdd(&cnt[(keys[idx] >> shift) & dmask], 1u);
    }
    __syncthreads();
    hist[(size_t)tid * nblocks + blockIdx.x] = cnt[tid];
}

// Exclusive scan of one value per thread over a 256-thread block; returns the
// block total through *total.
__device__ __forceinline__ unsigned block256_excl_scan(unsigned v, unsigned* total) {
    __shared__ unsigned wsum[RS_WARPS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    unsigned before = 0, all = 0;
#pragma unroll
    for (int k = 0; k < RS_WARPS; ++k) {
        before += k < w ? wsum[k] : 0u;
        all += wsum[k];
    }
    __syncthreads();
    *total = all;
    return before + incl - v;
}

// Block d: exclusive scan of hist[d * nblocks .. (d + 1) * nblocks) in place,
// the column total to tot[d].
__global__ void __launch_bounds__(RS_BLOCK) rs_digit_scan(unsigned* __restrict__ hist, int nblocks,
                                                          unsigned* __restrict__ tot) {
    pdl_entry();
    unsigned* col = hist + (size_t)blockIdx.x * nblocks;
    unsigned carry = 0;
    for (int b0 = 0; b0 < nblocks; b0 += RS_BLOCK) {
        const int b = b0 + threadIdx.x;
        const unsigned v = b < nblocks ? col[b] : 0u;
        unsigned sum;
        const unsigned ex = block256_excl_scan(v, &sum);
        if (b < nblocks) col[b] = carry + ex;
        carry += sum;
    }
    if (threadIdx.x == 0) tot[blockIdx.x] = carry;
}

// Single-block scan over n entries (exclusive or inclusive), 1024 threads, in
// segments of 32768 staged in (dynamic) shared memory: one coalesced load of
// the segment, each thread sums 32 consecutive entries (one padding word per
// 32 keeps those reads on distinct banks), a block scan of the sums (warp
// shuffles, then the 32 warp totals), each thread rewrites its 32, one
// coalesced store; the running total carries into the next segment.
constexpr int SCAN_SEG = 32768;
constexpr int SCAN_PER = SCAN_SEG / 1024;
constexpr size_t SCAN_SMEM = (size_t)(SCAN_SEG + SCAN_SEG / 32) * 4;

__device__ __forceinline__ int scan_slot(int i) { return i + (i >> 5); }

__global__ void __launch_bounds__(1024) scan_single_block(unsigned* data, int n, int inclusive) {
    pdl_entry();
    extern __shared__ unsigned seg[];
    __shared__ unsigned wsum[32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    unsigned carry = 0;
    for (int s0 = 0; s0 < n; s0 += SCAN_SEG) {
        const int m = min(SCAN_SEG, n - s0);
#pragma unroll 8
        for (int i = tid; i < SCAN_SEG; i += 1024) seg[scan_slot(i)] = i < m ? data[s0 + i] : 0u;
        __syncthreads();
        unsigned sum = 0;
#pragma unroll
        for (int k = 0; k < SCAN_PER; ++k) sum += seg[scan_slot(tid * SCAN_PER + k)];
        unsigned incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) wsum[w] = incl;
        __syncthreads();
        unsigned before = 0, total = 0;
        for (int k = 0; k < 32; ++k) {
            before += k < w ? wsum[k] : 0u;
            total += wsum[k];
        }
        unsigned run = carry + before + incl - sum;
#pragma unroll
        for (int k = 0; k < SCAN_PER; ++k) {
            const int j = scan_slot(tid * SCAN_PER + k);
            const unsigned x = seg[j];
            seg[j] = inclusive ? run + x : run;
            run += x;
        }
        __syncthreads();
#pragma unroll 8
        for (int i = tid; i < m; i += 1024) data[s0 + i] = seg[scan_slot(i)];
        carry += total;
        __syncthreads();
    }
}

// The shared-memory limit is raised once per process; sx_cell_bvh_init does it
// first, outside any stream capture.
static cudaError_t scan_smem_attr() {
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(scan_single_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SCAN_SMEM);
    });
    return attr;
}

static int launch_scan_single_block(unsigned* data, int n, int inclusive, cudaStream_t s) {
    const cudaError_t attr = scan_smem_attr();
    if (attr != cudaSuccess) return cuda_status(attr, "cudaFuncSetAttribute(scan_single_block)");
    launch(scan_single_block, 1, 1024, SCAN_SMEM, s, data, n, inclusive);
    return check_launch("scan_single_block");
}

__global__ void __launch_bounds__(RS_BLOCK) rs_scatter(const unsigned* __restrict__ kin,
                                                       const int* __restrict__ vin, unsigned* __restrict__ kout,
                                                       int* __restrict__ vout, int n, int shift, unsigned dmask,
                                                       const unsigned* __restrict__ hist,
                                                       const unsigned* __restrict__ tot, int nblocks) {
    pdl_entry();
    __shared__ unsigned s_off[RS_WARPS][256];
    __shared__ unsigned s_gbase[256], s_lbase[256];
    __shared__ unsigned s_key[RS_TILE];
    __shared__ int s_val[RS_TILE];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    unsigned all;
    const unsigned digit_base = block256_excl_scan(tot[tid], &all) + hist[(size_t)tid * nblocks + blockIdx.x];
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) s_off[w][tid] = 0;
    __syncthreads();
    // warp `warp` owns keys [tile + warp * 256, tile + (warp + 1) * 256)
    const long long tile = (long long)blockIdx.x * RS_TILE;
    const long long base = tile + warp * (RS_ITEMS * 32);
    unsigned key[RS_ITEMS], rank[RS_ITEMS];
    int val[RS_ITEMS];
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        const long long idx = base + r * 32 + lane;
        key[r] = idx < n ? kin[idx] : 0u;
        val[r] = idx < n ? vin[idx] : 0;
    }
    unsigned* cnt = s_off[warp];
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        const bool valid = base + r * 32 + lane < n;
        const unsigned digit = valid ? ((key[r] >> shift) & dmask) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, digit);
        const unsigned before = valid ? cnt[digit] : 0u;
        rank[r] = before + __popc(peers & lt_mask);
        __syncwarp();
        if (valid && (__ffs(peers) - 1) == lane) cnt[digit] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // per digit: the tile's count, its offset in the tile's digit order, and
    // each warp's offset within it
    unsigned tsum = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) tsum += s_off[w][tid];
    const unsigned lbase = block256_excl_scan(tsum, &all);
    s_lbase[tid] = lbase;
    s_gbase[tid] = digit_base;
    unsigned run = lbase;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) {
        const unsigned c = s_off[w][tid];
        s_off[w][tid] = run;
        run += c;
    }
    __syncthreads();
    // the tile in digit order (stable within a digit) in shared memory ...
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        if (base + r * 32 + lane < n) {
            const unsigned lp = cnt[(key[r] >> shift) & dmask] + rank[r];
            s_key[lp] = key[r];
            s_val[lp] = val[r];
        }
    }
    __syncthreads();
    // ... written out so that consecutive threads fill consecutive slots of
    // each digit's run
    const int count = (int)min((long long)RS_TILE, (long long)n - tile);
    for (int i = tid; i < count; i += RS_BLOCK) {
        const unsigned k = s_key[i];
        const unsigned d = (k >> shift) & dmask;
        const unsigned g = s_gbase[d] + ((unsigned)i - s_lbase[d]);
        kout[g] = k;
        vout[g] = s_val[i];
    }
}

int scan_u32(unsigned* data, int n, int inclusive, cudaStream_t s) {
    if (n <= 0) return SX_OK;
    return launch_scan_single_block(data, n, inclusive, s);
}

static inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }
static inline int rs_nblocks(int n) { return n <= 0 ? 1 : (n + RS_TILE - 1) / RS_TILE; }
static size_t rs_ws_bytes(int n) {
    size_t nn = (size_t)(n > 0 ? n : 1);
    return align256(nn * 4) * 2 + align256((size_t)256 * rs_nblocks(n) * 4) + align256(256 * 4);
}

static int radix_sort(unsigned* keys, int* vals, int n, int bits, void* ws, size_t ws_bytes, cudaStream_t s) {
    SX_REQUIRE(bits >= 1 && bits <= 32, "radix sort: bits must be in [1, 32]");
    if (n <= 1) return SX_OK;
    SX_REQUIRE(ws && ws_bytes >= rs_ws_bytes(n), "radix sort: workspace too small (%zu < %zu)", ws_bytes,
               rs_ws_bytes(n));
    char* p = (char*)ws;
    unsigned* kalt = (unsigned*)p;
    p += align256((size_t)n * 4);
    int* valt = (int*)p;
    p += align256((size_t)n * 4);
    unsigned* hist = (unsigned*)p;
    const int nb = rs_nblocks(n);
    p += align256((size_t)256 * nb * 4);
    unsigned* tot = (unsigned*)p;
    const int passes = (bits + 7) / 8;
    unsigned* ki = keys;
    int* vi = vals;
    unsigned* ko = kalt;
    int* vo = valt;
    for (int pass = 0; pass < passes; ++pass) {
        const int shift = 8 * pass;
        // the last digit keeps only the key bits below `bits`: keys are ordered
        // by their low `bits` bits, higher bits ride along unsorted
        const int width = bits - shift < 8 ? bits - shift : 8;
        const unsigned dmask = (1u << width) - 1u;
        launch(rs_upsweep, nb, RS_BLOCK, 0, s, ki, n, shift, dmask, hist, nb);
        launch(rs_digit_scan, 256, RS_BLOCK, 0, s, hist, nb, tot);
        launch(rs_scatter, nb, RS_BLOCK, 0, s, ki, vi, ko, vo, n, shift, dmask, (const unsigned*)hist,
               (const unsigned*)tot, nb);
        unsigned* tk = ki; ki = ko; ko = tk;
        int* tv = vi; vi = vo; vo = tv;
    }
    if (ki != keys) {
        SX_CUDA(cudaMemcpyAsync(keys, ki, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
        SX_CUDA(cudaMemcpyAsync(vals, vi, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
    }
    return check_launch("radix_sort");
}

// ---------------------------------------------------------------------------
// Karras 2012 hierarchy (lbvh_cell.py:256-336, :384-430)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int kdelta(int i, long long j, int n, const unsigned* c, int tie) {
    if (j > n - 1 || j < 0) return -1;
    unsigned x = c[i] ^ c[(int)j];
    if (x == 0) return tie ? 32 + __clz(i ^ (int)j) : 32;
    return __clz(x);
}

__global__ void karras_kernel(int n, const unsigned* __restrict__ c, int tie, int* child_a, int* child_b,
                              int* range_l, int* range_r, int* parent) {
    pdl_entry();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) parent[0] = -1;
    if (i >= n - 1) return;
    // determine_range
    int dl = kdelta(i, (long long)i - 1, n, c, tie), dr = kdelta(i, (long long)i + 1, n, c, tie);
    int d = 1, dmin = dl;
    if (dr < dl) { d = -1; dmin = dr; }
    long long lmax = 2;
    while (lmax < 4LL * n && kdelta(i, (long long)i + lmax * d, n, c, tie) > dmin) lmax <<= 2;
    long long l = 0;
    for (long long t = lmax / 2; t > 0; t /= 2) {
        long long j = (long long)i + (l + t) * d;
        int dd = (j >= 0 && j < n) ? kdelta(i, j, n, c, tie) : -1;
        if (dd > dmin) l += t;
    }
    int s = i, e = (int)(i + l * d);
    if (d == -1) { s = (int)(i + l * d); e = i; }
    // find_split
    int split;
    if (c[s] == c[e] && !tie) {
        split = (s + e) / 2;
    } else {
        int common = kdelta(s, e, n, c, tie);
        split = s;
        int step = e - s;
        while (step > 1) {
            step = (step + 1) / 2;
            int ns = split + step;
            if (ns < e && kdelta(s, ns, n, c, tie) > common) split = ns;
        }
    }
    int left = split, right = split + 1;
    if (split == s) left += n - 1;
    if (right == e) right += n - 1;
    child_a[i] = left;
    child_b[i] = right;
    range_l[i] = s;
    range_r[i] = e;
    parent[left] = i;
    parent[right] = i;
}

// ---------------------------------------------------------------------------
// Cell-grid BVH build (LBVH_CELL.build, lbvh_cell.py:637-653)
// ---------------------------------------------------------------------------
__global__ void face_cell_kernel(int F, const float4* __restrict__ mn4, const float4* __restrict__ mx4,
                                 const float* __restrict__ box6, unsigned* keys, int* ids, unsigned* counts,
                                 float* grid8) {
    pdl_entry();
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    V3 lo{box6[0], box6[1], box6[2]};
    V3 cs = cell_size_of(box6);
    if (f == 0) {
        grid8[0] = cs.x;
        grid8[1] = cs.y;
        grid8[2] = cs.z;
        grid8[3] = grid8[4] = grid8[5] = 0.0f;  // max leaf overhang, raised by the leaf kernel
        grid8[6] = grid8[7] = 0.0f;
    }
    if (f >= F) return;
    V3 c = scale(0.5f, add(mk(mn4[f]), mk(mx4[f])));
    int ix = min(max(f2i_sat((c.x - lo.x) / cs.x), 0), kGridRes - 1);
    int iy = min(max(f2i_sat((c.y - lo.y) / cs.y), 0), kGridRes - 1);
    int iz = min(max(f2i_sat((c.z - lo.z) / cs.z), 0), kGridRes - 1);
    int cell = ix * kGridRes * kGridRes + iy * kGridRes + iz;
    keys[f] = (unsigned)cell;
    ids[f] = f;
    atomicAdd(counts + cell, 1u);
}

// Node boxes are float4 pairs; min.w carries the node's face count (int bits)
// so that one 16-byte load gives a child's box corner and whether it is empty.
__device__ __forceinline__ void store_box(float4* nmin4, float4* nmax4, int i, V3 a, V3 b, int nf = 0) {
    nmin4[i] = make_float4(a.x, a.y, a.z, __int_as_float(nf));
    nmax4[i] = make_float4(b.x, b.y, b.z, 0.0f);
}
__device__ __forceinline__ V3 load_cg(const float4* p) {
    float4 v = __ldcg(p);
    return V3{v.x, v.y, v.z};
}

// assign_leaf_cell_nodes (:602-634) fused with a bottom-up refit that applies
// the rules of compute_cell_node_aabbs (:491-522).  The second thread to reach
// an internal node computes it from both (finished) children.  Each leaf also
// writes its faces' records (min.xyz + face id, max.xyz) in sorted order, the
// contiguous array the traversal scans.
// The cell tree is the perfect tree over the 32768 row-major cells (leaf slot
// i = cell i, child_a = lower half).  The Karras build numbers an internal
// node covering the aligned slot range [l, r] of size s >= 2 as 0 for the
// root, r when it is a left child (l / s even) and l when it is a right child;
// a leaf is slot + 32767.  The refit therefore needs no climbing: one block
// per z-column (32 leaves, an aligned subtree) fits its leaves and the
// subtree's 31 nodes in shared memory, and a second kernel fits the 1023
// nodes above the columns level by level.
__device__ __forceinline__ int cell_node_index(int l, int size) {
    if (size == kNumCells) return 0;
    if (size == 1) return l + kNumCells - 1;
    return ((l / size) & 1) == 0 ? l + size - 1 : l;
}

struct NodeBox {
    V3 a, b;
    int n;
};
// compute_cell_node_aabbs (lbvh_cell.py:491-522): union of the non-empty
// children; two empty children give the point at the mean of their corners
__device__ __forceinline__ NodeBox join_nodes(const NodeBox& l, const NodeBox& r) {
    NodeBox o;
    if (l.n > 0 && r.n > 0) {
        o.a = vmin(l.a, r.a);
        o.b = vmax(l.b, r.b);
    } else if (l.n > 0) {
        o.a = l.a;
        o.b = l.b;
    } else if (r.n > 0) {
        o.a = r.a;
        o.b = r.b;
    } else {
        o.a = scale(0.25f, add(add(add(l.a, l.b), r.a), r.b));
        o.b = o.a;
    }
    o.n = l.n + r.n;
    return o;
}

// Block = one z-column (cells col*32 .. col*32+31), a warp per cell: 8 warps
// taking 4 cells each, so that the 1024 columns fit one wave of blocks.
constexpr int kColumnRefitThreads = 256;

__global__ void __launch_bounds__(kColumnRefitThreads) cell_column_refit_kernel(
    const float* __restrict__ box6, const int* __restrict__ prefix, const int* __restrict__ sorted_face_ids,
    const float4* __restrict__ fmn4, const float4* __restrict__ fmx4, int* __restrict__ num_faces,
    float4* __restrict__ nmin4, float4* __restrict__ nmax4, float4* __restrict__ frec, float* grid8) {
    pdl_entry();
    __shared__ NodeBox tree[64];  // [32 + k]: leaf k; [16 + k], [8 + k], ...: levels above
    __shared__ unsigned ext_bits[3];
    const int col = blockIdx.x, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x < 3) ext_bits[threadIdx.x] = 0u;
    const V3 lo{box6[0], box6[1], box6[2]};
    const V3 cs = cell_size_of(box6);
    __syncthreads();  // ext_bits initialised
    // warp w takes the column's cells w, w + warps, ... (one warp per cell)
    for (int z = w; z < kGridRes; z += kColumnRefitThreads / 32) {
        const int i = col * kGridRes + z;
        const int rl = i == 0 ? 0 : prefix[i - 1];
        const int size = prefix[i] - rl;
        const V3 c = cell_center(i, cs, lo);
        V3 a = c, b = c;
        for (int j = lane; j < size; j += 32) {
            const int fid = sorted_face_ids[rl + j];
            const float4 fa = fmn4[fid], fb = fmx4[fid];
            a = vmin(a, mk(fa));
            b = vmax(b, mk(fb));
            frec[2 * (rl + j)] = make_float4(fa.x, fa.y, fa.z, __int_as_float(fid));
            frec[2 * (rl + j) + 1] = make_float4(fb.x, fb.y, fb.z, 0.0f);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a = vmin(a, V3{__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o),
                           __shfl_xor_sync(0xffffffffu, a.z, o)});
            b = vmax(b, V3{__shfl_xor_sync(0xffffffffu, b.x, o), __shfl_xor_sync(0xffffffffu, b.y, o),
                           __shfl_xor_sync(0xffffffffu, b.z, o)});
        }
        if (lane == 0) {
            const int leaf = i + kNumCells - 1;
            num_faces[leaf] = size;
            store_box(nmin4, nmax4, leaf, a, b, size);
            tree[32 + z] = NodeBox{a, b, size};
            // how far this leaf's box reaches beyond its cell (>= 0), maximised
            // over the grid: the traversal scans the cells within that reach
            if (size > 0) {
                const int x0 = i / (kGridRes * kGridRes), y0 = (i % (kGridRes * kGridRes)) / kGridRes, z0 = z;
                const float clo[3] = {lo.x + cs.x * (float)x0, lo.y + cs.y * (float)y0, lo.z + cs.z * (float)z0};
                const float chi[3] = {lo.x + cs.x * (float)(x0 + 1), lo.y + cs.y * (float)(y0 + 1),
                                      lo.z + cs.z * (float)(z0 + 1)};
                const float am[3] = {a.x, a.y, a.z}, bm[3] = {b.x, b.y, b.z};
                for (int k = 0; k < 3; ++k) {
                    const float ext = fmaxf(fmaxf(clo[k] - am[k], bm[k] - chi[k]), 0.0f);
                    if (ext > 0.0f) atomicMax(ext_bits + k, __float_as_uint(ext));
                }
            }
        }
    }
    __syncthreads();
    if (w == 0) {
        // occupancy word of the column, and the column's subtree, level by level
        const unsigned occ = __ballot_sync(0xffffffffu, tree[32 + lane].n > 0);
        if (lane == 0) reinterpret_cast<unsigned*>(grid8)[kGridHeader + col] = occ;
        if (lane < 3 && ext_bits[lane] != 0u) atomicMax(reinterpret_cast<unsigned*>(grid8) + 3 + lane, ext_bits[lane]);
        for (int half = 16, sz = 2; half >= 1; half >>= 1, sz <<= 1) {
            if (lane < half) {
                const NodeBox nb = join_nodes(tree[2 * half + 2 * lane], tree[2 * half + 2 * lane + 1]);
                tree[half + lane] = nb;
                const int node = cell_node_index(col * kGridRes + lane * sz, sz);
                num_faces[node] = nb.n;
                store_box(nmin4, nmax4, node, nb.a, nb.b, nb.n);
            }
            __syncwarp();
        }
    }
}

// The 1023 nodes above the columns (sizes 64 .. 32768), one block.
__global__ void __launch_bounds__(1024) cell_top_refit_kernel(int* __restrict__ num_faces,
                                                              float4* __restrict__ nmin4,
                                                              float4* __restrict__ nmax4) {
    pdl_entry();
    __shared__ float4 sa[kGridRes * kGridRes], sb[kGridRes * kGridRes];
    const int t = threadIdx.x;
    {
        const int node = cell_node_index(t * kGridRes, kGridRes);
        sa[t] = nmin4[node];
        sb[t] = nmax4[node];
    }
    __syncthreads();
    for (int half = kGridRes * kGridRes / 2, sz = 2 * kGridRes; half >= 1; half >>= 1, sz <<= 1) {
        NodeBox nb;
        if (t < half) {
            const float4 la = sa[2 * t], lb = sb[2 * t], ra = sa[2 * t + 1], rb = sb[2 * t + 1];
            nb = join_nodes(NodeBox{mk(la), mk(lb), __float_as_int(la.w)}, NodeBox{mk(ra), mk(rb), __float_as_int(ra.w)});
            const int node = cell_node_index(t * sz, sz);
            num_faces[node] = nb.n;
            store_box(nmin4, nmax4, node, nb.a, nb.b, nb.n);
        }
        __syncthreads();
        if (t < half) {
            sa[t] = make_float4(nb.a.x, nb.a.y, nb.a.z, __int_as_float(nb.n));
            sb[t] = make_float4(nb.b.x, nb.b.y, nb.b.z, 0.0f);
        }
        __syncthreads();
    }
}

// traverse_cell_bvh_single (lbvh_cell.py:662-714) as a walk over grid cells.
//
// The reference pops a node, skips it when empty or not overlapping, and
// otherwise scans a leaf's faces or pushes child_a then child_b.  The cell tree
// is always the perfect tree that the Karras build makes over the 32^3
// distinct cell codes, child_a covering the lower half of a node's leaf slots,
// and leaf slot i holds row-major cell i (lbvh_cell.py:604-634).  Its
// depth-first walk therefore reaches exactly the non-empty leaves whose boxes
// overlap the query (every ancestor of such a leaf contains its box), in
// descending slot = descending cell index.  A leaf's box is its cell grown by
// at most the build's maximum overhang (grid8[3..5]), so scanning the cells
// within that reach of the query box, in descending index, and applying the
// same leaf and face tests produces the same candidate list in the same order,
// with independent loads instead of a chain of dependent node fetches.
__device__ __forceinline__ void cell_range(float qa, float qb, float o, float c, float e, int* i0, int* i1) {
    // A leaf box lies within [o + c i - e, o + c (i + 1) + e] up to the
    // rounding of those bounds (relative 2^-24 of |o| + 64 c and of e); the
    // divisions below carry relative 2^-22 of (|q| + e + |o|) / c.  delta covers
    // both 64 times over, so a cell is left out only when no leaf box in it
    // can reach the query box.  A zero or non-finite cell size gives the full
    // range.
    const float delta = 1.5e-5f * ((fabsf(qa) + fabsf(qb) + 2.0f * e + 2.0f * fabsf(o) + 64.0f * c) / c);
    const float f0 = ceilf((qa - e - o) / c - 1.0f - delta), f1 = floorf((qb + e - o) / c + delta);
    *i0 = (int)fmaxf(f0, 0.0f);
    *i1 = (int)fminf(f1, (float)(kGridRes - 1));
}

// One warp per query.  The warp walks the (x, y) columns of the query's cell
// range in descending order.  In each column, lane l takes cell z = 31 - l, so
// that ascending lanes are the reference's descending-z visiting order: the
// occupied cells' leaf boxes are tested at once, a warp scan lays the faces of
// the cells that pass end to end in that order, and the lanes test those faces
// 32 at a time (each lane finds its cell by a binary search over the scan).  A
// ballot places each overlapping face after those of lower lanes, so
// candidates come out in descending cell order and, within a cell, in sorted
// face order -- the reference's visiting order -- with every lane busy.
constexpr int CT_BLOCK = 256;

__device__ __forceinline__ int warp_incl_scan(int v, int lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += o;
    }
    return v;
}
// lowest lane whose inclusive count exceeds k (31 when none does)
__device__ __forceinline__ int warp_owner(int incl, int k) {
    int lo = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1)
        if (__shfl_sync(0xffffffffu, incl, lo + step - 1) <= k) lo += step;
    return lo;
}

// EDGE: query q is the box of edge q (endpoints edges[2q], edges[2q+1] in p4)
// grown by pad (XPBD.py:221-232), else the box p4[q] +- pad.
template <bool EDGE>
__global__ void __launch_bounds__(CT_BLOCK, 4) cell_traverse_kernel(
    int Q, const float4* __restrict__ p4, float pad, const float* __restrict__ grid8, const float* __restrict__ box6,
    const float4* __restrict__ nmin4, const float4* __restrict__ nmax4, const int* __restrict__ prefix,
    const float4* __restrict__ frec, int cap, int* __restrict__ cand, int* __restrict__ num, int* status,
    const int* __restrict__ edges) {
    pdl_entry();
    // occupancy words: bit z of word x*32 + y = cell (x, y, z) holds faces
    __shared__ unsigned occ[kGridRes * kGridRes];
    const unsigned* gocc = reinterpret_cast<const unsigned*>(grid8) + kGridHeader;
    for (int k = threadIdx.x; k < kGridRes * kGridRes; k += blockDim.x) occ[k] = gocc[k];
    __syncthreads();
    const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (q >= Q) return;  // warp-uniform
    V3 a, b;
    if (EDGE) {
        const V3 p0 = mk(p4[edges[2 * q]]), p1 = mk(p4[edges[2 * q + 1]]);
        const V3 lo = vmin(p0, p1), hi = vmax(p0, p1);
        a = V3{lo.x - pad, lo.y - pad, lo.z - pad};
        b = V3{hi.x + pad, hi.y + pad, hi.z + pad};
    } else {
        const V3 p = mk(p4[q]);
        a = V3{p.x - pad, p.y - pad, p.z - pad};
        b = V3{p.x + pad, p.y + pad, p.z + pad};
    }
    const V3 pos = scale(0.5f, add(a, b));
    const V3 cs{grid8[0], grid8[1], grid8[2]}, org{box6[0], box6[1], box6[2]};
    const int ix = f2i_sat((pos.x - org.x) / cs.x), iy = f2i_sat((pos.y - org.y) / cs.y),
              iz = f2i_sat((pos.z - org.z) / cs.z);
    const int cid =
        (int)((unsigned)ix * (unsigned)(kGridRes * kGridRes) + (unsigned)iy * (unsigned)kGridRes + (unsigned)iz);
    int count = 0;  // warp-uniform
    int* out = cand + (size_t)q * cap;
    if (cid <= kNumCells - 1) {  // the reference's skip rule (lbvh_cell.py:665)
        int x0, x1, y0, y1, z0, z1;
        cell_range(a.x, b.x, org.x, cs.x, grid8[3], &x0, &x1);
        cell_range(a.y, b.y, org.y, cs.y, grid8[4], &y0, &y1);
        cell_range(a.z, b.z, org.z, cs.z, grid8[5], &z0, &z1);
        if (z0 <= z1 && x0 <= x1 && y0 <= y1) {
            const unsigned zmask = (z1 == 31 ? 0xffffffffu : ((1u << (z1 + 1)) - 1u)) & ~((1u << z0) - 1u);
            const int ny = y1 - y0 + 1, ncol = (x1 - x0 + 1) * ny;
            // columns in visiting order (x descending, then y descending), 32 at a time
            for (int c0 = 0; c0 < ncol; c0 += 32) {
                unsigned cm = 0u;  // this lane's column: occupied cells within the z range
                if (c0 + lane < ncol) {
                    const int cc = c0 + lane;
                    cm = occ[(x1 - cc / ny) * kGridRes + (y1 - cc % ny)] & zmask;
                }
                const int cn = __popc(cm);
                const int cincl = warp_incl_scan(cn, lane);
                const int ctotal = __shfl_sync(0xffffffffu, cincl, 31);
                // the occupied cells of these columns end to end (z descending
                // within a column), 32 at a time: lane k takes the k-th
                for (int k0 = 0; k0 < ctotal; k0 += 32) {
                    const int k = k0 + lane;
                    const int oc = warp_owner(cincl, k);
                    const unsigned m = __shfl_sync(0xffffffffu, cm, oc);
                    const int rank = k - (__shfl_sync(0xffffffffu, cincl, oc) - __shfl_sync(0xffffffffu, cn, oc));
                    int start = 0, n = 0;
                    if (k < ctotal) {
                        // position of the rank-th highest set bit of m
                        int cz = 0;
#pragma unroll
                        for (int step = 16; step >= 1; step >>= 1)
                            if (__popc(m >> (cz + step)) >= rank + 1) cz += step;
                        const int cc = c0 + oc;
                        const int i = (x1 - cc / ny) * kGridRes * kGridRes + (y1 - cc % ny) * kGridRes + cz;
                        const int leaf = i + kNumCells - 1;
                        if (overlap(a, b, mk(nmin4[leaf]), mk(nmax4[leaf]))) {
                            start = i == 0 ? 0 : prefix[i - 1];
                            n = prefix[i] - start;
                        }
                    }
                    const int incl = warp_incl_scan(n, lane);  // faces of the passing cells, in order
                    const int total = __shfl_sync(0xffffffffu, incl, 31);
                    for (int f0 = 0; f0 < total; f0 += 32) {
                        const int f = f0 + lane;
                        const int lo = warp_owner(incl, f);
                        const int o_incl = __shfl_sync(0xffffffffu, incl, lo);
                        const int o_n = __shfl_sync(0xffffffffu, n, lo);
                        const int o_start = __shfl_sync(0xffffffffu, start, lo);
                        bool hit = false;
                        float4 fa = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (f < total) {
                            const int j = o_start + (f - (o_incl - o_n));
                            fa = frec[2 * j];
                            hit = overlap(a, b, mk(fa), mk(frec[2 * j + 1]));
                        }
                        const unsigned hits = __ballot_sync(0xffffffffu, hit);
                        if (hit) {
                            const int slot = count + __popc(hits & ((1u << lane) - 1u));
                            if (slot < cap) out[slot] = __float_as_int(fa.w);
                        }
                        count += __popc(hits);
                    }
                }
            }
        }
    }
    if (lane == 0) {
        num[q] = count;
        if (count > cap) atomicOr(status, SX_STATUS_CAND_OVERFLOW);
    }
}

// ---------------------------------------------------------------------------
// Face-level LBVH refit and traversal
// ---------------------------------------------------------------------------
__global__ void face_refit_kernel(int n, const int* __restrict__ sorted_ids, const float4* __restrict__ fmn4,
                                  const float4* __restrict__ fmx4, const int* __restrict__ child_a,
                                  const int* __restrict__ child_b, const int* __restrict__ parent, float4* nmin4,
                                  float4* nmax4, int* flags, int* status) {
    pdl_entry();
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int leaf = n - 1 + j, f = sorted_ids[j];
    nmin4[leaf] = fmn4[f];
    nmax4[leaf] = fmx4[f];
    if (n == 1) return;
    int node = parent[leaf];
    for (int steps = 0; node >= 0; ++steps) {
        if (steps > n) {
            atomicOr(status, SX_STATUS_CLIMB_LIMIT);
            return;
        }
        __threadfence();
        if (atomicAdd(flags + node, 1) == 0) return;
        flags[node] = 0;
        const int l = child_a[node], r = child_b[node];
        V3 a = vmin(load_cg(nmin4 + l), load_cg(nmin4 + r));
        V3 b = vmax(load_cg(nmax4 + l), load_cg(nmax4 + r));
        store_box(nmin4, nmax4, node, a, b);
        node = parent[node];
    }
}

// The same refit with its lower levels in shared memory.  A Karras node
// covers a contiguous range of sorted leaves and carries the index of one of
// its ends, so every node whose range lies inside a block's tile of 256 leaves
// has its index in the tile as well: the block keeps those nodes' boxes and
// arrival counters in shared memory (block-scope fences, no global atomics).
// A thread that climbs out of the tile continues with the global protocol of
// face_refit_kernel.  Each thread carries its current box in registers; every
// internal box is also written to global memory.  Min and max are exact, so
// the boxes are the same as the one-thread-per-leaf climb's.
constexpr int FR_TILE = 256;

// node c (internal 0..n-2 or leaf n-1+j) has its slot in the tile [B, tile_end]
__device__ __forceinline__ bool in_tile(int c, int n, int B, int tile_end) {
    const int k = c >= n - 1 ? c - (n - 1) : c;
    return k >= B && k <= tile_end;
}

__global__ void __launch_bounds__(FR_TILE) face_refit_tiled_kernel(
    int n, const int* __restrict__ sorted_ids, const float4* __restrict__ fmn4, const float4* __restrict__ fmx4,
    const int* __restrict__ child_a, const int* __restrict__ child_b, const int* __restrict__ parent,
    const int* __restrict__ range_l, const int* __restrict__ range_r, float4* nmin4, float4* nmax4, int* flags,
    int* status) {
    pdl_entry();
    __shared__ float4 s_leaf[2][FR_TILE];
    __shared__ float4 s_node[2][FR_TILE];
    __shared__ int s_flag[FR_TILE];
    const int B = blockIdx.x * FR_TILE, t = threadIdx.x, j = B + t;
    s_flag[t] = 0;
    float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
    if (j < n) {
        const int f = sorted_ids[j];
        lo = fmn4[f];
        hi = fmx4[f];
        nmin4[n - 1 + j] = lo;
        nmax4[n - 1 + j] = hi;
        s_leaf[0][t] = lo;
        s_leaf[1][t] = hi;
    }
    __syncthreads();
    if (j >= n || n == 1) return;
    const int tile_end = min(B + FR_TILE, n) - 1;  // last leaf of the tile
    int me = n - 1 + j;
    int node = parent[me];
    bool local = true;
    // topology of the current node; the next level's is loaded before this
    // level's arrival counter, so that only the counter and the sibling's box
    // are round trips on the climb's critical path
    int ca = 0, cb = 0, up = -1, rl = 0, rr = 0;
    if (node >= 0) {
        ca = __ldg(child_a + node); cb = __ldg(child_b + node); up = __ldg(parent + node);
        rl = __ldg(range_l + node); rr = __ldg(range_r + node);
    }
    for (int steps = 0; node >= 0; ++steps) {
        if (steps > n) {
            atomicOr(status, SX_STATUS_CLIMB_LIMIT);
            return;
        }
        int nca = 0, ncb = 0, nup = -1, nrl = 0, nrr = 0;
        if (up >= 0) {
            nca = __ldg(child_a + up); ncb = __ldg(child_b + up); nup = __ldg(parent + up);
            nrl = __ldg(range_l + up); nrr = __ldg(range_r + up);
        }
        const int sib = ca == me ? cb : ca;
        float4 slo, shi;
        // local: the node and both children lie in the tile (decided from the
        // node alone, so both children agree; always true below a node whose
        // range is in the tile when the hierarchy is well formed)
        if (local && node >= B && node <= tile_end && rl >= B && rr <= tile_end && in_tile(ca, n, B, tile_end) &&
            in_tile(cb, n, B, tile_end)) {
            __threadfence_block();
            if (atomicAdd(s_flag + (node - B), 1) == 0) return;
            __threadfence_block();
            const bool sib_leaf = sib >= n - 1;
            const int k = sib_leaf ? sib - (n - 1) - B : sib - B;
            slo = sib_leaf ? s_leaf[0][k] : s_node[0][k];
            shi = sib_leaf ? s_leaf[1][k] : s_node[1][k];
        } else {
            local = false;
            // release: this thread's box stores are visible before the count;
            // acquire: the sibling's are visible to the loads below
            cuda::atomic_ref<int, cuda::thread_scope_device> cnt(flags[node]);
            if (cnt.fetch_add(1, cuda::memory_order_acq_rel) == 0) return;
            flags[node] = 0;
            slo = __ldcg(nmin4 + sib);
            shi = __ldcg(nmax4 + sib);
        }
        const V3 a = vmin(mk(lo), mk(slo)), b = vmax(mk(hi), mk(shi));
        store_box(nmin4, nmax4, node, a, b);
        lo = make_float4(a.x, a.y, a.z, 0.f);
        hi = make_float4(b.x, b.y, b.z, 0.f);
        if (local) {
            s_node[0][node - B] = lo;
            s_node[1][node - B] = hi;
        }
        me = node;
        node = up;
        ca = nca; cb = ncb; up = nup; rl = nrl; rr = nrr;
    }
}

__global__ void __launch_bounds__(128) face_traverse_kernel(int n, int Q, const float4* __restrict__ p4, float pad,
                                                            const int* __restrict__ child_a,
                                                            const int* __restrict__ child_b,
                                                            const int* __restrict__ sorted_ids,
                                                            const float4* __restrict__ nmin4,
                                                            const float4* __restrict__ nmax4, int cap,
                                                            int* __restrict__ cand, int* __restrict__ num,
                                                            int* status, const int* __restrict__ order) {
    pdl_entry();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Q) return;
    // order (optional): the queries in a spatially coherent order, so that a
    // warp's threads walk nearby parts of the tree
    const int q = order ? order[i] : i;
    V3 p = mk(p4[q]);
    V3 a{p.x - pad, p.y - pad, p.z - pad}, b{p.x + pad, p.y + pad, p.z + pad};
    int count = 0, flags = 0;
    int* out = cand + (size_t)q * cap;
    int stack[64];
    int sc = 0;
    // Children are tested before they are pushed (same visiting order as a
    // pop-time test, see cell_traverse_kernel).
    if (overlap(a, b, mk(nmin4[0]), mk(nmax4[0]))) stack[sc++] = 0;
    // A well-formed tree pops each of its 2n-1 nodes at most once; the bound
    // stops the walk on a malformed hierarchy (reference tie rule with repeated
    // codes can create cycles).
    long long pops = 0;
    const long long max_pops = 2LL * n;
    while (sc > 0) {
        if (++pops > max_pops) {
            flags |= SX_STATUS_STACK_OVERFLOW;
            break;
        }
        const int idx = stack[--sc];
        if (idx >= n - 1) {
            if (count < cap) out[count] = sorted_ids[idx - (n - 1)];
            ++count;
        } else {
            const int l = child_a[idx], r = child_b[idx];
            if (overlap(a, b, mk(nmin4[l]), mk(nmax4[l]))) {
                if (sc < 64) stack[sc++] = l; else flags |= SX_STATUS_STACK_OVERFLOW;
            }
            if (overlap(a, b, mk(nmin4[r]), mk(nmax4[r]))) {
                if (sc < 64) stack[sc++] = r; else flags |= SX_STATUS_STACK_OVERFLOW;
            }
        }
    }
    num[q] = count;
    if (count > cap) flags |= SX_STATUS_CAND_OVERFLOW;
    if (flags) atomicOr(status, flags);
}

}  // namespace sx

using namespace sx;

// ---- workspace layouts --------------------------------------------------------
// cell BVH: [keys F][radix ws F][flags NC] ; init uses [codes NC][radix ws NC]
extern "C" size_t sx_radix_sort_workspace_bytes(int n) { return rs_ws_bytes(n); }

extern "C" size_t sx_cell_bvh_workspace_bytes(int n_faces) {
    size_t build = align256((size_t)(n_faces > 0 ? n_faces : 1) * 4) + rs_ws_bytes(n_faces) +
                   align256((size_t)kNumCells * 4);
    size_t init = align256((size_t)kNumCells * 4) + rs_ws_bytes(kNumCells);
    return build > init ? build : init;
}

extern "C" int sx_radix_sort_pairs(unsigned* keys, int* vals, int n, int bits, void* ws, size_t ws_bytes,
                                   void* stream) {
    SX_REQUIRE(n >= 0, "sx_radix_sort_pairs: n < 0");
    if (n <= 1) return SX_OK;
    SX_REQUIRE(keys && vals, "sx_radix_sort_pairs: null pointer");
    return radix_sort(keys, vals, n, bits, ws, ws_bytes, as_stream(stream));
}

// ---------------------------------------------------------------------------
// Radix sort without a caller-provided workspace.
//
// Some callers cannot allocate device memory when they need to sort: hosts
// whose device memory belongs to another allocator with a fixed budget (a
// framework's caching pool, an engine's arena), where an extra cudaMalloc can
// fail or fragment the pool, and real-time loops that cannot afford the
// device-wide synchronisation cudaMalloc/cudaFree may cause.  For them the
// sort's scratch (two key/value ping-pong buffers and the digit histograms)
// lives in one fixed array in this library's device memory, sized for at most
// kNoAllocMaxKeys keys.  Every GPU that loads the library keeps the array
// (about 2.1 MB) until the process exits.
//
// In host code the array's name is only a host-side stand-in for the symbol, so
// its device address is looked up once per device, on the first call made with
// that device current, with cudaGetSymbolAddress; that first call should come
// before any stream capture.  The cached address is never refreshed: a
// cudaDeviceReset re-creates the context and may move the array, so callers
// must not use this entry point after resetting the device.  All calls share the array: calls that overlap on
// the GPU (different streams, or threads) race on it and must be ordered by the
// caller.  Nothing in it needs clearing: every pass overwrites the histogram
// and both ping-pong buffers before reading them.
// ---------------------------------------------------------------------------
constexpr int kNoAllocMaxKeys = 1 << 18;
constexpr size_t kNoAllocScratchBytes =
    2 * (((size_t)kNoAllocMaxKeys * 4 + 255) & ~(size_t)255) +
    (((size_t)256 * ((kNoAllocMaxKeys + RS_TILE - 1) / RS_TILE) * 4 + 255) & ~(size_t)255) + 256 * 4;
static __device__ __align__(256) unsigned char g_sort_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
static std::mutex g_scratch_mutex;
static void* g_scratch_addr[kMaxDevices] = {};

static int sort_scratch_for_current_device(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
    SX_REQUIRE(dev >= 0 && dev < kMaxDevices, "sx_radix_sort_pairs_noalloc: device %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_addr[dev] == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_sort_scratch)");
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return SX_OK;
}

extern "C" int sx_radix_sort_pairs_noalloc(unsigned* keys, int* vals, int n, int bits, void* stream) {
    SX_REQUIRE(n >= 0, "sx_radix_sort_pairs_noalloc: n < 0");
    SX_REQUIRE(n <= kNoAllocMaxKeys,
               "sx_radix_sort_pairs_noalloc: %d keys exceed the fixed scratch capacity of %d keys; "
               "use sx_radix_sort_pairs with a workspace",
               n, kNoAllocMaxKeys);
    if (n <= 1) return SX_OK;
    SX_REQUIRE(keys && vals, "sx_radix_sort_pairs_noalloc: null pointer");
    SX_REQUIRE(rs_ws_bytes(n) <= kNoAllocScratchBytes, "sx_radix_sort_pairs_noalloc: scratch layout mismatch");
    void* scratch = nullptr;
    int rc = sort_scratch_for_current_device(&scratch);
    if (rc) return rc;
    return radix_sort(keys, vals, n, bits, scratch, kNoAllocScratchBytes, as_stream(stream));
}

extern "C" int sx_face_morton(const float* fmin4, const float* fmax4, int n_faces, const float* box6,
                              unsigned* codes, int* ids, void* stream) {
    SX_REQUIRE(n_faces >= 0, "sx_face_morton: n_faces < 0");
    if (n_faces == 0) return SX_OK;
    SX_REQUIRE(fmin4 && fmax4 && box6 && codes && ids, "sx_face_morton: null pointer");
    launch(face_morton_kernel, grid_for(n_faces, 256), 256, 0, as_stream(stream), 
        n_faces, (const float4*)fmin4, (const float4*)fmax4, box6, codes, ids);
    return check_launch("face_morton_kernel");
}

extern "C" int sx_karras_build(const unsigned* codes, int n, int tie, int* child_a, int* child_b, int* range_l,
                               int* range_r, int* parent, void* stream) {
    SX_REQUIRE(n >= 1, "sx_karras_build: n must be >= 1");
    SX_REQUIRE(codes && parent && (n == 1 || (child_a && child_b && range_l && range_r)),
               "sx_karras_build: null pointer");
    launch(karras_kernel, grid_for(n, 256), 256, 0, as_stream(stream), n, codes, tie ? 1 : 0, child_a, child_b,
                                                                    range_l, range_r, parent);
    return check_launch("karras_kernel");
}

extern "C" int sx_cell_bvh_init(int* sorted_codes, int* sorted_ids, int* child_a, int* child_b, int* range_l,
                                int* range_r, int* parent, void* ws, size_t ws_bytes, void* stream) {
    SX_REQUIRE(sorted_codes && sorted_ids && child_a && child_b && range_l && range_r && parent,
               "sx_cell_bvh_init: null pointer");
    SX_REQUIRE(ws && ws_bytes >= sx_cell_bvh_workspace_bytes(0), "sx_cell_bvh_init: workspace too small");
    const cudaError_t attr = scan_smem_attr();  // for sx_cell_bvh_build's prefix scan
    if (attr != cudaSuccess) return cuda_status(attr, "cudaFuncSetAttribute(scan_single_block)");
    cudaStream_t s = as_stream(stream);
    launch(cell_morton_kernel, grid_for(kNumCells, 256), 256, 0, s, (unsigned*)sorted_codes, sorted_ids);
    int rc = check_launch("cell_morton_kernel");
    if (rc) return rc;
    rc = radix_sort((unsigned*)sorted_codes, sorted_ids, kNumCells, 30, ws, ws_bytes, s);
    if (rc) return rc;
    launch(karras_kernel, grid_for(kNumCells, 256), 256, 0, s, kNumCells, (const unsigned*)sorted_codes, 0, child_a,
                                                           child_b, range_l, range_r, parent);
    return check_launch("karras_kernel(cells)");
}

extern "C" int sx_cell_bvh_build(const float* fmin4, const float* fmax4, int n_faces, const float* box6,
                                 const int* child_a, const int* child_b, const int* parent, int* sorted_face_ids,
                                 int* prefix, int* num_faces, float* nmin4, float* nmax4, float* face_rec8,
                                 float* grid8, void* ws, size_t ws_bytes, void* stream) {
    SX_REQUIRE(n_faces >= 0, "sx_cell_bvh_build: n_faces < 0");
    SX_REQUIRE(box6 && child_a && child_b && parent && prefix && num_faces && nmin4 && nmax4 && grid8,
               "sx_cell_bvh_build: null pointer");
    SX_REQUIRE(n_faces == 0 || (fmin4 && fmax4 && sorted_face_ids && face_rec8),
               "sx_cell_bvh_build: null face arrays");
    SX_REQUIRE(ws && ws_bytes >= sx_cell_bvh_workspace_bytes(n_faces), "sx_cell_bvh_build: workspace too small");
    cudaStream_t s = as_stream(stream);
    char* p = (char*)ws;
    unsigned* keys = (unsigned*)p;
    p += align256((size_t)(n_faces > 0 ? n_faces : 1) * 4);
    void* rws = p;
    p += rs_ws_bytes(n_faces);
    SX_CUDA(cudaMemsetAsync(prefix, 0, sizeof(int) * kNumCells, s));
    launch(face_cell_kernel, grid_for(n_faces, 256), 256, 0, s, n_faces, (const float4*)fmin4, (const float4*)fmax4,
           box6, keys, sorted_face_ids, (unsigned*)prefix, grid8);
    int rc = check_launch("face_cell_kernel");
    if (rc) return rc;
    rc = launch_scan_single_block((unsigned*)prefix, kNumCells, 1, s);
    if (rc) return rc;
    if (n_faces > 1) {
        rc = radix_sort(keys, sorted_face_ids, n_faces, 15, rws, rs_ws_bytes(n_faces), s);
        if (rc) return rc;
    }
    launch(cell_column_refit_kernel, kGridRes * kGridRes, kColumnRefitThreads, 0, s, box6, (const int*)prefix,
           (const int*)sorted_face_ids, (const float4*)fmin4, (const float4*)fmax4, num_faces, (float4*)nmin4,
           (float4*)nmax4, (float4*)face_rec8, grid8);
    rc = check_launch("cell_column_refit_kernel");
    if (rc) return rc;
    launch(cell_top_refit_kernel, 1, 1024, 0, s, num_faces, (float4*)nmin4, (float4*)nmax4);
    return check_launch("cell_top_refit_kernel");
}

extern "C" int sx_cell_bvh_traverse(const float* p4, int n_queries, float padding, const float* grid8,
                                    const float* origin_box6, const float* nmin4, const float* nmax4,
                                    const int* prefix,
                                    const float* face_rec8, int cap, int* cand, int* num, int* status,
                                    void* stream) {
    SX_REQUIRE(n_queries >= 0 && cap >= 1, "sx_cell_bvh_traverse: bad sizes");
    if (n_queries == 0) return SX_OK;
    SX_REQUIRE(p4 && grid8 && origin_box6 && nmin4 && nmax4 && prefix && face_rec8 &&
                   cand && num && status,
               "sx_cell_bvh_traverse: null pointer");
    launch(cell_traverse_kernel<false>, grid_for(32LL * n_queries, CT_BLOCK), CT_BLOCK, 0, as_stream(stream),
           n_queries, (const float4*)p4, padding, grid8, origin_box6, (const float4*)nmin4, (const float4*)nmax4,
           prefix, (const float4*)face_rec8, cap, cand, num, status, (const int*)nullptr);
    return check_launch("cell_traverse_kernel");
}

extern "C" int sx_cell_bvh_traverse_edges(const int* edges, int n_edges, const float* p4, float padding,
                                          const float* grid8, const float* origin_box6, const float* nmin4,
                                          const float* nmax4, const int* prefix, const float* face_rec8, int cap,
                                          int* cand, int* num, int* status, void* stream) {
    SX_REQUIRE(n_edges >= 0 && cap >= 1, "sx_cell_bvh_traverse_edges: bad sizes");
    if (n_edges == 0) return SX_OK;
    SX_REQUIRE(edges && p4 && grid8 && origin_box6 && nmin4 && nmax4 && prefix && face_rec8 && cand && num &&
                   status,
               "sx_cell_bvh_traverse_edges: null pointer");
    launch(cell_traverse_kernel<true>, grid_for(32LL * n_edges, CT_BLOCK), CT_BLOCK, 0, as_stream(stream), n_edges,
           (const float4*)p4, padding, grid8, origin_box6, (const float4*)nmin4, (const float4*)nmax4, prefix,
           (const float4*)face_rec8, cap, cand, num, status, edges);
    return check_launch("cell_traverse_kernel");
}

extern "C" int sx_face_bvh_refit(int n, const int* sorted_ids, const float* fmin4, const float* fmax4,
                                 const int* child_a, const int* child_b, const int* parent, float* nmin4,
                                 float* nmax4, int* flags, int* status, void* stream) {
    SX_REQUIRE(n >= 1, "sx_face_bvh_refit: n must be >= 1");
    SX_REQUIRE(sorted_ids && fmin4 && fmax4 && parent && nmin4 && nmax4 && status &&
                   (n == 1 || (child_a && child_b && flags)),
               "sx_face_bvh_refit: null pointer");
    launch(face_refit_kernel, grid_for(n, 256), 256, 0, as_stream(stream), 
        n, sorted_ids, (const float4*)fmin4, (const float4*)fmax4, child_a, child_b, parent, (float4*)nmin4,
        (float4*)nmax4, flags, status);
    return check_launch("face_refit_kernel");
}

extern "C" int sx_face_bvh_refit_tiled(int n, const int* sorted_ids, const float* fmin4, const float* fmax4,
                                       const int* child_a, const int* child_b, const int* parent, const int* range_l,
                                       const int* range_r, float* nmin4, float* nmax4, int* flags, int* status,
                                       void* stream) {
    SX_REQUIRE(n >= 1, "sx_face_bvh_refit_tiled: n must be >= 1");
    SX_REQUIRE(sorted_ids && fmin4 && fmax4 && parent && nmin4 && nmax4 && status &&
                   (n == 1 || (child_a && child_b && flags && range_l && range_r)),
               "sx_face_bvh_refit_tiled: null pointer");
    launch(face_refit_tiled_kernel, grid_for(n, FR_TILE), FR_TILE, 0, as_stream(stream), n, sorted_ids,
           (const float4*)fmin4, (const float4*)fmax4, child_a, child_b, parent, range_l, range_r, (float4*)nmin4,
           (float4*)nmax4, flags, status);
    return check_launch("face_refit_tiled_kernel");
}

extern "C" int sx_face_bvh_traverse(int n, const float* p4, int n_queries, float padding, const int* child_a,
                                    const int* child_b, const int* sorted_ids, const float* nmin4,
                                    const float* nmax4, int cap, int* cand, int* num, int* status, void* stream) {
    SX_REQUIRE(n >= 1 && n_queries >= 0 && cap >= 1, "sx_face_bvh_traverse: bad sizes");
    if (n_queries == 0) return SX_OK;
    SX_REQUIRE(p4 && sorted_ids && nmin4 && nmax4 && cand && num && status && (n == 1 || (child_a && child_b)),
               "sx_face_bvh_traverse: null pointer");
    launch(face_traverse_kernel, grid_for(n_queries, 128), 128, 0, as_stream(stream), 
        n, n_queries, (const float4*)p4, padding, child_a, child_b, sorted_ids, (const float4*)nmin4,
        (const float4*)nmax4, cap, cand, num, status, (const int*)nullptr);
    return check_launch("face_traverse_kernel");
}

extern "C" int sx_face_bvh_traverse_ordered(int n, const float* p4, int n_queries, float padding,
                                            const int* child_a, const int* child_b, const int* sorted_ids,
                                            const float* nmin4, const float* nmax4, int cap, int* cand, int* num,
                                            int* status, const int* order, void* stream) {
    SX_REQUIRE(n >= 1 && n_queries >= 0 && cap >= 1, "sx_face_bvh_traverse_ordered: bad sizes");
    if (n_queries == 0) return SX_OK;
    SX_REQUIRE(p4 && sorted_ids && nmin4 && nmax4 && cand && num && status && order &&
                   (n == 1 || (child_a && child_b)),
               "sx_face_bvh_traverse_ordered: null pointer");
    launch(face_traverse_kernel, grid_for(n_queries, 128), 128, 0, as_stream(stream), n, n_queries,
           (const float4*)p4, padding, child_a, child_b, sorted_ids, (const float4*)nmin4, (const float4*)nmax4, cap,
           cand, num, status, order);
    return check_launch("face_traverse_kernel");
}
