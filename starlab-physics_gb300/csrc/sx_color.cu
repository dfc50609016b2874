// Constraint-graph colouring (framework/utilities/graph_coloring.py).
//
// The reference builds a dense E x E adjacency (initAdjEdges :112-129) and
// colours edges sequentially, first-fit, in edge-id order (colorEdgesGreedy
// :131-149), then sorts edges by colour with a stable counting sort
// (colorCountingSort :172-201).  Here: a vertex -> edge incidence list replaces
// the dense matrix, and the sequential first-fit is reproduced exactly by
// parallel rounds in which an edge takes its colour as soon as every adjacent
// edge with a smaller id has one (those are exactly the edges a sequential pass
// would have coloured before it).  One cooperative launch colours every edge,
// each as soon as its lower-id neighbours have colours (no rounds, no host
// synchronisation).  The stable sort is the library's radix sort.
#include "sx_common.cuh"

extern "C" size_t sx_radix_sort_workspace_bytes(int n);
extern "C" int sx_radix_sort_pairs(unsigned* keys, int* vals, int n, int bits, void* ws, size_t ws_bytes,
                                   void* stream);

namespace sx {

constexpr int kMaxColorWords = 4;  // up to 128 colours

static inline size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

__global__ void inc_count_kernel(int E, const int* __restrict__ edges, int* cnt) {
    pdl_entry();
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    atomicAdd(cnt + edges[2 * e], 1);
    atomicAdd(cnt + edges[2 * e + 1], 1);
}

__global__ void inc_fill_kernel(int E, const int* __restrict__ edges, const int* __restrict__ ptr, int* cursor,
                                int* inc) {
    pdl_entry();
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int a = edges[2 * e], b = edges[2 * e + 1];
    inc[ptr[a] + atomicAdd(cursor + a, 1)] = e;
    inc[ptr[b] + atomicAdd(cursor + b, 1)] = e;
}

__global__ void color_init_kernel(int E, int* color, unsigned* keys, int* ids) {
    pdl_entry();
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    color[e] = -1;
    ids[e] = e;
}

// Tries to colour edge e: false if an adjacent edge with a smaller id has no
// colour yet; otherwise e gets the smallest colour none of them has (or keeps
// the one it has).  Colours once set never change, so reading a neighbour's
// colour set earlier in the same round gives the same choice.
__device__ __forceinline__ bool color_try(int e, const int* __restrict__ edges, const int* __restrict__ ptr,
                                          const int* __restrict__ inc, int max_colors, int* color, int* blocker) {
    volatile int* vc = color;
    if (vc[e] != -1) return true;
    unsigned forbid[kMaxColorWords] = {0u, 0u, 0u, 0u};
    for (int s = 0; s < 2; ++s) {
        const int v = edges[2 * e + s];
        for (int k = ptr[v]; k < ptr[v + 1]; ++k) {
            const int o = inc[k];
            if (o >= e) continue;
            const int c = vc[o];
            if (c < 0) {
                *blocker = o;
                return false;
            }
            forbid[c >> 5] |= 1u << (c & 31);
        }
    }
    int pick = 0;
    for (int c = 0; c < max_colors; ++c) {
        if (!(forbid[c >> 5] & (1u << (c & 31)))) {
            pick = c;
            break;
        }
    }
    vc[e] = pick;
    return true;
}

// Every edge in one cooperative launch (all threads resident), without
// rounds: a thread takes its edges in ascending id order (grid stride) and
// colours each as soon as every adjacent edge with a smaller id has a
// colour.  The smallest uncoloured edge never waits (its thread has finished
// all its smaller edges), so the colouring always progresses; its critical
// path is the longest chain of adjacent edges with increasing ids (1529 links
// for the 256 x 256 cloth).  The cost of a link is the latency between one
// edge's colour store and the next edge's decision, so a thread gathers the
// ids of its edge's lower neighbours once (up to kMaxLower; more falls back
// to color_try's sequential scan), then reads all their colours with
// independent loads (one L2 round trip instead of one per neighbour), and
// when one is missing waits on that neighbour alone, re-reading with a short
// sleep.  Each wait is bounded: after kColorPolls re-reads the edge stays
// uncoloured and SX_STATUS_WAIT_TIMEOUT is set, which makes the edges waiting
// on it give up in turn.
constexpr int kColorPolls = 1 << 21;
constexpr int kMaxLower = 24;

__global__ void __launch_bounds__(256, 4) color_edges_kernel(int E, const int* __restrict__ edges,
                                                          const int* __restrict__ ptr, const int* __restrict__ inc,
                                                          int max_colors, int* color, int* status) {
    pdl_entry();
    const long long stride = (long long)gridDim.x * blockDim.x;
    volatile int* vc = color;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride) {
        int polls = 0;
        bool timed_out = false;
        // the lower neighbours of e, once
        int nb[kMaxLower];
        int n = 0;
        bool many = false;
        for (int s = 0; s < 2; ++s) {
            const int v = edges[2 * e + s];
            for (int k = ptr[v]; k < ptr[v + 1]; ++k) {
                const int o = inc[k];
                if (o >= e) continue;
                if (n < kMaxLower) {
                    nb[n++] = o;
                } else {
                    many = true;
                }
            }
        }
        if (many) {
            int blocker = -1;
            bool done = false;
            while (!done && !timed_out) {
                done = color_try((int)e, edges, ptr, inc, max_colors, color, &blocker);
                const volatile int* vb = color + blocker;
                while (!done && *vb < 0) {
                    if (++polls > kColorPolls) {
                        timed_out = true;
                        break;
                    }
                    __nanosleep(32);
                }
            }
        } else {
            for (;;) {
                int c[kMaxLower];
#pragma unroll
                for (int j = 0; j < kMaxLower; ++j) c[j] = j < n ? vc[nb[j]] : 0;
                int blocker = -1;
                unsigned forbid[kMaxColorWords] = {0u, 0u, 0u, 0u};
#pragma unroll
                for (int j = 0; j < kMaxLower; ++j) {
                    if (j < n) {
                        if (c[j] < 0) {
                            if (blocker < 0) blocker = nb[j];
                        } else {
                            forbid[c[j] >> 5] |= 1u << (c[j] & 31);
                        }
                    }
                }
                if (blocker < 0) {
                    int pick = 0;
                    for (int q = 0; q < max_colors; ++q) {
                        if (!(forbid[q >> 5] & (1u << (q & 31)))) {
                            pick = q;
                            break;
                        }
                    }
                    vc[e] = pick;
                    break;
                }
                const volatile int* vb = color + blocker;
                while (*vb < 0) {
                    if (++polls > kColorPolls) {
                        timed_out = true;
                        break;
                    }
                    __nanosleep(32);
                }
                if (timed_out) break;
            }
        }
        if (timed_out) atomicOr(status, SX_STATUS_WAIT_TIMEOUT);
    }
}

__global__ void color_hist_kernel(int E, const int* __restrict__ color, unsigned* keys, unsigned* hist) {
    pdl_entry();
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const int c = color[e];  // -1 only if a bounded wait gave up (status bit set)
    keys[e] = c < 0 ? 255u : (unsigned)c;
    if (c >= 0) atomicAdd(hist + c, 1u);
}

// exclusive scan of the colour histogram (max_colors <= 128) -> start offsets
__global__ void color_prefix_kernel(int max_colors, const unsigned* hist, int* prefix) {
    pdl_entry();
    if (threadIdx.x != 0) return;
    unsigned run = 0;
    for (int c = 0; c < max_colors; ++c) {
        prefix[c] = (int)run;
        run += hist[c];
    }
}

__global__ void scan_excl_small(int n, int* data) {
    pdl_entry();  // single thread; n = V+1 only for small V
    if (threadIdx.x != 0) return;
    int run = 0;
    for (int i = 0; i < n; ++i) {
        int t = data[i];
        data[i] = run;
        run += t;
    }
}

}  // namespace sx

using namespace sx;

// workspace: [status 1][unused 5][ptr V+1][cursor V][inc 2E][keys E][hist 128][radix ws E]
extern "C" size_t sx_color_workspace_bytes(int n_verts, int n_edges) {
    size_t V = (size_t)(n_verts > 0 ? n_verts : 1), E = (size_t)(n_edges > 0 ? n_edges : 1);
    return a256(4) + a256(5 * 4) + a256((V + 1) * 4) + a256(V * 4) + a256(2 * E * 4) + a256(E * 4) +
           a256(128 * 4) + sx_radix_sort_workspace_bytes(n_edges);
}

// exclusive scan of V+1 ints, reusing the radix-sort scan would need unsigned
// layout; a block-wide scan keeps it simple.
__global__ void scan_excl_block(int n, int* data) {
    pdl_entry();
    __shared__ int s[1024];
    const int tid = threadIdx.x;
    const int per = (n + 1023) / 1024;
    const int beg = min(tid * per, n), end = min(beg + per, n);
    int sum = 0;
    for (int i = beg; i < end; ++i) sum += data[i];
    s[tid] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        int v = tid >= off ? s[tid - off] : 0;
        __syncthreads();
        s[tid] += v;
        __syncthreads();
    }
    int run = tid ? s[tid - 1] : 0;
    for (int i = beg; i < end; ++i) {
        int t = data[i];
        data[i] = run;
        run += t;
    }
}

extern "C" int sx_color_edges_greedy(const int* edges, int n_edges, int n_verts, int max_colors, int* color,
                                     int* sorted_edges, int* prefix, void* ws, size_t ws_bytes, void* stream) {
    SX_REQUIRE(n_edges >= 0 && n_verts >= 0, "sx_color_edges_greedy: bad sizes");
    SX_REQUIRE(max_colors >= 1 && max_colors <= 32 * kMaxColorWords, "sx_color_edges_greedy: max_colors in [1, 128]");
    SX_REQUIRE(prefix, "sx_color_edges_greedy: null prefix");
    cudaStream_t s = as_stream(stream);
    if (n_edges == 0) {
        SX_CUDA(cudaMemsetAsync(prefix, 0, sizeof(int) * max_colors, s));
        return SX_OK;
    }
    SX_REQUIRE(edges && color && sorted_edges, "sx_color_edges_greedy: null pointer");
    SX_REQUIRE(ws && ws_bytes >= sx_color_workspace_bytes(n_verts, n_edges),
               "sx_color_edges_greedy: workspace too small");
    const size_t V = (size_t)(n_verts > 0 ? n_verts : 1), E = (size_t)n_edges;
    char* p = (char*)ws;
    int* status = (int*)p; p += a256(4);
    p += a256(5 * 4);  // unused
    int* ptr = (int*)p; p += a256((V + 1) * 4);
    int* cursor = (int*)p; p += a256(V * 4);
    int* inc = (int*)p; p += a256(2 * E * 4);
    unsigned* keys = (unsigned*)p; p += a256(E * 4);
    unsigned* hist = (unsigned*)p; p += a256(128 * 4);
    void* rws = p;

    SX_CUDA(cudaMemsetAsync(ws, 0, a256(4) + a256(5 * 4), s));
    SX_CUDA(cudaMemsetAsync(ptr, 0, (V + 1) * 4, s));
    SX_CUDA(cudaMemsetAsync(cursor, 0, V * 4, s));
    launch(inc_count_kernel, grid_for(n_edges, 256), 256, 0, s, n_edges, edges, ptr);
    launch(scan_excl_block, 1, 1024, 0, s, n_verts + 1, ptr);
    launch(inc_fill_kernel, grid_for(n_edges, 256), 256, 0, s, n_edges, edges, ptr, cursor, inc);
    launch(color_init_kernel, grid_for(n_edges, 256), 256, 0, s, n_edges, color, keys, sorted_edges);
    int rc = check_launch("colour setup");
    if (rc) return rc;
    // every edge in one cooperative launch (every block resident)
    {
        const int cap = resident_blocks(color_edges_kernel, 256);
        const int g = grid_for(n_edges, 256) < cap ? grid_for(n_edges, 256) : cap;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(g);
        cfg.blockDim = dim3(256);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        SX_CUDA(cudaLaunchKernelEx(&cfg, color_edges_kernel, n_edges, edges, (const int*)ptr, (const int*)inc,
                                   max_colors, color, status));
        note_launch();
    }
    SX_CUDA(cudaMemsetAsync(hist, 0, 128 * 4, s));
    launch(color_hist_kernel, grid_for(n_edges, 256), 256, 0, s, n_edges, color, keys, hist);
    launch(color_prefix_kernel, 1, 32, 0, s, max_colors, hist, prefix);
    rc = check_launch("colour histogram");
    if (rc) return rc;
    return sx_radix_sort_pairs(keys, sorted_edges, n_edges, 8, rws, sx_radix_sort_workspace_bytes(n_edges), s);
}
