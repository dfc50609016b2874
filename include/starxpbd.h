/*
 * starxpbd -- C ABI of the GB300 (sm_103a) XPBD cloth substep library.
 *
 * Every entry point takes raw device pointers, element counts and a CUDA
 * stream (cudaStream_t passed as void*; NULL = legacy default stream).  Calls
 * are enqueued on that stream and return without synchronising, except where
 * noted.  No entry point allocates or frees memory: scratch space comes from
 * caller-provided workspaces whose size is given by the *_workspace_bytes
 * functions.  Errors are returned as negative codes (below); the message of the
 * last error on the calling thread is available from sx_last_error().  No C++
 * exception crosses this boundary.
 *
 * Layout conventions
 *   positions / velocities : float4 per vertex (xyz + w).  For x4 and y4 the w
 *                            lane holds wf = fixed * m_inv; for v4 it is unused.
 *   face AABBs             : float4 per face for min and for max (w unused).
 *   boxes                  : box6 = {min x, min y, min z, max x, max y, max z}.
 *   indices                : int32.
 *   BVH nodes              : 2n-1 nodes; internal nodes 0..n-2, leaves n-1..2n-2.
 *
 * Each declaration cites the reference (medialab-ku/starlab-physics) function
 * it replaces, as path:line within that project.
 */
#ifndef STARXPBD_H
#define STARXPBD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SX_OK 0
#define SX_ERR_ARG (-1)      /* bad argument (null pointer, size, workspace)      */
#define SX_ERR_CAPACITY (-2) /* a fixed-capacity list overflowed (see status word) */
#define SX_ERR_TIMEOUT (-3)  /* a bounded device-side wait gave up                */
#define SX_ERR_CUDA (-4)     /* a CUDA runtime call failed                          */

/* status-word bits written by traversal / contact kernels (int32, device) */
#define SX_STATUS_CAND_OVERFLOW 1  /* a query found more candidates than `cap`     */
#define SX_STATUS_STACK_OVERFLOW 2 /* a traversal stack (64 entries) overflowed     */
#define SX_STATUS_FIXED_RANGE 4    /* a contact term was NaN or out of fixed range  */
#define SX_STATUS_CLIMB_LIMIT 8    /* a bottom-up refit walk exceeded n steps        */
#define SX_STATUS_WAIT_TIMEOUT 16  /* a bounded device-side wait gave up             */

int sx_version(void);
const char* sx_last_error(void);
/* Number of CUDA kernels this library has launched in the process so far
 * (all threads); benchmarks difference it around a timed region. */
long long sx_kernel_launches(void);

/* ---- cloth state (framework/physics/XPBD.py) ------------------------------ */

/* compute_y, XPBD.py:116-118: y = x + fixed*v*dt + g*dt*dt; y.w = x.w */
int sx_predict(const float* x4, const float* v4, const float* fixed, float* y4, int n_verts, float dt,
               float gx, float gy, float gz, void* stream);

/* One Jacobi sweep: init_variables + solve_spring_constraints_x + update_dx,
 * XPBD.py:345-348, :141-184, :384-387.  Springs read y_in4; bending pairs read
 * x4 as in the reference (XPBD.py:169) when bend_on_y == 0, or y_in4 when
 * bend_on_y == 1.  Vertex-centric gather over adj_ptr[n_verts+1] /
 * adj[2*nnz] = (neighbour | 0x80000000 for bending, float bits of rest length)
 * in ascending constraint index; writes y_out4 (must not alias y_in4).
 * k_spring, k_bend = stiffness * dt^2 of the two constraint types. */
int sx_jacobi_sweep(const float* x4, const float* y_in4, float* y_out4, const float* fixed, const int* adj_ptr,
                    const int* adj, int n_verts, float k_spring, float k_bend, int bend_on_y, void* stream);

/* Launch configurations of the sweep (entries whose loads are issued together,
 * threads per block) for an autotuner; no counterpart in the reference.  All
 * variants give bit-identical results; variant 0 is the one sx_jacobi_sweep
 * uses. */
/* Programmatic dependent launch for the library's kernels: each may be
 * scheduled while its predecessor on the stream finishes, and waits on the
 * device for the predecessor's results (griddepcontrol) before it touches
 * memory.  Kernels recorded into a device-side loop body (sx_loop_begin ..
 * sx_loop_end) are plain launches.  On by default; returns the previous
 * setting.  Results do not depend on it. */
int sx_set_programmatic_launch(int enable);
int sx_jacobi_sweep_variants(void);
int sx_jacobi_sweep_variant_info(int variant, int* g, int* block);
/* The form of that variant: *lanes = lanes of a warp that evaluate one vertex
 * (1, or 2/4/8: the vertex's entries are split across the lanes and their
 * terms added in ascending entry order through shuffles, for meshes with too
 * few vertices to fill the SMs); *streaming = 1 if the adjacency entries are
 * read with the evict-first cache policy (for batches larger than L2).  Every
 * form gives the same result bit for bit. */
int sx_jacobi_sweep_variant_form(int variant, int* lanes, int* streaming);
int sx_jacobi_sweep_v(const float* x4, const float* y_in4, float* y_out4, const float* fixed, const int* adj_ptr,
                      const int* adj, int n_verts, float k_spring, float k_bend, int bend_on_y, int variant,
                      void* stream);
/* sx_jacobi_sweep_v with a choice of arithmetic (no counterpart in the
 * reference): fast = 0 is the exact, reference-order float arithmetic of
 * sx_jacobi_sweep_v (bit for bit); fast != 0 uses fused multiply-adds, the
 * hardware reciprocal square root, a fast divide and n.n taken as 1 --
 * within float rounding of the exact sweep, not bit-identical, and held to
 * the substep's position and residual tolerance instead. */
int sx_jacobi_sweep_mode(const float* x4, const float* y_in4, float* y_out4, const float* fixed, const int* adj_ptr,
                         const int* adj, int n_verts, float k_spring, float k_bend, int bend_on_y, int variant,
                         int fast, void* stream);
/* The same sweep over the packed adjacency (6 bytes per entry instead of 8):
 * for entry k of the CSR adj_ptr, nbr16[k] = neighbour - owner (int16) and
 * rest32[k] = bits(rest length) | 0x80000000 for a bending pair.  Both arrays
 * are 16-byte aligned and hold at least ((adj_ptr[n_verts] + 7) & ~7) entries
 * (the kernel reads whole 16-byte groups; padding entries are never used).
 * Each block copies its vertices' range of entries into shared memory with
 * coalesced streaming loads before the gather.  Results equal
 * sx_jacobi_sweep_mode's bit for bit (fast = 0) or its fast arithmetic. */
int sx_jacobi_sweep_packed(const float* x4, const float* y_in4, float* y_out4, const float* fixed, const int* adj_ptr,
                           const short* nbr16, const unsigned* rest32, int n_verts, float k_spring, float k_bend,
                           int bend_on_y, int fast, void* stream);
/* sx_jacobi_sweep_packed in one of sx_jacobi_sweep_packed_forms() forms
 * (bit-identical): form 0 stages each block's entries in shared memory
 * (sx_jacobi_sweep_packed); forms 1.. read them straight from global memory,
 * one vertex per thread, in several launch configurations (entries whose loads
 * are issued together, threads per block) for an autotuner. */
int sx_jacobi_sweep_packed_forms(void);
int sx_jacobi_sweep_packed_v(const float* x4, const float* y_in4, float* y_out4, const float* fixed,
                             const int* adj_ptr, const short* nbr16, const unsigned* rest32, int n_verts,
                             float k_spring, float k_bend, int bend_on_y, int form, int fast, void* stream);

/* solve_sewing_constraints_x (XPBD.py:425-441) + update_dx over sewn vertex
 * pairs (zero rest length, k = compliance argument of the reference):
 * sewn[n_sewn] the vertices with partners, partner[sptr[i] .. sptr[i+1]) the
 * partners of sewn[i] in ascending pair index; scratch4 holds n_sewn float4.
 * Coincident pairs add nothing. */
int sx_sewing_sweep(float* y4, const float* fixed, int n_sewn, const int* sewn, const int* sptr, const int* partner,
                    float k, float* scratch4, void* stream);

/* compute_velocity + update_x, XPBD.py:341-343 and :333-337:
 * v = (1-damping)*fixed*(y-x)/dt ; x += dt*v */
int sx_velocity_update(float* x4, const float* y4, float* v4, const float* fixed, int n_verts, float damping,
                       float dt, void* stream);

/* Constraint residual (the reference defines none; it runs a fixed number of
 * sweeps, XPBD.py:350-369): out3 (device) = {S, n, sqrt(S/n)} where n is the
 * number of adjacency entries (each spring and bending pair counted from both
 * endpoints) and S the sum of C^2 over them, C = |p_self - p_other| - l0
 * evaluated in float as the sweep evaluates it.  Per-vertex and per-block
 * sums are float in a fixed order, the sum over blocks is FP64 in a fixed
 * order, so the value is deterministic.  Workspace:
 * sx_residual_workspace_bytes(n_verts), zero-filled before its first use (its
 * block counter is left zero after every call). */
size_t sx_residual_workspace_bytes(int n_verts);
int sx_constraint_residual(const float* p4, const int* adj_ptr, const int* adj, int n_verts, double* out3, void* ws,
                           size_t ws_bytes, void* stream);

/* System energy in FP64 (no counterpart in the reference): out3 (device) =
 * {kinetic 1/2 sum m |v|^2, gravitational -sum m (g . x), elastic
 * 1/2 sum k C^2} with m = 1/m_inv over vertices with m_inv > 0, C = |x_a - x_b|
 * - l0 over the springs (k = k_spring) and bending pairs (k = k_bend) of the
 * adjacency (adj_ptr/adj as for sx_jacobi_sweep).  Every term in double from
 * the float inputs, sums in a fixed order (deterministic).  Workspace:
 * sx_energy_workspace_bytes(n_verts). */
size_t sx_energy_workspace_bytes(int n_verts);
int sx_system_energy(const float* x4, const float* v4, const float* m_inv, const int* adj_ptr, const int* adj,
                     int n_verts, float k_spring, float k_bend, float gx, float gy, float gz, double* out3, void* ws,
                     size_t ws_bytes, void* stream);

/* Iterating to a residual (no counterpart in the reference, which runs one
 * sweep per substep).  conv is a device int[8]:
 *   conv[0] stop iteration of the current substep (-1: not converged),
 *   conv[2] checks made this substep, conv[3] sum of stop iterations and
 *   conv[4] converged substeps since the last reset_totals, conv[5] the next
 *   check's iteration and conv[6] the check interval (device-side loops).
 * sx_convergence_begin starts a substep with checks every check_every (even)
 * iterations.  sx_jacobi_sweep_checked is sx_jacobi_sweep with bending on y,
 * launched for Jacobi iteration `iter` of the substep.  With check != 0 (iter
 * a multiple of check_every) it also computes the residual of its input y_in4
 * (the state after iteration iter-1) into res3, as sx_constraint_residual
 * would, and if that is <= tol (ref3 NULL) or <= tol * ref3[2] (ref3 = a
 * residual from sx_constraint_residual, e.g. of the substep's cold start) sets
 * conv[0] = iter.  The rest of that block of check_every iterations runs;
 * every kernel of a later iteration iter' (this sweep, and the contact sweeps
 * given the same conv and iter') returns at once, so y ends in the buffer it
 * would have ended in after an even number of sweeps.  No host
 * synchronisation is involved.
 *
 * Inside a CUDA graph the remaining iterations can run as a device-side loop
 * instead (nothing is launched after convergence): sx_loop_begin, while
 * `stream` is being captured, appends a conditional WHILE node and captures
 * its body on body_stream; the caller issues one block of check_every
 * iterations there -- the first a checked sweep given loop = *handle_out and
 * the cap n_iter, the contact sweeps with conv NULL -- and sx_loop_end closes
 * the body.  The checked sweep ends the loop once converged or when the next
 * block would start at n_iter.  Same iterations as the gated form. */
int sx_convergence_begin(int* conv, int check_every, int reset_totals, void* stream);
int sx_jacobi_sweep_checked(const float* x4, const float* y_in4, float* y_out4, const float* fixed, const int* adj_ptr,
                            const int* adj, int n_verts, float k_spring, float k_bend, int iter, int check, double tol,
                            const double* ref3, int* conv, double* res3, void* ws, size_t ws_bytes,
                            unsigned long long loop, int n_iter, void* stream);
/* sx_jacobi_sweep_checked with the arithmetic choice of sx_jacobi_sweep_mode */
int sx_jacobi_sweep_checked_mode(const float* x4, const float* y_in4, float* y_out4, const float* fixed,
                                 const int* adj_ptr, const int* adj, int n_verts, float k_spring, float k_bend,
                                 int iter, int check, double tol, const double* ref3, int* conv, double* res3,
                                 void* ws, size_t ws_bytes, unsigned long long loop, int n_iter, int fast,
                                 void* stream);
int sx_loop_begin(void* stream, void* body_stream, unsigned long long* handle_out, void** ctx_out);
int sx_loop_end(void* ctx);

/* the two halves of sx_velocity_update, for substeps with the velocity-level
 * contact pass between them: compute_velocity (XPBD.py:341-343) and update_x
 * (XPBD.py:333-337) */
int sx_compute_velocity(const float* x4, const float* y4, float* v4, const float* fixed, int n_verts, float damping,
                        float dt, void* stream);
int sx_update_x(float* x4, const float* v4, int n_verts, float dt, void* stream);

/* computeAABB_faces, meshTaichiWrapper.py:351-365 (positions p4) */
int sx_face_aabbs(const float* p4, const int* faces, int n_faces, float padding, float* aabb_min4,
                  float* aabb_max4, void* stream);
/* The same, plus chunk boxes: chunk_min4/max4[c] (float4, ceil(n_faces / 32)
 * of each) = the union of the padded boxes of faces 32c .. 32c+31, for broad
 * phases that test chunks before faces (no counterpart in the reference). */
int sx_face_aabbs_chunked(const float* p4, const int* faces, int n_faces, float padding, float* aabb_min4,
                          float* aabb_max4, float* chunk_min4, float* chunk_max4, void* stream);

/* computeAABB, meshTaichiWrapper.py:335-347: box6 (device) = vertex AABB +- padding.
 * The reference returns the box to the host; here it stays on the device. */
int sx_scene_aabb(const float* p4, int n_verts, float padding, float* box6, void* stream);

/* ---- LBVH over the 32^3 cell grid (framework/collision/lbvh_cell.py) ------- */

/* LBVH_CELL.__init__, lbvh_cell.py:78-80: Morton codes of the 32768 cell
 * centres (assign_cell_morton :123-152), radix sort (radix_sort_cells
 * :553-562) and Karras build (assign_internal_nodes_Karras12_cells :408-430).
 * Outputs are 32768 (codes, ids) and 32767 internal nodes; parent has 65535. */
size_t sx_cell_bvh_workspace_bytes(int n_faces);
int sx_cell_bvh_init(int* sorted_codes, int* sorted_ids, int* child_a, int* child_b, int* range_l, int* range_r,
                     int* parent, void* ws, size_t ws_bytes, void* stream);

/* LBVH_CELL.build, lbvh_cell.py:637-653: cell size from box6
 * (assign_cell_centers :105-120), faces binned by AABB centre
 * (assign_face_cell_ids :577-586), inclusive scan, stable counting sort
 * (counting_sort_cells :589-598), leaves = row-major cells with
 * AABB = centre U faces (assign_leaf_cell_nodes :602-634) and a single-launch
 * bottom-up refit with the rules of compute_cell_node_aabbs :491-522.
 * Outputs: sorted_face_ids[n_faces], prefix[32768] (inclusive),
 * num_faces[65535], nmin4/nmax4[65535] (nmin4.w = the node's face count as
 * int bits), face_rec8[8*n_faces] (per sorted face: min xyz + face id bits,
 * max xyz + 0; what the traversal scans), grid8[1032] = {cell size xyz, the
 * largest distance any leaf box reaches beyond its cell per axis, 0, 0,
 * then 1024 uint32 occupancy words: bit z of word x*32 + y set when cell
 * (x, y, z) holds faces}. */
int sx_cell_bvh_build(const float* fmin4, const float* fmax4, int n_faces, const float* box6, const int* child_a,
                      const int* child_b, const int* parent, int* sorted_face_ids, int* prefix, int* num_faces,
                      float* nmin4, float* nmax4, float* face_rec8, float* grid8, void* ws, size_t ws_bytes,
                      void* stream);

/* traverse_cell_bvh_single, lbvh_cell.py:656-714, for query boxes
 * p4[i] +- padding (Solver.broadphase_lbvh, XPBD.py:187-215), over a build's
 * nodes, grid8 and face records.  origin = box6 of the build (its min corner is
 * the grid origin).  cand[q*cap + j] for j < cap; num[q] = total overlaps
 * found (num > cap: list truncated, status bit 1).  Candidates come out in
 * the reference's depth-first visiting order, which for the cell tree is
 * descending cell index; the walk visits the cells within the leaves' reach of
 * each query box in that order. */
int sx_cell_bvh_traverse(const float* p4, int n_queries, float padding, const float* grid8, const float* origin_box6,
                         const float* nmin4, const float* nmax4, const int* prefix, const float* face_rec8, int cap,
                         int* cand, int* num, int* status, void* stream);

/* The same walk for edge boxes (the reference's commented-out edge broad
 * phase, XPBD.py:217-232): query q is the box of edge (edges[2q], edges[2q+1])
 * of the points p4, min - padding .. max + padding per axis. */
int sx_cell_bvh_traverse_edges(const int* edges, int n_edges, const float* p4, float padding, const float* grid8,
                               const float* origin_box6, const float* nmin4, const float* nmax4, const int* prefix,
                               const float* face_rec8, int cap, int* cand, int* num, int* status, void* stream);

/* ---- face-level LBVH (standalone broad phase) ------------------------------ */

/* Morton codes of face-AABB centres normalised by box6 (intended form of
 * LBVH_CELL.assign_morton, lbvh_cell.py:196-232; morton_3d :87-102). ids[i]=i */
int sx_face_morton(const float* fmin4, const float* fmax4, int n_faces, const float* box6, unsigned* codes,
                   int* ids, void* stream);

/* Stable LSD radix sort of (key, value) pairs on the low `bits` key bits
 * (radix_sort_cells, lbvh_cell.py:525-562: the reference uses 6-bit digits and
 * a serialised scatter; here 8-bit digits, per-block histograms and a
 * warp-ranked stable scatter give the same permutation). In place. Key bits
 * at and above `bits` take no part in the order: they move with their key. */
size_t sx_radix_sort_workspace_bytes(int n);
int sx_radix_sort_pairs(unsigned* keys, int* vals, int n, int bits, void* ws, size_t ws_bytes, void* stream);

/* The same sort for callers that cannot allocate device memory when they
 * sort -- e.g. hosts whose device memory belongs to another allocator with a
 * fixed budget, or real-time loops that cannot take the synchronisation a
 * cudaMalloc may cause.  It takes no workspace and allocates nothing: its
 * scratch is a fixed array in the library's own device memory (about 2.1 MB,
 * held on every GPU that loads the library until the process exits).
 * n is limited to 262144 (2^18) keys; larger n returns SX_ERR_ARG.  The first
 * call on a device looks up the array's device address with that device
 * current; make that first call before any stream capture.  The address is
 * kept for the life of the process: after cudaDeviceReset (or anything else
 * that re-creates the device's primary context) this entry point must not be
 * called again in that process.  All calls share the array, so calls that
 * overlap on the GPU race and must be ordered by the caller.  This entry point
 * has no counterpart in the reference. */
int sx_radix_sort_pairs_noalloc(unsigned* keys, int* vals, int n, int bits, void* stream);

/* Karras 2012 hierarchy over sorted codes (assign_internal_nodes_Karras12,
 * lbvh_cell.py:384-405, with delta/find_split/determine_range :256-336).
 * tie = 0: the reference's rule (equal codes give delta = 32, split at the
 * midpoint); tie = 1: equal codes compare by index (always a valid tree).
 * parent has 2n-1 entries; parent[0] = -1. */
int sx_karras_build(const unsigned* codes, int n, int tie, int* child_a, int* child_b, int* range_l,
                    int* range_r, int* parent, void* stream);

/* Bottom-up refit of a face-level LBVH (one face per leaf; leaf n-1+j holds
 * face sorted_ids[j]): node box = union of children, single launch with
 * per-node arrival counters (flags: n-1 ints scratch, zero on entry, left
 * zero on exit). */
int sx_face_bvh_refit(int n, const int* sorted_ids, const float* fmin4, const float* fmax4, const int* child_a,
                      const int* child_b, const int* parent, float* nmin4, float* nmax4, int* flags, int* status,
                      void* stream);

/* sx_face_bvh_refit with the tree's lower levels in shared memory: nodes
 * whose leaf range [range_l, range_r] (from sx_karras_build) lies in one tile
 * of 256 sorted leaves are refit inside the tile's block; the rest as above.
 * Same boxes, same scratch contract. */
int sx_face_bvh_refit_tiled(int n, const int* sorted_ids, const float* fmin4, const float* fmax4,
                            const int* child_a, const int* child_b, const int* parent, const int* range_l,
                            const int* range_r, float* nmin4, float* nmax4, int* flags, int* status, void* stream);

/* Stack traversal of a face-level LBVH for query boxes p4[i] +- padding, same
 * visiting order as traverse_cell_bvh_single (lbvh_cell.py:662-714). */
int sx_face_bvh_traverse(int n, const float* p4, int n_queries, float padding, const int* child_a,
                         const int* child_b, const int* sorted_ids, const float* nmin4, const float* nmax4, int cap,
                         int* cand, int* num, int* status, void* stream);
/* sx_face_bvh_traverse visiting the queries in the order order[0..n_queries)
 * (a permutation, e.g. the queries sorted by Morton code: a warp then walks
 * nearby parts of the tree).  Results are per query and do not depend on it. */
int sx_face_bvh_traverse_ordered(int n, const float* p4, int n_queries, float padding, const int* child_a,
                                 const int* child_b, const int* sorted_ids, const float* nmin4, const float* nmax4,
                                 int cap, int* cand, int* num, int* status, const int* order, void* stream);

/* ---- narrow phase + contact projection ------------------------------------ */

/* solve_collision_constraints_x (XPBD.py:237-264) -> __vt_st / __vt_dy /
 * __tv_st (collision_constraints_x.py:6-310; distance.py:5-47, :102-184,
 * :413-459), then update_dx (XPBD.py:384-387) on the dynamic mesh y4.
 * Candidate blocks: vt_st and vt_dy are n_dy x cap, tv_st is n_st x cap.
 * Corrections are accumulated in 64-bit fixed point (40 fractional bits) in
 * dx_fix[3*n_dy] and nc[n_dy], which must be zero on entry and are zero again
 * on return.  Pair records (pair[2], pair_g[16 floats], pair_schur, pair_num;
 * blocks vt_st | vt_dy | tv_st, each query x cap) are optional: pass NULL. */
int sx_collision_sweep(int n_dy, int n_st, const int* faces_dy, const int* faces_st, float* y4, const float* xs4,
                       const float* fixed, const float* m_inv, float dHat, float compliance, int cap,
                       const int* vt_st_cand, const int* vt_st_num, const int* vt_dy_cand, const int* vt_dy_num,
                       const int* tv_st_cand, const int* tv_st_num, long long* dx_fix, int* nc, int* pair,
                       float* pair_g, float* pair_schur, int* pair_num, int* status, void* stream);

/* The same contact projection over a dense pair list.  The candidate lists do
 * not change between the Jacobi iterations of a substep (the broad phase runs
 * once per substep), so sx_contact_pairs_build flattens them once -- in query
 * order, dropping the incident faces __vt_dy skips (XPBD.py:258) -- into
 * pairs[max_pairs] (int4: query vertex, triangle vertices;
 * max_pairs >= (2*n_dy + n_st) * cap), and sx_contact_pairs_sweep then runs
 * one thread per pair followed by update_dx.  Same arithmetic and the same
 * order-independent accumulation as sx_collision_sweep, hence the same result;
 * pair records are only available from sx_collision_sweep.
 * cull_d2 > 0 skips a pair before its region classification when the squared
 * distance from the point to the triangle's bounding box exceeds cull_d2; the
 * point-triangle distance of every region is at least that distance, so with
 * cull_d2 a margin above dHat (the solver passes dHat * 1.0625) a culled pair
 * is one whose projection adds nothing.  cull_d2 <= 0 evaluates every pair.
 * conv/iter: convergence gate of sx_jacobi_sweep_checked (conv NULL: always
 * runs). */
size_t sx_contact_pairs_workspace_bytes(int n_dy, int n_st);
int sx_contact_pairs_build(int n_dy, int n_st, const int* faces_dy, const int* faces_st, int cap,
                           const int* vt_st_cand, const int* vt_st_num, const int* vt_dy_cand, const int* vt_dy_num,
                           const int* tv_st_cand, const int* tv_st_num, int* pairs, long long max_pairs, void* ws,
                           size_t ws_bytes, void* stream);
int sx_contact_pairs_sweep(int n_dy, int n_st, const int* pairs, const void* ws, float* y4, const float* xs4,
                           const float* fixed, const float* m_inv, float dHat, float compliance, float cull_d2,
                           long long* dx_fix, int* nc, int* status, const int* conv, int iter, void* stream);
/* The two halves of sx_contact_pairs_sweep: the projection, which only adds
 * to dx_fix / nc, and update_dx (XPBD.py:384-387), which applies and clears
 * them. */
int sx_contact_pairs_project(int n_dy, int n_st, const int* pairs, const void* ws, const float* y4, const float* xs4,
                             const float* fixed, const float* m_inv, float dHat, float compliance, float cull_d2,
                             long long* dx_fix, int* nc, int* status, const int* conv, int iter, void* stream);
/* sx_contact_pairs_project in one of its compiled launch configurations
 * (identical results): pair batches box-tested per warp step and resident
 * blocks per SM, as sx_contact_pairs_project_variant_info reports. */
int sx_contact_pairs_project_variants(void);
int sx_contact_pairs_project_variant_info(int variant, int* unroll, int* blocks_per_sm);
/* 1 if that variant is the pipelined form: the vertex-vs-obstacle and
 * obstacle-vertex pairs one per lane with their positions kept in registers,
 * and the next step's pair records loaded while the current step's positions
 * are gathered; 0 for the stacked form.  Same sums either way. */
int sx_contact_pairs_project_variant_pipelined(int variant);
int sx_contact_pairs_project_v(int n_dy, int n_st, const int* pairs, const void* ws, const float* y4,
                               const float* xs4, const float* fixed, const float* m_inv, float dHat, float compliance,
                               float cull_d2, long long* dx_fix, int* nc, int* status, const int* conv, int iter,
                               int variant, void* stream);
int sx_contact_apply(int n_dy, float* y4, const float* fixed, long long* dx_fix, int* nc, const int* conv, int iter,
                     void* stream);


/* Edge-edge contacts: __ee_st / __ee_dy (collision_constraints_x.py:313-588;
 * d_type_EE distance.py:50-99, d_EE :119-124; the gradient in closed form)
 * as the reference's commented-out solver code would call them
 * (XPBD.py:266-281): for every cloth edge e and candidate face f (ee_st:
 * static faces, ee_dy: cloth faces; n_edges_dy x cap each), the three edges
 * face_edges[3f + k] of f; ee_dy skips edges sharing a vertex with e.  Only
 * d_type_EE == 8 with |x01 x x23| > 1e-3 and d_EE < dHat projects:
 * ld = compliance (dHat - d) / (compliance schur + 1), dx += fixed m_inv ld g
 * on the cloth's vertices (ee_st: e's two; ee_dy: all four).  Terms are
 * ADDED to dx_fix / nc; no update_dx -- run before sx_collision_sweep or
 * sx_contact_pairs_sweep of the same iteration, which apply both.  ee_st_cand
 * NULL: no static mesh.  Records (optional): blocks ee_st | ee_dy of
 * n_edges_dy queries x cap, (partner edge, dtype), gradients, schur; records
 * past cap are dropped (the reference writes past its cache).  conv/iter: the
 * convergence gate of sx_jacobi_sweep_checked. */
int sx_edge_edge_sweep(int n_edges_dy, const int* edges_dy, const int* edges_st, const int* face_edges_dy,
                       const int* face_edges_st, const float* y4, const float* xs4, const float* fixed,
                       const float* m_inv, float dHat, float compliance, int cap, const int* ee_st_cand,
                       const int* ee_st_num, const int* ee_dy_cand, const int* ee_dy_num, long long* dx_fix, int* nc,
                       int* pair, float* pair_g, float* pair_schur, int* pair_num, int* status, const int* conv,
                       int iter, void* stream);
/* d_type_EE, the projected distance (dHat unless dtype 8 with
 * |x01 x x23| > 1e-3) and its gradient for n quadruples p12[12 i ..] = x0, x1
 * (edge 0), x2, x3 (edge 1): dtype[n], d[n], g12[12 n]. */
int sx_edge_edge_classify(int n, const float* p12, float dHat, int* dtype, float* d, float* g12, void* stream);

/* Persistent batched substep (no counterpart in the reference, whose batching
 * is mesh concatenation, framework/meshio/concat.py:11-58): one launch runs a
 * whole substep of every instance of a batch.  Each CTA (or, in the cluster
 * variants, each thread-block cluster) takes instances from a queue in the
 * order `order` (largest first), and for its instance alone
 * computes the cloth box (sx_segment_aabbs) and padded face boxes on x, with
 * predict != 0 the prediction y = compute_y(x, v) (sx_predict; 0: y already
 * holds the start, e.g. a learned warm start), n_iter Jacobi iterations --
 * the sweep with bending on y (sx_jacobi_sweep_v / sx_jacobi_sweep_mode with
 * `fast`), in the first iteration the obstacle broad phase
 * (sx_batched_obstacle_broadphase), then the obstacle contacts and update_dx
 * (sx_batched_obstacle_contacts) -- and the velocity update
 * (sx_velocity_update), with block (cluster) barriers between the phases.  y and
 * y_other ping-pong: after an even n_iter the final positions are in y, after
 * an odd one in y_other.  The result equals those grid-wide launches bit for
 * bit.  Chunk boxes are per instance: cmin4 / cmax4 hold cptr[n_inst] boxes,
 * instance i's chunks of 32 faces at cptr[i] .. cptr[i+1].  queue: two ints,
 * zero before the first launch and left zero by every launch.  Fixed
 * iteration counts only (iterating to a residual uses the grid-wide
 * launches).  adj_nbr16 / adj_rest32: the packed adjacency
 * (sx_jacobi_sweep_packed) or both null. */
typedef struct SxBatchedSubstep {
    int n_inst, n_iter, predict, cap;
    const int *order, *vptr, *fptr, *cptr, *optr, *ob_fptr;
    float *x4, *y4, *y_other4, *v4;
    const float *fixed, *m_inv;
    const int *adj_ptr, *adj;
    const short* adj_nbr16;      /* the packed adjacency (sx_jacobi_sweep_packed), or */
    const unsigned* adj_rest32;  /* null: the sweep then reads adj                    */
    const int *faces, *ob_faces;
    const float* xs4;
    float *fmin4, *fmax4, *cmin4, *cmax4, *cl_box6;
    const float *ob_box6, *ob_fmin4, *ob_fmax4;
    unsigned* vmask;
    int *tv_cand, *tv_num;
    long long* dx_fix;
    int *nc, *status, *queue;
    float padding, dt, gx, gy, gz, k_spring, k_bend, dHat, compliance, damping;
} SxBatchedSubstep;
int sx_batched_substep_variants(void);
int sx_batched_substep_variant_info(int variant, int* block, int* blocks_per_sm);
/* CTAs per instance of a variant: 1 = an instance per CTA (block barriers);
 * more = an instance per thread-block cluster of that many CTAs (hardware
 * cluster barriers; fewer instances in flight, so their working set stays in
 * L2 across the iterations).  Results are identical for every variant. */
int sx_batched_substep_variant_cluster(int variant);
int sx_batched_substep(const SxBatchedSubstep* args, int variant, int fast, void* stream);

/* solve_constraints_v (XPBD.py:374-381, :398-404; collision_constraints_v.py
 * __vt_st :6-133, __tv_st :137-330, __vt_dy :334-570): velocity-level contact
 * and friction over the pair records of the last sx_collision_sweep (pair,
 * pair_g, pair_schur, pair_num as written there), velocities v4 of the dynamic
 * mesh and vs4 of the static one, friction coefficient mu; then update_dv
 * (v += fixed * dv / nc where m_inv > 0).  dv_fix/nc: zero on entry, left
 * zero.  m_inv_st: the static mesh's inverse masses (read by __vt_st region
 * 3, as the reference does). */
int sx_velocity_contacts(int n_dy, int n_st, const int* faces_dy, const int* faces_st, int cap, const int* pair,
                         const float* pair_g, const float* pair_schur, const int* pair_num, float* v4, const float* vs4,
                         const float* fixed, const float* m_inv, const float* m_inv_st, float mu, long long* dv_fix,
                         int* nc, int* status, void* stream);

/* ---- batched independent cloths with obstacles ---------------------------- */

/* computeAABB (meshTaichiWrapper.py:335-347) for each segment
 * [seg_ptr[s], seg_ptr[s+1]) of a point array: box6[6*s..] = AABB +- padding. */
int sx_segment_aabbs(const float* p4, const int* seg_ptr, int n_seg, float padding, float* box6, void* stream);

/* Broad phase of the obstacle contacts of a batch (Solver.broadphase_lbvh,
 * XPBD.py:187-215, restricted to each instance): for cloth vertex v of
 * instance vinst[v], vmask[v] bit k = obstacle face ob_fptr[inst] + k is a
 * candidate (padded boxes overlap, and the query is not skipped by the rule of
 * lbvh_cell.py:665 on the obstacle's grid ob_box6[inst]); for obstacle vertex
 * s of instance svinst[s], tv_cand[s*cap..] lists its cloth faces in
 * [cl_fptr[inst], cl_fptr[inst+1]) (ascending, grid cl_box6[inst]).  These are
 * the candidate sets the reference's cell-BVH traversal returns.  At most 32
 * obstacle faces per instance.  cl_cmin4/cl_cmax4: the cloth faces' chunk
 * boxes (sx_face_aabbs_chunked); a chunk that misses the query is skipped
 * whole, which leaves the candidate lists unchanged. */
int sx_batched_obstacle_broadphase(int n_verts, const float* y4, const int* vinst, const float* ob_box6,
                                   const int* ob_fptr, const float* ob_fmin4, const float* ob_fmax4, float padding,
                                   unsigned* vmask, int n_ob_verts, const float* xs4, const int* svinst,
                                   const float* cl_box6, const int* cl_fptr, const float* cl_fmin4,
                                   const float* cl_fmax4, const float* cl_cmin4, const float* cl_cmax4, int cap,
                                   int* tv_cand, int* tv_num, int* status, void* stream);

/* __vt_st / __tv_st (collision_constraints_x.py:6-173) over those candidates,
 * fixed-point accumulation, then update_dx (XPBD.py:384-387). */
int sx_batched_obstacle_contacts(int n_verts, float* y4, const float* fixed, const float* m_inv, const int* vinst,
                                 const int* ob_fptr, const int* ob_faces, const float* xs4, const unsigned* vmask,
                                 int n_ob_verts, const int* tv_cand, const int* tv_num, int cap, const int* cl_faces,
                                 float dHat, float compliance, long long* dx_fix, int* nc, int* status, const int* conv,
                                 int iter, void* stream);

/* ---- constraint-graph colouring (framework/utilities/graph_coloring.py) --- */

/* initAdjEdges + colorEdgesGreedy + colorCountingSort, graph_coloring.py:112-201:
 * colour = first-fit over edges in id order (edges sharing a vertex are
 * adjacent; all max_colors forbidden -> 0), computed in parallel: an edge is
 * coloured once all its lower-id neighbours are; then a
 * stable sort by colour.  prefix[max_colors] = start offset of each colour.
 * One cooperative launch colours every edge as soon as its lower-id
 * neighbours have colours (bounded waits, no host synchronisation).  After
 * the call the first int of ws holds status bits: SX_STATUS_WAIT_TIMEOUT if a
 * wait gave up, the colours then being incomplete. */
size_t sx_color_workspace_bytes(int n_verts, int n_edges);
int sx_color_edges_greedy(const int* edges, int n_edges, int n_verts, int max_colors, int* color, int* sorted_edges,
                          int* prefix, void* ws, size_t ws_bytes, void* stream);

/* ---- colour-ordered Gauss-Seidel sweep (consumer of the colouring) ----------
 * The reference colours its constraints for a parallel Gauss-Seidel solver it
 * marks as work in progress (README.md:20-22, graph_coloring.py:8-97); its
 * solver runs only the Jacobi sweep.  Springs 0..E-1 and bending pairs
 * E..E+B-1 are coloured together as one edge list (sx_color_edges_greedy on
 * [edges; bend]) and packed in colour order by sx_gs_pack:
 * cons[i] = {v0, v1 | 0x80000000 for a bending pair, bits(rest length), id}
 * for id = sorted[i]; *bad gets 1 if an id is out of range.
 *
 * sx_gs_sweep: one sweep, one launch per colour c over
 * cons[colour_start[c] .. colour_start[c+1]) (colour_start: n_colors + 1 HOST
 * ints).  Each constraint is projected on the current positions and both
 * endpoints move at once: y0 -= (w0*ld)*n, y1 += (w1*ld)*n, with n, ld as in
 * the Jacobi sweep (XPBD.py:141-184), w = y4.w, k = k_spring or k_bend.
 * Constraints of one colour share no vertex, so y4 is updated in place
 * without races and the result is independent of thread order. */
int sx_gs_pack(const int* edges, const float* l0, int E, const int* bend, const float* bend_l0, int B,
               const int* sorted, int* cons, int* bad, void* stream);
int sx_gs_sweep(float* y4, const int* cons, const int* colour_start, int n_colors, float k_spring, float k_bend,
                void* stream);

/* ---- learned warm start (no counterpart in the reference) -----------------
 * The reference starts every Jacobi solve from the predicted positions
 * (XPBD.py:116-118).  Here a per-vertex MLP 24 -> 64 -> 64 -> 3 (SiLU, BF16
 * weights and activations, FP32 accumulation on tensor cores) predicts a
 * position correction in units of L (the vertex's mean spring rest length);
 * the solve starts from y_pred + fixed * L * correction, or from y_pred when
 * that raises the constraint residual.
 *
 * Parameters: FP32 master blob of sx_mlp_param_count() floats
 * (W1[64][32] | b1[64] | W2[64][64] | b2[64] | W3[8][64] | b3[8]) and its BF16
 * copy of the three matrices (sx_mlp_bf16_count() values, 2 bytes each).
 * Feature rows: BF16[n][32] (24 features, 8 zeros). */
int sx_mlp_param_count(void);
int sx_mlp_bf16_count(void);
/* features of every vertex from y4 (predicted), x4, c4 (previous solve
 * correction), fixed, the constraint CSR and Lref; also copies y4 to y_pred4
 * when that is not NULL */
int sx_warm_features(const float* x4, const float* y4, const float* c4, const float* fixed, const int* adj_ptr,
                     const int* adj, const float* Lref, int n_verts, float gx, float gy, float gz, float dt,
                     void* feat, float* y_pred4, void* stream);
/* out4[n][4] (columns 0..2 used) = MLP(feat) */
int sx_mlp_forward(const void* feat, int n_rows, const void* w16, const float* p32, float* out4, void* stream);
/* The same network on tcgen05 tensor cores (128-row tiles, accumulators in
 * tensor memory); same outputs up to the order of FP32 accumulation and the
 * bias being added after the products.  A device-side wait that gives up
 * (1 s) sets SX_STATUS_WAIT_TIMEOUT in status. */
int sx_mlp_forward_tc(const void* feat, int n_rows, const void* w16, const float* p32, float* out4, int* status,
                      void* stream);
/* y4 = y_pred4 + fixed * (Lref * out4[:, :3]) */
int sx_warm_apply(const float* y_pred4, const float* out4, const float* fixed, const float* Lref, int n_verts,
                  float* y4, void* stream);
/* if res_warm3[2] > res_cold3[2] (residuals from sx_constraint_residual),
 * y4 = y_pred4; flags2[0] counts such fallbacks, flags2[1] kept warm starts */
int sx_warm_select(const double* res_warm3, const double* res_cold3, const float* y_pred4, float* y4, int n_verts,
                   int* flags2, void* stream);
/* after the solve: c4 = y4 - y_pred4, and (when target4 is not NULL) the
 * training target target4 = ((y4 - y_pred4) / Lref, fixed) */
int sx_warm_record(const float* y4, const float* y_pred4, const float* fixed, const float* Lref, int n_verts,
                   float* c4, float* target4, void* stream);
/* Training over the rows idx[n_rows] of (feat, target4): loss = sum of
 * target4.w * |out[:3] - target4.xyz|^2 / n_valid.  sx_mlp_gradients writes
 * the gradient (sx_mlp_param_count() floats) and stats[0] = n_valid * loss;
 * sx_mlp_train_step also applies one Adam step (bias corrections for `step`,
 * 1-based) to p32 and refreshes w16.  Partial sums are combined in a fixed
 * order.  Workspace: sx_mlp_train_workspace_bytes(n_rows). */
size_t sx_mlp_train_workspace_bytes(int max_rows);
int sx_mlp_gradients(const void* feat, const float* target4, const int* idx, int n_rows, int n_valid, const void* w16,
                     const float* p32, float* grad, float* stats, void* ws, size_t ws_bytes, void* stream);
int sx_mlp_train_step(const void* feat, const float* target4, const int* idx, int n_rows, int n_valid, void* w16,
                      float* p32, float* adam_m, float* adam_v, float lr, float beta1, float beta2, float eps, int step,
                      float* stats, void* ws, size_t ws_bytes, void* stream);
/* w16 = BF16(p32) for the three weight matrices */
int sx_mlp_sync_bf16(const float* p32, void* w16, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* STARXPBD_H */
