/*
 * ikdg.h - C ABI of the GB300 incremental k-d tree (libikdg.so).
 *
 * A drop-in replacement for the hot path of hku-mars/ikd-Tree's
 * KD_TREE<PointType> (ikd-Tree/ikd_Tree.h:59-249): the tree lives in GPU memory
 * and every call below runs CUDA kernels on one GPU.  There is no CPU fallback:
 * without a usable CUDA device ikdg_create fails with IKDG_NO_DEVICE.
 *
 * Conventions
 *   - Points are float xyz triples; `stride` is the distance in floats between
 *     consecutive points (3 for packed xyz, 4 for pcl::PointXYZ, ...).
 *   - Boxes are 6 floats {min x, min y, min z, max x, max y, max z}
 *     (BoxPointType, ikd-Tree/ikd_Tree.h:32-35); box tests are half-open,
 *     min <= p < max, as in the reference.
 *   - Every point gets a 32-bit id when it enters the tree: Build numbers its
 *     points 0..n-1, later insertions continue the sequence.  Searches report
 *     ids; distance ties are broken by the smaller id.
 *   - Functions taking host pointers are synchronous.  *_device variants take
 *     device pointers and are asynchronous on the tree's stream.
 *   - All functions return an ikdg_status code.
 *
 * Thread safety: calls on one tree are serialised by an internal mutex; the
 * reference's concurrent Nearest_Search callers (ikd_Tree.cpp:875-884) are
 * therefore safe, and mutations from several threads are ordered.
 */
#ifndef IKDG_H
#define IKDG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ikdg_tree ikdg_tree;
typedef struct ikdg_batch ikdg_batch;

enum ikdg_status {
    IKDG_OK = 0,
    IKDG_BAD_ARG = 2,        /* invalid argument (null pointer, k <= 0, NaN / inf point ...) */
    IKDG_CAPACITY = 3,       /* an output buffer is too small; the required size is reported */
    IKDG_DEVICE_TIMEOUT = 4, /* a bounded device-side wait gave up */
    IKDG_CUDA_ERR = 5,       /* a CUDA runtime call failed; see ikdg_last_error */
    IKDG_NO_DEVICE = 6,      /* no usable CUDA device */
    IKDG_INTERNAL = 7        /* an internal invariant failed; see ikdg_last_error */
};

const char* ikdg_status_string(int status);
/* Text of the last error on this tree (thread-unsafe across trees: per tree). */
const char* ikdg_last_error(const ikdg_tree* t);

/* KD_TREE(float delete_param, float balance_param, float box_length)
 * (ikd-Tree/ikd_Tree.h:226, ikd_Tree.cpp:9-17).  `device` selects the CUDA
 * device (-1: the current one). */
int ikdg_create(float delete_param, float balance_param, float box_length, int device, ikdg_tree** out);
/* ~KD_TREE (ikd_Tree.cpp:19-27). */
int ikdg_destroy(ikdg_tree* t);

/* Set_delete_criterion_param / Set_balance_criterion_param /
 * set_downsample_param (ikd_Tree.h:228-230, ikd_Tree.cpp:29-42). */
int ikdg_set_delete_criterion_param(ikdg_tree* t, float delete_param);
int ikdg_set_balance_criterion_param(ikdg_tree* t, float balance_param);
int ikdg_set_downsample_param(ikdg_tree* t, float box_length);
/* Tuning knobs (no counterpart in the reference): points per leaf bucket
 * written by (re)builds, 8..32 (default 16); threads cooperating on one kNN
 * query, 1, 2 or 4 (default 1); tree levels used to sort a kNN batch into
 * spatially coherent order before the search: -1 (default) sorts by 16
 * levels from 262,144 queries up and not below, 0 never sorts, 1..16 sorts
 * every batch of at least 2048 queries. */
int ikdg_set_leaf_fill(ikdg_tree* t, int fill);
int ikdg_set_knn_lanes(ikdg_tree* t, int lanes);
int ikdg_set_knn_bin_bits(ikdg_tree* t, int bits);

/* Build(PointVector) (ikd_Tree.h:235, ikd_Tree.cpp:352-364). */
int ikdg_build(ikdg_tree* t, const float* xyz, int64_t n, int32_t stride);

/* Add_Points(PointVector&, bool downsample_on) (ikd_Tree.h:239,
 * ikd_Tree.cpp:413-489).  *n_added receives the reference's return value: the
 * number of downsampling insertions, 0 without downsampling.  Unlike the
 * reference (which dereferences a null root, ikd_Tree.cpp:472) adding to an
 * empty tree works. */
int ikdg_add_points(ikdg_tree* t, const float* xyz, int64_t n, int32_t stride, int downsample_on, int64_t* n_added);

/* Delete_Points(PointVector&) (ikd_Tree.h:241, ikd_Tree.cpp:513-533): each
 * input point deletes one valid point within 1e-6 per axis, if any. */
int ikdg_delete_points(ikdg_tree* t, const float* xyz, int64_t n, int32_t stride);

/* Delete_Point_Boxes(vector<BoxPointType>&) (ikd_Tree.h:242,
 * ikd_Tree.cpp:535-556).  *n_deleted = number of valid points deleted. */
int ikdg_delete_boxes(ikdg_tree* t, const float* boxes, int64_t m, int64_t* n_deleted);

/* Add_Point_Boxes(vector<BoxPointType>&) (ikd_Tree.h:240,
 * ikd_Tree.cpp:491-511): restores points inside the boxes that were deleted by
 * box or point deletion and are still stored. */
int ikdg_add_boxes(ikdg_tree* t, const float* boxes, int64_t m);

/* Nearest_Search(point, k, Nearest_Points, Point_Distance, max_dist)
 * (ikd_Tree.h:236, ikd_Tree.cpp:366-397), batched over nq queries.  Row i of
 * the outputs holds the k nearest valid points whose float squared distance
 * is <= max_dist * max_dist evaluated in double, as the reference does
 * (ikd_Tree.cpp:872, :887; INFINITY: unbounded), ascending; missing
 * entries have id -1 and distance +inf.  out_xyz (nq*k*3) and out_count (nq)
 * may be NULL.  k >= 1 (k <= 64 keeps the candidates in registers). */
int ikdg_knn(ikdg_tree* t, const float* q, int64_t nq, int32_t stride, int32_t k, double max_dist,
             int32_t* out_ids, float* out_d2, float* out_xyz, int32_t* out_count);
/* Same with device pointers; asynchronous on the tree's stream. */
int ikdg_knn_device(ikdg_tree* t, const float* q, int64_t nq, int32_t stride, int32_t k, double max_dist,
                    int32_t* out_ids, float* out_d2, float* out_xyz, int32_t* out_count);

/* kNN for callers that cannot allocate device memory (no counterpart in the
 * reference).  Some integrations may not call cudaMalloc while they search:
 * a real-time loop (a LiDAR odometry step, for instance) cannot accept the
 * device-wide synchronisation and unbounded latency a cudaMalloc / cudaFree
 * may bring, and a host whose framework reserves and manages all device
 * memory itself leaves no room for allocations of its own.  This variant of
 * ikdg_knn_device calls no cudaMalloc / cudaFree and no allocating library
 * routine.  Batches of 2,048 queries or more are sorted into spatially
 * coherent order first, and that sort's scratch lives in one static device
 * array of the library (about 2.7 MB, held on every GPU that loads libikdg
 * until the process exits); smaller batches are searched unsorted and use no
 * scratch.  Limits: nq <= 262144 queries and k <= 64 per call; larger
 * requests fail with IKDG_BAD_ARG.  The first call on a device looks the
 * array up (cudaGetSymbolAddress).  All calls share the array and it keeps
 * the last call's contents: calls that can overlap on the GPU (for example on
 * two trees with different streams) race on it and must be serialised by the
 * caller.  Pointers are
 * device pointers; asynchronous on the tree's stream; results equal
 * ikdg_knn_device's. */
int ikdg_knn_device_noalloc(ikdg_tree* t, const float* q, int64_t nq, int32_t stride, int32_t k, double max_dist,
                            int32_t* out_ids, float* out_d2, float* out_xyz, int32_t* out_count);

/* Box_Search(const BoxPointType&, PointVector&) (ikd_Tree.h:237,
 * ikd_Tree.cpp:399-404), batched over nb boxes.  Results are CSR: hits of box
 * i are ids[offsets[i] .. offsets[i+1]) (and xyz, 3 floats each, may be NULL).
 * offsets has nb + 1 entries.  When *total exceeds `capacity`, nothing but
 * offsets and *total is written and IKDG_CAPACITY is returned. */
int ikdg_box_search(ikdg_tree* t, const float* boxes, int64_t nb, int64_t* offsets, int32_t* ids, float* xyz,
                    int64_t capacity, int64_t* total);

/* Radius_Search(point, radius, PointVector&) (ikd_Tree.h:238,
 * ikd_Tree.cpp:406-411), batched: query i uses radius[i * radius_stride]
 * (radius_stride 0: one radius for all).  CSR output as ikdg_box_search. */
int ikdg_radius_search(ikdg_tree* t, const float* centers, int64_t nq, int32_t stride, const float* radius,
                       int32_t radius_stride, int64_t* offsets, int32_t* ids, float* xyz, int64_t capacity,
                       int64_t* total);

/* Device-pointer forms of ikdg_box_search / ikdg_radius_search (the reference
 * has only the per-point host calls above): every pointer is a device pointer,
 * the call is asynchronous on the tree's stream and never waits for the GPU.
 * offsets (nq + 1 entries) and *total (nullable) are always written; a query
 * whose hits would end past `capacity` writes no ids / xyz, so compare *total
 * with capacity after synchronising.  Hits come in the same order as from the
 * host-pointer calls. */
int ikdg_box_search_device(ikdg_tree* t, const float* boxes, int64_t nb, int64_t* offsets, int32_t* ids, float* xyz,
                           int64_t capacity, int64_t* total);
int ikdg_radius_search_device(ikdg_tree* t, const float* centers, int64_t nq, int32_t stride, const float* radius,
                              int32_t radius_stride, int64_t* offsets, int32_t* ids, float* xyz, int64_t capacity,
                              int64_t* total);

/* ---- Multi-tree batches (no counterpart in the reference) -------------------
 * A batch is a list of search requests over any number of trees (same
 * device), each with the semantics and results of the per-call device entry
 * points (ikdg_knn_device, ikdg_box_search_device, ikdg_radius_search_device).
 * ikdg_batch_run issues the whole list at once as one CUDA graph: the trees'
 * descriptors are refreshed, one persistent search kernel per register class
 * (kNN k <= 1, 2, 4, 8, 16 and box / radius) runs on its own graph branch, and
 * box / radius requests then get a device prefix sum and one persistent write
 * kernel.  The graph is built at the first run after requests change.
 *
 * All query / output pointers are device pointers owned by the caller; they
 * must stay valid until the batch is cleared or destroyed, and their contents
 * may change between runs (the graph reads them at run time).  Trees may be
 * mutated between runs: a run waits for work already queued on each tree's
 * stream, and later work on those streams waits for the run.  A tree must not
 * be destroyed while a batch holds requests on it.  `request` (nullable)
 * receives the request's index. */
int ikdg_batch_create(int device, ikdg_batch** out);
int ikdg_batch_destroy(ikdg_batch* b);
int ikdg_batch_clear(ikdg_batch* b);
const char* ikdg_batch_last_error(const ikdg_batch* b);
/* kNN request, k <= 16; outputs as ikdg_knn. */
int ikdg_batch_add_knn(ikdg_batch* b, ikdg_tree* t, const float* queries, int64_t nq, int32_t stride, int32_t k,
                       double max_dist, int32_t* out_ids, float* out_d2, float* out_xyz, int32_t* out_count,
                       int32_t* request);
/* Box / radius requests: CSR output as ikdg_box_search_device, per request. */
int ikdg_batch_add_box_search(ikdg_batch* b, ikdg_tree* t, const float* boxes, int64_t nb, int64_t* offsets,
                              int32_t* ids, float* xyz, int64_t capacity, int32_t* request);
int ikdg_batch_add_radius_search(ikdg_batch* b, ikdg_tree* t, const float* centers, int64_t nq, int32_t stride,
                                 const float* radius, int32_t radius_stride, int64_t* offsets, int32_t* ids,
                                 float* xyz, int64_t capacity, int32_t* request);
/* Lanes per kNN query of one request (1, 2, 4; 0 = the tree's setting). */
int ikdg_batch_set_knn_lanes(ikdg_batch* b, int32_t request, int32_t lanes);
/* use_graph 0: issue the same kernels directly at every run (no graph). */
int ikdg_batch_set_graph(ikdg_batch* b, int use_graph);
/* ordered 1: each run first sorts every request's queries by a Morton code
 * in its tree's box (one key pass and one radix sort for the whole batch) and
 * searches them in that order, so neighbouring lanes walk nearby nodes;
 * results are unchanged and stay in query order.  0 (default): queries are searched in
 * the order given. */
int ikdg_batch_set_query_order(ikdg_batch* b, int ordered);
/* Asynchronous on the batch's stream. */
int ikdg_batch_run(ikdg_batch* b);
/* Waits for the last run.  range_totals (nullable, host) receives one total
 * per box / radius request, in the order they were added.  IKDG_CAPACITY when
 * a request's hits exceeded its capacity (those queries wrote no ids). */
int ikdg_batch_synchronize(ikdg_batch* b, int64_t* range_totals);
/* Autotuner: per tree of the batch, times that tree's requests alone for
 * every leaf fill in {8, 12, 16, 24, 32} (the tree is rebuilt at each) and
 * every lanes-per-kNN-query in {1, 2, 4} (median of `reps` runs), then keeps
 * the fastest pair: the tree stays rebuilt at that fill, its kNN requests get
 * those lanes.  chosen (nullable, host) receives {fill, lanes} per distinct
 * tree, in order of first use.  Results do not depend on either setting. */
int ikdg_batch_autotune(ikdg_batch* b, int32_t reps, int32_t* chosen);
int ikdg_batch_num_trees(ikdg_batch* b, int32_t* n);
int ikdg_batch_get_stream(ikdg_batch* b, void** stream);

/* Scan-to-map point-to-plane residuals on top of Nearest_Search (no
 * counterpart in the reference; the step its main consumer, FAST-LIO2, runs on
 * every kNN result).  Device pointers except pose / loss / grad_pose (host).
 * pose = {omega_x, omega_y, omega_z, t_x, t_y, t_z}: w_i = Exp(omega) p_i + t.
 * Forward: kNN (k, max_dist) of every w_i; least-squares plane n.q + d = 0
 * through the k neighbours (A x = -1, n = x/|x|, d = 1/|x|), valid when every
 * neighbour lies within plane_thresh; planes[8i..8i+7] = {n, d, c, 0} with c
 * a point on the plane; r_i = n.(w_i - c) (= n.w_i + d); *loss = 1/2 sum
 * over valid points of r_i^2.
 * Adjoint (neighbours and planes held fixed): grad_points[i] = dL/dp_i (may
 * be NULL) and grad_pose = dL/d(omega, t), scaled by grad_loss. */
int ikdg_p2p_forward(ikdg_tree* t, const float* scan, int64_t n, const double* pose, int32_t k, double max_dist,
                     float plane_thresh, float* planes, float* residuals, int32_t* valid, double* loss);
int ikdg_p2p_adjoint(ikdg_tree* t, const float* scan, int64_t n, const double* pose, const float* planes,
                     const float* residuals, const int32_t* valid, double grad_loss, float* grad_points,
                     double* grad_pose);

/* size() (ikd_Tree.cpp:78-96): stored points, deleted ones not yet dropped by a
 * rebuild included.  validnum() (ikd_Tree.cpp:128-145): valid points. */
int ikdg_size(ikdg_tree* t, int64_t* out);
int ikdg_validnum(ikdg_tree* t, int64_t* out);

/* tree_range() (ikd_Tree.cpp:98-126): AABB of the valid points (zeros when
 * the tree is empty). */
int ikdg_tree_range(ikdg_tree* t, float* box6);
/* root_alpha() (ikd_Tree.cpp:147-165): balance and deleted share at the root. */
int ikdg_root_alpha(ikdg_tree* t, float* alpha_bal, float* alpha_del);

/* flatten(Root_Node, Storage, NOT_RECORD) (ikd_Tree.cpp:1325-1352): all valid
 * points (order unspecified).  IKDG_CAPACITY with *n = required size when
 * `capacity` is too small.  ids may be NULL. */
int ikdg_flatten(ikdg_tree* t, float* xyz, int32_t* ids, int64_t capacity, int64_t* n);

/* acquire_removed_points (ikd_Tree.cpp:558-571): drains the points deleted by
 * box or point deletion that rebuilds have dropped since the last call, with
 * their ids (xyz or ids may be NULL, not both).  IKDG_CAPACITY with *n =
 * required size (nothing drained) when too small. */
int ikdg_acquire_removed_points(ikdg_tree* t, float* xyz, int32_t* ids, int64_t capacity, int64_t* n);

/* Ids of every point the tree can still hand back (no counterpart in the
 * reference, whose nodes carry the whole PointType): the stored points, valid
 * or deleted but not yet dropped by a rebuild (Add_Point_Boxes can restore
 * those), followed by the removed points ikdg_acquire_removed_points has not
 * drained yet.  Bindings that keep per-point payloads on the host, keyed by
 * id, use it to drop payloads no search can return any more.  IKDG_CAPACITY
 * with *n = required size when ids is NULL or capacity is too small. */
int ikdg_live_ids(ikdg_tree* t, int32_t* ids, int64_t capacity, int64_t* n);

/* Rebuilds the whole tree from its valid points (compaction). */
int ikdg_rebuild(ikdg_tree* t);

/* Diagnostics (no counterpart in the reference): checks the device tree's
 * structure - parent / child links, per-child counts and AABBs, leaf fill - and
 * reports the number of violations (0 for a sound tree). */
int ikdg_debug_validate(ikdg_tree* t, int64_t* violations);

/* Stream control: the tree runs all work on one CUDA stream. */
int ikdg_get_stream(ikdg_tree* t, void** stream);
int ikdg_set_stream(ikdg_tree* t, void* stream);
int ikdg_synchronize(ikdg_tree* t);

#ifdef __cplusplus
}
#endif

#endif /* IKDG_H */
