// Launchers for the mutation kernels (update.cu).
#pragma once
#include "kernels.cuh"

namespace ikdg {

// Per-node / per-leaf bookkeeping arrays used by mutations (sized with the
// pools; all entries idle at 0 or -1 between calls).
struct UpdateAux {
    int* pend;          // [node_cap] refit: number of dirty children    (0)
    int* arrive;        // [node_cap] refit: arrivals so far            (0)
    int* viol_flag;     // [node_cap] criterion violated                (0)
    int* job_of_node;   // [node_cap] job rooted here                   (-1)
    int* node_job;      // [node_cap] scratch: job containing the node
    int* dirty_flag;    // [leaf_cap] leaf queued for refit             (0)
    int* job_of_leaf;   // [leaf_cap] job rooted at this leaf           (-1)
    int* leaf_job;      // [leaf_cap] scratch: job containing the leaf
    int* items;         // [leaf_cap + node_cap] refit start codes
    int* viol;          // [leaf_cap + node_cap] violator codes
    int* jobs;          // [leaf_cap + node_cap] job root codes
    int* job_link;      // [leaf_cap + node_cap]
    int* job_count;     // [leaf_cap + node_cap + 1]
    int* job_off;       // [leaf_cap + node_cap + 1]
    int* job_fill;      // [leaf_cap + node_cap]
    int list_cap;       // entries of items / viol / jobs / job_link
};

struct Criteria {
    float alpha_del;
    float alpha_bal;
    int min_size;   // subtrees with at most this many slots are never rebuilt
    int fill;       // leaf fill of the builder (height guard)
};

// Marks / queues leaf L for refit.
void launch_route_append(const DevTree& t, const UpdateAux& a, const float4* pts, long long n, int4* ovf_leaf_pt,
                         float4* ovf_pts, cudaStream_t s);
// Refit from the codes in a.items[0 .. st->n_items) and record violators;
// clears the dirty flags of the listed leaves.
void launch_refit(const DevTree& t, const UpdateAux& a, const int* items, const int* n_items, int max_items,
                  const Criteria& c, cudaStream_t s);
// Select topmost violators as rebuild jobs (st->n_jobs = job count).
void launch_select_jobs(const DevTree& t, const UpdateAux& a, int max_viol, cudaStream_t s);
// Clears the criterion flags of the recorded violators without selecting jobs.
void launch_clear_viol(const DevTree& t, const UpdateAux& a, int max_viol, cudaStream_t s);
// Count / gather the valid points of every job (plus overflow points).
void launch_job_count(const DevTree& t, const UpdateAux& a, int leaf_top, int node_top, const int4* ovf_leaf,
                      int max_ovf, int max_jobs, void* scan_temp, cudaStream_t s);
// Job selection and counting launched before the host knows the violator
// count (st->n_viol, st->n_jobs read on the device; nothing happens when they
// are zero): one status read then returns the violators, the jobs and their
// sizes.  leaf_top / node_top must be current (no build since the last read).
void launch_select_and_count(const DevTree& t, const UpdateAux& a, int leaf_top, int node_top, const int4* ovf_leaf,
                             int max_ovf, cudaStream_t s);
void launch_job_gather(const DevTree& t, const UpdateAux& a, int leaf_top, int node_top, const int4* ovf_leaf,
                       const float4* ovf_pts, int max_ovf, float4* out, float4* removed, long long removed_cap,
                       cudaStream_t s);
void launch_job_finish(const DevTree& t, const UpdateAux& a, int max_jobs, cudaStream_t s);
// Delete every valid point inside each box; `flags` = F_DEL or F_DEL|F_DSDEL.
void launch_delete_boxes(const DevTree& t, const UpdateAux& a, const float* boxes, long long m, uint32_t flags,
                         long long* total, cudaStream_t s);
void launch_delete_points(const DevTree& t, const UpdateAux& a, const float* pts, int stride, long long n,
                          cudaStream_t s);
void launch_add_boxes(const DevTree& t, const UpdateAux& a, const float* boxes, long long m, cudaStream_t s);
void launch_snapshot_root(const DevTree& t, cudaStream_t s);
// *p = v on the stream (no host wait; the value travels as a kernel argument).
void launch_set_ll(long long* p, long long v, cudaStream_t s);
void launch_route_append_dev_count(const DevTree& t, const UpdateAux& a, const float4* pts, long long n_bound,
                                   const int* n_dev, int4* ovf_leaf, float4* ovf_pts, cudaStream_t s);
// Packs strided xyz input into {x, y, z, first_id + i} and flags non-finite
// coordinates (st->err |= ERR_INPUT).
void launch_pack_points(const DevTree& t, const float* in, int stride, long long n, long long first_id, float4* out,
                        cudaStream_t s);
// Flags non-finite values among n * width floats (st->err |= ERR_INPUT).
void launch_check_finite(const DevTree& t, const float* in, long long count, cudaStream_t s);
// Copies every valid point ({x, y, z, id}) to out; *counter += count.
void launch_flatten(const DevTree& t, float4* out, long long* counter, cudaStream_t s);
// Writes the id of every stored slot (valid or deleted) to out[0 .. cap);
// *counter += the number of stored slots.
void launch_stored_ids(const DevTree& t, int* out, long long cap, long long* counter, cudaStream_t s);
// Structural check of the whole tree; *bad += number of violations.
// Structural check (links, counts, AABBs) plus the bookkeeping flags; at_rest
// (between calls) also requires cleared violation / job tags and leaves within
// their slots.
void launch_validate(const DevTree& t, const UpdateAux& a, bool at_rest, long long* bad, cudaStream_t s);
// Makes the whole tree the single rebuild job (st->n_jobs = 1).
void launch_select_root_job(const DevTree& t, const UpdateAux& a, cudaStream_t s);

// ---- voxel downsampling ----------------------------------------------------
struct DsScratch {
    float4* pts;        // [n] input points {x, y, z, -}
    float4* box_lo;     // [n] {lo x, lo y, lo z, -}
    float4* box_hi;     // [n]
    float4* mid;        // [n]
    int4* key;          // [n] {kx, ky, kz, clean}
    int4* s_key;        // [n] key in sorted (hash) order
    float4* s_pts;      // [n] {x, y, z, input index} in sorted order
    uint32_t* hkey[2];  // [n]
    uint32_t* hval[2];  // [n]
    int* groups;        // [n] leader positions in sorted order
    int4* g_info;       // [n] {n0, best slot, best id, hazard}
    float4* g_best;     // [n] best S0 point {x, y, z, d}
    int4* g_out;        // [n] {delete S0, insert, triggers, -}
    float4* ins;        // [n] points to insert {x, y, z, id}
    int* big;           // [n] groups deferred to the warp fold
    int* n_big;         // [1]
    int2* pairs;        // [pair_cap] {group, slot}: the stored points each voxel search found
    int* n_pairs;       // [1] entries written (may pass pair_cap: then the deletion walks)
    int pair_cap;
    void* temp;
};
// pair_cap: room for the (voxel, stored point) pairs of a call's searches
// (the stored points plus the call's insertions suffice unless float slivers
// put points in several voxel boxes; beyond it the deletion walks the tree).
size_t ds_scratch_bytes(long long n, long long pair_cap);
void carve_ds_scratch(void* base, long long n, long long pair_cap, DsScratch* d);
// Prepares keys and groups (once per batch).  st->n_groups = group count;
// a non-finite input sets ERR_INPUT, after which the kernels below change
// nothing.  The kernels read the group count and the sub-batch end on the
// device: max_groups only sizes their grids (any bound on the group count).
void launch_ds_prepare(const DevTree& t, const float* in, int stride, long long n, float ds, DsScratch& d,
                       cudaStream_t s);
// S0 search for all groups and the hazard split of the sub-batch [a, n):
// st->count = first index where the sub-batch must end.
void launch_ds_search(const DevTree& t, long long n, float ds, long long a, DsScratch& d, int max_groups,
                      cudaStream_t s);
// Folds [a, e) per group, with e = min(max(st->count, a + 1), n) the end
// launch_ds_search found, deletes the S0 sets that must go, and queues the
// surviving winners in d.ins (st->n_ins = count); st->count2 += triggers.
void launch_ds_fold(const DevTree& t, const UpdateAux& aux, long long n, long long a, long long first_id,
                    DsScratch& d, int max_groups, cudaStream_t s);

}  // namespace ikdg
