// Oracle C API: one interface, two implementations.
//
//   * oracle/_ref/libikd_ref.so  - the unmodified ikd-Tree reference
//     (ikd-Tree/ikd_Tree.cpp) wrapped by oracle/ref_capi.cpp.  It can only be
//     built where the reference sources are present.
//   * oracle/libikd_port.so      - oracle/ikd_port.cpp, a CPU restatement of
//     the same algorithm that builds anywhere (used as the timed CPU baseline
//     on machines without the reference sources).
//
// TEST INFRASTRUCTURE ONLY: the GPU library never links, loads or calls
// anything declared here.
//
// Points are packed float xyz triples; boxes are packed {min x,y,z, max x,y,z}
// (BoxPointType, ikd-Tree/ikd_Tree.h:32-35).
#pragma once
#ifdef __cplusplus
extern "C" {
#endif

void* ora_create(float delete_param, float balance_param, float box_length);
void ora_destroy(void* h);
void ora_build(void* h, const float* xyz, int n);
// Returns the reference's Add_Points return value, or -1 when the tree is
// empty (the reference dereferences a null root there, ikd_Tree.cpp:472).
int ora_add_points(void* h, const float* xyz, int n, int downsample_on);
void ora_delete_points(void* h, const float* xyz, int n);
int ora_delete_boxes(void* h, const float* boxes, int m);
void ora_add_boxes(void* h, const float* boxes, int m);
// out_xyz[nq*k*3], out_d2[nq*k], out_cnt[nq]; rows are ascending as the
// reference emits them (ikd_Tree.cpp:388-395).
void ora_knn(void* h, const float* q, int nq, int k, double max_dist, float* out_xyz,
             float* out_d2, int* out_cnt, int nthreads);
// Box / radius searches keep their results inside the handle; ora_fetch copies
// them out, concatenated in query order.  Returns the total hit count.
long long ora_box_search(void* h, const float* boxes, int nb, long long* counts, int nthreads);
long long ora_radius_search(void* h, const float* q, const float* radius, int nq,
                            long long* counts, int nthreads);
void ora_fetch(void* h, float* out_xyz);
int ora_flatten(void* h, float* out_xyz, int cap);
int ora_size(void* h);
int ora_validnum(void* h);
void ora_settle(void* h);
// async = 1: mutations and searches run as the reference's own calls do,
// without waiting for its background rebuild thread (timing the caller-visible
// cost; the reference lets searches run during a rebuild, ikd_Tree.cpp:875-884);
// flatten / size / validnum / removed points still wait for it.  async = 0 (default): every mutation waits for
// the rebuild thread before and after, so results are deterministic.  The
// port has no background thread; it accepts the call and ignores it.
void ora_set_async(void* h, int async);
int ora_acquire_removed(void* h);  // drains into a staging buffer, returns its size
void ora_fetch_removed(void* h, float* out_xyz);
void ora_tree_range(void* h, float* box6);
void ora_root_alpha(void* h, float* out2);

#ifdef __cplusplus
}
#endif
