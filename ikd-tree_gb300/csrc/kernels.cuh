// Host-side launchers shared between the translation units of libikdg.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace ikdg {

// ---- scan.cu / sort.cu ------------------------------------------------------
// Exclusive prefix sum of n int32 / int64 values; `total` (device, nullable) receives
// the sum.  `temp` must hold scan_temp_bytes(n) bytes.
size_t scan_temp_bytes(long long n);
void exclusive_scan(const int* in, int* out, long long n, int* total, void* temp, cudaStream_t s);
void exclusive_scan(const long long* in, long long* out, long long n, long long* total, void* temp, cudaStream_t s);

// Stable LSD radix sort of `batch` independent (key, value) arrays of length n
// stored `stride` elements apart, on the low `bits` bits of the key (a
// multiple of 8).  The result lands back in keys / vals; the *_alt buffers are
// scratch of the same shape.  `temp` must hold sort_temp_bytes(n, batch).
size_t sort_temp_bytes(long long n, int batch);
// With copy_back = false an odd number of passes leaves the result in the
// alt buffers, and the call returns true.
bool radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, long long n,
                      int batch, long long stride, int bits, void* temp, cudaStream_t s, bool copy_back = true);

// ---- build.cu ---------------------------------------------------------------
// Batched subtree build.  `pts` holds the points of `njobs` jobs back to back
// (job j = [job_off[j], job_off[j+1])), each as {x, y, z, id}.  Every job
// becomes a balanced subtree of leaves holding at most `fill` points, split at
// the median of the longest AABB axis, and is linked into the child slot
// `job_link[j]` (= parent * 2 + side) together with its AABB and counts.
struct BuildScratch {
    uint32_t* ord[2];    // 2 x [3 * n] point indices sorted per axis
    uint32_t* keys[2];   // 2 x [3 * n]
    int* segpos[2];      // 2 x [n]
    int* flag;           // [n]
    int* scan_in;        // [3 * n]
    int* scan_out;       // [3 * n]
    int4* segs[2];       // 2 x [max_segs]  {s, e, link, pad}
    int4* seginfo;       // [max_segs]      {kind, axis/leaf, mid, child_base}
    int4* local_jobs;    // [max_segs]      {s, e, link} for the CTA-local builder
    int* nseg;           // [4] device counters (two levels, local jobs)
    void* temp;          // scan / sort temp
    float4* mid_pts[2];  // 2 x [n] points of the medium-job splitter (alias ord / keys)
};
size_t build_scratch_bytes(long long n, int njobs, int fill);
void carve_build_scratch(void* base, long long n, int njobs, int fill, BuildScratch* bs);
int build_levels(long long max_job, int fill);
void build_subtrees(const DevTree& t, const float4* pts, long long n, const int* job_off, const int* job_link,
                    int njobs, long long max_job, int fill, const BuildScratch& bs, cudaStream_t s);

// ---- query.cu ---------------------------------------------------------------
// Batched kNN.  `temp` must hold knn_temp_bytes(nq, k) bytes of device
// scratch: the query binning (QBIN_BINS counters, a key and a permutation
// entry per query, for batches of at least QBIN_MIN_QUERIES) and, for
// k > KNN_SMEM_MAX, k slot indices per query.  The candidate lists live in
// registers for k <= KNN_REG_MAX, in shared memory for k <= KNN_SMEM_MAX and
// in the output rows beyond.
#ifndef IKDG_KNN_REG_MAX
#define IKDG_KNN_REG_MAX 8
#endif
constexpr int KNN_REG_MAX = IKDG_KNN_REG_MAX;
constexpr int KNN_SMEM_MAX = 64;
constexpr int QBIN_BITS = 16;
constexpr int QBIN_BINS = 1 << QBIN_BITS;
constexpr long long QBIN_MIN_QUERIES = 2048;
constexpr long long QBIN_AUTO_QUERIES = 262144;  // default: sort batches from this size
size_t knn_temp_bytes(long long nq, int k);
// Host-pointer kNN calls of at most this many queries (and k <= KNN_SMEM_MAX)
// run on pooled per-call streams with the tree's lock held shared, so
// concurrent callers search at the same time.
constexpr long long SMALL_KNN_QUERIES = 4096;
// Allocation-free kNN: limit on the batch size and the device address of the
// shared scratch array (looked up on the first call per device).
constexpr long long NOALLOC_MAX_QUERIES = 1 << 18;
cudaError_t noalloc_scratch(int device, void** ptr);
size_t noalloc_scratch_bytes();
// `lanes` (1, 2 or 4) threads cooperate on each query; `bin_bits` (0 = off,
// at most QBIN_BITS) levels of the tree order the queries before the search.
// host_out: the outputs are host memory the GPU writes directly (each warp's
// rows then leave as coalesced 16-byte spans through shared memory).
void launch_knn(const DevTree& t, const float* q, int q_stride, long long nq, int k, float max_sq,
                int* out_id, float* out_d2, float* out_xyz, int* out_cnt, void* temp, int lanes, int bin_bits,
                cudaStream_t s, bool host_out = false);
// Box (mode 0) and radius (mode 1) search.  Pass 1 (ids == nullptr) writes
// per-query hit counts into `counts`; pass 2 writes ids / xyz starting at
// offsets[i].  Boxes are {min xyz, max xyz}; radius queries are {x, y, z} with
// a per-query radius (r_stride floats apart).  With capacity >= 0, pass 2
// reads counts and skips (raising ERR_OUTPUT) every query whose results would
// end past `capacity`.
void launch_range(const DevTree& t, int mode, const float* q, int q_stride, const float* radius, int r_stride,
                  long long nq, long long* counts, const long long* offsets, int* ids, float* xyz,
                  long long capacity, cudaStream_t s);

// ---- batch.cu ---------------------------------------------------------------------
// One request of a multi-tree batch: a kNN, box or radius search of nq queries
// on trees[tree].  Phase 1 (search) covers chunks [c1, c1 + n1) of the
// phase's chunk numbering; range requests also take phase-2 (write) chunks
// [c2, c2 + n2).  A chunk is one warp, BATCH_CHUNK threads: 32 / lanes kNN
// queries, or 32 range queries.
constexpr int BATCH_THREADS = 128;
constexpr int BATCH_CHUNK = 32;
constexpr int BATCH_KMAX = 16;
constexpr int BATCH_SMEM_CLASS = 4;   // kNN with 8 < k <= 16: lists in shared memory
constexpr int BATCH_RANGE_CLASS = 5;  // box / radius requests
enum BatchKind : int { BATCH_KNN = 0, BATCH_BOX = 1, BATCH_RADIUS = 2 };

struct BatchReq {
    long long c1, n1, c2, n2;
    const float* q;
    const float* radius;
    long long nq;
    int kind, tree, q_stride, r_stride;
    int k, kclass, lanes;
    float max_sq;
    int* ids;
    float* d2;
    float* xyz;
    int* cnt;
    long long* offsets;  // range: nq + 1 entries, CSR within the request
    long long cbase;     // range: first entry of this request in the batch count array
    long long capacity;  // range: ids / xyz capacity
    long long* total;    // range: device total (nullable)
    const int* perm;     // query at position i of the request's run order (nullptr: in order)
};

// Register class of a kNN request with this k (k <= BATCH_KMAX): 0..4;
// range requests are class BATCH_RANGE_CLASS.
int batch_kclass(int k);
// Resident CTAs (whole GPU) of the persistent search kernel of a class.
int batch_search_grid(int kclass, int lanes);
int batch_write_grid();
// Phase 1 over requests [r0, r1), all of register class kclass and `lanes`
// lanes per query, whose chunks are [c_begin, c_end); ctr: a zeroed device
// counter.
void launch_batch_search(const DevTree* trees, const BatchReq* reqs, const long long* req_c1, int r0, int r1,
                         long long c_begin, long long c_end, int kclass, int lanes, long long* counts,
                         unsigned long long* ctr, int grid, cudaStream_t s);
// Spatial order of every request's queries: key = request position in the
// high bits, Morton code of the query (kNN / radius: the point; box: its
// centre) in the tree's root box below; vals = query index in its request.
// qstart: first query of each request in [0, total) (n + 1 entries).
void launch_batch_keys(const DevTree* trees, const BatchReq* reqs, const long long* qstart, int n, long long total,
                       int req_bits, uint32_t* keys, uint32_t* vals, cudaStream_t s);
// Phase 2 over the range requests listed in ridx[0..nr) (ascending c2, chunks
// [0, c_end)); goff: exclusive scan of the batch count array.
void launch_batch_write(const DevTree* trees, const BatchReq* reqs, const int* ridx, const long long* req_c2, int nr,
                        long long c_end, const long long* goff, unsigned long long* ctr, int grid, cudaStream_t s);

// ---- register.cu ---------------------------------------------------------------
// Rt_dev: 12 doubles, R row-major then t.  planes: 2 float4 per point ({n,d}
// and a point c on the plane).  partial: per-block double sums (reg_blocks(n)
// entries of 1 (loss) or 6 (adjoint) doubles).
int reg_blocks(long long n);
void launch_transform(const float* p, long long n, const double* Rt_dev, float* w, cudaStream_t s);
void launch_plane_residual(const float* p, const double* Rt_dev, long long n, int k, const float* nb, const int* cnt,
                           float thresh, float4* planes, float* res, int* valid, double* partial, cudaStream_t s);
void launch_adjoint(const float* p, long long n, const double* Rt_dev, const float4* planes, const float* res,
                    const int* valid, float dl, float* grad_p, double* partial, cudaStream_t s);

// ---- update.cu --------------------------------------------------------------
struct UpdateScratch;
}  // namespace ikdg
