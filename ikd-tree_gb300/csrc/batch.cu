// Multi-tree batched searches: many kNN / box / radius requests over many
// trees in one persistent launch per phase.  The reference has no batched
// form; every request has the semantics of its per-call search (search.cuh).
//
// Work is cut into chunks of one warp (BATCH_CHUNK threads); each warp takes
// the next chunk index from a device counter, finds the request it belongs to
// by a binary search over the requests' first chunks, and runs that request's
// search body on it.  So small requests of many trees fill the GPU together,
// no launch is spent per request, and no warp waits for another (a warp with
// a heavy query does not hold up the rest of its CTA).
#include <cuda_runtime.h>

#include <mutex>

#include "search.cuh"

namespace ikdg {
namespace {

constexpr int WARPS_PER_CTA = BATCH_THREADS / BATCH_CHUNK;

// Last r in [lo, hi) with starts[r] <= c (starts ascending, starts[lo] <= c).
__device__ __forceinline__ int find_req(const long long* __restrict__ starts, int lo, int hi, long long c) {
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(starts + mid) <= c)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// Phase 1 for one class: KC 0..3 are kNN requests with k <= 1, 2, 4, 8 (lists
// in registers), KC = BATCH_SMEM_CLASS kNN with k <= 16 (lists in shared
// memory), all producing their final rows; KC = BATCH_RANGE_CLASS box and
// radius requests (per-query hit counts in counts[cbase + qi]).  One kernel
// per class keeps each at its own register count.
template <int KC, int G>
__global__ void __launch_bounds__(BATCH_THREADS) batch_search_kernel(const DevTree* __restrict__ trees,
                                                                     const BatchReq* __restrict__ reqs,
                                                                     const long long* __restrict__ req_c1, int r0,
                                                                     int r1, long long c_begin, long long c_end,
                                                                     long long* __restrict__ counts,
                                                                     unsigned long long* __restrict__ ctr) {
    constexpr int KM = KC == 0 ? 1 : KC == 1 ? 2 : KC == 2 ? 4 : 8;
    const int lane = threadIdx.x & 31;
    for (;;) {
        // Each warp takes its own chunk: no warp waits for another.
        long long c = 0;
        int r = -1;
        if (lane == 0) {
            c = c_begin + (long long)atomicAdd(ctr, 1ull);
            r = c < c_end ? find_req(req_c1, r0, r1, c) : -1;
        }
        c = __shfl_sync(0xffffffffu, c, 0);
        r = __shfl_sync(0xffffffffu, r, 0);
        if (c >= c_end) break;
        const BatchReq& R = reqs[r];
        const DevTree t = trees[R.tree];
        if constexpr (KC == BATCH_SMEM_CLASS) {
            // 8 < k <= 16: each group's sorted list in shared memory, entry j
            // of group g at [j * groups + g] (as the per-call kernel does)
            extern __shared__ float batch_sm[];
            constexpr int groups = BATCH_THREADS / G;
            float* sd = batch_sm;
            int* si = reinterpret_cast<int*>(sd + groups * BATCH_KMAX);
            int* ss = si + groups * BATCH_KMAX;
            const int g = threadIdx.x / G;
            const long long tid = (c - R.c1) * (BATCH_CHUNK / G) + lane / G;
            search::knn_body<0, G>(t, tid, R.q, R.q_stride, R.nq, R.k, R.max_sq, R.ids, R.d2, R.xyz, R.cnt, nullptr,
                                   R.perm, sd + g, si + g, ss + g, groups);
        } else if constexpr (KC < BATCH_RANGE_CLASS) {
            const long long tid = (c - R.c1) * (BATCH_CHUNK / G) + lane / G;
            search::knn_body<KM, G>(t, tid, R.q, R.q_stride, R.nq, R.k, R.max_sq, R.ids, R.d2, R.xyz, R.cnt, nullptr,
                                    R.perm);
        } else {
            // warp-collective body: every lane calls it
            long long qi = (c - R.c1) * BATCH_CHUNK + lane;
            const bool valid = qi < R.nq;
            if (valid && R.perm != nullptr) qi = __ldg(R.perm + qi);
            const long long n =
                R.kind == BATCH_BOX
                    ? search::range_body<0, search::RANGE_COUNT>(t, R.q, R.q_stride, nullptr, 0, qi, valid, 0, 0,
                                                                 nullptr, nullptr)
                    : search::range_body<1, search::RANGE_COUNT>(t, R.q, R.q_stride, R.radius, R.r_stride, qi, valid,
                                                                 0, 0,
                                                   nullptr, nullptr);
            if (valid) counts[R.cbase + qi] = n;
        }
    }
}

// Phase 2: range requests write their CSR offsets and, where the request's
// capacity holds the query's results, the ids / points.
__global__ void __launch_bounds__(BATCH_THREADS) batch_write_kernel(const DevTree* __restrict__ trees,
                                                                    const BatchReq* __restrict__ reqs,
                                                                    const int* __restrict__ ridx,
                                                                    const long long* __restrict__ req_c2, int nr,
                                                                    long long c_end,
                                                                    const long long* __restrict__ goff,
                                                                    unsigned long long* __restrict__ ctr) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        long long c = 0;
        int r = -1;
        if (lane == 0) {
            c = (long long)atomicAdd(ctr, 1ull);
            r = c < c_end ? __ldg(ridx + find_req(req_c2, 0, nr, c)) : -1;
        }
        c = __shfl_sync(0xffffffffu, c, 0);
        r = __shfl_sync(0xffffffffu, r, 0);
        if (c >= c_end) break;
        const BatchReq& R = reqs[r];
        const DevTree t = trees[R.tree];
        const long long pos = (c - R.c2) * BATCH_CHUNK + lane;
        const long long qi = pos < R.nq && R.perm != nullptr ? (long long)__ldg(R.perm + pos) : pos;
        const long long base = goff[R.cbase];
        if (pos == 0) {
            const long long tot = goff[R.cbase + R.nq] - base;
            R.offsets[R.nq] = tot;
            if (R.total != nullptr) *R.total = tot;
        }
        // warp-collective body: every lane calls it, lanes without work idle
        bool go = pos < R.nq;
        long long o = 0, n = 0;
        if (go) {
            o = goff[R.cbase + qi] - base;
            n = goff[R.cbase + qi + 1] - goff[R.cbase + qi];
            R.offsets[qi] = o;
            if (n == 0 || R.ids == nullptr) {
                go = false;
            } else if (o + n > R.capacity) {
                atomicOr(&t.st->err, ERR_OUTPUT);
                go = false;
            }
        }
        if (R.kind == BATCH_BOX)
            search::range_body<0, search::RANGE_WRITE>(t, R.q, R.q_stride, nullptr, 0, qi, go, o, o + n, R.ids,
                                                       R.xyz);
        else
            search::range_body<1, search::RANGE_WRITE>(t, R.q, R.q_stride, R.radius, R.r_stride, qi, go, o, o + n,
                                                       R.ids, R.xyz);
    }
}

// Every third bit of a 10-bit value (Morton interleave).
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void batch_key_kernel(const DevTree* __restrict__ trees, const BatchReq* __restrict__ reqs,
                                 const long long* __restrict__ qstart, int n, long long total, int req_bits,
                                 uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    const int p = find_req(qstart, 0, n, g);
    const BatchReq& R = reqs[p];
    const long long qi = g - qstart[p];
    float c[3];
    const float* q = R.q + qi * R.q_stride;
    for (int a = 0; a < 3; ++a) c[a] = R.kind == BATCH_BOX ? 0.5f * (q[a] + q[3 + a]) : q[a];
    // the root's box is the left-child box of the sentinel record (node 0)
    const float4 f0 = trees[R.tree].node[0], f1 = trees[R.tree].node[1];
    const float lo[3] = {f0.x, f0.y, f0.z}, hi[3] = {f0.w, f1.x, f1.y};
    uint32_t m = 0;
    for (int a = 0; a < 3; ++a) {
        const float t = (c[a] - lo[a]) / (hi[a] - lo[a]);
        const int v = hi[a] > lo[a] && t > 0.f ? (t < 1.f ? (int)(t * 1024.f) : 1023) : 0;
        m |= spread3((uint32_t)min(v, 1023)) << a;
    }
    const int mb = 32 - req_bits;  // Morton bits kept below the request position
    keys[g] = ((uint32_t)p << mb) | (mb >= 30 ? m : m >> (30 - mb));
    vals[g] = (uint32_t)qi;
}

std::mutex g_grid_mu;

// Dynamic shared memory of a search kernel class (the k <= 16 lists).
size_t class_smem(int kc, int lanes) {
    return kc == BATCH_SMEM_CLASS ? (size_t)(BATCH_THREADS / lanes) * BATCH_KMAX * 12 : 0;
}

int resident_grid(const void* fn, size_t smem = 0) {
    // On a failed query the grid falls back to one CTA per SM (or 1); the
    // kernels are correct for any grid size.
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, BATCH_THREADS, smem) != cudaSuccess) per_sm = 1;
    cudaGetLastError();
    return (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
}

}  // namespace

int batch_kclass(int k) { return k <= 1 ? 0 : k <= 2 ? 1 : k <= 4 ? 2 : k <= 8 ? 3 : 4; }

namespace {

template <int KC, int G>
void search_variant(bool launch, int* grid, const DevTree* trees, const BatchReq* reqs, const long long* req_c1,
                    int r0, int r1, long long c_begin, long long c_end, long long* counts, unsigned long long* ctr,
                    unsigned g, cudaStream_t s) {
    const size_t smem = class_smem(KC, G);
    if (!launch) {
        *grid = resident_grid((const void*)batch_search_kernel<KC, G>, smem);
        return;
    }
    batch_search_kernel<KC, G><<<g, BATCH_THREADS, smem, s>>>(trees, reqs, req_c1, r0, r1, c_begin, c_end, counts,
                                                              ctr);
}

template <int KC>
void search_lanes(int lanes, bool launch, int* grid, const DevTree* trees, const BatchReq* reqs,
                  const long long* req_c1, int r0, int r1, long long c_begin, long long c_end, long long* counts,
                  unsigned long long* ctr, unsigned g, cudaStream_t s) {
    if (lanes >= 4)
        search_variant<KC, 4>(launch, grid, trees, reqs, req_c1, r0, r1, c_begin, c_end, counts, ctr, g, s);
    else if (lanes == 2)
        search_variant<KC, 2>(launch, grid, trees, reqs, req_c1, r0, r1, c_begin, c_end, counts, ctr, g, s);
    else
        search_variant<KC, 1>(launch, grid, trees, reqs, req_c1, r0, r1, c_begin, c_end, counts, ctr, g, s);
}

void search_dispatch(int kc, int lanes, bool launch, int* grid, const DevTree* trees, const BatchReq* reqs,
                     const long long* req_c1, int r0, int r1, long long c_begin, long long c_end, long long* counts,
                     unsigned long long* ctr, unsigned g, cudaStream_t s) {
#define IKDG_BKC(KC) search_lanes<KC>(lanes, launch, grid, trees, reqs, req_c1, r0, r1, c_begin, c_end, counts, ctr, g, s)
    switch (kc) {
        case 0: IKDG_BKC(0); break;
        case 1: IKDG_BKC(1); break;
        case 2: IKDG_BKC(2); break;
        case 3: IKDG_BKC(3); break;
        case 4: IKDG_BKC(4); break;
        default:
            search_variant<BATCH_RANGE_CLASS, 1>(launch, grid, trees, reqs, req_c1, r0, r1, c_begin, c_end, counts,
                                                 ctr, g, s);
            break;
    }
#undef IKDG_BKC
}

}  // namespace

int batch_search_grid(int kclass, int lanes) {
    std::lock_guard<std::mutex> lock(g_grid_mu);
    int grid = 0;
    search_dispatch(kclass, lanes, false, &grid, nullptr, nullptr, nullptr, 0, 0, 0, 0, nullptr, nullptr, 0, nullptr);
    return grid;
}

int batch_write_grid() {
    std::lock_guard<std::mutex> lock(g_grid_mu);
    return resident_grid((const void*)batch_write_kernel);
}

void launch_batch_search(const DevTree* trees, const BatchReq* reqs, const long long* req_c1, int r0, int r1,
                         long long c_begin, long long c_end, int kclass, int lanes, long long* counts,
                         unsigned long long* ctr, int grid, cudaStream_t s) {
    if (c_end <= c_begin || r1 <= r0) return;
    const long long ctas = (c_end - c_begin + WARPS_PER_CTA - 1) / WARPS_PER_CTA;
    const unsigned g = (unsigned)(ctas < grid ? ctas : grid);
    search_dispatch(kclass, lanes, true, nullptr, trees, reqs, req_c1, r0, r1, c_begin, c_end, counts, ctr, g, s);
}

void launch_batch_keys(const DevTree* trees, const BatchReq* reqs, const long long* qstart, int n, long long total,
                       int req_bits, uint32_t* keys, uint32_t* vals, cudaStream_t s) {
    if (total <= 0 || n <= 0) return;
    batch_key_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(trees, reqs, qstart, n, total, req_bits, keys,
                                                                      vals);
}

void launch_batch_write(const DevTree* trees, const BatchReq* reqs, const int* ridx, const long long* req_c2, int nr,
                        long long c_end, const long long* goff, unsigned long long* ctr, int grid, cudaStream_t s) {
    if (c_end <= 0 || nr <= 0) return;
    const long long ctas = (c_end + WARPS_PER_CTA - 1) / WARPS_PER_CTA;
    const unsigned g = (unsigned)(ctas < grid ? ctas : grid);
    batch_write_kernel<<<g, BATCH_THREADS, 0, s>>>(trees, reqs, ridx, req_c2, nr, c_end, goff, ctr);
}

}  // namespace ikdg
