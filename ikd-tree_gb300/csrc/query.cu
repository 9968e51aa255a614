// Batched searches: Nearest_Search, Box_Search, Radius_Search, one launch per
// call; the traversal bodies and their semantics are in search.cuh.
#include <cuda_runtime.h>

#include <mutex>

#include "search.cuh"

namespace ikdg {
namespace {

using search::FINF;

// Threads per CTA of the per-call kNN kernel.
#ifndef IKDG_KNN_THREADS
#define IKDG_KNN_THREADS 128
#endif
constexpr int KNN_THREADS = IKDG_KNN_THREADS;


// STAGED: the outputs are host memory (rows leave through shared memory as
// coalesced 16-byte stores; see knn_body).
template <int KMAX, int G, bool STAGED = false, int PAIRS = search::knn_leaf_pairs<KMAX>()>
__global__ void __launch_bounds__(KNN_THREADS) knn_kernel(DevTree t, const float* __restrict__ q, int q_stride,
                                                  long long nq, int k, float max_sq, int* __restrict__ out_id,
                                                  float* __restrict__ out_d2, float* __restrict__ out_xyz,
                                                  int* __restrict__ out_cnt, int* __restrict__ slots,
                                                  const int* __restrict__ perm) {
    const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (KMAX > 0 && G == 1 && STAGED) {
        // rows of a warp's consecutive queries leave through shared memory
        __shared__ __align__(16) float stage[KNN_THREADS / 32][search::knn_stage_floats(KMAX)];
        search::knn_body<KMAX, G, PAIRS>(t, gtid, q, q_stride, nq, k, max_sq, out_id, out_d2, out_xyz, out_cnt, slots,
                                         perm, nullptr, nullptr, nullptr, 1,
                                         perm == nullptr ? stage[threadIdx.x >> 5] : nullptr);
    } else {
        search::knn_body<KMAX, G, PAIRS>(t, gtid / G, q, q_stride, nq, k, max_sq, out_id, out_d2, out_xyz, out_cnt,
                                         slots, perm);
    }
}

// WRITE = false stores counts[qi]; true emits at [offsets[qi],
// offsets[qi + 1]) (offsets has nq + 1 entries).  With a capacity (>= 0), a
// query whose results would end past it writes nothing and raises ERR_OUTPUT.
template <int MODE, bool WRITE>
__global__ void __launch_bounds__(128) range_kernel(DevTree t, const float* __restrict__ q, int q_stride,
                                                    const float* __restrict__ radius, int r_stride, long long nq,
                                                    long long* __restrict__ counts,
                                                    const long long* __restrict__ offsets, int* __restrict__ ids,
                                                    float* __restrict__ xyz, long long capacity) {
    // No early exit: the search body is warp-collective.
    const long long qi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = qi < nq;
    if (!WRITE) {
        const long long c =
            search::range_body<MODE, search::RANGE_COUNT>(t, q, q_stride, radius, r_stride, qi, valid, 0, 0, nullptr, nullptr);
        if (valid) counts[qi] = c;
        return;
    }
    long long o = 0, o_lim = 0;
    bool go = valid;
    if (valid) {
        o = offsets[qi];
        o_lim = offsets[qi + 1];
        if (capacity >= 0 && o_lim > capacity) {
            atomicOr(&t.st->err, ERR_OUTPUT);
            go = false;
        }
    }
    search::range_body<MODE, search::RANGE_WRITE>(t, q, q_stride, radius, r_stride, qi, go, o, o_lim, ids, xyz);
}

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

// Blocks of `fn` resident on the whole GPU (0 if the query fails).
inline int knn_resident(const void* fn) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, KNN_THREADS, 0) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return sms * per_sm;
}

template <int KMAX>
void knn_launch(const DevTree& t, const float* q, int q_stride, long long nq, int k, float max_sq, int* out_id,
                float* out_d2, float* out_xyz, int* out_cnt, int* slots, const int* perm, int lanes, cudaStream_t s,
                bool host_out = false) {
    const int G = lanes >= 4 ? 4 : lanes == 2 ? 2 : 1;
    const unsigned grid = blocks_for(nq * G, KNN_THREADS);
    if constexpr (KMAX > 0) {
        if (G == 1) {
            // Four slot pairs per leaf step while every block of the batch is
            // resident at once (the occupancy of a kernel does not change:
            // looked up once; the library drives one kind of GPU).
            const bool staged = host_out && perm == nullptr;
            static int resident[2] = {-1, -1};
            int& r = resident[staged ? 1 : 0];
            if (r < 0)
                r = staged ? knn_resident((const void*)knn_kernel<KMAX, 1, true, 4>)
                           : knn_resident((const void*)knn_kernel<KMAX, 1, false, 4>);
            const bool wide = grid <= (unsigned)r;
#define IKDG_KNN_P(ST, P)                                                                                     \
    knn_kernel<KMAX, 1, ST, P><<<grid, KNN_THREADS, 0, s>>>(t, q, q_stride, nq, k, max_sq, out_id, out_d2, out_xyz, \
                                                            out_cnt, slots, perm)
            if (staged && wide)
                IKDG_KNN_P(true, 4);
            else if (staged)
                IKDG_KNN_P(true, 2);
            else if (wide)
                IKDG_KNN_P(false, 4);
            else
                IKDG_KNN_P(false, 2);
#undef IKDG_KNN_P
            return;
        }
    }
#define IKDG_KNN_G(GG)                                                                                              \
    knn_kernel<KMAX, GG><<<grid, KNN_THREADS, 0, s>>>(t, q, q_stride, nq, k, max_sq, out_id, out_d2, out_xyz, out_cnt, \
                                                      slots, perm)
    if (G == 4)
        IKDG_KNN_G(4);
    else if (G == 2)
        IKDG_KNN_G(2);
    else
        IKDG_KNN_G(1);
#undef IKDG_KNN_G
}

// KNN_REG_MAX < k <= KNN_SMEM_MAX: each group's sorted candidate list lives
// in shared memory, entry j of group g at [j * groups + g] (threads of a warp
// touching the same entry hit different banks).  64 threads per CTA keep
// 64 entries x 12 bytes x 64 groups within the default 48 KB.
constexpr int KNN_SMEM_THREADS = 64;

template <int G>
__global__ void __launch_bounds__(KNN_SMEM_THREADS) knn_smem_kernel(DevTree t, const float* __restrict__ q,
                                                                    int q_stride, long long nq, int k, float max_sq,
                                                                    int* __restrict__ out_id,
                                                                    float* __restrict__ out_d2,
                                                                    float* __restrict__ out_xyz,
                                                                    int* __restrict__ out_cnt,
                                                                    const int* __restrict__ perm) {
    extern __shared__ float knn_sm[];
    constexpr int groups = KNN_SMEM_THREADS / G;
    float* sd = knn_sm;
    int* si = reinterpret_cast<int*>(sd + groups * k);
    int* ss = si + groups * k;
    const int g = threadIdx.x / G;
    const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    search::knn_body<0, G>(t, gtid / G, q, q_stride, nq, k, max_sq, out_id, out_d2, out_xyz, out_cnt, nullptr, perm,
                           sd + g, si + g, ss + g, groups);
}

void knn_smem_launch(const DevTree& t, const float* q, int q_stride, long long nq, int k, float max_sq, int* out_id,
                     float* out_d2, float* out_xyz, int* out_cnt, const int* perm, int lanes, cudaStream_t s) {
    const int G = lanes >= 4 ? 4 : lanes == 2 ? 2 : 1;
    const size_t smem = (size_t)(KNN_SMEM_THREADS / G) * k * 12;
    const unsigned grid = blocks_for(nq * G, KNN_SMEM_THREADS);
    if (G == 4)
        knn_smem_kernel<4><<<grid, KNN_SMEM_THREADS, smem, s>>>(t, q, q_stride, nq, k, max_sq, out_id, out_d2,
                                                                out_xyz, out_cnt, perm);
    else if (G == 2)
        knn_smem_kernel<2><<<grid, KNN_SMEM_THREADS, smem, s>>>(t, q, q_stride, nq, k, max_sq, out_id, out_d2,
                                                                out_xyz, out_cnt, perm);
    else
        knn_smem_kernel<1><<<grid, KNN_SMEM_THREADS, smem, s>>>(t, q, q_stride, nq, k, max_sq, out_id, out_d2,
                                                                out_xyz, out_cnt, perm);
}

// ---- query binning -----------------------------------------------------------
// Each query descends the top QBIN_BITS levels of the tree by the split planes;
// the left/right path, left-aligned to QBIN_BITS bits, is an in-order index of
// a k-d cell.  A counting sort on it puts queries of the same or neighbouring
// cells into the same warp, so the threads of a warp traverse nearly the same
// nodes and leaves.
__global__ void qbin_kernel(DevTree t, const float* __restrict__ q, int q_stride, long long nq, int* __restrict__ key,
                            int* __restrict__ hist, int nbits) {
    long long qi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    const float p[3] = {q[qi * q_stride], q[qi * q_stride + 1], q[qi * q_stride + 2]};
    int code = __float_as_int(__ldg(&t.node[3].x));
    int bits = 0, depth = 0;
    while (code > 0 && depth < nbits) {
        const float4 f3 = __ldg(t.node + 4 * code + 3);
        const int go = p[__float_as_int(f3.w)] < f3.z ? 0 : 1;
        bits = (bits << 1) | go;
        code = go ? __float_as_int(f3.y) : __float_as_int(f3.x);
        ++depth;
    }
    bits <<= (nbits - depth);
    key[qi] = bits;
    atomicAdd(hist + bits, 1);
}

__global__ void qbin_scatter_kernel(const int* __restrict__ key, long long nq, int* __restrict__ cursor,
                                    int* __restrict__ perm) {
    long long qi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    int pos = atomicAdd(cursor + key[qi], 1);
    perm[pos] = (int)qi;
}

}  // namespace

size_t knn_temp_bytes(long long nq, int k) {
    size_t b = 0;
    if (nq >= QBIN_MIN_QUERIES) b += sizeof(int) * (2 * QBIN_BINS + 2 * nq) + scan_temp_bytes(QBIN_BINS) + 1024;
    if (k > KNN_SMEM_MAX) b += sizeof(int) * nq * k + 256;
    return b;
}

void launch_knn(const DevTree& t, const float* q, int q_stride, long long nq, int k, float max_sq, int* out_id,
                float* out_d2, float* out_xyz, int* out_cnt, void* temp, int lanes, int bin_bits, cudaStream_t s,
                bool host_out) {
    if (nq <= 0) return;
    char* tp = (char*)temp;
    const int* perm = nullptr;
    const int nbins = 1 << bin_bits;
    if (nq >= QBIN_MIN_QUERIES && bin_bits > 0) {
        int* hist = (int*)tp;
        int* offs = hist + nbins;
        int* key = offs + nbins;
        int* pm = key + nq;
        char* stemp = (char*)(pm + nq);
        stemp = (char*)(((uintptr_t)stemp + 255) & ~(uintptr_t)255);
        tp = stemp + ((scan_temp_bytes(QBIN_BINS) + 255) / 256) * 256;
        cudaMemsetAsync(hist, 0, sizeof(int) * nbins, s);
        qbin_kernel<<<blocks_for(nq, 256), 256, 0, s>>>(t, q, q_stride, nq, key, hist, bin_bits);
        exclusive_scan(hist, offs, nbins, nullptr, stemp, s);
        qbin_scatter_kernel<<<blocks_for(nq, 256), 256, 0, s>>>(key, nq, offs, pm);
        perm = pm;
    }
    int* slots = k > KNN_SMEM_MAX ? (int*)tp : nullptr;
#define IKDG_KNN(KM) \
    knn_launch<KM>(t, q, q_stride, nq, k, max_sq, out_id, out_d2, out_xyz, out_cnt, slots, perm, lanes, s, host_out)
    if (k > KNN_SMEM_MAX)
        IKDG_KNN(0);
    else if (k > KNN_REG_MAX)
        knn_smem_launch(t, q, q_stride, nq, k, max_sq, out_id, out_d2, out_xyz, out_cnt, perm, lanes, s);
    else if (k <= 1)
        IKDG_KNN(1);
    else if (k <= 2)
        IKDG_KNN(2);
    else if (k <= 4)
        IKDG_KNN(4);
    else if (k <= 5)
        IKDG_KNN(5);
    else if (k <= 8)
        IKDG_KNN(8);
    else if (k <= 16)
        IKDG_KNN(16);
    else if constexpr (KNN_REG_MAX >= 32)
        IKDG_KNN(32);
#undef IKDG_KNN
}

// ---- kNN without allocation -----------------------------------------------------
// Scratch of the allocation-free kNN entry point (ikdg_knn_device_noalloc): the
// query sort's bin counters, bin offsets, per-query keys and permutation, and
// the prefix-sum partials, for at most NOALLOC_MAX_QUERIES queries.  It is a
// file-scope device array, so it exists on every GPU that loads the library
// until the process exits, and every call shares it.
constexpr size_t NOALLOC_SCRATCH_BYTES = ((size_t)(2 * QBIN_BINS + 2 * NOALLOC_MAX_QUERIES) * sizeof(int) + 4096 +
                                          64 * 1024);
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[256] = {};
}  // namespace

// Device address of the scratch array on the current device.  Looked up once
// per device (the first call on a device does this set-up, which is why that
// first call must not happen inside a stream capture); later calls reuse it.
cudaError_t noalloc_scratch(int device, void** ptr) {
    if (device < 0 || device >= 256) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_noalloc_ptr[device] == nullptr) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[device] = p;
    }
    *ptr = g_noalloc_ptr[device];
    return cudaSuccess;
}

size_t noalloc_scratch_bytes() { return NOALLOC_SCRATCH_BYTES; }

void launch_range(const DevTree& t, int mode, const float* q, int q_stride, const float* radius, int r_stride,
                  long long nq, long long* counts, const long long* offsets, int* ids, float* xyz,
                  long long capacity, cudaStream_t s) {
    if (nq <= 0) return;
    unsigned g = blocks_for(nq, 128);
#define IKDG_RANGE(M, W) \
    range_kernel<M, W><<<g, 128, 0, s>>>(t, q, q_stride, radius, r_stride, nq, counts, offsets, ids, xyz, capacity)
    if (mode == 0) {
        if (ids == nullptr)
            IKDG_RANGE(0, false);
        else
            IKDG_RANGE(0, true);
    } else {
        if (ids == nullptr)
            IKDG_RANGE(1, false);
        else
            IKDG_RANGE(1, true);
    }
#undef IKDG_RANGE
}

}  // namespace ikdg
