// Prefix sums and LSD radix sort used by the tree builder, the query sorter and
// the downsampling grouper.  Both are three-phase (per-tile reduce, scan of the
// tile partials, per-tile downsweep / scatter): no block ever waits on
// another, so nothing here can spin.
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace ikdg {
namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;   // 4096

constexpr int SORT_THREADS = 256;
constexpr int SORT_MAX_ROUNDS = 16;
constexpr int RADIX = 256;

// Rounds of SORT_THREADS keys per tile: 16 for large sorts; small sorts (the
// downsampling grouper's ~15k keys per scan) take smaller tiles, so that more
// blocks share each pass while the histogram (tiles x RADIX x batch) still
// fits the single-block scan.
inline int sort_rounds(long long n, int batch) {
    const long long per = (long long)SORT_MAX_ROUNDS * SORT_THREADS;
    long long r = (n * batch + per - 1) / per;
    return (int)(r < 1 ? 1 : r > SORT_MAX_ROUNDS ? SORT_MAX_ROUNDS : r);
}

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and writes the block total into *total.
template <int THREADS, typename T>
__device__ __forceinline__ T block_excl_scan(T v, T* total) {
    __shared__ T warp_sums[THREADS / 32];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T inc = warp_incl_scan(v);
    if (lane == 31) warp_sums[w] = inc;
    __syncthreads();
    if (w == 0) {
        T s = lane < THREADS / 32 ? warp_sums[lane] : T(0);
        T si = warp_incl_scan(s);
        if (lane < THREADS / 32) warp_sums[lane] = si - s;
        if (lane == THREADS / 32 - 1) *total = si;
    }
    __syncthreads();
    T r = inc - v + warp_sums[w];
    __syncthreads();
    return r;
}

template <typename T>
__global__ void scan_reduce_kernel(const T* __restrict__ in, long long n, T* __restrict__ partial) {
    long long base = (long long)blockIdx.x * SCAN_TILE;
    T s = 0;
    for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
        long long g = base + i;
        if (g < n) s += in[g];
    }
    __shared__ T tot;
    block_excl_scan<SCAN_THREADS>(s, &tot);
    if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

// Single block: exclusive scan of the tile partials.
template <typename T>
__global__ void scan_partials_kernel(T* partial, int ntiles, T* total) {
    __shared__ T carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < ntiles; base += 1024) {
        int i = base + threadIdx.x;
        T v = i < ntiles ? partial[i] : T(0);
        __shared__ T tot;
        T ex = block_excl_scan<1024>(v, &tot);
        if (i < ntiles) partial[i] = ex + carry;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total != nullptr) *total = carry;
}

template <typename T>
__global__ void scan_down_kernel(const T* __restrict__ in, T* __restrict__ out, long long n,
                                 const T* __restrict__ partial) {
    __shared__ T tile[SCAN_TILE];
    long long base = (long long)blockIdx.x * SCAN_TILE;
    for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
        long long g = base + i;
        tile[i] = g < n ? in[g] : T(0);
    }
    __syncthreads();
    T local[SCAN_ITEMS];
    T s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        local[j] = s;
        s += tile[threadIdx.x * SCAN_ITEMS + j];
    }
    __shared__ T tot;
    T ex = block_excl_scan<SCAN_THREADS>(s, &tot) + partial[blockIdx.x];
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) tile[threadIdx.x * SCAN_ITEMS + j] = local[j] + ex;
    __syncthreads();
    for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
        long long g = base + i;
        if (g < n) out[g] = tile[i];
    }
}

// One tile (n <= SCAN_TILE): the whole scan in one block, one launch.
template <typename T>
__global__ void scan_single_kernel(const T* __restrict__ in, T* __restrict__ out, int n, T* total) {
    __shared__ T tile[SCAN_TILE];
    for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) tile[i] = i < n ? in[i] : T(0);
    __syncthreads();
    T local[SCAN_ITEMS];
    T sum = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        local[j] = sum;
        sum += tile[threadIdx.x * SCAN_ITEMS + j];
    }
    __shared__ T tot;
    const T ex = block_excl_scan<SCAN_THREADS>(sum, &tot);
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) tile[threadIdx.x * SCAN_ITEMS + j] = local[j] + ex;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += SCAN_THREADS) out[i] = tile[i];
    if (threadIdx.x == 0 && total != nullptr) *total = tot;
}

template <typename T>
void exclusive_scan_t(const T* in, T* out, long long n, T* total, void* temp, cudaStream_t s) {
    if (n <= 0) {
        if (total) cudaMemsetAsync(total, 0, sizeof(T), s);
        return;
    }
    if (n <= SCAN_TILE) {
        scan_single_kernel<T><<<1, SCAN_THREADS, 0, s>>>(in, out, (int)n, total);
        return;
    }
    int tiles = (int)((n + SCAN_TILE - 1) / SCAN_TILE);
    T* partial = (T*)temp;
    scan_reduce_kernel<T><<<tiles, SCAN_THREADS, 0, s>>>(in, n, partial);
    scan_partials_kernel<T><<<1, 1024, 0, s>>>(partial, tiles, total);
    scan_down_kernel<T><<<tiles, SCAN_THREADS, 0, s>>>(in, out, n, partial);
}

// ---- radix sort --------------------------------------------------------------

__global__ void sort_hist_kernel(const uint32_t* __restrict__ keys, long long n, long long stride, int shift,
                                 int ntiles, int rounds, int* __restrict__ hist) {
    __shared__ int h[RADIX];
    for (int i = threadIdx.x; i < RADIX; i += SORT_THREADS) h[i] = 0;
    __syncthreads();
    const uint32_t* k = keys + (long long)blockIdx.y * stride;
    const int tile = rounds * SORT_THREADS;
    long long base = (long long)blockIdx.x * tile;
    for (int i = threadIdx.x; i < tile; i += SORT_THREADS) {
        long long g = base + i;
        if (g < n) atomicAdd(&h[(k[g] >> shift) & 0xff], 1);
    }
    __syncthreads();
    // Digit-major layout per batch: hist[b][digit][tile].
    int* hb = hist + (long long)blockIdx.y * RADIX * ntiles;
    for (int d = threadIdx.x; d < RADIX; d += SORT_THREADS) hb[(long long)d * ntiles + blockIdx.x] = h[d];
}

__global__ void sort_scatter_kernel(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                                    uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, long long n,
                                    long long stride, int shift, int ntiles, int rounds,
                                    const int* __restrict__ offs) {
    __shared__ int wcnt[SORT_THREADS / 32][RADIX];
    __shared__ int dbase[RADIX];
    const int b = blockIdx.y;
    const uint32_t* kin = keys + (long long)b * stride;
    const uint32_t* vin = vals + (long long)b * stride;
    uint32_t* kout = keys_out + (long long)b * stride;
    uint32_t* vout = vals_out + (long long)b * stride;
    // Scanned offsets were computed over all batches back to back; batch b's
    // first element sits at b * n.
    const int* ob = offs + (long long)b * RADIX * ntiles;
    for (int d = threadIdx.x; d < RADIX; d += SORT_THREADS)
        dbase[d] = ob[(long long)d * ntiles + blockIdx.x] - (int)((long long)b * n);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    long long base = (long long)blockIdx.x * rounds * SORT_THREADS;
    for (int r = 0; r < rounds; ++r) {
        for (int i = threadIdx.x; i < (SORT_THREADS / 32) * RADIX; i += SORT_THREADS) (&wcnt[0][0])[i] = 0;
        __syncthreads();
        long long g = base + (long long)r * SORT_THREADS + threadIdx.x;
        bool valid = g < n;
        uint32_t key = valid ? kin[g] : 0u;
        uint32_t val = valid ? vin[g] : 0u;
        int d = valid ? (int)((key >> shift) & 0xff) : RADIX;  // RADIX = out-of-range group
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int lrank = __popc(peers & lt_mask);
        if (valid && lrank == 0) wcnt[w][d] = __popc(peers);
        __syncthreads();
        if (threadIdx.x < RADIX) {
            int dd = threadIdx.x;
            int run = dbase[dd];
#pragma unroll
            for (int ww = 0; ww < SORT_THREADS / 32; ++ww) {
                int c = wcnt[ww][dd];
                wcnt[ww][dd] = run;
                run += c;
            }
            dbase[dd] = run;
        }
        __syncthreads();
        if (valid) {
            int pos = wcnt[w][d] + lrank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
    }
}

inline int ceil_div_ll(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace

size_t scan_temp_bytes(long long n) {
    long long tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    return (size_t)((tiles + 64) * sizeof(long long) + 256);
}

void exclusive_scan(const int* in, int* out, long long n, int* total, void* temp, cudaStream_t s) {
    exclusive_scan_t<int>(in, out, n, total, temp, s);
}

void exclusive_scan(const long long* in, long long* out, long long n, long long* total, void* temp, cudaStream_t s) {
    exclusive_scan_t<long long>(in, out, n, total, temp, s);
}

size_t sort_temp_bytes(long long n, int batch) {
    const long long tile = (long long)sort_rounds(n, batch) * SORT_THREADS;
    long long tiles = (n + tile - 1) / tile;
    long long hn = tiles * RADIX * batch;
    return (size_t)(hn * sizeof(int) * 2 + scan_temp_bytes(hn) + 512);
}

bool radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, long long n,
                      int batch, long long stride, int bits, void* temp, cudaStream_t s, bool copy_back) {
    if (n <= 1 || batch <= 0) return false;
    const int rounds = sort_rounds(n, batch);
    int tiles = ceil_div_ll(n, (long long)rounds * SORT_THREADS);
    long long hn = (long long)tiles * RADIX * batch;
    int* hist = (int*)temp;
    int* offs = hist + hn;
    void* stemp = (void*)(offs + hn);
    uint32_t *ki = keys, *vi = vals, *ko = keys_alt, *vo = vals_alt;
    int passes = (bits + 7) / 8;
    dim3 grid(tiles, batch);
    for (int p = 0; p < passes; ++p) {
        int shift = 8 * p;
        sort_hist_kernel<<<grid, SORT_THREADS, 0, s>>>(ki, n, stride, shift, tiles, rounds, hist);
        exclusive_scan(hist, offs, hn, nullptr, stemp, s);
        sort_scatter_kernel<<<grid, SORT_THREADS, 0, s>>>(ki, vi, ko, vo, n, stride, shift, tiles, rounds, offs);
        uint32_t* t;
        t = ki; ki = ko; ko = t;
        t = vi; vi = vo; vo = t;
    }
    if (ki == keys) return false;
    if (!copy_back) return true;
    cudaMemcpyAsync(keys, ki, sizeof(uint32_t) * (size_t)((batch - 1) * stride + n), cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(vals, vi, sizeof(uint32_t) * (size_t)((batch - 1) * stride + n), cudaMemcpyDeviceToDevice, s);
    return false;
}

}  // namespace ikdg
