// Batched, level-synchronous subtree builder.
//
// Replaces the recursive BuildTree (ikd-Tree/ikd_Tree.cpp:573-622), used both
// by Build (:352-364) and by the rebuilds of Rebuild (:624-645).  The split
// rule is kept: every segment is cut at its median on the longest axis of its
// AABB (first axis wins ties, :593-595).  Unlike the reference, internal nodes
// hold no point: segments of at most `fill` points become leaf buckets.
//
// Method (all jobs of a call at once): each of the three coordinates is
// radix-sorted once; the three sorted index arrays are then stably partitioned
// level by level, so every segment stays a contiguous range in each array and
// its AABB is read off the ends of the three ranges.  Per level: one thread per
// segment allocates its node or leaf and links it into its parent; one thread
// per position marks left / right; a prefix sum and a scatter partition the
// three arrays.
#include <cuda_runtime.h>

#include <atomic>

#include "kernels.cuh"

namespace ikdg {
namespace {

constexpr int LB_MAX = 4096;  // segments this small go to the CTA-local builder

constexpr int KIND_LEAF = 0;
constexpr int KIND_NODE = 1;
constexpr int KIND_LOCAL = 2;  // handed to the CTA-local builder

__device__ __forceinline__ float coord4(const float4& p, int a) { return a == 0 ? p.x : (a == 1 ? p.y : p.z); }

__global__ void init_keys_kernel(const float4* __restrict__ pts, long long n, uint32_t* keys, uint32_t* ord) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int b = blockIdx.y;
    if (i >= n) return;
    float4 p = pts[i];
    keys[b * n + i] = float_key(coord4(p, b));
    ord[b * n + i] = (uint32_t)i;
}

__global__ void job_of_point_kernel(const int* __restrict__ job_off, int njobs, long long n, int* jp) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int lo = 0, hi = njobs - 1;  // last j with job_off[j] <= i
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (job_off[mid] <= i) lo = mid; else hi = mid - 1;
    }
    jp[i] = lo;
}

__global__ void job_keys_kernel(const int* __restrict__ jp, const uint32_t* __restrict__ ord, long long n,
                                uint32_t* keys) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int b = blockIdx.y;
    if (i >= n) return;
    keys[b * n + i] = (uint32_t)jp[ord[b * n + i]];
}

__global__ void init_segs_kernel(const int* __restrict__ job_off, const int* __restrict__ job_link, int njobs,
                                 int4* segs, int* nseg) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j == 0) nseg[0] = njobs;
    if (j >= njobs) return;
    segs[j] = make_int4(job_off[j], job_off[j + 1], job_link[j], 0);
}

__global__ void init_segpos_kernel(const uint32_t* __restrict__ job_keys, long long n, int single, int* segpos) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    segpos[i] = single ? 0 : (int)job_keys[i];
}

// One thread per segment of the current level.
__global__ void level_seg_kernel(DevTree t, const float4* __restrict__ pts, const uint32_t* __restrict__ ord,
                                 long long n, const int4* __restrict__ segs, const int* nseg_cur,
                                 int4* __restrict__ segs_next, int* nseg_next, int4* __restrict__ seginfo,
                                 int fill, int max_next, int4* __restrict__ local_jobs, int* nlocal) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *nseg_cur) return;
    int4 sg = segs[i];
    int s = sg.x, e = sg.y, link = sg.z;
    int cnt = e - s;
    if (cnt <= LB_MAX) {
        int r = atomicAdd(nlocal, 1);
        if (r >= max_next) {
            atomicOr(&t.st->err, ERR_SEG);
            seginfo[i] = make_int4(-1, 0, 0, 0);
            return;
        }
        local_jobs[r] = make_int4(s, e, link, 0);
        seginfo[i] = make_int4(KIND_LOCAL, 0, 0, 0);
        return;
    }
    int parent = link >> 1, side = link & 1;
    Box3 b = empty_box();
    if (cnt > 0) {
        for (int a = 0; a < 3; ++a) {
            b.lo[a] = coord4(pts[ord[a * n + s]], a);
            b.hi[a] = coord4(pts[ord[a * n + e - 1]], a);
        }
    }
    if (cnt <= fill) {
        int L = alloc_leaf(t);
        if (L < 0) {
            seginfo[i] = make_int4(-1, 0, 0, 0);
            return;
        }
        t.leaf_n[L] = cnt;
        t.lparent[L] = link;
        write_child_box(t.node, parent, side, b);
        write_child_code(t.node, parent, side, leaf_code(L));
        write_child_cnt(t.ncnt, parent, side, cnt, 0);
        seginfo[i] = make_int4(KIND_LEAF, L, s, 0);
        return;
    }
    int X = alloc_node(t);
    if (X < 0) {
        seginfo[i] = make_int4(-1, 0, 0, 0);
        return;
    }
    float ext[3];
    for (int a = 0; a < 3; ++a) ext[a] = __fsub_rn(b.hi[a], b.lo[a]);
    int axis = 0;
    if (ext[1] > ext[axis]) axis = 1;
    if (ext[2] > ext[axis]) axis = 2;
    int mid = s + cnt / 2;
    float split = coord4(pts[ord[axis * n + mid]], axis);
    float4* rec = t.node + 4 * X;
    rec[3] = make_float4(__int_as_float(0), __int_as_float(0), split, __int_as_float(axis));
    t.nparent[X] = link;
    int h = 0;
    for (int m = cnt; m > fill; m -= m / 2) ++h;
    t.nheight[X] = h;
    write_child_box(t.node, parent, side, b);
    write_child_code(t.node, parent, side, X);
    write_child_cnt(t.ncnt, parent, side, cnt, 0);
    int r = atomicAdd(nseg_next, 2);
    if (r + 1 >= max_next) {  // cannot happen with the host's bound; guard anyway
        atomicOr(&t.st->err, ERR_SEG);
        seginfo[i] = make_int4(-1, 0, 0, 0);
        return;
    }
    segs_next[r] = make_int4(s, mid, X * 2 + 0, 0);
    segs_next[r + 1] = make_int4(mid, e, X * 2 + 1, 0);
    seginfo[i] = make_int4(KIND_NODE, axis, mid, r);
}

// One thread per position: leaves copy their points; internal segments mark
// which of their points go left.
__global__ void level_pos_kernel(DevTree t, const float4* __restrict__ pts, const uint32_t* __restrict__ ord,
                                 long long n, const int* __restrict__ segpos, const int4* __restrict__ seginfo,
                                 int* __restrict__ flag) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int sg = segpos[i];
    if (sg < 0) return;
    int4 info = seginfo[sg];
    if (info.x == KIND_LEAF) {
        float4 p = pts[ord[i]];
        p.w = __uint_as_float(__float_as_uint(p.w) & ID_MASK);
        t.pts[(long long)info.y * LEAF_CAP + (i - info.z)] = p;
    } else if (info.x == KIND_NODE) {
        uint32_t pt = ord[(long long)info.y * n + i];
        flag[pt] = i < info.z ? 1 : 0;
    }
}

__global__ void level_scanin_kernel(const uint32_t* __restrict__ ord, long long n, const int* __restrict__ segpos,
                                    const int4* __restrict__ seginfo, const int* __restrict__ flag,
                                    int* __restrict__ scan_in) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int b = blockIdx.y;
    if (i >= n) return;
    int sg = segpos[i];
    int v = 0;
    if (sg >= 0 && seginfo[sg].x == KIND_NODE) v = flag[ord[b * n + i]];
    scan_in[b * n + i] = v;
}

__global__ void level_scatter_kernel(const uint32_t* __restrict__ ord, uint32_t* __restrict__ ord_next, long long n,
                                     const int* __restrict__ segpos, int* __restrict__ segpos_next,
                                     const int4* __restrict__ segs, const int4* __restrict__ seginfo,
                                     const int* __restrict__ flag, const int* __restrict__ scan_out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int b = blockIdx.y;
    if (i >= n) return;
    int sg = segpos[i];
    int4 info = sg >= 0 ? seginfo[sg] : make_int4(-1, 0, 0, 0);
    if (info.x != KIND_NODE) {
        ord_next[b * n + i] = ord[b * n + i];  // keeps the local builder's three arrays whole
        if (b == 0) segpos_next[i] = -1;
        return;
    }
    int s = segs[sg].x, mid = info.z;
    uint32_t pt = ord[b * n + i];
    int in_left = flag[pt];
    int base = scan_out[b * n + s];
    int pl = scan_out[b * n + i] - base;
    long long np = in_left ? (long long)s + pl : (long long)mid + (i - s - pl);
    ord_next[b * n + np] = pt;
    if (b == 0) segpos_next[np] = info.w + (in_left ? 0 : 1);
}

// ---- CTA-local builder ----------------------------------------------------------
// One block builds a whole subtree of up to LB_MAX points in shared memory,
// with the method of the global levels: three index arrays, each sorted on
// one coordinate, are stably partitioned level by level, so every open
// segment is the same position range in all three and its AABB is read off
// the ends of the ranges.  Per level: one thread per open segment allocates
// its node or leaf (the split point is the middle of the range on the split
// axis, which already holds the left half in place); one pass over positions
// marks each point's side and fills the leaves; a block prefix sum of the
// left flags of the two other arrays and a scatter partition them.  Each
// thread owns LB_PPT consecutive positions.
//
// The arrays arrive sorted from the global levels (`idx` != nullptr: the
// three arrays of the level scatter, stride `stride`); jobs that never went
// through the global levels (`idx` == nullptr: points pts[x .. y)) are sorted
// here first, one bitonic sort per axis on (coordinate key, input position).
//
// With leaves of at most `fill` >= 8 points an open segment holds >= 9
// points, so a level has at most 2 * LB_MAX / 9 < LB_SEGS open segments.
constexpr int LB_THREADS = 1024;
constexpr int LB_PPT = LB_MAX / LB_THREADS;
constexpr int LB_SEGS = 1024;
constexpr uint16_t LB_DONE = 0xffff;
static_assert(LB_MAX % LB_THREADS == 0 && LB_MAX <= 65535, "local builder shape");
static_assert(2 * LB_MAX / 9 < LB_SEGS, "segment table too small");

struct LbShared {
    float4 P[LB_MAX];                 // the job's points by local id (input order)
    uint16_t ord0[3][LB_MAX];         // index arrays, one per axis (local ids)
    union {
        struct {
            uint16_t ord1[3][LB_MAX];  // the other buffer of the partition
            uint16_t seg_of[LB_MAX];   // open segment of a position, LB_DONE once in a leaf
        } a;
        unsigned long long K[LB_MAX];  // sort keys, only before the first level
    } u;
    uint32_t scanv[LB_MAX];           // exclusive prefix of packed left flags
    uint8_t side[LB_MAX];             // per local id: 1 = goes right
    uint16_t ss[2][LB_SEGS], se[2][LB_SEGS];
    int slink[2][LB_SEGS];
    int snode[LB_SEGS];               // node or leaf index, -1 when allocation failed
    uint16_t snext[LB_SEGS];          // first child segment of a node
    int8_t saxis[LB_SEGS];            // split axis, -1 for leaves
    uint32_t wsum[LB_THREADS / 32];
    int nseg[2];
    int overflow;
};
static_assert(sizeof(((LbShared*)0)->u.a) == sizeof(((LbShared*)0)->u.K), "sort keys alias the second buffer");

__device__ __forceinline__ float key_float(uint32_t k) {
    uint32_t u = (k & 0x80000000u) ? (k ^ 0x80000000u) : ~k;
    return __uint_as_float(u);
}

// Ascending bitonic sort of K[0 .. size), size a power of two; one
// compare-exchange per pair, pairs spread over the block.
__device__ void lb_bitonic(unsigned long long* K, int size) {
    const int half = size >> 1;
    for (int kk = 2; kk <= size; kk <<= 1) {
        for (int j = kk >> 1; j > 0; j >>= 1) {
            for (int p = threadIdx.x; p < half; p += LB_THREADS) {
                const int i = ((p & ~(j - 1)) << 1) | (p & (j - 1));
                const int ixj = i | j;
                const unsigned long long a = K[i], c = K[ixj];
                if ((a > c) == ((i & kk) == 0)) {
                    K[i] = c;
                    K[ixj] = a;
                }
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(LB_THREADS) local_build_kernel(DevTree t, const float4* __restrict__ pts,
                                                                 const uint32_t* __restrict__ idx,
                                                                 long long stride, int* loc,
                                                                 const int4* __restrict__ jobs, const int* njobs,
                                                                 int fill) {
    extern __shared__ __align__(16) unsigned char lb_raw[];
    LbShared& sm = *reinterpret_cast<LbShared*>(lb_raw);
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int nj = *njobs;
    for (int job = blockIdx.x; job < nj; job += gridDim.x) {
        const int4 jb = jobs[job];
        const int n = jb.y - jb.x;
        if (n > LB_MAX || n < 0 || fill < 8) {  // cannot happen: the host guarantees all three
            if (tid == 0) atomicOr(&t.st->err, ERR_SEG);
            continue;
        }
        if (idx == nullptr) {
            for (int i = tid; i < n; i += LB_THREADS) sm.P[i] = pts[(long long)jb.x + i];
            int size = 2;
            while (size < n) size <<= 1;
            for (int a = 0; a < 3; ++a) {
                __syncthreads();
                for (int i = tid; i < size; i += LB_THREADS)
                    sm.u.K[i] = i < n ? ((unsigned long long)float_key(coord4(sm.P[i], a)) << 32) | (unsigned)i
                                      : ~0ull;
                __syncthreads();
                lb_bitonic(sm.u.K, size);
                for (int i = tid; i < n; i += LB_THREADS) sm.ord0[a][i] = (uint16_t)sm.u.K[i];
            }
        } else {
            for (int i = tid; i < n; i += LB_THREADS) {
                const uint32_t g = idx[jb.x + i];
                sm.P[i] = pts[g];
                sm.ord0[0][i] = (uint16_t)i;
                loc[g] = i;
            }
            __syncthreads();
            for (int b = 1; b < 3; ++b)
                for (int i = tid; i < n; i += LB_THREADS) sm.ord0[b][i] = (uint16_t)loc[idx[b * stride + jb.x + i]];
        }
        __syncthreads();  // the sort keys are dead from here on
        for (int i = tid; i < n; i += LB_THREADS) sm.u.a.seg_of[i] = 0;
        if (tid == 0) {
            sm.nseg[0] = 1;
            sm.nseg[1] = 0;
            sm.overflow = 0;
            sm.ss[0][0] = 0;
            sm.se[0][0] = (uint16_t)n;
            sm.slink[0][0] = jb.z;
        }
        __syncthreads();
        uint16_t(*oc)[LB_MAX] = sm.ord0;
        uint16_t(*on)[LB_MAX] = sm.u.a.ord1;
        int cb = 0;
        const int i0 = tid * LB_PPT;
        for (int level = 0; level < 64; ++level) {
            const int S = sm.nseg[cb];
            if (S == 0) break;
            // One thread per open segment: a leaf, or a node with its axis,
            // its split value and two child segments.
            for (int sg = tid; sg < S; sg += LB_THREADS) {
                const int s = sm.ss[cb][sg], e = sm.se[cb][sg], link = sm.slink[cb][sg];
                const int cnt = e - s;
                const int parent = link >> 1, side = link & 1;
                Box3 b = empty_box();
                if (cnt > 0)
                    for (int a = 0; a < 3; ++a) {
                        b.lo[a] = coord4(sm.P[oc[a][s]], a);
                        b.hi[a] = coord4(sm.P[oc[a][e - 1]], a);
                    }
                sm.saxis[sg] = -1;
                sm.snode[sg] = -1;
                if (cnt <= fill) {
                    const int L = alloc_leaf(t);
                    sm.snode[sg] = L;
                    if (L >= 0) {
                        t.leaf_n[L] = cnt;
                        t.lparent[L] = link;
                        write_child_box(t.node, parent, side, b);
                        write_child_code(t.node, parent, side, leaf_code(L));
                        write_child_cnt(t.ncnt, parent, side, cnt, 0);
                    }
                    continue;
                }
                const int X = alloc_node(t);
                if (X < 0) continue;
                float ext[3];
                for (int a = 0; a < 3; ++a) ext[a] = __fsub_rn(b.hi[a], b.lo[a]);
                int axis = 0;
                if (ext[1] > ext[axis]) axis = 1;
                if (ext[2] > ext[axis]) axis = 2;
                const int mid = s + cnt / 2;
                const int r = atomicAdd(&sm.nseg[cb ^ 1], 2);
                if (r + 1 >= LB_SEGS) {  // cannot happen by the bound above; guard anyway
                    atomicOr(&t.st->err, ERR_SEG);
                    sm.overflow = 1;
                    continue;
                }
                sm.snode[sg] = X;
                sm.saxis[sg] = (int8_t)axis;
                sm.snext[sg] = (uint16_t)r;
                t.node[4 * X + 3] = make_float4(__int_as_float(0), __int_as_float(0),
                                                coord4(sm.P[oc[axis][mid]], axis), __int_as_float(axis));
                t.nparent[X] = link;
                int h = 0;
                for (int m = cnt; m > fill; m -= m / 2) ++h;
                t.nheight[X] = h;
                write_child_box(t.node, parent, side, b);
                write_child_code(t.node, parent, side, X);
                write_child_cnt(t.ncnt, parent, side, cnt, 0);
                sm.ss[cb ^ 1][r] = (uint16_t)s;
                sm.se[cb ^ 1][r] = (uint16_t)mid;
                sm.slink[cb ^ 1][r] = X * 2;
                sm.ss[cb ^ 1][r + 1] = (uint16_t)mid;
                sm.se[cb ^ 1][r + 1] = (uint16_t)e;
                sm.slink[cb ^ 1][r + 1] = X * 2 + 1;
            }
            __syncthreads();
            if (sm.overflow) break;
            // Leaves take their points; node segments mark each point's side
            // from its position in the split axis's array.
#pragma unroll
            for (int r = 0; r < LB_PPT; ++r) {
                const int i = i0 + r;
                if (i >= n) break;
                const int sg = sm.u.a.seg_of[i];
                if (sg == LB_DONE) continue;
                const int ax = sm.saxis[sg];
                const int s = sm.ss[cb][sg];
                if (ax < 0) {
                    const int L = sm.snode[sg];
                    if (L >= 0) {
                        float4 q = sm.P[oc[0][i]];
                        q.w = __uint_as_float(__float_as_uint(q.w) & ID_MASK);
                        t.pts[(long long)L * LEAF_CAP + (i - s)] = q;
                    }
                } else {
                    const int mid = s + (sm.se[cb][sg] - s) / 2;
                    sm.side[oc[ax][i]] = i >= mid ? 1 : 0;
                }
            }
            __syncthreads();
            // Packed left flags of the two arrays that are not the split
            // axis's: (axis + 1) % 3 in the low half, (axis + 2) % 3 in the high.
            uint32_t v[LB_PPT];
            uint32_t sum = 0;
#pragma unroll
            for (int r = 0; r < LB_PPT; ++r) {
                const int i = i0 + r;
                uint32_t f = 0;
                if (i < n) {
                    const int sg = sm.u.a.seg_of[i];
                    if (sg != LB_DONE) {
                        const int ax = sm.saxis[sg];
                        if (ax >= 0) {
                            const int b1 = ax == 2 ? 0 : ax + 1, b2 = ax == 0 ? 2 : ax - 1;
                            f = (uint32_t)(sm.side[oc[b1][i]] ^ 1) | ((uint32_t)(sm.side[oc[b2][i]] ^ 1) << 16);
                        }
                    }
                }
                v[r] = sum;
                sum += f;
            }
            uint32_t inc = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += y;
            }
            if (lane == 31) sm.wsum[warp] = inc;
            __syncthreads();
            if (warp == 0) {
                uint32_t w = lane < LB_THREADS / 32 ? sm.wsum[lane] : 0u;
                uint32_t wi = w;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
                    if (lane >= o) wi += y;
                }
                if (lane < LB_THREADS / 32) sm.wsum[lane] = wi - w;
            }
            __syncthreads();
            const uint32_t tbase = sm.wsum[warp] + inc - sum;
#pragma unroll
            for (int r = 0; r < LB_PPT; ++r)
                if (i0 + r < n) sm.scanv[i0 + r] = tbase + v[r];
            __syncthreads();
            // Scatter: the split axis's array keeps its order, the other two
            // are partitioned stably; positions move to the child segments.
            if (tid == 0) sm.nseg[cb] = 0;  // every thread read it at the top of the level
#pragma unroll
            for (int r = 0; r < LB_PPT; ++r) {
                const int i = i0 + r;
                if (i >= n) break;
                const int sg = sm.u.a.seg_of[i];
                if (sg == LB_DONE) continue;
                const int ax = sm.saxis[sg];
                if (ax < 0) {
                    sm.u.a.seg_of[i] = LB_DONE;
                    continue;
                }
                const int s = sm.ss[cb][sg];
                const int mid = s + (sm.se[cb][sg] - s) / 2;
                const int b1 = ax == 2 ? 0 : ax + 1, b2 = ax == 0 ? 2 : ax - 1;
                const uint32_t rel = sm.scanv[i] - sm.scanv[s];
                on[ax][i] = oc[ax][i];
                const uint16_t j1 = oc[b1][i], j2 = oc[b2][i];
                const int c1 = (int)(rel & 0xffffu), c2 = (int)(rel >> 16);
                on[b1][sm.side[j1] ? mid + (i - s - c1) : s + c1] = j1;
                on[b2][sm.side[j2] ? mid + (i - s - c2) : s + c2] = j2;
                sm.u.a.seg_of[i] = (uint16_t)(sm.snext[sg] + (i < mid ? 0 : 1));
            }
            __syncthreads();
            uint16_t(*tmp)[LB_MAX] = oc;
            oc = on;
            on = tmp;
            cb ^= 1;
        }
        __syncthreads();
    }
}

size_t lb_smem_bytes() { return sizeof(LbShared); }

// The block's shared memory is above the 48 KB default: opt in once per device.
void lb_prepare() {
    static std::atomic<unsigned long long> done{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return;
    cudaFuncSetAttribute(local_build_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(LbShared));
    done.fetch_or(bit, std::memory_order_release);
}

__global__ void finish_alloc_kernel(DevStatus* st) {
    st->free_node_n = max(0, st->free_node_n - st->free_node_taken);
    st->free_leaf_n = max(0, st->free_leaf_n - st->free_leaf_taken);
    st->free_node_taken = 0;
    st->free_leaf_taken = 0;
}

__global__ void reset_count_kernel(int* c) { *c = 0; }

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

long long max_segs_bound(long long n, int njobs, int fill) {
    long long b = 2 * (n / (fill + 1)) + 2;
    return b > njobs ? b : njobs;
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

int build_levels(long long max_job, int fill) {
    int d = 0;
    while (max_job > fill) {
        max_job = max_job - max_job / 2;
        ++d;
    }
    return d + 1;
}

size_t build_scratch_bytes(long long n, int njobs, int fill) {
    long long ms = max_segs_bound(n, njobs, fill);
    size_t b = 0;
    b += 2 * align_up(sizeof(uint32_t) * 3 * n);   // ord
    b += 2 * align_up(sizeof(uint32_t) * 3 * n);   // keys
    b += 2 * align_up(sizeof(int) * n);            // segpos
    b += align_up(sizeof(int) * n);                // flag
    b += 2 * align_up(sizeof(int) * 3 * n);        // scan in / out
    b += 4 * align_up(sizeof(int4) * ms);          // segs x2, seginfo, local jobs
    b += align_up(sizeof(int) * 4);                // nseg
    size_t tmp = sort_temp_bytes(n, 3);
    size_t st = scan_temp_bytes(3 * n);
    b += align_up(tmp > st ? tmp : st);
    return b;
}

void carve_build_scratch(void* base, long long n, int njobs, int fill, BuildScratch* bs) {
    long long ms = max_segs_bound(n, njobs, fill);
    char* p = (char*)base;
    auto take = [&](size_t bytes) {
        void* r = p;
        p += align_up(bytes);
        return r;
    };
    bs->ord[0] = (uint32_t*)take(sizeof(uint32_t) * 3 * n);
    bs->ord[1] = (uint32_t*)take(sizeof(uint32_t) * 3 * n);
    bs->keys[0] = (uint32_t*)take(sizeof(uint32_t) * 3 * n);
    bs->keys[1] = (uint32_t*)take(sizeof(uint32_t) * 3 * n);
    bs->segpos[0] = (int*)take(sizeof(int) * n);
    bs->segpos[1] = (int*)take(sizeof(int) * n);
    bs->flag = (int*)take(sizeof(int) * n);
    bs->scan_in = (int*)take(sizeof(int) * 3 * n);
    bs->scan_out = (int*)take(sizeof(int) * 3 * n);
    bs->segs[0] = (int4*)take(sizeof(int4) * ms);
    bs->segs[1] = (int4*)take(sizeof(int4) * ms);
    bs->seginfo = (int4*)take(sizeof(int4) * ms);
    bs->local_jobs = (int4*)take(sizeof(int4) * ms);
    bs->nseg = (int*)take(sizeof(int) * 4);
    bs->temp = (void*)p;
}

void build_subtrees(const DevTree& t, const float4* pts, long long n, const int* job_off, const int* job_link,
                    int njobs, long long max_job, int fill, const BuildScratch& bs, cudaStream_t s) {
    if (njobs <= 0) return;
    lb_prepare();
    const int T = 256;
    long long nn = n > 0 ? n : 1;
    long long ms = max_segs_bound(nn, njobs, fill);
    const unsigned lb_grid = (unsigned)(njobs < 4096 ? njobs : 4096);
    if (max_job <= LB_MAX) {
        // Every job fits one block: a single launch builds them all.
        init_segs_kernel<<<blocks_for(njobs, T), T, 0, s>>>(job_off, job_link, njobs, bs.segs[0], bs.nseg);
        local_build_kernel<<<lb_grid, LB_THREADS, lb_smem_bytes(), s>>>(t, pts, nullptr, 0, nullptr, bs.segs[0],
                                                                         bs.nseg, fill);
        finish_alloc_kernel<<<1, 1, 0, s>>>(t.st);
        return;
    }
    init_keys_kernel<<<dim3(blocks_for(n, T), 3), T, 0, s>>>(pts, n, bs.keys[0], bs.ord[0]);
    radix_sort_pairs(bs.keys[0], bs.ord[0], bs.keys[1], bs.ord[1], n, 3, n, 32, bs.temp, s);
    if (njobs > 1) {
        int* jp = bs.segpos[1];
        job_of_point_kernel<<<blocks_for(n, T), T, 0, s>>>(job_off, njobs, n, jp);
        job_keys_kernel<<<dim3(blocks_for(n, T), 3), T, 0, s>>>(jp, bs.ord[0], n, bs.keys[0]);
        int bits = 8;
        while (bits < 32 && (1ll << bits) < njobs) bits += 8;
        radix_sort_pairs(bs.keys[0], bs.ord[0], bs.keys[1], bs.ord[1], n, 3, n, bits, bs.temp, s);
    }
    init_segpos_kernel<<<blocks_for(n, T), T, 0, s>>>(bs.keys[0], n, njobs == 1, bs.segpos[0]);
    init_segs_kernel<<<blocks_for(njobs, T), T, 0, s>>>(job_off, job_link, njobs, bs.segs[0], bs.nseg);
    reset_count_kernel<<<1, 1, 0, s>>>(bs.nseg + 2);
    // Global levels until every segment fits the local builder.
    int levels = build_levels(max_job, LB_MAX);
    int cur = 0;
    long long seg_bound = njobs;
    for (int lv = 0; lv < levels; ++lv) {
        int nxt = cur ^ 1;
        reset_count_kernel<<<1, 1, 0, s>>>(bs.nseg + nxt);
        level_seg_kernel<<<blocks_for(seg_bound, 128), 128, 0, s>>>(t, pts, bs.ord[cur], nn, bs.segs[cur],
                                                                    bs.nseg + cur, bs.segs[nxt], bs.nseg + nxt,
                                                                    bs.seginfo, fill, (int)ms, bs.local_jobs,
                                                                    bs.nseg + 2);
        level_pos_kernel<<<blocks_for(n, T), T, 0, s>>>(t, pts, bs.ord[cur], n, bs.segpos[cur], bs.seginfo, bs.flag);
        level_scanin_kernel<<<dim3(blocks_for(n, T), 3), T, 0, s>>>(bs.ord[cur], n, bs.segpos[cur], bs.seginfo,
                                                                   bs.flag, bs.scan_in);
        exclusive_scan(bs.scan_in, bs.scan_out, 3 * n, nullptr, bs.temp, s);
        level_scatter_kernel<<<dim3(blocks_for(n, T), 3), T, 0, s>>>(bs.ord[cur], bs.ord[nxt], n, bs.segpos[cur],
                                                                    bs.segpos[nxt], bs.segs[cur], bs.seginfo,
                                                                    bs.flag, bs.scan_out);
        long long nb = seg_bound * 2;
        seg_bound = nb < ms ? nb : ms;
        cur = nxt;
    }
    // The three index arrays of the last level hold every local segment.
    unsigned g = (unsigned)(ms < 4096 ? ms : 4096);
    local_build_kernel<<<g, LB_THREADS, lb_smem_bytes(), s>>>(t, pts, bs.ord[cur], n, bs.flag, bs.local_jobs,
                                                               bs.nseg + 2, fill);
    finish_alloc_kernel<<<1, 1, 0, s>>>(t.st);
}

}  // namespace ikdg
