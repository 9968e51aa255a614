// Batched, level-synchronous subtree builder.
//
// Replaces the recursive BuildTree (ikd-Tree/ikd_Tree.cpp:573-622), used both
// by Build (:352-364) and by the rebuilds of Rebuild (:624-645).  The split
// rule is kept: every segment is cut at its median on the longest axis of its
// AABB (first axis wins ties, :593-595).  Unlike the reference, internal nodes
// hold no point: segments of at most `fill` points become leaf buckets.
//
// All jobs of a call are built together, on one of three paths chosen by the
// largest job:
// * small (every job <= LB_SMALL points): one CTA per job builds the whole
//   subtree in shared memory (local_build_kernel<LB_SMALL, 256>);
// * medium (jobs <= MID_MAX): one launch per tree level splits every open
//   segment of every job, one CTA per segment, down to LB_SMALL-point segments
//   (mid_level_kernel: radix-selected median, stable partition), then the
//   small local builder finishes them;
// * large: each of the three coordinates is radix-sorted once; the three sorted
//   index arrays are then stably partitioned level by level, so every segment
//   stays a contiguous range in each array and its AABB is read off the ends of
//   the three ranges.  Per level: one thread per segment allocates its node or
//   leaf and links it into its parent; one thread per position marks left /
//   right; a prefix sum and a scatter partition the three arrays.  Segments of
//   at most LB_MAX points go, with their sorted arrays, to
//   local_build_kernel<LB_MAX, 1024>.
// All three cut a segment of n points at the point of rank n / 2 on its axis,
// ties in input order (every partition is stable), so they follow one split
// rule.
#include <cuda_runtime.h>

#include <algorithm>
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
    if (i >= *nseg_cur || i >= max_next) return;  // the count runs past the capacity only on overflow (flagged)
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
// One block builds a whole subtree of up to MAXN points in shared memory,
// with the method of the global levels: three index arrays, each sorted on
// one coordinate, are stably partitioned level by level, so every open
// segment is the same position range in all three and its AABB is read off
// the ends of the ranges.  Per level: one thread per open segment allocates
// its node or leaf (the split point is the middle of the range on the split
// axis, which already holds the left half in place); one pass over positions
// marks each point's side and fills the leaves; a block prefix sum of the
// left flags of the two other arrays and a scatter partition them.
//
// The arrays arrive sorted from the global levels (`idx` != nullptr: the
// three arrays of the level scatter, stride `stride`); jobs that never went
// through the global levels (`idx` == nullptr: points pts[x .. y)) are sorted
// here first: one bitonic network sorts the three arrays of (coordinate key,
// input position) together.
//
// With leaves of at most `fill` >= 8 points an open segment holds >= 9
// points, so a level has at most 2 * MAXN / 9 < SEGS open segments.
//
// Two shapes: 4,096 points on 1,024 threads (about 207 KB of shared memory,
// one block per SM) and 1,024 points on 256 threads (about 52 KB, four per
// SM); each thread owns four positions and one open segment at most.
constexpr int LB_SMALL = 1024;
constexpr uint16_t LB_DONE = 0xffff;

template <int MAXN, int THREADS>
struct LbShared {
    static constexpr int SEGS = THREADS;
    float4 P[MAXN];            // the job's points by local id (input order)
    uint16_t ord0[3][MAXN];    // index arrays, one per axis (local ids)
    union {
        struct {
            uint16_t ord1[3][MAXN];  // the other buffer of the partition
            uint16_t seg_of[MAXN];   // open segment of a position, LB_DONE once in a leaf
            uint32_t scanv[MAXN];    // exclusive prefix of packed left flags
            uint8_t side[MAXN];      // per local id: 1 = goes right
        } a;
        unsigned long long K[3][MAXN];  // sort keys, only before the first level
    } u;
    uint16_t ss[2][SEGS], se[2][SEGS];
    int slink[2][SEGS];
    int snode[SEGS];           // node or leaf index, -1 when allocation failed
    uint16_t snext[SEGS];      // first child segment of a node
    int8_t saxis[SEGS];        // split axis, -1 for leaves
    uint32_t wsum[THREADS / 32];
    PoolRun run_leaf, run_node;
    int free_leaf_n, free_node_n;  // free-stack sizes when the runs were taken
    uint32_t level_total;          // leaves (low 16 bits) and nodes of the current level
    int nseg[2];
    int overflow;
};
static_assert(sizeof(LbShared<LB_MAX, 1024>) <= 227 * 1024, "local builder shared memory");

__device__ __forceinline__ float key_float(uint32_t k) {
    uint32_t u = (k & 0x80000000u) ? (k ^ 0x80000000u) : ~k;
    return __uint_as_float(u);
}

// Ascending bitonic sort of K[a][0 .. size) for the three arrays at once,
// size a power of two; one compare-exchange per pair, pairs spread over the
// block.
template <int MAXN, int THREADS>
__device__ void lb_bitonic3(unsigned long long (*K)[MAXN], int size) {
    const int half = size >> 1;
    for (int kk = 2; kk <= size; kk <<= 1) {
        for (int j = kk >> 1; j > 0; j >>= 1) {
            for (int p = threadIdx.x; p < half; p += THREADS) {
                const int i = ((p & ~(j - 1)) << 1) | (p & (j - 1));
                const int ixj = i | j;
                const bool up = (i & kk) == 0;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const unsigned long long x = K[a][i], y = K[a][ixj];
                    if ((x > y) == up) {
                        K[a][i] = y;
                        K[a][ixj] = x;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Nodes and leaves of the subtree the builders make from n points with leaf
// fill `fill`: a segment of more than `fill` points is a node whose children
// hold n / 2 and n - n / 2 points, so the sizes of one level take at most two
// consecutive values.
__device__ __forceinline__ void subtree_counts(int n, int fill, int* nodes, int* leaves) {
    int lo = n, c_lo = 1, c_hi = 0;  // c_lo segments of lo points, c_hi of lo + 1
    int nn = 0, nl = 0;
    for (int guard = 0; guard < 40 && c_lo + c_hi > 0; ++guard) {
        int n_lo = 0, n_hi = 0, next = 0;
        bool have = false;
        for (int h = 0; h < 2; ++h) {
            const int size = lo + h, c = h ? c_hi : c_lo;
            if (c == 0) continue;
            if (size <= fill) {
                nl += c;
                continue;
            }
            nn += c;
            const int a = size / 2, b = size - size / 2;  // b == a or a + 1
            if (!have) {
                next = a;
                have = true;
            }
            // children sizes at this level are next or next + 1
            n_lo += (a == next ? c : 0) + (b == next ? c : 0);
            n_hi += (a == next + 1 ? c : 0) + (b == next + 1 ? c : 0);
        }
        lo = next;
        c_lo = n_lo;
        c_hi = n_hi;
    }
    *nodes = nn;
    *leaves = nl;
}

template <int MAXN, int THREADS>
__global__ void __launch_bounds__(THREADS, THREADS >= 1024 ? 1 : 4) local_build_kernel(DevTree t, const float4* __restrict__ pts,
                                                                 const uint32_t* __restrict__ idx,
                                                                 long long stride, int* loc,
                                                                 const int4* __restrict__ jobs, const int* njobs,
                                                                 int max_jobs, int fill) {
    extern __shared__ __align__(16) unsigned char lb_raw[];
    constexpr int PPT = MAXN / THREADS;
    constexpr int SEGS = THREADS;
    static_assert(MAXN % THREADS == 0 && PPT == 4 && MAXN <= 65535, "local builder shape");
    static_assert(2 * MAXN / 9 < SEGS, "segment table too small");
    LbShared<MAXN, THREADS>& sm = *reinterpret_cast<LbShared<MAXN, THREADS>*>(lb_raw);
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    // The producers count past the capacity when it overflows (and flag it):
    // never read beyond the job array.
    const int nj = min(*njobs, max_jobs);
    for (int job = blockIdx.x; job < nj; job += gridDim.x) {
        const int4 jb = jobs[job];
        const int n = jb.y - jb.x;
        if (n > MAXN || n < 0 || fill < 8) {  // cannot happen: the host guarantees all three
            if (tid == 0) atomicOr(&t.st->err, ERR_SEG);
            continue;
        }
        if (idx == nullptr) {
            for (int i = tid; i < n; i += THREADS) sm.P[i] = pts[(long long)jb.x + i];
            int size = 2;
            while (size < n) size <<= 1;
            __syncthreads();
            for (int i = tid; i < size; i += THREADS) {
                if (i < n) {
                    const float4 p = sm.P[i];
                    sm.u.K[0][i] = ((unsigned long long)float_key(p.x) << 32) | (unsigned)i;
                    sm.u.K[1][i] = ((unsigned long long)float_key(p.y) << 32) | (unsigned)i;
                    sm.u.K[2][i] = ((unsigned long long)float_key(p.z) << 32) | (unsigned)i;
                } else {
                    sm.u.K[0][i] = sm.u.K[1][i] = sm.u.K[2][i] = ~0ull;
                }
            }
            __syncthreads();
            lb_bitonic3<MAXN, THREADS>(sm.u.K, size);
            for (int i = tid; i < n; i += THREADS) {
                sm.ord0[0][i] = (uint16_t)sm.u.K[0][i];
                sm.ord0[1][i] = (uint16_t)sm.u.K[1][i];
                sm.ord0[2][i] = (uint16_t)sm.u.K[2][i];
            }
        } else {
            for (int i = tid; i < n; i += THREADS) {
                const uint32_t g = idx[jb.x + i];
                sm.P[i] = pts[g];
                sm.ord0[0][i] = (uint16_t)i;
                loc[g] = i;
            }
            __syncthreads();
            for (int b = 1; b < 3; ++b)
                for (int i = tid; i < n; i += THREADS) sm.ord0[b][i] = (uint16_t)loc[idx[b * stride + jb.x + i]];
        }
        __syncthreads();  // the sort keys are dead from here on
        for (int i = tid; i < n; i += THREADS) sm.u.a.seg_of[i] = 0;
        if (tid == 0) {
            sm.nseg[0] = 1;
            sm.nseg[1] = 0;
            sm.overflow = 0;
            sm.ss[0][0] = 0;
            sm.se[0][0] = (uint16_t)n;
            sm.slink[0][0] = jb.z;
            // The whole subtree's nodes and leaves from the pools at once
            // (its shape follows from n and the fill); level l takes the
            // indices after those of levels 0 .. l-1.
            int nn = 0, nl = 0;
            subtree_counts(n, fill, &nn, &nl);
            sm.free_leaf_n = t.st->free_leaf_n;
            sm.free_node_n = t.st->free_node_n;
            sm.run_leaf = pool_reserve(&t.st->free_leaf_taken, sm.free_leaf_n, &t.st->leaf_top, nl);
            sm.run_node = pool_reserve(&t.st->free_node_taken, sm.free_node_n, &t.st->node_top, nn);
        }
        __syncthreads();
        uint16_t(*oc)[MAXN] = sm.ord0;
        uint16_t(*on)[MAXN] = sm.u.a.ord1;
        int cb = 0;
        const int i0 = tid * PPT;
        int leaf_base = 0, node_base = 0;  // indices of the runs taken by earlier levels
        for (int level = 0; level < 64; ++level) {
            const int S = sm.nseg[cb];
            if (S == 0) break;
            // One thread per open segment: a leaf, or a node with its axis,
            // its split value and two child segments.  The level's leaves and
            // nodes are ranked by ballots and taken from the pools with one
            // reservation each.
            const int sg = tid;
            const bool live = sg < S;
            int s = 0, e = 0, link = 0;
            if (live) {
                s = sm.ss[cb][sg];
                e = sm.se[cb][sg];
                link = sm.slink[cb][sg];
            }
            const int cnt = e - s;
            const bool is_leaf = live && cnt <= fill, is_node = live && cnt > fill;
            const unsigned lm = __ballot_sync(0xffffffffu, is_leaf), nm = __ballot_sync(0xffffffffu, is_node);
            if (lane == 0) sm.wsum[warp] = (uint32_t)__popc(lm) | ((uint32_t)__popc(nm) << 16);
            __syncthreads();
            if (warp == 0) {
                const uint32_t w = lane < THREADS / 32 ? sm.wsum[lane] : 0u;
                uint32_t wi = w;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
                    if (lane >= o) wi += y;
                }
                if (lane < THREADS / 32) sm.wsum[lane] = wi - w;
                if (lane == 31) sm.level_total = wi;
            }
            __syncthreads();
            const uint32_t level_total = sm.level_total;
            if (live) {
                const uint32_t wb = sm.wsum[warp];
                const unsigned below = (1u << lane) - 1u;
                const int parent = link >> 1, side = link & 1;
                Box3 b = empty_box();
                if (cnt > 0)
                    for (int a = 0; a < 3; ++a) {
                        b.lo[a] = coord4(sm.P[oc[a][s]], a);
                        b.hi[a] = coord4(sm.P[oc[a][e - 1]], a);
                    }
                sm.saxis[sg] = -1;
                sm.snode[sg] = -1;
                if (is_leaf) {
                    const int L = pool_pick(sm.run_leaf, t.free_leaf, sm.free_leaf_n, t.leaf_cap,
                                            leaf_base + (int)(wb & 0xffffu) + __popc(lm & below), t.st,
                                            ERR_POOL_LEAF);
                    sm.snode[sg] = L;
                    if (L >= 0) {
                        t.leaf_n[L] = cnt;
                        t.lparent[L] = link;
                        write_child_box(t.node, parent, side, b);
                        write_child_code(t.node, parent, side, leaf_code(L));
                        write_child_cnt(t.ncnt, parent, side, cnt, 0);
                    }
                } else {
                    const int X = pool_pick(sm.run_node, t.free_node, sm.free_node_n, t.node_cap,
                                            node_base + (int)(wb >> 16) + __popc(nm & below), t.st, ERR_POOL);
                    float ext[3];
                    for (int a = 0; a < 3; ++a) ext[a] = __fsub_rn(b.hi[a], b.lo[a]);
                    int axis = 0;
                    if (ext[1] > ext[axis]) axis = 1;
                    if (ext[2] > ext[axis]) axis = 2;
                    const int mid = s + cnt / 2;
                    const int r = X >= 0 ? atomicAdd(&sm.nseg[cb ^ 1], 2) : 0;
                    if (X >= 0 && r + 1 >= SEGS) {  // cannot happen by the bound above; guard anyway
                        atomicOr(&t.st->err, ERR_SEG);
                        sm.overflow = 1;
                    } else if (X >= 0) {
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
                }
            }
            __syncthreads();
            if (sm.overflow) break;
            leaf_base += (int)(level_total & 0xffffu);
            node_base += (int)(level_total >> 16);
            // Leaves take their points; node segments mark each point's side
            // from its position in the split axis's array.
#pragma unroll
            for (int r = 0; r < PPT; ++r) {
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
                    sm.u.a.side[oc[ax][i]] = i >= mid ? 1 : 0;
                }
            }
            __syncthreads();
            // Packed left flags of the two arrays that are not the split
            // axis's: (axis + 1) % 3 in the low half, (axis + 2) % 3 in the high.
            uint32_t v[PPT];
            uint32_t sum = 0;
#pragma unroll
            for (int r = 0; r < PPT; ++r) {
                const int i = i0 + r;
                uint32_t f = 0;
                if (i < n) {
                    const int sg = sm.u.a.seg_of[i];
                    if (sg != LB_DONE) {
                        const int ax = sm.saxis[sg];
                        if (ax >= 0) {
                            const int b1 = ax == 2 ? 0 : ax + 1, b2 = ax == 0 ? 2 : ax - 1;
                            f = (uint32_t)(sm.u.a.side[oc[b1][i]] ^ 1) | ((uint32_t)(sm.u.a.side[oc[b2][i]] ^ 1) << 16);
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
                uint32_t w = lane < THREADS / 32 ? sm.wsum[lane] : 0u;
                uint32_t wi = w;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
                    if (lane >= o) wi += y;
                }
                if (lane < THREADS / 32) sm.wsum[lane] = wi - w;
            }
            __syncthreads();
            const uint32_t tbase = sm.wsum[warp] + inc - sum;
#pragma unroll
            for (int r = 0; r < PPT; ++r)
                if (i0 + r < n) sm.u.a.scanv[i0 + r] = tbase + v[r];
            __syncthreads();
            // Scatter: the split axis's array keeps its order, the other two
            // are partitioned stably; positions move to the child segments.
            if (tid == 0) sm.nseg[cb] = 0;  // every thread read it at the top of the level
#pragma unroll
            for (int r = 0; r < PPT; ++r) {
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
                const uint32_t rel = sm.u.a.scanv[i] - sm.u.a.scanv[s];
                on[ax][i] = oc[ax][i];
                const uint16_t j1 = oc[b1][i], j2 = oc[b2][i];
                const int c1 = (int)(rel & 0xffffu), c2 = (int)(rel >> 16);
                on[b1][sm.u.a.side[j1] ? mid + (i - s - c1) : s + c1] = j1;
                on[b2][sm.u.a.side[j2] ? mid + (i - s - c2) : s + c2] = j2;
                sm.u.a.seg_of[i] = (uint16_t)(sm.snext[sg] + (i < mid ? 0 : 1));
            }
            __syncthreads();
            uint16_t(*tmp)[MAXN] = oc;
            oc = on;
            on = tmp;
            cb ^= 1;
        }
        __syncthreads();
    }
}

// ---- level-by-level splitter for medium jobs -------------------------------------------
// Jobs of up to MID_MAX points skip the global sort: they are split one tree
// level per launch until every open segment fits the small local builder
// (LB_SMALL points), each open segment of a level by a block of its own (the
// open segments of every job of the call share the launch).  Per segment: the AABB by a block reduction of
// order-preserving keys; the median key on the longest axis by a four-pass
// radix select (8-bit digits, shared histogram); then one stable partition
// pass.  Keys below the median go left, keys equal to it go left in position
// order until the left half holds n / 2 points, so the split is the same
// (point of rank n / 2 on the axis, ties by position) as in the sorted
// builders.  Points move between two scratch buffers (level 0 reads the
// input); segments that fit the small local builder are copied to buffer 0
// if they are not there and handed to it as jobs.
constexpr int MID_MAX = 1 << 17;
constexpr int MID_THREADS = 1024;
constexpr int MID_PPT = 4;
constexpr int MID_TILE = MID_THREADS * MID_PPT;

struct MidShared {
    int hist[256];
    uint32_t red[MID_THREADS / 32][6];
    uint32_t wsum[MID_THREADS / 32];
    uint32_t tot;
    uint32_t box[6];
    int node, axis, digit, rank;
};

// Exclusive block prefix of a per-thread value; the block total goes to
// *total.  The shared words are free for reuse when it returns.
__device__ __forceinline__ uint32_t mid_block_scan(uint32_t v, uint32_t* wsum, uint32_t* tot, uint32_t* total) {
    static_assert(MID_THREADS == 32 * 32, "one warp scans the warp sums");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = wsum[lane];
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        wsum[lane] = wi - w;
        if (lane == 31) *tot = wi;
    }
    __syncthreads();
    const uint32_t r = wsum[warp] + inc - v;
    *total = *tot;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(MID_THREADS, 1) mid_level_kernel(DevTree t, const float4* src, float4* dst,
                                                                float4* buf0, uint32_t* keys,
                                                                const int4* __restrict__ segs_in,
                                                                const int* nseg_in, int4* __restrict__ segs_out,
                                                                int* nseg_out, int max_segs,
                                                                int4* __restrict__ local_jobs, int* nlocal,
                                                                int max_local, int fill) {
    __shared__ MidShared sm;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int S = min(*nseg_in, max_segs);
    for (int q = blockIdx.x; q < S; q += gridDim.x) {
        const int4 sg = segs_in[q];
        const int s = sg.x, e = sg.y, link = sg.z;
        const int cnt = e - s;
        __syncthreads();  // the previous segment's shared words are free again
        if (cnt <= LB_SMALL) {  // only at level 0: a small job goes straight to the local builder
            for (int i = s + tid; i < e; i += MID_THREADS) buf0[i] = src[i];
            if (tid == 0) {
                const int r = atomicAdd(nlocal, 1);
                if (r < max_local) local_jobs[r] = make_int4(s, e, link, 0);
                else atomicOr(&t.st->err, ERR_SEG);
            }
            continue;
        }
        // AABB.
        uint32_t mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0u, 0u, 0u};
        for (int i = s + tid; i < e; i += MID_THREADS) {
            const float4 p = src[i];
            const uint32_t kx = float_key(p.x), ky = float_key(p.y), kz = float_key(p.z);
            mn[0] = min(mn[0], kx), mx[0] = max(mx[0], kx);
            mn[1] = min(mn[1], ky), mx[1] = max(mx[1], ky);
            mn[2] = min(mn[2], kz), mx[2] = max(mx[2], kz);
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            mn[a] = __reduce_min_sync(0xffffffffu, mn[a]);
            mx[a] = __reduce_max_sync(0xffffffffu, mx[a]);
        }
        if (lane == 0)
            for (int a = 0; a < 3; ++a) sm.red[warp][a] = mn[a], sm.red[warp][3 + a] = mx[a];
        __syncthreads();
        if (warp == 0) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                uint32_t lo = lane < MID_THREADS / 32 ? sm.red[lane][a] : 0xffffffffu;
                uint32_t hi = lane < MID_THREADS / 32 ? sm.red[lane][3 + a] : 0u;
                lo = __reduce_min_sync(0xffffffffu, lo);
                hi = __reduce_max_sync(0xffffffffu, hi);
                if (lane == 0) sm.box[a] = lo, sm.box[3 + a] = hi;
            }
        }
        __syncthreads();
        // The node: axis, allocation, links into its parent.
        if (tid == 0) {
            Box3 b;
            for (int a = 0; a < 3; ++a) {
                b.lo[a] = key_float(sm.box[a]);
                b.hi[a] = key_float(sm.box[3 + a]);
            }
            float ext[3];
            for (int a = 0; a < 3; ++a) ext[a] = __fsub_rn(b.hi[a], b.lo[a]);
            int axis = 0;
            if (ext[1] > ext[axis]) axis = 1;
            if (ext[2] > ext[axis]) axis = 2;
            const int X = alloc_node(t);
            sm.node = X;
            sm.axis = axis;
            if (X >= 0) {
                const int parent = link >> 1, side = link & 1;
                t.nparent[X] = link;
                int h = 0;
                for (int m = cnt; m > fill; m -= m / 2) ++h;
                t.nheight[X] = h;
                write_child_box(t.node, parent, side, b);
                write_child_code(t.node, parent, side, X);
                write_child_cnt(t.ncnt, parent, side, cnt, 0);
            }
        }
        __syncthreads();
        const int X = sm.node, axis = sm.axis;
        if (X < 0) continue;  // the pool is exhausted (flagged by alloc_node): the points are dropped
        // Radix select of the key of rank m = cnt / 2.
        const int m = cnt / 2;
        uint32_t prefix = 0, pmask = 0;
        int rank = m;
        for (int pass = 0; pass < 4; ++pass) {
            const int shift = 24 - 8 * pass;
            if (tid < 256) sm.hist[tid] = 0;
            __syncthreads();
            for (int base = s; base < e; base += MID_THREADS) {
                const int i = base + tid;
                bool ok = false;
                uint32_t k = 0;
                if (i < e) {
                    if (pass == 0) {
                        k = float_key(coord4(src[i], axis));
                        keys[i] = k;
                    } else {
                        k = keys[i];
                    }
                    ok = (k & pmask) == prefix;
                }
                const int d = ok ? (int)((k >> shift) & 255u) : 256 + lane;
                const unsigned peers = __match_any_sync(0xffffffffu, d);
                if (ok && lane == __ffs(peers) - 1) atomicAdd(&sm.hist[d], __popc(peers));
            }
            __syncthreads();
            if (warp == 0) {
                int c[8], sum = 0;
#pragma unroll
                for (int j = 0; j < 8; ++j) c[j] = sm.hist[lane * 8 + j], sum += c[j];
                int inc = sum;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) inc += y;
                }
                const int before = inc - sum;
                if (rank >= before && rank < inc) {  // exactly one lane
                    int r = rank - before, d = lane * 8;
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        if (r < c[j]) {
                            d = lane * 8 + j;
                            break;
                        }
                        r -= c[j];
                    }
                    sm.digit = d;
                    sm.rank = r;
                }
            }
            __syncthreads();
            prefix |= (uint32_t)sm.digit << shift;
            pmask |= 255u << shift;
            rank = sm.rank;
        }
        const uint32_t v = prefix;
        const uint32_t need = (uint32_t)rank;  // keys equal to v that go left
        if (tid == 0)
            t.node[4 * X + 3] = make_float4(__int_as_float(0), __int_as_float(0), key_float(v),
                                            __int_as_float(axis));
        // Stable partition: left = keys below v, then the first `need`
        // keys equal to v.  Packed counts: below v low, equal high.
        uint32_t carry_lt = 0, carry_eq = 0;
        for (int base = s; base < e; base += MID_TILE) {
            const int i0 = base + tid * MID_PPT;
            uint32_t kk[MID_PPT];
            uint32_t sum = 0;
#pragma unroll
            for (int r = 0; r < MID_PPT; ++r) {
                const int i = i0 + r;
                kk[r] = i < e ? keys[i] : 0xffffffffu;
                if (i < e) sum += kk[r] < v ? 1u : (kk[r] == v ? 0x10000u : 0u);
            }
            uint32_t total;
            const uint32_t ex = mid_block_scan(sum, sm.wsum, &sm.tot, &total);
            uint32_t lt = carry_lt + (ex & 0xffffu), eq = carry_eq + (ex >> 16);
#pragma unroll
            for (int r = 0; r < MID_PPT; ++r) {
                const int i = i0 + r;
                if (i >= e) break;
                const uint32_t k = kk[r];
                const bool left = k < v || (k == v && eq < need);
                const uint32_t lb = lt + (eq < need ? eq : need);
                const int dest = left ? s + (int)lb : s + m + (i - s - (int)lb);
                if (dest >= s && dest < e) dst[dest] = src[i];
                else atomicOr(&t.st->err, ERR_SEG);  // cannot happen: the select found rank m
                if (k < v) ++lt;
                else if (k == v) ++eq;
            }
            carry_lt += total & 0xffffu;
            carry_eq += total >> 16;
        }
        __syncthreads();  // the partition is complete before the children are read
        // Children: small ones go to the local builder (from buffer 0),
        // the others stay open.
#pragma unroll 1
        for (int c = 0; c < 2; ++c) {
            const int cs = c == 0 ? s : s + m, ce = c == 0 ? s + m : e;
            if (ce - cs <= LB_SMALL) {
                if (dst != buf0)
                    for (int i = cs + tid; i < ce; i += MID_THREADS) buf0[i] = dst[i];
                if (tid == 0) {
                    const int r = atomicAdd(nlocal, 1);
                    if (r < max_local) local_jobs[r] = make_int4(cs, ce, X * 2 + c, 0);
                    else atomicOr(&t.st->err, ERR_SEG);
                }
            } else if (tid == 0) {
                const int r = atomicAdd(nseg_out, 1);
                if (r < max_segs) segs_out[r] = make_int4(cs, ce, X * 2 + c, 0);
                else atomicOr(&t.st->err, ERR_SEG);
            }
        }
    }
}

template <int MAXN, int THREADS>
void launch_local(unsigned grid, const DevTree& t, const float4* pts, const uint32_t* idx, long long stride, int* loc,
                  const int4* jobs, const int* njobs, int max_jobs, int fill, cudaStream_t s) {
    local_build_kernel<MAXN, THREADS><<<grid, THREADS, sizeof(LbShared<MAXN, THREADS>), s>>>(t, pts, idx, stride, loc,
                                                                                          jobs, njobs, max_jobs, fill);
}

// The local builders' shared memory is above the 48 KB default: opt in once
// per device.  Returns the device's SM count: the block-per-job kernels run
// one block per SM at most, each looping over jobs (idle blocks of 1,024
// threads and 200 KB of shared memory still cost a wave each to launch).
int lb_prepare() {
    static std::atomic<int> sms[64];
    int dev = 0;
    cudaGetDevice(&dev);
    dev &= 63;
    int n = sms[dev].load(std::memory_order_acquire);
    if (n > 0) return n;
    cudaFuncSetAttribute(local_build_kernel<LB_MAX, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(LbShared<LB_MAX, 1024>));
    cudaFuncSetAttribute(local_build_kernel<LB_SMALL, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(LbShared<LB_SMALL, 256>));
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
    sms[dev].store(n, std::memory_order_release);
    return n;
}

__global__ void finish_alloc_kernel(DevStatus* st) {
    st->free_node_n = max(0, st->free_node_n - st->free_node_taken);
    st->free_leaf_n = max(0, st->free_leaf_n - st->free_leaf_taken);
    st->free_node_taken = 0;
    st->free_leaf_taken = 0;
}

__global__ void reset_count_kernel(int* c) { *c = 0; }

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

// Bound on the segments of a level and on the local builders' jobs of one
// call: a level holds at most two segments per node of the level above (each
// node has more than `fill` points); a local job is a whole job or a piece of
// at least 512 points (half of a segment above LB_SMALL or LB_MAX points).
long long max_segs_bound(long long n, int njobs, int fill) {
    long long b = 2 * (n / (fill + 1)) + 2;
    long long j = (long long)njobs + n / 512 + 2;
    return b > j ? b : j;
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
    // The splitter of medium jobs uses none of the sort arrays: its two point
    // buffers (32 n bytes) lie over ord[0 .. 1] and keys[0 .. 1] (>= 48 n bytes).
    bs->mid_pts[0] = (float4*)bs->ord[0];
    bs->mid_pts[1] = (float4*)((char*)bs->ord[0] + align_up(sizeof(float4) * n));
}

void build_subtrees(const DevTree& t, const float4* pts, long long n, const int* job_off, const int* job_link,
                    int njobs, long long max_job, int fill, const BuildScratch& bs, cudaStream_t s) {
    if (njobs <= 0) return;
    const long long sms = lb_prepare();
    const int T = 256;
    long long nn = n > 0 ? n : 1;
    long long ms = max_segs_bound(nn, njobs, fill);
    // Block-per-job grids: the small local builder fits four blocks per SM,
    // the splitter and the large local builder one.
    auto grid = [&](long long jobs, long long per_sm) { return (unsigned)std::min(jobs, per_sm * sms); };
    if (max_job <= LB_SMALL) {
        // Every job fits the small local builder: one launch builds them all.
        init_segs_kernel<<<blocks_for(njobs, T), T, 0, s>>>(job_off, job_link, njobs, bs.segs[0], bs.nseg);
        launch_local<LB_SMALL, 256>(grid(njobs, 4), t, pts, nullptr, 0, nullptr, bs.segs[0], bs.nseg, njobs, fill, s);
        finish_alloc_kernel<<<1, 1, 0, s>>>(t.st);
        return;
    }
    if (max_job <= MID_MAX) {
        // Medium jobs: one launch per level splits every open segment (one
        // block each) until all of them fit the small local builder.
        reset_count_kernel<<<1, 1, 0, s>>>(bs.nseg + 2);
        init_segs_kernel<<<blocks_for(njobs, T), T, 0, s>>>(job_off, job_link, njobs, bs.segs[0], bs.nseg);
        int levels = 0;
        for (long long m = max_job; m > LB_SMALL; m -= m / 2) ++levels;
        long long open = njobs;  // bound on the open segments of a level
        for (int lv = 0; lv < std::max(levels, 1); ++lv) {
            const float4* src = lv == 0 ? pts : ((lv & 1) ? bs.mid_pts[0] : bs.mid_pts[1]);
            float4* dst = (lv & 1) ? bs.mid_pts[1] : bs.mid_pts[0];
            reset_count_kernel<<<1, 1, 0, s>>>(bs.nseg + ((lv + 1) & 1));
            mid_level_kernel<<<grid(std::min(open, ms), 1), MID_THREADS, 0, s>>>(
                t, src, dst, bs.mid_pts[0], (uint32_t*)bs.flag, bs.segs[lv & 1], bs.nseg + (lv & 1),
                bs.segs[(lv + 1) & 1], bs.nseg + ((lv + 1) & 1), (int)ms, bs.local_jobs, bs.nseg + 2, (int)ms, fill);
            open = std::min(2 * open, ms);
        }
        launch_local<LB_SMALL, 256>(grid(ms, 4), t, bs.mid_pts[0], nullptr, 0, nullptr, bs.local_jobs, bs.nseg + 2,
                                    (int)ms, fill, s);
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
    launch_local<LB_MAX, 1024>(grid(ms, 1), t, pts, bs.ord[cur], n, bs.flag, bs.local_jobs, bs.nseg + 2, (int)ms,
                               fill, s);
    finish_alloc_kernel<<<1, 1, 0, s>>>(t.st);
}

}  // namespace ikdg
