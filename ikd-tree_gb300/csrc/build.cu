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

#include "kernels.cuh"

namespace ikdg {
namespace {

constexpr int KIND_LEAF = 0;
constexpr int KIND_NODE = 1;

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
                                 int fill, int max_next) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *nseg_cur) return;
    int4 sg = segs[i];
    int s = sg.x, e = sg.y, link = sg.z;
    int cnt = e - s;
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
    b += 3 * align_up(sizeof(int4) * ms);          // segs x2, seginfo
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
    bs->nseg = (int*)take(sizeof(int) * 4);
    bs->temp = (void*)p;
}

void build_subtrees(const DevTree& t, const float4* pts, long long n, const int* job_off, const int* job_link,
                    int njobs, long long max_job, int fill, const BuildScratch& bs, cudaStream_t s) {
    if (njobs <= 0) return;
    const int T = 256;
    long long nn = n > 0 ? n : 1;
    if (n > 0) {
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
    }
    init_segs_kernel<<<blocks_for(njobs, T), T, 0, s>>>(job_off, job_link, njobs, bs.segs[0], bs.nseg);
    long long ms = max_segs_bound(nn, njobs, fill);
    int levels = build_levels(max_job, fill);
    int cur = 0;
    long long seg_bound = njobs;
    for (int lv = 0; lv < levels; ++lv) {
        int nxt = cur ^ 1;
        reset_count_kernel<<<1, 1, 0, s>>>(bs.nseg + nxt);
        level_seg_kernel<<<blocks_for(seg_bound, 128), 128, 0, s>>>(t, pts, bs.ord[cur], nn, bs.segs[cur],
                                                                    bs.nseg + cur, bs.segs[nxt], bs.nseg + nxt,
                                                                    bs.seginfo, fill, (int)ms);
        if (n > 0) {
            level_pos_kernel<<<blocks_for(n, T), T, 0, s>>>(t, pts, bs.ord[cur], n, bs.segpos[cur], bs.seginfo,
                                                            bs.flag);
            if (lv + 1 < levels) {
                level_scanin_kernel<<<dim3(blocks_for(n, T), 3), T, 0, s>>>(bs.ord[cur], n, bs.segpos[cur],
                                                                           bs.seginfo, bs.flag, bs.scan_in);
                exclusive_scan(bs.scan_in, bs.scan_out, 3 * n, nullptr, bs.temp, s);
                level_scatter_kernel<<<dim3(blocks_for(n, T), 3), T, 0, s>>>(
                    bs.ord[cur], bs.ord[nxt], n, bs.segpos[cur], bs.segpos[nxt], bs.segs[cur], bs.seginfo,
                    bs.flag, bs.scan_out);
            }
        }
        long long nb = seg_bound * 2;
        seg_bound = nb < ms ? nb : ms;
        cur = nxt;
    }
    finish_alloc_kernel<<<1, 1, 0, s>>>(t.st);
}

}  // namespace ikdg
