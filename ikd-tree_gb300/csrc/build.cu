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

constexpr int LB_MAX_GLOBAL = 1024;  // = LB_MAX: segments this small go to the local builder

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
    if (cnt <= LB_MAX_GLOBAL) {
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
        if (b == 0) {
            segpos_next[i] = -1;
            ord_next[i] = ord[i];  // keeps the local builder's index array whole
        }
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
// One block builds a whole subtree of up to LB_MAX points in shared memory.
// Per level: every open segment's AABB by shared atomics on order-preserving
// keys, the longest axis, then one bitonic sort of (segment start, coordinate
// on the segment's axis, position) over the block's points, which sorts every
// segment along its own axis in place; the median split is at the segment's
// middle.  seg_of[i] names the open segment holding position i (-1 once the
// point sits in a leaf).  With leaves of at most `fill` >= 8 points an open
// segment holds >= 9 points, so a level never has more than
// 2 * LB_MAX / 9 < LB_SEGS open segments.
constexpr int LB_MAX = 1024;
constexpr int LB_THREADS = 256;
constexpr int LB_SEGS = 256;
static_assert(2 * LB_MAX / 9 < LB_SEGS, "segment table too small");

__device__ __forceinline__ float key_float(uint32_t k) {
    uint32_t u = (k & 0x80000000u) ? (k ^ 0x80000000u) : ~k;
    return __uint_as_float(u);
}

__global__ void __launch_bounds__(LB_THREADS) local_build_kernel(DevTree t, const float4* __restrict__ pts,
                                                                 const uint32_t* __restrict__ idx,
                                                                 const int4* __restrict__ jobs, const int* njobs,
                                                                 int fill) {
    __shared__ float4 P[LB_MAX];
    __shared__ unsigned long long K[LB_MAX];
    __shared__ short seg_of[LB_MAX];
    __shared__ int seg_s[LB_SEGS], seg_e[LB_SEGS], seg_link[LB_SEGS], seg_axis[LB_SEGS], seg_node[LB_SEGS];
    __shared__ uint32_t bx[LB_SEGS][6];
    __shared__ int nseg;
    int* next_pos = reinterpret_cast<int*>(&bx[0][0]);  // reuses the dead box keys
    const int tid = threadIdx.x;
    const int nj = *njobs;
    for (int job = blockIdx.x; job < nj; job += gridDim.x) {
        const int4 jb = jobs[job];
        const int n = jb.y - jb.x;
        if (n > LB_MAX || fill < 8) {  // cannot happen: the host guarantees both
            if (tid == 0) atomicOr(&t.st->err, ERR_SEG);
            continue;
        }
        for (int i = tid; i < n; i += LB_THREADS) {
            const long long src = idx != nullptr ? (long long)idx[jb.x + i] : (long long)jb.x + i;
            P[i] = pts[src];
            seg_of[i] = 0;
        }
        if (tid == 0) {
            nseg = 1;
            seg_s[0] = 0;
            seg_e[0] = n;
            seg_link[0] = jb.z;
        }
        __syncthreads();
        int size = 1;
        while (size < n) size <<= 1;
        for (int level = 0; level < 64; ++level) {
            const int S = nseg;
            if (tid < S) {
                bx[tid][0] = bx[tid][1] = bx[tid][2] = 0xffffffffu;
                bx[tid][3] = bx[tid][4] = bx[tid][5] = 0u;
            }
            __syncthreads();
            for (int i = tid; i < n; i += LB_THREADS) {
                const int sg = seg_of[i];
                if (sg < 0) continue;
                const float4 p = P[i];
                atomicMin(&bx[sg][0], float_key(p.x));
                atomicMin(&bx[sg][1], float_key(p.y));
                atomicMin(&bx[sg][2], float_key(p.z));
                atomicMax(&bx[sg][3], float_key(p.x));
                atomicMax(&bx[sg][4], float_key(p.y));
                atomicMax(&bx[sg][5], float_key(p.z));
            }
            __syncthreads();
            // One thread per open segment: a leaf, or a node with its axis.
            if (tid < S) {
                const int sg = tid;
                const int s = seg_s[sg], e = seg_e[sg], link = seg_link[sg];
                const int cnt = e - s;
                const int parent = link >> 1, side = link & 1;
                Box3 b = empty_box();
                if (cnt > 0)
                    for (int a = 0; a < 3; ++a) {
                        b.lo[a] = key_float(bx[sg][a]);
                        b.hi[a] = key_float(bx[sg][3 + a]);
                    }
                seg_axis[sg] = -1;
                seg_node[sg] = -1;
                if (cnt <= fill) {
                    const int L = alloc_leaf(t);
                    seg_node[sg] = L;
                    if (L >= 0) {
                        t.leaf_n[L] = cnt;
                        t.lparent[L] = link;
                        write_child_box(t.node, parent, side, b);
                        write_child_code(t.node, parent, side, leaf_code(L));
                        write_child_cnt(t.ncnt, parent, side, cnt, 0);
                    }
                } else {
                    const int X = alloc_node(t);
                    seg_node[sg] = X;
                    if (X >= 0) {
                        float ext[3];
                        for (int a = 0; a < 3; ++a) ext[a] = __fsub_rn(b.hi[a], b.lo[a]);
                        int axis = 0;
                        if (ext[1] > ext[axis]) axis = 1;
                        if (ext[2] > ext[axis]) axis = 2;
                        seg_axis[sg] = axis;
                        t.nparent[X] = link;
                        int h = 0;
                        for (int m = cnt; m > fill; m -= m / 2) ++h;
                        t.nheight[X] = h;
                        write_child_box(t.node, parent, side, b);
                        write_child_code(t.node, parent, side, X);
                        write_child_cnt(t.ncnt, parent, side, cnt, 0);
                    }
                }
            }
            __syncthreads();
            // Leaves take their points; open points get sort keys.
            for (int i = tid; i < size; i += LB_THREADS) {
                if (i >= n) {
                    K[i] = ~0ull;
                    continue;
                }
                const int sg = seg_of[i];
                uint32_t ck = 0;
                unsigned long long seg_key = 0;
                if (sg >= 0) {
                    const float4 p = P[i];
                    const int axis = seg_axis[sg];
                    seg_key = (unsigned long long)seg_s[sg];
                    if (axis < 0) {
                        const int L = seg_node[sg];
                        if (L >= 0) {
                            float4 q = p;
                            q.w = __uint_as_float(__float_as_uint(p.w) & ID_MASK);
                            t.pts[(long long)L * LEAF_CAP + (i - seg_s[sg])] = q;
                        }
                    } else {
                        ck = float_key(axis == 0 ? p.x : (axis == 1 ? p.y : p.z));
                    }
                } else {
                    seg_key = (unsigned long long)i;  // done points keep their place
                }
                K[i] = (seg_key << 43) | ((unsigned long long)ck << 11) | (unsigned long long)i;
            }
            __syncthreads();
            // Bitonic sort of K[0 .. size).
            for (int kk = 2; kk <= size; kk <<= 1) {
                for (int j = kk >> 1; j > 0; j >>= 1) {
                    for (int i = tid; i < size; i += LB_THREADS) {
                        const int ixj = i ^ j;
                        if (ixj > i) {
                            const unsigned long long a = K[i], c = K[ixj];
                            if ((a > c) == ((i & kk) == 0)) {
                                K[i] = c;
                                K[ixj] = a;
                            }
                        }
                    }
                    __syncthreads();
                }
            }
            // Permute the points into sorted order.
            float4 tmp[LB_MAX / LB_THREADS];
#pragma unroll
            for (int r = 0; r < LB_MAX / LB_THREADS; ++r) {
                const int i = tid + r * LB_THREADS;
                if (i < n) tmp[r] = P[K[i] & 2047ull];
            }
            __syncthreads();
#pragma unroll
            for (int r = 0; r < LB_MAX / LB_THREADS; ++r) {
                const int i = tid + r * LB_THREADS;
                if (i < n) P[i] = tmp[r];
            }
            // Positions of the next level's open segments (two per node).
            if (tid == 0) {
                int acc = 0;
                for (int sg = 0; sg < S; ++sg) {
                    next_pos[sg] = acc;
                    acc += (seg_axis[sg] >= 0 && seg_node[sg] >= 0) ? 2 : 0;
                }
                next_pos[S] = acc;
            }
            __syncthreads();
            const int S2 = next_pos[S];
            // Split: the node's split value, the children's ranges, seg_of.
            int ns = 0, ne = 0, nmid = 0, nX = -1, npos = -1;
            if (tid < S && seg_axis[tid] >= 0 && seg_node[tid] >= 0) {
                ns = seg_s[tid];
                ne = seg_e[tid];
                nX = seg_node[tid];
                nmid = ns + (ne - ns) / 2;
                const int axis = seg_axis[tid];
                const float4 pm = P[nmid];
                t.node[4 * nX + 3] = make_float4(__int_as_float(0), __int_as_float(0),
                                                 axis == 0 ? pm.x : (axis == 1 ? pm.y : pm.z), __int_as_float(axis));
                npos = next_pos[tid];
            }
            for (int i = tid; i < n; i += LB_THREADS) {
                const int sg = seg_of[i];
                if (sg < 0) continue;
                if (seg_axis[sg] < 0 || seg_node[sg] < 0) {
                    seg_of[i] = -1;
                } else {
                    const int mid = seg_s[sg] + (seg_e[sg] - seg_s[sg]) / 2;
                    seg_of[i] = (short)(next_pos[sg] + (i < mid ? 0 : 1));
                }
            }
            __syncthreads();
            if (S2 == 0 || S2 > LB_SEGS) {
                if (S2 > LB_SEGS && tid == 0) atomicOr(&t.st->err, ERR_SEG);
                break;
            }
            if (npos >= 0) {
                seg_s[npos] = ns;
                seg_e[npos] = nmid;
                seg_link[npos] = nX * 2;
                seg_s[npos + 1] = nmid;
                seg_e[npos + 1] = ne;
                seg_link[npos + 1] = nX * 2 + 1;
            }
            if (tid == 0) nseg = S2;
            __syncthreads();
        }
        __syncthreads();
    }
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
    const int T = 256;
    long long nn = n > 0 ? n : 1;
    long long ms = max_segs_bound(nn, njobs, fill);
    const unsigned lb_grid = (unsigned)(njobs < 4096 ? njobs : 4096);
    if (max_job <= LB_MAX) {
        // Every job fits one block: a single launch builds them all.
        init_segs_kernel<<<blocks_for(njobs, T), T, 0, s>>>(job_off, job_link, njobs, bs.segs[0], bs.nseg);
        local_build_kernel<<<lb_grid, LB_THREADS, 0, s>>>(t, pts, nullptr, bs.segs[0], bs.nseg, fill);
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
    // The axis-0 index array of the last level holds every local segment.
    unsigned g = (unsigned)(ms < 4096 ? ms : 4096);
    local_build_kernel<<<g, LB_THREADS, 0, s>>>(t, pts, bs.ord[cur], bs.local_jobs, bs.nseg + 2, fill);
    finish_alloc_kernel<<<1, 1, 0, s>>>(t.st);
}

}  // namespace ikdg
