// Batched searches: Nearest_Search, Box_Search, Radius_Search.
//
// Semantics (the drop-in contract):
//   * kNN (Nearest_Search / Search, ikd-Tree/ikd_Tree.cpp:366-397, :868-1013):
//     the k valid points with the smallest squared distance, among those with
//     sq_dist <= max_dist^2, ascending.  Ties at equal distance are broken by
//     the smaller point id (the reference leaves them to traversal order).  A
//     subtree is skipped only when its AABB lower bound exceeds the current
//     k-th distance or max_dist^2, so the result is exact.
//   * Box_Search (:399-404, :1015-1044): every valid p with min <= p < max.
//   * Radius_Search (:406-411, :1046-1087): every valid p with
//     sq_dist(p, q) <= r*r in float.  Whole subtrees are taken when their
//     farthest corner is inside (an exact float bound), so no point at the
//     boundary is admitted or lost by rounding.
#include <cuda_runtime.h>

#include <mutex>

#include "kernels.cuh"

namespace ikdg {
namespace {

constexpr float FINF = __builtin_huge_valf();

__device__ __forceinline__ bool cand_less(float d, int id, float d2, int id2) {
    return d < d2 || (d == d2 && id < id2);
}

// KMAX > 0: the best k candidates live sorted in registers (k <= KMAX).
// KMAX == 0: any k; the sorted candidates live in the query's output rows
// (global memory), with the slot index parked in out_cnt-independent scratch
// `slots` (k ints per query).
// Traversal of one query by a group of G consecutive lanes: nearer child
// first, the farther one pushed with its box distance; a subtree is skipped
// when that distance exceeds min(max_dist^2, current k-th distance).  The loop
// is "while-while": a node phase steps every group through nodes until it holds
// a leaf (or is finished), then the warp scans leaves together, so the leaf
// scans run with most lanes active.  The G lanes of a group keep identical
// copies of the traversal state; in a leaf, lane s takes slots s, s+G, ...
// and the G candidates of each round are broadcast and offered to every copy
// in lane order, which keeps the copies identical.
template <int KMAX, int G>
__global__ void __launch_bounds__(128) knn_kernel(DevTree t, const float* __restrict__ q, int q_stride,
                                                  long long nq, int k, float max_sq, int* __restrict__ out_id,
                                                  float* __restrict__ out_d2, float* __restrict__ out_xyz,
                                                  int* __restrict__ out_cnt, int* __restrict__ slots,
                                                  const int* __restrict__ perm) {
    const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long tid = gtid / G;
    const int sub = threadIdx.x & (G - 1);
    const int lane = threadIdx.x & 31;
    const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
    const bool valid = tid < nq;
    long long qi = valid ? tid : 0;
    if (valid && perm != nullptr) qi = __ldg(perm + tid);
    const float qx = valid ? q[qi * q_stride + 0] : 0.f;
    const float qy = valid ? q[qi * q_stride + 1] : 0.f;
    const float qz = valid ? q[qi * q_stride + 2] : 0.f;

    constexpr int KR = KMAX > 0 ? KMAX : 1;
    float bd[KR];
    int bi[KR], bsl[KR];
#pragma unroll
    for (int j = 0; j < KR; ++j) {
        bd[j] = FINF;
        bi[j] = 0x7fffffff;
        bsl[j] = -1;
    }
    float* gd = out_d2 + qi * k;
    int* gi = out_id + qi * k;
    int* gs = slots != nullptr ? slots + qi * k : nullptr;
    int gcnt = 0;
    float worst = FINF;
    int worst_id = 0x7fffffff;

    int st_code[MAX_STACK];
    float st_d[MAX_STACK];
    int sp = 0;
    int cur = 0;  // node code (>= 0; 0 = the sentinel record) or leaf code (< 0)
    bool done = !valid;
    int visits = 0;
    const float4* __restrict__ P = t.pts;

    // Next stacked subtree that can still hold a result, or done.
    auto pop = [&]() {
        const float lim = fminf(max_sq, worst);
        while (sp > 0) {
            --sp;
            if (st_d[sp] <= lim) {
                cur = st_code[sp];
                return;
            }
        }
        done = true;
    };

    // Offers a candidate to this lane's copy of the k best.
    auto offer = [&](float d, int id, int sl) {
        if (!(d <= max_sq && cand_less(d, id, worst, worst_id))) return;
        if (KMAX == 0) {
            // Large k: the sorted list lives in the output rows; only the
            // group's first lane owns them.
            if (sub == 0) {
                int pos = gcnt < k ? gcnt : k - 1;
                while (pos > 0 && cand_less(d, id, gd[pos - 1], gi[pos - 1])) {
                    gd[pos] = gd[pos - 1];
                    gi[pos] = gi[pos - 1];
                    gs[pos] = gs[pos - 1];
                    --pos;
                }
                gd[pos] = d;
                gi[pos] = id;
                gs[pos] = sl;
            }
            if (gcnt < k) ++gcnt;
            if (gcnt == k) {
                __syncwarp(gmask);
                worst = __shfl_sync(gmask, sub == 0 ? gd[k - 1] : 0.f, lane & ~(G - 1));
                worst_id = __shfl_sync(gmask, sub == 0 ? gi[k - 1] : 0, lane & ~(G - 1));
            }
            return;
        }
        float cd = d;
        int cid = id, cs = sl;
#pragma unroll
        for (int m = 0; m < KR; ++m) {
            const bool sw = cand_less(cd, cid, bd[m], bi[m]);
            const float td = bd[m];
            const int ti = bi[m], ts = bsl[m];
            bd[m] = sw ? cd : td;
            bi[m] = sw ? cid : ti;
            bsl[m] = sw ? cs : ts;
            cd = sw ? td : cd;
            cid = sw ? ti : cid;
            cs = sw ? ts : cs;
        }
#pragma unroll
        for (int m = 0; m < KR; ++m)
            if (m == k - 1) {
                worst = bd[m];
                worst_id = bi[m];
            }
    };

    while (true) {
        // Node phase.
        while (true) {
            const bool nodework = !done && cur >= 0;
            if (!__any_sync(0xffffffffu, nodework)) break;
            if (!nodework) continue;
            if (++visits > MAX_VISITS) {
                atomicOr(&t.st->err, ERR_LOOP);
                done = true;
                continue;
            }
            NodeRec r = load_node(t.node, cur);
            const int cl = r.left(), cr = r.right();
            const float lim = fminf(max_sq, worst);
            float dl = FINF, dr = FINF;
            bool vl = false, vr = false;
            if (cl != 0 && r.f0.x <= r.f0.w) {
                dl = box_dist(qx, qy, qz, r.f0.x, r.f0.y, r.f0.z, r.f0.w, r.f1.x, r.f1.y);
                vl = dl <= lim;
            }
            if (cr != 0 && r.f1.z <= r.f2.y) {
                dr = box_dist(qx, qy, qz, r.f1.z, r.f1.w, r.f2.x, r.f2.y, r.f2.z, r.f2.w);
                vr = dr <= lim;
            }
            if (vl && vr) {
                const bool left_first = dl <= dr;
                if (sp < MAX_STACK) {
                    st_code[sp] = left_first ? cr : cl;
                    st_d[sp] = left_first ? dr : dl;
                    ++sp;
                } else {
                    atomicOr(&t.st->err, ERR_STACK);
                }
                cur = left_first ? cl : cr;
            } else if (vl) {
                cur = cl;
            } else if (vr) {
                cur = cr;
            } else {
                pop();
            }
        }
        // Leaf phase.
        const bool leafwork = !done && cur < 0;
        if (!__any_sync(0xffffffffu, leafwork)) break;
        if (!leafwork) continue;
        const int L = code_leaf(cur);
        const int n = min(__ldg(t.leaf_n + L), LEAF_CAP);
        const float4* lp = P + (long long)L * LEAF_CAP;
        for (int j0 = 0; j0 < n; j0 += G) {
            const int j = j0 + sub;
            float d = FINF;
            int id = 0x7fffffff, sl = -1;
            if (j < n) {
                const float4 p = __ldg(lp + j);
                const uint32_t w = __float_as_uint(p.w);
                if (!(w & F_DEL)) {
                    d = sq_dist(qx, qy, qz, p.x, p.y, p.z);
                    id = (int)(w & ID_MASK);
                    sl = L * LEAF_CAP + j;
                }
            }
            if (G == 1) {
                if (sl >= 0) offer(d, id, sl);
            } else {
#pragma unroll
                for (int s = 0; s < G; ++s) {
                    const int src = (lane & ~(G - 1)) + s;
                    const float ds = __shfl_sync(gmask, d, src);
                    const int is = __shfl_sync(gmask, id, src);
                    const int ss = __shfl_sync(gmask, sl, src);
                    if (ss >= 0) offer(ds, is, ss);
                }
            }
        }
        pop();
    }
    if (!valid || sub != 0) return;

    if (KMAX == 0) {
        for (int j = 0; j < k; ++j) {
            const bool ok = j < gcnt;
            const int sl = ok ? gs[j] : -1;
            if (!ok) {
                gi[j] = -1;
                gd[j] = FINF;
            }
            if (out_xyz != nullptr) {
                float4 p = ok ? __ldg(P + sl) : make_float4(0.f, 0.f, 0.f, 0.f);
                out_xyz[(qi * k + j) * 3 + 0] = p.x;
                out_xyz[(qi * k + j) * 3 + 1] = p.y;
                out_xyz[(qi * k + j) * 3 + 2] = p.z;
            }
        }
        if (out_cnt != nullptr) out_cnt[qi] = gcnt;
        return;
    }
    int cnt = 0;
#pragma unroll
    for (int j = 0; j < KR; ++j) {
        if (j < k) {
            const bool ok = bsl[j] >= 0;
            out_id[qi * k + j] = ok ? bi[j] : -1;
            out_d2[qi * k + j] = ok ? bd[j] : FINF;
            if (out_xyz != nullptr) {
                float4 p = ok ? __ldg(P + bsl[j]) : make_float4(0.f, 0.f, 0.f, 0.f);
                out_xyz[(qi * k + j) * 3 + 0] = p.x;
                out_xyz[(qi * k + j) * 3 + 1] = p.y;
                out_xyz[(qi * k + j) * 3 + 2] = p.z;
            }
            cnt += ok ? 1 : 0;
        }
    }
    if (out_cnt != nullptr) out_cnt[qi] = cnt;
}

// MODE 0: box, MODE 1: radius.  WRITE = false counts, true emits.
template <int MODE, bool WRITE>
__global__ void __launch_bounds__(128) range_kernel(DevTree t, const float* __restrict__ q, int q_stride,
                                                    const float* __restrict__ radius, long long nq,
                                                    long long* __restrict__ counts,
                                                    const long long* __restrict__ offsets, int* __restrict__ ids,
                                                    float* __restrict__ xyz) {
    long long qi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    Box3 qb;
    float cx = 0.f, cy = 0.f, cz = 0.f, r2 = 0.f;
    if (MODE == 0) {
        for (int a = 0; a < 3; ++a) {
            qb.lo[a] = q[qi * q_stride + a];
            qb.hi[a] = q[qi * q_stride + 3 + a];
        }
    } else {
        cx = q[qi * q_stride + 0];
        cy = q[qi * q_stride + 1];
        cz = q[qi * q_stride + 2];
        const float r = radius[qi];
        r2 = __fmul_rn(r, r);
    }
    long long count = 0;
    long long o = WRITE ? offsets[qi] : 0;
    int stack[MAX_STACK];
    int sp = 0;
    int cur = 0;        // code; the sentinel record first
    bool covered = false;
    bool is_start = true;
    const float4* __restrict__ P = t.pts;
    int visits = 0;
    while (true) {
        if (++visits > MAX_VISITS) {
            atomicOr(&t.st->err, ERR_LOOP);
            break;
        }
        if (is_start || cur > 0) {
            const int X = is_start ? 0 : cur;
            is_start = false;
            NodeRec r = load_node(t.node, X);
            int4 c4 = WRITE ? make_int4(0, 0, 0, 0) : __ldg(t.ncnt + X);
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const int c = side == 0 ? r.left() : r.right();
                if (c == 0) continue;
                const Box3 b = r.box(side);
                if (box_empty(b)) continue;
                bool cov = covered;
                if (!cov) {
                    if (MODE == 0) {
                        if (qbox_disjoint(qb, b)) continue;
                        cov = qbox_covers(qb, b);
                    } else {
                        if (box_dist(cx, cy, cz, b.lo[0], b.lo[1], b.lo[2], b.hi[0], b.hi[1], b.hi[2]) > r2) continue;
                        cov = box_far(cx, cy, cz, b.lo[0], b.lo[1], b.lo[2], b.hi[0], b.hi[1], b.hi[2]) <= r2;
                    }
                }
                if (cov && !WRITE) {
                    count += side == 0 ? (c4.x - c4.y) : (c4.z - c4.w);
                    continue;
                }
                if (sp < MAX_STACK) {
                    stack[sp++] = c * 2 + (cov ? 1 : 0);
                } else {
                    atomicOr(&t.st->err, ERR_STACK);
                }
            }
        } else {
            const int L = code_leaf(cur);
            const int n = min(__ldg(t.leaf_n + L), LEAF_CAP);
            const float4* lp = P + (long long)L * LEAF_CAP;
            for (int j = 0; j < n; ++j) {
                const float4 p = __ldg(lp + j);
                const uint32_t w = __float_as_uint(p.w);
                if (w & F_DEL) continue;
                bool in = covered;
                if (!in) {
                    if (MODE == 0)
                        in = qbox_holds(qb, p.x, p.y, p.z);
                    else
                        in = sq_dist(p.x, p.y, p.z, cx, cy, cz) <= r2;
                }
                if (!in) continue;
                if (WRITE) {
                    ids[o] = (int)(w & ID_MASK);
                    if (xyz != nullptr) {
                        xyz[o * 3 + 0] = p.x;
                        xyz[o * 3 + 1] = p.y;
                        xyz[o * 3 + 2] = p.z;
                    }
                    ++o;
                }
                ++count;
            }
        }
        if (sp == 0) break;
        const int item = stack[--sp];
        cur = item >> 1;
        covered = item & 1;
    }
    if (!WRITE) counts[qi] = count;
}

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

template <int KMAX>
void knn_launch(const DevTree& t, const float* q, int q_stride, long long nq, int k, float max_sq, int* out_id,
                float* out_d2, float* out_xyz, int* out_cnt, int* slots, const int* perm, int lanes, cudaStream_t s) {
    if (lanes >= 4)
        knn_kernel<KMAX, 4><<<blocks_for(nq * 4, 128), 128, 0, s>>>(t, q, q_stride, nq, k, max_sq, out_id, out_d2,
                                                                    out_xyz, out_cnt, slots, perm);
    else if (lanes == 2)
        knn_kernel<KMAX, 2><<<blocks_for(nq * 2, 128), 128, 0, s>>>(t, q, q_stride, nq, k, max_sq, out_id, out_d2,
                                                                    out_xyz, out_cnt, slots, perm);
    else
        knn_kernel<KMAX, 1><<<blocks_for(nq, 128), 128, 0, s>>>(t, q, q_stride, nq, k, max_sq, out_id, out_d2,
                                                                out_xyz, out_cnt, slots, perm);
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
    if (k > KNN_REG_MAX) b += sizeof(int) * nq * k + 256;
    return b;
}

void launch_knn(const DevTree& t, const float* q, int q_stride, long long nq, int k, float max_sq, int* out_id,
                float* out_d2, float* out_xyz, int* out_cnt, void* temp, int lanes, int bin_bits, cudaStream_t s) {
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
    int* slots = k > KNN_REG_MAX ? (int*)tp : nullptr;
#define IKDG_KNN(KM) \
    knn_launch<KM>(t, q, q_stride, nq, k, max_sq, out_id, out_d2, out_xyz, out_cnt, slots, perm, lanes, s)
    if (k > KNN_REG_MAX)
        IKDG_KNN(0);
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
    else if (k <= 32)
        IKDG_KNN(32);
    else
        IKDG_KNN(64);
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

void launch_range(const DevTree& t, int mode, const float* q, int q_stride, const float* radius, long long nq,
                  long long* counts, const long long* offsets, int* ids, float* xyz, cudaStream_t s) {
    if (nq <= 0) return;
    unsigned g = blocks_for(nq, 128);
    if (mode == 0) {
        if (ids == nullptr)
            range_kernel<0, false><<<g, 128, 0, s>>>(t, q, q_stride, radius, nq, counts, offsets, ids, xyz);
        else
            range_kernel<0, true><<<g, 128, 0, s>>>(t, q, q_stride, radius, nq, counts, offsets, ids, xyz);
    } else {
        if (ids == nullptr)
            range_kernel<1, false><<<g, 128, 0, s>>>(t, q, q_stride, radius, nq, counts, offsets, ids, xyz);
        else
            range_kernel<1, true><<<g, 128, 0, s>>>(t, q, q_stride, radius, nq, counts, offsets, ids, xyz);
    }
}

}  // namespace ikdg
