// Device bodies of the searches, shared by the per-call kernels (query.cu)
// and the persistent multi-tree batch kernel (batch.cu).
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
#pragma once

#include "kernels.cuh"

namespace ikdg {
namespace search {

constexpr float FINF = __builtin_huge_valf();

// Two consecutive 16-byte slots from a 32-byte-aligned address, one 256-bit
// load (read-only data: the compiler may schedule it freely).
__device__ __forceinline__ void ld_slot_pair(const float4* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
                 : "l"(p));
}

// Slot pairs (256-bit loads) the kNN leaf scan issues together: the default
// for the register lists is two; the per-call kNN picks four when the whole
// batch is resident at once (measured, 1M-point map, k = 5: 100k queries
// 0.155 -> 0.146 ms with four; 1M queries 0.851 -> 0.825 ms with two, 0.896
// with four, whose extra registers cost resident blocks).  The shared-memory
// and row lists take four.
template <int KMAX>
__host__ __device__ constexpr int knn_leaf_pairs() {
    return KMAX > 0 ? 2 : 4;
}

// Leaves a warp scans per step of the range search's leaf phase.
#ifndef IKDG_RANGE_LEAF_BATCH
#define IKDG_RANGE_LEAF_BATCH 4
#endif
constexpr int RANGE_LEAF_BATCH = IKDG_RANGE_LEAF_BATCH;


// Stores n floats (or int bits) from shared memory to dst with the whole warp:
// 16-byte stores where dst is 16-byte aligned, lane-consecutive 4-byte stores
// otherwise.  src is 16-byte aligned shared memory.
__device__ __forceinline__ void warp_store(float* dst, const float* src, int n) {
    const int lane = threadIdx.x & 31;
    int done = 0;
    if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
        const int n4 = n >> 2;
        for (int i = lane; i < n4; i += 32)
            reinterpret_cast<float4*>(dst)[i] = reinterpret_cast<const float4*>(src)[i];
        done = n4 << 2;
    }
    for (int i = done + lane; i < n; i += 32) dst[i] = src[i];
}

// Shared-memory floats per warp for the staged kNN output (k <= kmax).
__host__ __device__ constexpr int knn_stage_floats(int kmax) { return 32 * (5 * kmax + 1); }

__device__ __forceinline__ bool cand_less(float d, int id, float d2, int id2) {
    return d < d2 || (d == d2 && id < id2);
}

// KMAX > 0: the best k candidates live sorted in registers (k <= KMAX).
// KMAX == 0: any k; the sorted candidates live in memory: in kd / ki / ks
// (entry j of the list at index j * kst; shared memory in the per-call
// kernel for k <= KNN_SMEM_MAX), or, when kd is null, in the query's output
// rows with the slot index parked in `slots` (k ints per query).
// Traversal of one query by a group of G consecutive lanes: nearer child
// first, the farther one pushed with its box distance; a subtree is skipped
// when that distance exceeds min(max_dist^2, current k-th distance).  The loop
// is "while-while": a node phase steps every group through nodes until it holds
// a leaf (or is finished), then the warp scans leaves together, so the leaf
// scans run with most lanes active.  The G lanes of a group keep identical
// copies of the traversal state; in a leaf, lane s takes slots s, s+G, ...
// and the G candidates of each round are broadcast and offered to every copy
// in lane order, which keeps the copies identical.
// `tid` is the query (before the optional permutation `perm`) of this
// thread's group; every lane of the warp must call this together.
template <int KMAX, int G, int PAIRS = knn_leaf_pairs<KMAX>()>
__device__ __forceinline__ void knn_body(const DevTree& t, long long tid, const float* __restrict__ q, int q_stride,
                                         long long nq, int k, float max_sq, int* __restrict__ out_id,
                                         float* __restrict__ out_d2, float* __restrict__ out_xyz,
                                         int* __restrict__ out_cnt, int* __restrict__ slots,
                                         const int* __restrict__ perm, float* kd = nullptr, int* ki = nullptr,
                                         int* ks = nullptr, int kst = 1, float* wstage = nullptr) {
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
    const bool in_rows = kd == nullptr;
    float* gd = in_rows ? out_d2 + qi * k : kd;
    int* gi = in_rows ? out_id + qi * k : ki;
    int* gs = in_rows ? (slots != nullptr ? slots + qi * k : nullptr) : ks;
    const int gst = in_rows ? 1 : kst;
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
                while (pos > 0 && cand_less(d, id, gd[(pos - 1) * gst], gi[(pos - 1) * gst])) {
                    gd[pos * gst] = gd[(pos - 1) * gst];
                    gi[pos * gst] = gi[(pos - 1) * gst];
                    gs[pos * gst] = gs[(pos - 1) * gst];
                    --pos;
                }
                gd[pos * gst] = d;
                gi[pos * gst] = id;
                gs[pos * gst] = sl;
            }
            if (gcnt < k) ++gcnt;
            if (gcnt == k) {
                __syncwarp(gmask);
                worst = __shfl_sync(gmask, sub == 0 ? gd[(k - 1) * gst] : 0.f, lane & ~(G - 1));
                worst_id = __shfl_sync(gmask, sub == 0 ? gi[(k - 1) * gst] : 0, lane & ~(G - 1));
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
                const int far = left_first ? cr : cl;
                if (sp < MAX_STACK) {
                    st_code[sp] = far;
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
        if (G == 1) {
            // Two passes.  First every slot's distance is checked against the
            // current bound, marking the slots that can enter the list (no
            // branch: lanes stay converged); then only the marked slots are
            // offered, re-read from L1.  Offering in one pass made the warp run
            // the insertion for every slot at which any lane had a candidate.
            // The final list does not depend on the order of the offers, and
            // the bound only tightens, so the marks miss nothing.
            // Two slots per 256-bit load (slot pairs are 32-byte aligned), and
            // PAIRS loads issued together before any is used.
            // A bucket always has LEAF_CAP slots in the pool, so loads past
            // the fill count stay inside it; their slots are ignored.
            static_assert(LEAF_CAP % (2 * PAIRS) == 0, "a batch of pairs must not leave the bucket");
            static_assert(LEAF_CAP <= 32, "one mark bit per slot");
            uint32_t marks = 0;
            for (int j0 = 0; j0 < n; j0 += 2 * PAIRS) {
                float4 pa[PAIRS], pb[PAIRS];
#pragma unroll
                for (int u = 0; u < PAIRS; ++u) ld_slot_pair(lp + j0 + 2 * u, pa[u], pb[u]);
#pragma unroll
                for (int u = 0; u < PAIRS; ++u) {
                    const int j = j0 + 2 * u;
                    const uint32_t wa = __float_as_uint(pa[u].w);
                    const float da = sq_dist(qx, qy, qz, pa[u].x, pa[u].y, pa[u].z);
                    const bool ma = j < n && !(wa & F_DEL) && da <= max_sq &&
                                    cand_less(da, (int)(wa & ID_MASK), worst, worst_id);
                    const uint32_t wb = __float_as_uint(pb[u].w);
                    const float db = sq_dist(qx, qy, qz, pb[u].x, pb[u].y, pb[u].z);
                    const bool mb = j + 1 < n && !(wb & F_DEL) && db <= max_sq &&
                                    cand_less(db, (int)(wb & ID_MASK), worst, worst_id);
                    marks |= (ma ? 1u : 0u) << j;
                    marks |= (mb ? 1u : 0u) << (j + 1);
                }
            }
            while (marks) {
                const int j = __ffs(marks) - 1;
                marks &= marks - 1;
                const float4 p = __ldg(lp + j);
                const uint32_t w = __float_as_uint(p.w);
                offer(sq_dist(qx, qy, qz, p.x, p.y, p.z), (int)(w & ID_MASK), L * LEAF_CAP + j);
            }
        } else {
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
            {
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
        }
        pop();
    }
    if constexpr (KMAX > 0 && G == 1) {
        if (wstage != nullptr) {
            // The warp's 32 queries are consecutive (no permutation): their
            // rows form one contiguous span of every output array.  Stage the
            // rows in shared memory, then write each span with coalesced,
            // 16-byte stores (the outputs may be host memory over the chip
            // link, where scattered 4-byte stores are slow).
            const long long q0 = tid - lane;
            const int nrows = (int)min(32ll, nq - q0);
            if (nrows <= 0) return;
            float* s_id = wstage;
            float* s_d2 = s_id + 32 * KMAX;
            float* s_xyz = s_d2 + 32 * KMAX;
            float* s_cnt = s_xyz + 96 * KMAX;
            if (valid) {
                int cnt = 0;
#pragma unroll
                for (int j = 0; j < KR; ++j) {
                    if (j < k) {
                        const bool ok = bsl[j] >= 0;
                        const int id = ok ? bi[j] : -1;
                        const float dd = ok ? bd[j] : FINF;
                        s_id[lane * k + j] = __int_as_float(id);
                        s_d2[lane * k + j] = dd;
                        if (out_xyz != nullptr) {
                            const float4 p = ok ? __ldg(P + bsl[j]) : make_float4(0.f, 0.f, 0.f, 0.f);
                            s_xyz[(lane * k + j) * 3 + 0] = p.x;
                            s_xyz[(lane * k + j) * 3 + 1] = p.y;
                            s_xyz[(lane * k + j) * 3 + 2] = p.z;
                        }
                        cnt += ok ? 1 : 0;
                    }
                }
                s_cnt[lane] = __int_as_float(cnt);
            }
            __syncwarp();
            warp_store(reinterpret_cast<float*>(out_id + q0 * k), s_id, nrows * k);
            warp_store(out_d2 + q0 * k, s_d2, nrows * k);
            if (out_xyz != nullptr) warp_store(out_xyz + q0 * k * 3, s_xyz, nrows * k * 3);
            if (out_cnt != nullptr) warp_store(reinterpret_cast<float*>(out_cnt + q0), s_cnt, nrows);
            return;
        }
    }
    if (!valid || sub != 0) return;

    if (KMAX == 0) {
        for (int j = 0; j < k; ++j) {
            const bool ok = j < gcnt;
            const int sl = ok ? gs[j * gst] : -1;
            out_id[qi * k + j] = ok ? gi[j * gst] : -1;
            out_d2[qi * k + j] = ok ? gd[j * gst] : FINF;
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

constexpr int RANGE_COUNT = 0, RANGE_WRITE = 1;

// MODE 0: box, MODE 1: radius.  OUT = RANGE_COUNT counts, RANGE_WRITE emits at
// the query's CSR offset.
// Box (MODE 0) / radius (MODE 1) search of query qi by this thread, with the
// leaves scanned by the whole warp.  Every lane of the warp calls this
// together; lanes without a query pass valid = false.  "While-while": in the
// node phase each thread walks its own query's nodes (a fully covered subtree
// adds its valid count from ncnt when counting, and is enumerated when
// writing) until it holds a leaf; in the leaf phase the warp takes the held
// leaves one at a time, one lane per slot (one 512-byte load per leaf), tests
// the slots against the holder's query and counts them with a ballot.  So a
// query with thousands of hits costs one warp step per leaf instead of one
// thread step per slot, while light queries keep one thread each.
// Returns this lane's hit count.  WRITE emits the hits at ids[o..],
// xyz[3 o..] in traversal order, never at or past o_lim (a hit there raises
// ERR_OUTPUT instead).  radius: one float per query, r_stride floats apart.
template <int MODE, int OUT>
__device__ __forceinline__ long long range_body(const DevTree& t, const float* __restrict__ q, int q_stride,
                                                const float* __restrict__ radius, int r_stride, long long qi,
                                                bool valid, long long o, long long o_lim, int* __restrict__ ids,
                                                float* __restrict__ xyz) {
    constexpr bool WRITE = OUT != RANGE_COUNT;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    // The query in six floats: box {lo, hi}, or radius {centre, r^2, -, -}.
    float qa[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (valid) {
        if (MODE == 0) {
            for (int a = 0; a < 6; ++a) qa[a] = q[qi * q_stride + a];
        } else {
            for (int a = 0; a < 3; ++a) qa[a] = q[qi * q_stride + a];
            const float r = radius[qi * r_stride];
            qa[3] = __fmul_rn(r, r);
        }
    }
    long long count = 0;
    int stack[MAX_STACK];
    int sp = 0;
    int cur = 0;  // item = code * 2 + covered; code 0 is the sentinel record
    bool done = !valid;
    int visits = 0;
    const float4* __restrict__ P = t.pts;
    auto pop = [&]() {
        if (sp > 0)
            cur = stack[--sp];
        else
            done = true;
    };

    while (true) {
        // Node phase.
        while (true) {
            const bool nodework = !done && (cur >> 1) >= 0;
            if (!__any_sync(0xffffffffu, nodework)) break;
            if (!nodework) continue;
            if (++visits > MAX_VISITS) {
                atomicOr(&t.st->err, ERR_LOOP);
                done = true;
                continue;
            }
            const int X = cur >> 1;
            const bool covered = cur & 1;
            const NodeRec r = load_node(t.node, X);
            const int4 c4 = WRITE ? make_int4(0, 0, 0, 0) : __ldg(t.ncnt + X);
            int next = 0;
            bool have_next = false;
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const int c = side == 0 ? r.left() : r.right();
                if (c == 0) continue;
                const Box3 b = r.box(side);
                if (box_empty(b)) continue;
                bool cov = covered;
                if (!cov) {
                    if (MODE == 0) {
                        Box3 qb;
                        for (int a = 0; a < 3; ++a) {
                            qb.lo[a] = qa[a];
                            qb.hi[a] = qa[3 + a];
                        }
                        if (qbox_disjoint(qb, b)) continue;
                        cov = qbox_covers(qb, b);
                    } else {
                        if (box_dist(qa[0], qa[1], qa[2], b.lo[0], b.lo[1], b.lo[2], b.hi[0], b.hi[1], b.hi[2]) >
                            qa[3])
                            continue;
                        cov = box_far(qa[0], qa[1], qa[2], b.lo[0], b.lo[1], b.lo[2], b.hi[0], b.hi[1], b.hi[2]) <=
                              qa[3];
                    }
                }
                if (cov && !WRITE) {
                    count += side == 0 ? (c4.x - c4.y) : (c4.z - c4.w);
                    continue;
                }
                const int it = c * 2 + (cov ? 1 : 0);
                if (!have_next) {
                    next = it;
                    have_next = true;
                } else if (sp < MAX_STACK) {
                    stack[sp++] = it;
                } else {
                    atomicOr(&t.st->err, ERR_STACK);
                }
            }
            if (have_next)
                cur = next;
            else
                pop();
        }
        // Leaf phase: the held leaves, RANGE_LEAF_BATCH at a time, one lane per
        // slot.  A bucket always has LEAF_CAP slots in the pool, so each slot
        // load is issued together with the leaf's fill count.
        const bool leafwork = !done && (cur >> 1) < 0;
        unsigned lb = __ballot_sync(0xffffffffu, leafwork);
        if (lb == 0) break;
        while (lb) {
            int src[RANGE_LEAF_BATCH];
#pragma unroll
            for (int u = 0; u < RANGE_LEAF_BATCH; ++u) {
                src[u] = lb ? __ffs(lb) - 1 : -1;
                lb &= lb - 1;
            }
            float4 p[RANGE_LEAF_BATCH];
            int nl[RANGE_LEAF_BATCH], it[RANGE_LEAF_BATCH];
#pragma unroll
            for (int u = 0; u < RANGE_LEAF_BATCH; ++u) {
                if (src[u] < 0) break;
                it[u] = __shfl_sync(0xffffffffu, cur, src[u]);
                const int L = code_leaf(it[u] >> 1);
                p[u] = __ldg(P + (long long)L * LEAF_CAP + lane);
                nl[u] = __ldg(t.leaf_n + L);
            }
#pragma unroll
            for (int u = 0; u < RANGE_LEAF_BATCH; ++u) {
                if (src[u] < 0) break;
                float h[6];
#pragma unroll
                for (int a = 0; a < 6; ++a) h[a] = __shfl_sync(0xffffffffu, qa[a], src[u]);
                bool hit = false;
                if (lane < nl[u] && !(__float_as_uint(p[u].w) & F_DEL)) {
                    if (it[u] & 1) {
                        hit = true;
                    } else if (MODE == 0) {
                        hit = p[u].x >= h[0] && p[u].x < h[3] && p[u].y >= h[1] && p[u].y < h[4] &&
                              p[u].z >= h[2] && p[u].z < h[5];
                    } else {
                        hit = sq_dist(p[u].x, p[u].y, p[u].z, h[0], h[1], h[2]) <= h[3];
                    }
                }
                const unsigned hb = __ballot_sync(0xffffffffu, hit);
                if (OUT == RANGE_WRITE) {
                    const long long base = __shfl_sync(0xffffffffu, o + count, src[u]);
                    const long long lim = __shfl_sync(0xffffffffu, o_lim, src[u]);
                    if (hit) {
                        const long long pos = base + __popc(hb & lt);
                        if (pos < lim) {
                            ids[pos] = (int)(__float_as_uint(p[u].w) & ID_MASK);
                            if (xyz != nullptr) {
                                xyz[pos * 3 + 0] = p[u].x;
                                xyz[pos * 3 + 1] = p[u].y;
                                xyz[pos * 3 + 2] = p[u].z;
                            }
                        } else {
                            atomicOr(&t.st->err, ERR_OUTPUT);
                        }
                    }
                }
                if (lane == src[u]) count += __popc(hb);
            }
        }
        if (leafwork) pop();
    }
    return count;
}

}  // namespace search
}  // namespace ikdg
