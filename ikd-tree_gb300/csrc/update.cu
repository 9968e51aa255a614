// Mutations of the device tree: point insertion, box / point deletion, box
// re-insertion, bottom-up refit with the rebalancing criteria, rebuild-job
// collection, and the exact voxel downsampling of Add_Points.
//
// Reference behaviour replaced here:
//   Add_by_point (ikd-Tree/ikd_Tree.cpp:817-866): descend by `p[axis] < split`
//     to a leaf bucket and append; a full bucket becomes a rebuild job.
//   Delete_by_range / Delete_Point_Boxes (:535-556, :647-710): every valid
//     point in the half-open box is flagged; the count of newly deleted points
//     is returned.  Whole covered subtrees are flagged without box tests.
//   Delete_by_point (:712-760): one valid point within EPSS = 1e-6 per axis is
//     flagged per input point (same_point, :1368-1371).
//   Add_by_range (:762-815): points deleted by box / point deletion (not by
//     downsampling) inside the box are restored.
//   Update / Criterion_Check / Rebuild (:1183-1323, :1089-1107, :624-645):
//     counts and AABBs are refit bottom-up along the touched paths only; a
//     node whose deleted share of slots exceeds alpha_del or whose left share
//     of valid points leaves [1 - alpha_bal, alpha_bal] is rebuilt, topmost
//     first.
#include <cuda_runtime.h>

#include <climits>
#include <utility>

#include "update.cuh"

namespace ikdg {
namespace {

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

__device__ __forceinline__ float coord4(const float4& p, int a) { return a == 0 ? p.x : (a == 1 ? p.y : p.z); }

// Appends `v` to a work list, or flags ERR_LIST when the list is full.
__device__ __forceinline__ void list_push(DevStatus* st, int* counter, int* list, int cap, int v) {
    int i = atomicAdd(counter, 1);
    if (i < cap)
        list[i] = v;
    else
        atomicOr(&st->err, ERR_LIST);
}

__device__ __forceinline__ void mark_dirty(const UpdateAux& a, DevStatus* st, int L) {
    if (atomicExch(&a.dirty_flag[L], 1) == 0) list_push(st, &st->n_items, a.items, a.list_cap, leaf_code(L));
}

// ---- insertion -----------------------------------------------------------------

__global__ void route_append_kernel(DevTree t, UpdateAux a, const float4* __restrict__ pts, long long n,
                                    const int* n_dev, int4* __restrict__ ovf_leaf, float4* __restrict__ ovf_pts) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long lim = n_dev != nullptr ? (long long)*n_dev : n;
    if (i >= lim) return;
    if (t.st->err & ERR_INPUT) return;  // a non-finite input: the call changes nothing
    float4 p = pts[i];
    int code = __float_as_int(t.node[3].x);  // sentinel's left child = root
    if (code == 0) {
        atomicOr(&t.st->err, ERR_ROUTE);
        return;
    }
    int steps = 0;
    while (code > 0) {
        if (++steps > MAX_WALK) {
            atomicOr(&t.st->err, ERR_LOOP);
            return;
        }
        float4 f3 = t.node[4 * code + 3];
        int axis = __float_as_int(f3.w);
        code = coord4(p, axis) < f3.z ? __float_as_int(f3.x) : __float_as_int(f3.y);
    }
    int L = code_leaf(code);
    int slot = atomicAdd(&t.leaf_n[L], 1);
    if (slot < LEAF_CAP) {
        t.pts[(long long)L * LEAF_CAP + slot] = p;
    } else {
        int o = atomicAdd(&t.st->n_ovf, 1);
        ovf_leaf[o] = make_int4(L, 0, 0, 0);
        ovf_pts[o] = p;
    }
    mark_dirty(a, t.st, L);
}

// ---- refit -------------------------------------------------------------------

__global__ void refit_mark_kernel(DevTree t, UpdateAux a, const int* __restrict__ items, const int* n_items) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *n_items || i >= a.list_cap) return;
    int code = items[i];
    int X;
    if (code < 0) {
        int lp = t.lparent[code_leaf(code)];
        if (lp < 0) return;
        X = lp >> 1;
    } else {
        X = code;
    }
    for (int steps = 0; X > 0; ++steps) {
        if (steps > MAX_WALK) {
            atomicOr(&t.st->err, ERR_LOOP);
            return;
        }
        if (atomicAdd(&a.pend[X], 1) > 0) break;
        X = t.nparent[X] >> 1;
    }
}

__device__ __forceinline__ int child_height(const DevTree& t, int code) {
    return code > 0 ? __ldcg(&t.nheight[code]) : 0;
}

__device__ __forceinline__ int log2_ceil(int x) {
    int r = 0;
    while ((1 << r) < x && r < 30) ++r;
    return r;
}

__global__ void refit_compute_kernel(DevTree t, UpdateAux a, const int* __restrict__ items, const int* n_items,
                                     Criteria c, int fill) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *n_items || i >= a.list_cap) return;
    int code = items[i];
    // Per node X on the walk: its child codes, its parent link and its
    // expected arrival count do not change during a refit (pend[X] is reset
    // only by X's last walker, after every walker has arrived).  They are
    // fetched one level ahead, in the same round trip as the level below's
    // record, so each level costs the arrival and one load round trip.
    auto invariants = [&](int X, float2& kids, int& lp, int& expect) {
        kids = __ldcg(reinterpret_cast<const float2*>(t.node + 4 * X + 3));
        lp = __ldcg(&t.nparent[X]);
        expect = __ldcg(&a.pend[X]);
    };
    int X;
    float2 kids = make_float2(0.f, 0.f);
    int lp = 0, expect = 0;
    if (code < 0) {
        int L = code_leaf(code);
        // the dirty list is consumed by this refit (nothing below reads the flag)
        a.dirty_flag[L] = 0;
        int llp = t.lparent[L];
        if (llp < 0) return;
        X = llp >> 1;
        if (X > 0) invariants(X, kids, lp, expect);
        int n = __ldcg(&t.leaf_n[L]);
        int m = n < LEAF_CAP ? n : LEAF_CAP;
        Box3 b = empty_box();
        int del = 0;
        const float4* lpn = t.pts + (long long)L * LEAF_CAP;
        for (int j = 0; j < m; ++j) {
            float4 p = __ldcg(lpn + j);
            if (__float_as_uint(p.w) & F_DEL)
                ++del;
            else
                box_grow(b, p.x, p.y, p.z);
        }
        write_child_box(t.node, X, llp & 1, b);
        write_child_cnt(t.ncnt, X, llp & 1, n, del);
        if (n > LEAF_CAP)  // an overflowing bucket must be split
            list_push(t.st, &t.st->n_viol, a.viol, a.list_cap, code);
    } else {
        X = code;
        if (X > 0) invariants(X, kids, lp, expect);
    }
    for (int steps = 0; X > 0; ++steps) {
        if (steps > MAX_WALK) {
            atomicOr(&t.st->err, ERR_LOOP);
            return;
        }
        // One acq_rel atomic: it releases this walker's writes into X's record
        // and, for the last walker, acquires the other children's (the
        // fence.sc / atomic / fence.sc form it replaces cost ~20 us per LiDAR
        // scan).
        int old;
        asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(&a.arrive[X]) : "memory");
        if (old + 1 < expect) return;
        a.pend[X] = 0;
        a.arrive[X] = 0;
        const int P = lp >> 1;
        const int hl = child_height(t, __float_as_int(kids.x)), hr = child_height(t, __float_as_int(kids.y));
        NodeRec r = load_node_cg(t.node, X);
        int4 cc = __ldcg(t.ncnt + X);
        float2 kids_p = make_float2(0.f, 0.f);
        int lp_p = 0, expect_p = 0;
        if (P > 0) invariants(P, kids_p, lp_p, expect_p);
        Box3 b = empty_box();
        Box3 bl = r.box(0), br = r.box(1);
        if (!box_empty(bl)) box_union(b, bl);
        if (!box_empty(br)) box_union(b, br);
        int slots = cc.x + cc.z, del = cc.y + cc.w;
        int h = 1 + max(hl, hr);
        t.nheight[X] = h;
        bool viol = false;
        if (slots > c.min_size) {
            // alpha_del on stored slots; alpha_bal on valid points.  (The
            // reference weighs balance by sizes that still include lazily
            // deleted nodes; here a rebuild that purges deleted points below
            // would then unbalance the ancestors and cascade into rebuilds of
            // ever larger subtrees, round after round.)
            const float fd = (float)del / (float)slots;
            const int valid = slots - del;
            const float fb = valid > 0 ? (float)(cc.x - cc.y) / (float)valid : 0.5f;
            viol = fd > c.alpha_del || fb > c.alpha_bal || fb < 1.0f - c.alpha_bal;
        }
        // Height guard: keeps every traversal stack within MAX_STACK.
        int ideal = log2_ceil(slots / (fill > 0 ? fill : 1) + 1);
        if (h > 2 * ideal + 8) viol = true;
        if (viol) {
            a.viol_flag[X] = 1;
            list_push(t.st, &t.st->n_viol, a.viol, a.list_cap, X);
        }
        write_child_box(t.node, P, lp & 1, b);
        write_child_cnt(t.ncnt, P, lp & 1, slots, del);
        X = P;
        kids = kids_p;
        lp = lp_p;
        expect = expect_p;
    }
}


// ---- rebuild jobs ----------------------------------------------------------------

__device__ __forceinline__ void select_job(const DevTree& t, const UpdateAux& a, int i) {
    int code = a.viol[i];
    int link = code < 0 ? t.lparent[code_leaf(code)] : t.nparent[code];
    if (link < 0) return;
    int X = link >> 1;
    for (int steps = 0; X > 0; ++steps) {
        if (steps > MAX_WALK) {
            atomicOr(&t.st->err, ERR_LOOP);
            return;
        }
        if (a.viol_flag[X]) return;  // an ancestor is rebuilt instead
        X = t.nparent[X] >> 1;
    }
    // One job per subtree even if the violator was listed twice.
    int* tag = code < 0 ? &a.job_of_leaf[code_leaf(code)] : &a.job_of_node[code];
    if (atomicCAS(tag, -1, -2) != -1) return;
    int j = atomicAdd(&t.st->n_jobs, 1);
    if (j >= a.list_cap) {
        atomicOr(&t.st->err, ERR_LIST);
        return;
    }
    a.jobs[j] = code;
    a.job_link[j] = link;
    if (code < 0)
        a.job_of_leaf[code_leaf(code)] = j;
    else
        a.job_of_node[code] = j;
}

// Grid-stride over the violators: the grid may be sized by a host bound or,
// when the selection runs before the host has read the violator count, by a
// fixed number of blocks.
__global__ void select_jobs_kernel(DevTree t, UpdateAux a, const int* n_viol) {
    const int nv = min(*n_viol, a.list_cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) select_job(t, a, i);
}

__global__ void clear_viol_kernel(UpdateAux a, const int* n_viol) {
    const int nv = min(*n_viol, a.list_cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
        int code = a.viol[i];
        if (code > 0) a.viol_flag[code] = 0;
    }
}


__device__ __forceinline__ int find_job_up(const DevTree& t, const UpdateAux& a, int X) {
    for (int steps = 0; X > 0; ++steps) {
        if (steps > MAX_WALK) {
            atomicOr(&t.st->err, ERR_LOOP);
            return -1;
        }
        int j = a.job_of_node[X];
        if (j >= 0) return j;
        X = t.nparent[X] >> 1;
    }
    return -1;
}

__device__ __forceinline__ int count_valid(const DevTree& t, int L) {
    int n = t.leaf_n[L];
    int m = n < LEAF_CAP ? n : LEAF_CAP;
    int v = 0;
    const float* lw = reinterpret_cast<const float*>(t.pts + (long long)L * LEAF_CAP) + 3;
    // eight flag words in flight (slots past the fill count stay in the bucket)
    for (int j0 = 0; j0 < m; j0 += 8) {
        float w[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) w[u] = lw[4 * (j0 + u)];
#pragma unroll
        for (int u = 0; u < 8; ++u) v += (j0 + u < m && !(__float_as_uint(w[u]) & F_DEL)) ? 1 : 0;
    }
    return v;
}

__global__ void job_count_leaf_kernel(DevTree t, UpdateAux a, int leaf_top) {
    int L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= leaf_top || t.st->n_jobs == 0) return;  // nothing selected: the speculative count ends here
    int lp = t.lparent[L];
    if (lp < 0) {
        a.leaf_job[L] = -1;
        return;
    }
    int j = a.job_of_leaf[L];
    if (j < 0) j = find_job_up(t, a, lp >> 1);
    a.leaf_job[L] = j;
    if (j >= 0) atomicAdd(&a.job_count[j], count_valid(t, L));
}

__global__ void job_count_node_kernel(DevTree t, UpdateAux a, int node_top) {
    int X = blockIdx.x * blockDim.x + threadIdx.x;
    if (X < 1 || X >= node_top || t.st->n_jobs == 0) return;
    if (t.nparent[X] < 0) {
        a.node_job[X] = -1;
        return;
    }
    a.node_job[X] = find_job_up(t, a, X);
}

__global__ void job_count_ovf_kernel(DevTree t, UpdateAux a, const int4* __restrict__ ovf_leaf, const int* n_ovf) {
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= *n_ovf || t.st->n_jobs == 0) return;
    int L = ovf_leaf[o].x;
    int j = a.leaf_job[L];
    if (j < 0) {
        if (atomicOr(&t.st->err, ERR_OVF_JOB) == 0 || true) {
            int* d = t.st->dbg;
            if (atomicCAS(&d[0], 0, 1) == 0) {
                d[1] = L;
                d[2] = t.lparent[L];
                d[3] = t.leaf_n[L];
                d[4] = a.job_of_leaf[L];
                d[5] = a.dirty_flag[L];
                int lp = t.lparent[L];
                d[6] = lp >= 0 ? a.viol_flag[lp >> 1] : -7;
                d[7] = *n_ovf;
            }
        }
        return;
    }
    atomicAdd(&a.job_count[j], 1);
}

// job_off = exclusive prefix sum of job_count over the selected jobs (count
// read on the device), job_off[n_jobs] = st->job_total = the sum, st->max_job
// = the largest job: one block, 1,024 jobs per step.
__global__ void __launch_bounds__(1024) job_scan_kernel(DevTree t, UpdateAux a) {
    __shared__ int wsum[32];
    __shared__ int carry, mx;
    const int n = min(t.st->n_jobs, a.list_cap);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        carry = 0;
        mx = 0;
    }
    __syncthreads();
    for (int base = 0; base < n; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < n ? a.job_count[i] : 0;
        int inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) wsum[w] = inc;
        if (v > 0) atomicMax(&mx, v);
        __syncthreads();
        if (w == 0) {
            const int ws = wsum[lane];
            int wi = ws;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += y;
            }
            wsum[lane] = wi - ws;
        }
        __syncthreads();
        const int c = carry;
        if (i < n) a.job_off[i] = c + wsum[w] + inc - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = c + wsum[w] + inc;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.job_off[n] = carry;
        t.st->job_total = carry;
        t.st->max_job = mx;
    }
}

__global__ void job_max_kernel(DevTree t, UpdateAux a, const int* n_jobs, const int* total) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j == 0) {
        t.st->job_total = *total;
        a.job_off[*n_jobs] = *total;
    }
    if (j >= *n_jobs) return;
    atomicMax(&t.st->max_job, a.job_count[j]);
}

__global__ void job_gather_leaf_kernel(DevTree t, UpdateAux a, int leaf_top, float4* __restrict__ out,
                                       float4* __restrict__ removed, long long removed_cap) {
    int L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= leaf_top) return;
    int j = a.leaf_job[L];
    if (j < 0) return;
    int n = t.leaf_n[L];
    int m = n < LEAF_CAP ? n : LEAF_CAP;
    const float4* lp = t.pts + (long long)L * LEAF_CAP;
    int nv = count_valid(t, L);
    int pos = a.job_off[j] + atomicAdd(&a.job_fill[j], nv);
    for (int s0 = 0; s0 < m; s0 += 8) {
        float4 pb[8];  // eight slots in flight (the bucket always has LEAF_CAP slots)
#pragma unroll
        for (int u = 0; u < 8; ++u) pb[u] = lp[s0 + u];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (s0 + u >= m) break;
            const float4 p = pb[u];
            const uint32_t w = __float_as_uint(p.w);
            if (!(w & F_DEL)) {
                out[pos++] = p;
            } else if (!(w & F_DSDEL)) {
                // Dropped deleted points are kept for acquire_removed_points
                // (flatten with DELETE_POINTS_REC, ikd_Tree.cpp:1338-1342).
                long long r = atomicAdd((unsigned long long*)&t.st->removed_n, 1ull);
                if (r < removed_cap) removed[r] = make_float4(p.x, p.y, p.z, __uint_as_float(w & ID_MASK));
            }
        }
    }
    t.lparent[L] = -1;
    t.leaf_n[L] = 0;
    int f = atomicAdd(&t.st->free_leaf_n, 1);
    t.free_leaf[f] = L;
}

__global__ void job_gather_node_kernel(DevTree t, UpdateAux a, int node_top) {
    int X = blockIdx.x * blockDim.x + threadIdx.x;
    if (X < 1 || X >= node_top) return;
    if (a.node_job[X] < 0) return;
    t.nparent[X] = -1;
    int f = atomicAdd(&t.st->free_node_n, 1);
    t.free_node[f] = X;
}

__global__ void job_gather_ovf_kernel(DevTree t, UpdateAux a, const int4* __restrict__ ovf_leaf,
                                      const float4* __restrict__ ovf_pts, const int* n_ovf, float4* __restrict__ out) {
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= *n_ovf) return;
    int j = a.leaf_job[ovf_leaf[o].x];
    if (j < 0) return;
    int pos = a.job_off[j] + atomicAdd(&a.job_fill[j], 1);
    out[pos] = ovf_pts[o];
}

// Resets per-job state and queues each job's parent for the follow-up refit.
__global__ void job_finish_kernel(DevTree t, UpdateAux a, const int* n_jobs) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j == 0) {
        t.st->max_job = 0;
        t.st->n_ovf = 0;
    }
    if (j >= *n_jobs) return;
    int code = a.jobs[j];
    if (code < 0)
        a.job_of_leaf[code_leaf(code)] = -1;
    else
        a.job_of_node[code] = -1;
    a.job_count[j] = 0;
    a.job_fill[j] = 0;
    int P = a.job_link[j] >> 1;
    if (P > 0) list_push(t.st, &t.st->n_items, a.items, a.list_cap, P);
}

// ---- box / point deletion, box re-insertion ----------------------------------------

constexpr int DB_THREADS = 128;
constexpr int DB_WARPS = DB_THREADS / 32;
constexpr int DB_STACK = DB_THREADS * (MAX_STACK + 2);
constexpr int DB_SPLIT_BITS_MAX = 6;
constexpr long long DB_TARGET_UNITS = 1024;

// Whether child `side` of node record r (code: its index, 0 = sentinel) can
// hold points that box qb edits.  MODE 0 prunes by the child's AABB (which
// bounds valid points) and reports full cover in ccov; MODE 1 looks for
// deleted points, which only the split planes bound: the left subtree holds
// coordinates <= split, the right >= split.
template <int MODE>
__device__ __forceinline__ bool box_child(const Box3& qb, const NodeRec& r, int code, int side, bool cov,
                                          bool& ccov) {
    ccov = cov;
    if (MODE == 0) {
        Box3 b = r.box(side);
        if (box_empty(b)) return false;
        if (!ccov) {
            if (qbox_disjoint(qb, b)) return false;
            ccov = qbox_covers(qb, b);
        }
    } else if (code > 0) {
        int ax = r.axis();
        float sp = r.split();
        if (side == 0 && sp < qb.lo[ax]) return false;
        if (side == 1 && qb.hi[ax] <= sp) return false;
    }
    return true;
}

// Work unit (box bi, part): the CTA walks split_bits levels down from the
// root, taking the side that bit d of `part` names at depth d, and edits the
// subtree it reaches.  A leaf met above that depth belongs to the part whose
// remaining bits are zero.  Returns the stack item (code * 2 + covered) or
// INT_MIN when the walk was pruned.
template <int MODE>
__device__ int box_seed(const DevTree& t, const Box3& qb, int part, int split_bits) {
    NodeRec r = load_node_cg(t.node, 0);
    int code = r.left();
    bool cov = false, ccov;
    if (code == 0 || !box_child<MODE>(qb, r, 0, 0, cov, ccov)) return INT_MIN;
    cov = ccov;
    for (int d = 0; d < split_bits; ++d) {
        if (code < 0) return (part >> d) == 0 ? code * 2 + (cov ? 1 : 0) : INT_MIN;
        r = load_node_cg(t.node, code);
        int side = (part >> d) & 1;
        int c = side == 0 ? r.left() : r.right();
        if (c == 0 || !box_child<MODE>(qb, r, code, side, cov, ccov)) return INT_MIN;
        code = c;
        cov = ccov;
    }
    return code * 2 + (cov ? 1 : 0);
}

// One CTA per work unit (box, top-level subtree).  Each round the CTA pops up
// to DB_THREADS items off a shared stack; threads expand nodes (pushing the
// children that overlap the box, tagged when fully covered) and queue leaves,
// then each warp edits queued leaves one slot per lane.  MODE 0 deletes
// (flags |= del_flags), MODE 1 restores box-deleted points (Add_by_range).
template <int MODE>
__global__ void __launch_bounds__(DB_THREADS) box_edit_kernel(DevTree t, UpdateAux a, const float* __restrict__ boxes,
                                                              long long m, int split_bits, uint32_t del_flags,
                                                              long long* __restrict__ total) {
    __shared__ int stack[DB_STACK];
    __shared__ int leafq[2 * DB_THREADS];
    __shared__ int top, nleaf;
    __shared__ long long block_cnt;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long units = m << split_bits;
    for (long long u = blockIdx.x; u < units; u += gridDim.x) {
        const long long bi = u >> split_bits;
        const int part = (int)(u & ((1 << split_bits) - 1));
        Box3 qb;
        for (int k = 0; k < 3; ++k) {
            qb.lo[k] = boxes[bi * 6 + k];
            qb.hi[k] = boxes[bi * 6 + 3 + k];
        }
        if (threadIdx.x == 0) {
            top = 0;
            nleaf = 0;
            block_cnt = 0;
            int seed = box_seed<MODE>(t, qb, part, split_bits);
            if (seed != INT_MIN) stack[top++] = seed;
        }
        __syncthreads();
        long long my_cnt = 0;
        for (int rounds = 0;; ++rounds) {
            int cur_top = top;
            if (cur_top == 0) break;
            if (rounds > MAX_VISITS / DB_THREADS) {
                if (threadIdx.x == 0) atomicOr(&t.st->err, ERR_LOOP);
                break;
            }
            int n = cur_top < DB_THREADS ? cur_top : DB_THREADS;
            int base = cur_top - n;
            int item = threadIdx.x < n ? stack[base + threadIdx.x] : 0;
            __syncthreads();
            if (threadIdx.x == 0) top = base;
            __syncthreads();
            if (threadIdx.x < n) {
                int code = item >> 1;  // arithmetic shift: floor(item / 2)
                bool cov = item & 1;
                if (code >= 0) {
                    NodeRec r = load_node_cg(t.node, code);
                    for (int side = 0; side < 2; ++side) {
                        int c = side == 0 ? r.left() : r.right();
                        bool ccov;
                        if (c == 0 || !box_child<MODE>(qb, r, code, side, cov, ccov)) continue;
                        int it = c * 2 + (ccov ? 1 : 0);
                        if (c < 0) {
                            leafq[atomicAdd(&nleaf, 1)] = it;  // <= 2 per thread
                        } else {
                            int pos = atomicAdd(&top, 1);
                            if (pos < DB_STACK)
                                stack[pos] = it;
                            else
                                atomicOr(&t.st->err, ERR_STACK);
                        }
                    }
                } else {
                    leafq[atomicAdd(&nleaf, 1)] = item;
                }
            }
            __syncthreads();
            const int nq = nleaf;
            for (int q = warp; q < nq; q += DB_WARPS) {
                const int it = leafq[q];
                const int L = code_leaf(it >> 1);
                const bool cov = it & 1;
                const int nl = t.leaf_n[L];
                float4* lp = t.pts + (long long)L * LEAF_CAP;
                bool hit = false;
                if (lane < nl && lane < LEAF_CAP) {
                    float4 p = __ldcg(lp + lane);
                    uint32_t w = __float_as_uint(p.w);
                    if (MODE == 0) {
                        if (!(w & F_DEL) && (cov || qbox_holds(qb, p.x, p.y, p.z))) {
                            unsigned old = atomicOr((unsigned*)&lp[lane].w, del_flags);
                            hit = !(old & F_DEL);
                        }
                    } else {
                        if ((w & F_DEL) && !(w & F_DSDEL) && (cov || qbox_holds(qb, p.x, p.y, p.z))) {
                            atomicAnd((unsigned*)&lp[lane].w, ~F_DEL);
                            hit = true;
                        }
                    }
                }
                unsigned bal = __ballot_sync(0xffffffffu, hit);
                if (bal && lane == 0) {
                    mark_dirty(a, t.st, L);
                    my_cnt += __popc(bal);
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) nleaf = 0;
        }
        if (MODE == 0 && my_cnt) atomicAdd((unsigned long long*)&block_cnt, (unsigned long long)my_cnt);
        __syncthreads();
        if (MODE == 0 && threadIdx.x == 0 && block_cnt) atomicAdd((unsigned long long*)total, (unsigned long long)block_cnt);
        __syncthreads();
    }
}

// Subtree split for box edits: enough (box, subtree) units to fill the GPU
// when there are few boxes, none when there are many.
int box_split_bits(long long m) {
    int bits = 0;
    while (bits < DB_SPLIT_BITS_MAX && (m << bits) < DB_TARGET_UNITS) ++bits;
    return bits;
}

unsigned box_grid(long long units) { return (unsigned)(units < (1LL << 20) ? units : (1LL << 20)); }

// same_point (ikd_Tree.cpp:1368-1371): |a - b| < 1e-6 per axis, the float
// difference compared in double.
__device__ __forceinline__ bool same_point(float ax, float ay, float az, float bx, float by, float bz) {
    return (double)fabsf(__fsub_rn(ax, bx)) < 1e-6 && (double)fabsf(__fsub_rn(ay, by)) < 1e-6 &&
           (double)fabsf(__fsub_rn(az, bz)) < 1e-6;
}

__global__ void __launch_bounds__(128) delete_points_kernel(DevTree t, UpdateAux a, const float* __restrict__ in,
                                                            int stride, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float px = in[i * stride], py = in[i * stride + 1], pz = in[i * stride + 2];
    // A match differs by < 1e-6 per axis; 2e-6 bounds the search box safely
    // (a larger coordinate rounds p +- 2e-6 only where no match can exist).
    Box3 sb;
    sb.lo[0] = __fsub_rn(px, 2e-6f); sb.hi[0] = __fadd_rn(px, 2e-6f);
    sb.lo[1] = __fsub_rn(py, 2e-6f); sb.hi[1] = __fadd_rn(py, 2e-6f);
    sb.lo[2] = __fsub_rn(pz, 2e-6f); sb.hi[2] = __fadd_rn(pz, 2e-6f);
    int stack[MAX_STACK];
    int sp = 0;
    stack[sp++] = 0;
    bool start = true;
    int visits = 0;
    while (sp > 0) {
        if (++visits > MAX_VISITS) {
            atomicOr(&t.st->err, ERR_LOOP);
            break;
        }
        int code = stack[--sp];
        if (start || code > 0) {
            start = false;
            NodeRec r = load_node_cg(t.node, code);
            for (int side = 0; side < 2; ++side) {
                int c = side == 0 ? r.left() : r.right();
                if (c == 0) continue;
                Box3 b = r.box(side);
                if (box_empty(b)) continue;
                bool far = false;
                for (int k = 0; k < 3; ++k) far = far || b.lo[k] > sb.hi[k] || b.hi[k] < sb.lo[k];
                if (far) continue;
                if (sp < MAX_STACK)
                    stack[sp++] = c;
                else
                    atomicOr(&t.st->err, ERR_STACK);
            }
        } else {
            int L = code_leaf(code);
            int nl = t.leaf_n[L];
            int ml = nl < LEAF_CAP ? nl : LEAF_CAP;
            float4* lp = t.pts + (long long)L * LEAF_CAP;
            for (int s = 0; s < ml; ++s) {
                float4 p = __ldcg(lp + s);
                unsigned w = __float_as_uint(p.w);
                if (w & F_DEL) continue;
                if (!same_point(p.x, p.y, p.z, px, py, pz)) continue;
                unsigned old = atomicCAS((unsigned*)&lp[s].w, w, w | F_DEL);
                if (old == w) {
                    mark_dirty(a, t.st, L);
                    return;
                }
            }
        }
    }
}

__global__ void flatten_kernel(DevTree t, float4* __restrict__ out, long long* counter) {
    int L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= t.st->leaf_top) return;
    if (t.lparent[L] < 0) return;
    int n = t.leaf_n[L];
    int m = n < LEAF_CAP ? n : LEAF_CAP;
    const float4* lp = t.pts + (long long)L * LEAF_CAP;
    int nv = count_valid(t, L);
    if (nv == 0) return;
    long long pos = (long long)atomicAdd((unsigned long long*)counter, (unsigned long long)nv);
    for (int s = 0; s < m; ++s) {
        float4 p = lp[s];
        if (!(__float_as_uint(p.w) & F_DEL)) out[pos++] = p;
    }
}

// Ids of every stored slot (valid or deleted) of the leaves in use; slots
// past `cap` are counted but not written.
__global__ void stored_ids_kernel(DevTree t, int* __restrict__ out, long long cap, long long* counter) {
    int L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= t.st->leaf_top) return;
    if (t.lparent[L] < 0) return;
    const int m = min(t.leaf_n[L], LEAF_CAP);
    if (m == 0) return;
    const long long pos = (long long)atomicAdd((unsigned long long*)counter, (unsigned long long)m);
    const float4* lp = t.pts + (long long)L * LEAF_CAP;
    for (int s = 0; s < m; ++s)
        if (pos + s < cap) out[pos + s] = (int)(__float_as_uint(lp[s].w) & ID_MASK);
}

__global__ void select_root_job_kernel(DevTree t, UpdateAux a) {
    int code = __float_as_int(t.node[3].x);
    if (code == 0) return;
    a.jobs[0] = code;
    a.job_link[0] = 0;
    if (code < 0)
        a.job_of_leaf[code_leaf(code)] = 0;
    else
        a.job_of_node[code] = 0;
    t.st->n_jobs = 1;
}

// ---- structural validation (diagnostics) ---------------------------------------------

__device__ __forceinline__ bool same_box(const Box3& a, const Box3& b) {
    for (int k = 0; k < 3; ++k)
        if (__float_as_uint(a.lo[k]) != __float_as_uint(b.lo[k]) || __float_as_uint(a.hi[k]) != __float_as_uint(b.hi[k]))
            return false;
    return true;
}

// For every live node: both children exist and point back; the child box and
// counts stored in the node equal what the child itself holds.
__device__ __forceinline__ void note_bad(DevStatus* st, int kind, int X, int side, int a0, int a1, int a2, int a3) {
    if (atomicCAS(&st->dbg[0], 0, kind) == 0) {
        st->dbg[1] = X;
        st->dbg[2] = side;
        st->dbg[3] = a0;
        st->dbg[4] = a1;
        st->dbg[5] = a2;
        st->dbg[6] = a3;
    }
}

// For every live node: both children exist and point back; the child box and
// counts stored in the node equal what the child itself holds.
__global__ void validate_nodes_kernel(DevTree t, bool at_rest, unsigned long long* bad) {
    int X = blockIdx.x * blockDim.x + threadIdx.x;
    if (X >= t.st->node_top) return;
    if (X > 0 && t.nparent[X] < 0) return;
    NodeRec r = load_node_cg(t.node, X);
    int4 cc = __ldcg(t.ncnt + X);
    unsigned long long nbad = 0;
    for (int side = 0; side < 2; ++side) {
        int c = side == 0 ? r.left() : r.right();
        int slots = side == 0 ? cc.x : cc.z, del = side == 0 ? cc.y : cc.w;
        Box3 stored = r.box(side);
        if (X == 0 && side == 1) {
            if (c != 0) {
                ++nbad;
                note_bad(t.st, 101, X, side, c, 0, 0, 0);
            }
            continue;
        }
        if (c == 0) {
            if (X != 0) {  // only an empty tree has no root
                ++nbad;
                note_bad(t.st, 102, X, side, 0, 0, 0, 0);
            }
            continue;
        }
        Box3 b = empty_box();
        int s2 = 0, d2 = 0;
        if (c > 0) {
            if (c >= t.st->node_top || t.nparent[c] != X * 2 + side) {
                ++nbad;
                note_bad(t.st, 103, X, side, c, c < t.st->node_top ? t.nparent[c] : -9, 0, 0);
                continue;
            }
            NodeRec rc = load_node_cg(t.node, c);
            int4 c4 = __ldcg(t.ncnt + c);
            Box3 bl = rc.box(0), br = rc.box(1);
            if (!box_empty(bl)) box_union(b, bl);
            if (!box_empty(br)) box_union(b, br);
            s2 = c4.x + c4.z;
            d2 = c4.y + c4.w;
        } else {
            int L = code_leaf(c);
            if (L >= t.st->leaf_top || t.lparent[L] != X * 2 + side) {
                ++nbad;
                note_bad(t.st, 104, X, side, c, L < t.st->leaf_top ? t.lparent[L] : -9, 0, 0);
                continue;
            }
            int n = t.leaf_n[L];
            // Between a refit and its rebuild jobs a leaf may hold more
            // points than slots (its overflow is queued for the rebuild).
            if ((n > LEAF_CAP && at_rest) || n < 0) {
                ++nbad;
                note_bad(t.st, 105, X, side, c, n, 0, 0);
                continue;
            }
            s2 = n;
            const int m = n < LEAF_CAP ? n : LEAF_CAP;
            for (int j = 0; j < m; ++j) {
                float4 p = __ldcg(t.pts + (long long)L * LEAF_CAP + j);
                if (__float_as_uint(p.w) & F_DEL)
                    ++d2;
                else
                    box_grow(b, p.x, p.y, p.z);
            }
        }
        if (s2 != slots || d2 != del) {
            ++nbad;
            note_bad(t.st, 106, X, side, slots, s2, del, d2);
        } else if (!same_box(b, stored)) {
            ++nbad;
            int k = 0;
            while (k < 3 && __float_as_uint(b.lo[k]) == __float_as_uint(stored.lo[k]) &&
                   __float_as_uint(b.hi[k]) == __float_as_uint(stored.hi[k]))
                ++k;
            note_bad(t.st, 107, X, side, c, k, __float_as_int(k < 3 ? b.lo[k] : 0.f),
                     __float_as_int(k < 3 ? stored.lo[k] : 0.f));
        }
    }
    if (nbad) atomicAdd(bad, nbad);
}

// Every live leaf is the child its parent record names.
__global__ void validate_leaves_kernel(DevTree t, unsigned long long* bad) {
    int L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= t.st->leaf_top) return;
    int lp = t.lparent[L];
    if (lp < 0) return;
    int P = lp >> 1;
    bool ok = P < t.st->node_top && (P == 0 || t.nparent[P] >= 0);
    if (ok) {
        const int* codes = reinterpret_cast<const int*>(t.node + 4 * P + 3);
        ok = codes[lp & 1] == leaf_code(L);
    }
    if (!ok) {
        atomicAdd(bad, 1ull);
        note_bad(t.st, 108, P, lp & 1, L, lp, 0, 0);
    }
}

// Refit / rebuild bookkeeping that must be clear between refits (arrival
// counters) or between calls (violation and job tags, dirty flags).
__global__ void validate_aux_nodes_kernel(DevTree t, UpdateAux a, bool at_rest, unsigned long long* bad) {
    int X = blockIdx.x * blockDim.x + threadIdx.x;
    if (X >= t.node_cap) return;
    if (a.pend[X] != 0 || a.arrive[X] != 0) {
        atomicAdd(bad, 1ull);
        note_bad(t.st, 109, X, a.pend[X], a.arrive[X], X < t.st->node_top ? t.nparent[X] : -9, 0, 0);
    }
    if (at_rest && (a.viol_flag[X] != 0 || a.job_of_node[X] != -1)) {
        atomicAdd(bad, 1ull);
        note_bad(t.st, 110, X, a.viol_flag[X], a.job_of_node[X], 0, 0, 0);
    }
}

__global__ void validate_aux_leaves_kernel(DevTree t, UpdateAux a, unsigned long long* bad) {
    int L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= t.leaf_cap) return;
    if (a.dirty_flag[L] != 0 || a.job_of_leaf[L] != -1) {
        atomicAdd(bad, 1ull);
        note_bad(t.st, 111, L, a.dirty_flag[L], a.job_of_leaf[L], L < t.st->leaf_top ? t.lparent[L] : -9, 0, 0);
    }
}

__global__ void set_ll_kernel(long long* p, long long v) { *p = v; }

__global__ void snapshot_root_kernel(DevTree t) {
    int4 c = t.ncnt[0];
    t.st->root_code = __float_as_int(t.node[3].x);
    t.st->root_slots = c.x;
    t.st->root_deleted = c.y;
    int rc = t.st->root_code;
    t.st->root_height = rc > 0 ? t.nheight[rc] : 0;
}

// ---- voxel downsampling ------------------------------------------------------------
//
// Sequential semantics (Add_Points with downsample_on, ikd_Tree.cpp:422-449),
// for new point p_i in order: box = the voxel of p_i, with
// lo = floor(x / ds) * ds and hi = lo + ds in float, centre = lo + (hi - lo) / 2
// in double rounded to float; S = valid points in the half-open box; the
// winner is p_i unless a point of S is strictly closer to the centre; if
// |S| > 1 or the winner is p_i (within EPSS), S is deleted (downsample flag)
// and the winner is inserted as a new point.
//
// Parallel form: points are grouped by voxel.  A voxel's outcome depends only
// on its own S and its own new points, taken in input order, as long as no
// point lies in two voxel boxes or outside its own (float rounding can make the
// boxes of neighbouring voxels overlap or leave gaps by one ulp).  Such points
// are detected and processed alone, in input order, which keeps the result
// identical to the sequential loop.  Among points of S at the same distance
// the smaller id wins (the reference takes the first in traversal order).  A
// winner that was already in the map is re-inserted under its own id; a new
// point i of the batch gets id first_id + i.

// Bits of the voxel hash the grouper sorts by (and compares: entries of one
// hash run are the sorted neighbours with equal masked hash).
constexpr int DS_HASH_BITS = 24;
// Hash runs longer than this go to ds_fold_big_kernel (a warp per group,
// DS_BIG_BLOCKS blocks of four warps walking the deferred list).
constexpr int DS_BIG_RUN = 64;
constexpr int DS_BIG_BLOCKS = 38;
// Blocks of the job selection when it runs before the violator count is known.
constexpr int SPEC_BLOCKS = 152;

__device__ __forceinline__ uint32_t mix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

__device__ __forceinline__ void voxel_axis(float c, float ds, float& f, float& lo, float& hi, float& mid) {
    f = floorf(__fdiv_rn(c, ds));
    lo = __fmul_rn(f, ds);
    hi = __fadd_rn(lo, ds);
    mid = __double2float_rn(__dadd_rn((double)lo, __dmul_rn((double)__fsub_rn(hi, lo), 0.5)));
}

// Is coordinate c inside the box range of voxel index f + df on this axis?
__device__ __forceinline__ bool in_voxel_range(float c, float f, float df, float ds) {
    float lo = __fmul_rn(__fadd_rn(f, df), ds);
    float hi = __fadd_rn(lo, ds);
    return lo <= c && c < hi;
}

__global__ void ds_prepare_kernel(DevTree t, const float* __restrict__ in, int stride, long long n, float ds,
                                  DsScratch d) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float c[3] = {in[i * stride], in[i * stride + 1], in[i * stride + 2]};
    if (!(isfinite(c[0]) && isfinite(c[1]) && isfinite(c[2]))) atomicOr(&t.st->err, ERR_INPUT);
    float f[3], lo[3], hi[3], mid[3];
    bool clean = true;
    for (int a = 0; a < 3; ++a) {
        voxel_axis(c[a], ds, f[a], lo[a], hi[a], mid[a]);
        clean = clean && lo[a] <= c[a] && c[a] < hi[a];
        if (!(fabsf(f[a]) < 8388608.0f)) clean = false;  // f +- 1 must stay exact
    }
    if (clean)
        for (int a = 0; a < 3; ++a)
            if (in_voxel_range(c[a], f[a], -1.f, ds) || in_voxel_range(c[a], f[a], 1.f, ds)) clean = false;
    d.pts[i] = make_float4(c[0], c[1], c[2], 0.f);
    d.box_lo[i] = make_float4(lo[0], lo[1], lo[2], f[0]);
    d.box_hi[i] = make_float4(hi[0], hi[1], hi[2], f[1]);
    d.mid[i] = make_float4(mid[0], mid[1], mid[2], f[2]);
    // Grouping key: the voxel's float indices (bit patterns), exact.
    // -0.0 and +0.0 give the same box; adding +0.0 maps both to +0.0.
    int kb[3];
    for (int a = 0; a < 3; ++a) kb[a] = __float_as_int(__fadd_rn(f[a], 0.0f));
    d.key[i] = make_int4(kb[0], kb[1], kb[2], clean ? 1 : 0);
    // The bit patterns of integral floats end in long runs of zeros: each
    // component goes through the full mixer (a product of them kept only
    // ~16 bits and put up to 7 voxels on one hash).
    uint32_t h = mix32((uint32_t)kb[2] ^ 0x9e3779b9u);
    h = mix32(h ^ (uint32_t)kb[1]);
    d.hkey[0][i] = mix32(h ^ (uint32_t)kb[0]) & ((1u << DS_HASH_BITS) - 1u);
    d.hval[0][i] = (uint32_t)i;
}

__device__ __forceinline__ bool same_key(const int4& a, const int4& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

// Also lays the keys and points out in sorted order (s_key, s_pts), so the
// per-group walks below read consecutive entries instead of gathering through
// hval one dependent load at a time.
__global__ void ds_leaders_kernel(long long n, DsScratch d, DevStatus* st) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t h = d.hkey[0][j];
    const uint32_t idx = d.hval[0][j];
    int4 k = d.key[idx];
    const float4 p = d.pts[idx];
    d.s_key[j] = k;
    d.s_pts[j] = make_float4(p.x, p.y, p.z, __int_as_float((int)idx));
    for (long long jj = j - 1; jj >= 0 && d.hkey[0][jj] == h; --jj)
        if (same_key(d.key[d.hval[0][jj]], k)) return;
    int g = atomicAdd(&st->n_groups, 1);
    d.groups[g] = (int)j;
}

// Entries of the hash run starting at sorted position j, four per step
// (independent loads); f(jj, key, point) sees them in sorted order, which
// within one voxel is input order, and returns false to stop.
template <class F>
__device__ __forceinline__ void for_run(const DsScratch& d, long long n, long long j, uint32_t h, F f) {
    for (long long base = j; base < n; base += 4) {
        uint32_t hh[4];
        int4 kk[4];
        float4 pp[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const long long jj = base + u;
            hh[u] = jj < n ? __ldg(d.hkey[0] + jj) : ~h;
            kk[u] = jj < n ? __ldg(d.s_key + jj) : make_int4(0, 0, 0, 0);
            pp[u] = jj < n ? __ldg(d.s_pts + jj) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (hh[u] != h) return;
            if (!f(base + u, kk[u], pp[u])) return;
        }
    }
}

// First member index >= a of group g (members are in increasing index order).
__device__ __forceinline__ long long group_first_from(const DsScratch& d, long long n, int j, long long a) {
    const uint32_t h = __ldg(d.hkey[0] + j);
    const int4 k = __ldg(d.s_key + j);
    long long r = -1;
    for_run(d, n, j, h, [&](long long, const int4& kk, const float4& p) {
        if (!same_key(kk, k)) return true;
        const long long idx = __float_as_int(p.w);
        if (idx >= a) {
            r = idx;
            return false;
        }
        return true;
    });
    return r;
}

__global__ void ds_h1_kernel(long long n, long long a, DsScratch d, DevStatus* st) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *d.n_pairs = 0;  // ds_search_kernel lists its pairs afresh
    long long i = a + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (d.key[i].w) return;
    long long cut = i > a ? i : a + 1;
    atomicMin((long long*)&st->count, cut);
}

// Warp-collective walk of every lane's box (half-open, {lo, hi}) down the
// tree: a node phase steps each lane through its own nodes until it holds a
// leaf, then the warp scans the held leaves together, one lane per slot (one
// coalesced 512-byte load per leaf).  For every held leaf every lane calls
// leaf(src, L, p, nl): src = the lane holding leaf L, p = slot `lane` of L,
// nl = L's fill count.  Every lane of the warp must call it; lanes without a
// box pass active = false.  Slots are read with plain loads: ds_delete_kernel
// flags slots of the leaves it walks.
template <class F>
__device__ __forceinline__ void warp_box_walk(const DevTree& t, bool active, const Box3& qb, F leaf) {
    const int lane = threadIdx.x & 31;
    int stack[MAX_STACK];
    int sp = 0;
    int cur = 0;  // node code (0 = the sentinel record, where the walk starts) or leaf code (< 0)
    bool done = !active;
    int visits = 0;
    auto pop = [&]() {
        if (sp > 0)
            cur = stack[--sp];
        else
            done = true;
    };
    while (true) {
        while (true) {
            const bool nodework = !done && cur >= 0;
            if (!__any_sync(0xffffffffu, nodework)) break;
            if (!nodework) continue;
            if (++visits > MAX_VISITS) {
                atomicOr(&t.st->err, ERR_LOOP);
                done = true;
                continue;
            }
            const NodeRec r = load_node(t.node, cur);
            int next = 0;
            bool have_next = false;
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const int c = side == 0 ? r.left() : r.right();
                if (c == 0) continue;
                const Box3 b = r.box(side);
                if (box_empty(b) || qbox_disjoint(qb, b)) continue;
                if (!have_next) {
                    next = c;
                    have_next = true;
                } else if (sp < MAX_STACK) {
                    stack[sp++] = c;
                } else {
                    atomicOr(&t.st->err, ERR_STACK);
                }
            }
            if (have_next)
                cur = next;
            else
                pop();
        }
        const bool leafwork = !done && cur < 0;
        unsigned lb = __ballot_sync(0xffffffffu, leafwork);
        if (lb == 0) break;
        while (lb) {
            // two held leaves per step: their slot loads go out together
            const int s0 = __ffs(lb) - 1;
            lb &= lb - 1;
            const int s1 = lb ? __ffs(lb) - 1 : -1;
            if (lb) lb &= lb - 1;
            const int L0 = code_leaf(__shfl_sync(0xffffffffu, cur, s0));
            const int L1 = code_leaf(__shfl_sync(0xffffffffu, cur, s1 < 0 ? s0 : s1));
            const float4 p0 = t.pts[(long long)L0 * LEAF_CAP + lane];
            const int n0 = __ldg(t.leaf_n + L0);
            float4 p1 = p0;
            int n1 = 0;
            if (s1 >= 0) {
                p1 = t.pts[(long long)L1 * LEAF_CAP + lane];
                n1 = __ldg(t.leaf_n + L1);
            }
            leaf(s0, L0, p0, min(n0, LEAF_CAP));
            if (s1 >= 0) leaf(s1, L1, p1, min(n1, LEAF_CAP));
        }
        if (leafwork) pop();
    }
}

__device__ __forceinline__ Box3 group_box(const DsScratch& d, int lead) {
    const float4 blo = d.box_lo[lead], bhi = d.box_hi[lead];
    Box3 qb;
    qb.lo[0] = blo.x; qb.lo[1] = blo.y; qb.lo[2] = blo.z;
    qb.hi[0] = bhi.x; qb.hi[1] = bhi.y; qb.hi[2] = bhi.z;
    return qb;
}

__device__ __forceinline__ Box3 shfl_box(const Box3& b, int src) {
    Box3 o;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        o.lo[k] = __shfl_sync(0xffffffffu, b.lo[k], src);
        o.hi[k] = __shfl_sync(0xffffffffu, b.hi[k], src);
    }
    return o;
}

// Per voxel group: S = the valid stored points in the voxel's box, |S|, the
// point of S closest to the voxel centre (smaller id on ties), and whether a
// point of S also lies in a neighbouring voxel's box range on some axis (a
// float-rounding sliver: the group is then folded alone).
__global__ void __launch_bounds__(128) ds_search_kernel(DevTree t, long long n, long long a, DsScratch d, float ds) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    if (g == 0) *d.n_big = 0;  // ds_fold_kernel lists its deferred groups afresh
    bool active = g < t.st->n_groups && !(t.st->err & ERR_INPUT);  // a non-finite input: the call changes nothing
    long long first = -1;
    int lead = 0;
    if (active) {
        const int j = d.groups[g];
        first = group_first_from(d, n, j, a);
        if (first < 0) {
            d.g_info[g] = make_int4(0, -1, 0, 0);
            active = false;
        } else {
            lead = d.hval[0][j];
        }
    }
    const Box3 qb = active ? group_box(d, lead) : empty_box();
    const float4 mid = active ? d.mid[lead] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float fk0 = active ? d.box_lo[lead].w : 0.f, fk1 = active ? d.box_hi[lead].w : 0.f;
    int n0 = 0, best_slot = -1, best_id = 0x7fffffff;
    float best_d = __int_as_float(0x7f800000);
    float4 best_p = make_float4(0.f, 0.f, 0.f, 0.f);
    bool hazard = false;
    warp_box_walk(t, active, qb, [&](int src, int L, const float4& p, int nl) {
        const Box3 hb = shfl_box(qb, src);
        const uint32_t w = __float_as_uint(p.w);
        const bool in = lane < nl && !(w & F_DEL) && qbox_holds(hb, p.x, p.y, p.z);
        const unsigned inb = __ballot_sync(0xffffffffu, in);
        if (inb == 0) return;
        const float mx = __shfl_sync(0xffffffffu, mid.x, src), my = __shfl_sync(0xffffffffu, mid.y, src),
                    mz = __shfl_sync(0xffffffffu, mid.z, src);
        const float f0 = __shfl_sync(0xffffffffu, fk0, src), f1 = __shfl_sync(0xffffffffu, fk1, src),
                    f2 = __shfl_sync(0xffffffffu, mid.w, src);
        bool hz = false;
        if (in) {
            const float pc[3] = {p.x, p.y, p.z};
            const float fk[3] = {f0, f1, f2};
#pragma unroll
            for (int k = 0; k < 3; ++k)
                if (in_voxel_range(pc[k], fk[k], -1.f, ds) || in_voxel_range(pc[k], fk[k], 1.f, ds)) hz = true;
        }
        const unsigned hzb = __ballot_sync(0xffffffffu, hz);
        // the pairs (voxel, slot) of this leaf's hits, for ds_delete_pairs_kernel
        int pbase = 0;
        if (lane == src) pbase = atomicAdd(d.n_pairs, __popc(inb));
        pbase = __shfl_sync(0xffffffffu, pbase, src);
        const int gsrc = __shfl_sync(0xffffffffu, g, src);
        if (in) {
            const int pos = pbase + __popc(inb & ((1u << lane) - 1u));
            if (pos < d.pair_cap) d.pairs[pos] = make_int2(gsrc, L * LEAF_CAP + lane);
        }
        // (distance, id) minimum over the hits: squared distances are >= 0, so
        // their bit patterns order like the values
        const float dd = in ? sq_dist(p.x, p.y, p.z, mx, my, mz) : __int_as_float(0x7f800000);
        const unsigned db = __float_as_uint(dd);
        const unsigned dmin = __reduce_min_sync(0xffffffffu, db);
        const unsigned id = in ? (w & ID_MASK) : 0xffffffffu;
        const unsigned imin = __reduce_min_sync(0xffffffffu, db == dmin ? id : 0xffffffffu);
        const int wl = __ffs(__ballot_sync(0xffffffffu, in && db == dmin && id == imin)) - 1;
        const float bx = __shfl_sync(0xffffffffu, p.x, wl), by = __shfl_sync(0xffffffffu, p.y, wl),
                    bz = __shfl_sync(0xffffffffu, p.z, wl);
        if (lane == src) {
            n0 += __popc(inb);
            hazard = hazard || hzb != 0;
            const float d0 = __uint_as_float(dmin);
            if (d0 < best_d || (d0 == best_d && (int)imin < best_id)) {
                best_d = d0;
                best_id = (int)imin;
                best_slot = L * LEAF_CAP + wl;
                best_p = make_float4(bx, by, bz, 0.f);
            }
        }
    });
    if (!active) return;
    d.g_info[g] = make_int4(n0, best_slot, best_id, hazard ? 1 : 0);
    d.g_best[g] = make_float4(best_p.x, best_p.y, best_p.z, best_d);
    if (hazard) {
        long long cut = first > a ? first : a + 1;
        atomicMin((long long*)&t.st->count, cut);
    }
}

__global__ void __launch_bounds__(128) ds_fold_kernel(DevTree t, long long n, long long a, long long first_id,
                                                      DsScratch d) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= t.st->n_groups) return;
    if (t.st->err & ERR_INPUT) return;  // a non-finite input: the call changes nothing
    // the sub-batch ends where ds_h1_kernel found the first point that must
    // be folded alone (st->count), and holds at least one point
    const long long e = min(max((long long)t.st->count, a + 1), n);
    int j = d.groups[g];
    int4 info = d.g_info[g];
    d.g_out[g] = make_int4(0, 0, 0, 0);
    const uint32_t h = __ldg(d.hkey[0] + j);
    if (j + DS_BIG_RUN < n && __ldg(d.hkey[0] + j + DS_BIG_RUN) == h) {
        // a long hash run (a voxel with many points): folded by a warp
        d.big[atomicAdd(d.n_big, 1)] = g;
        return;
    }
    if (info.y == -1 && info.x == 0 && group_first_from(d, n, j, a) < 0) return;
    const int lead = d.hval[0][j];
    const int4 k = __ldg(d.s_key + j);
    float4 mid = d.mid[lead];
    float4 best = d.g_best[g];
    const int n0 = info.x;
    bool s_is_s0 = true, del_s0 = false, have_ins = false;
    float cx = 0.f, cy = 0.f, cz = 0.f, cd = 0.f;
    long long cid = -1;  // id of the current winner c: a stored point keeps its id
    int triggers = 0;
    for_run(d, n, j, h, [&](long long, const int4& kk, const float4& p) {
        if (!same_key(kk, k)) return true;
        const long long idx = __float_as_int(p.w);
        if (idx < a) return true;
        if (idx >= e) return false;  // members come in increasing index order
        float pd = sq_dist(p.x, p.y, p.z, mid.x, mid.y, mid.z);
        float wx = p.x, wy = p.y, wz = p.z, wd = pd;
        long long wid = first_id + idx;
        bool trig;
        if (s_is_s0) {
            if (n0 > 0 && best.w < pd) {
                wx = best.x; wy = best.y; wz = best.z; wd = best.w;
                wid = info.z;
            }
            trig = n0 > 1 || same_point(p.x, p.y, p.z, wx, wy, wz);
            if (trig) {
                del_s0 = n0 > 0;
                s_is_s0 = false;
            }
        } else {
            if (cd < pd) {
                wx = cx; wy = cy; wz = cz; wd = cd;
                wid = cid;
            }
            trig = same_point(p.x, p.y, p.z, wx, wy, wz);
        }
        if (trig) {
            ++triggers;
            cx = wx; cy = wy; cz = wz; cd = wd;
            cid = wid;
            have_ins = true;
        }
        return true;
    });
    d.g_out[g] = make_int4(del_s0 ? 1 : 0, have_ins ? 1 : 0, triggers, 0);
    if (triggers) atomicAdd((unsigned long long*)&t.st->count2, (unsigned long long)triggers);
    if (have_ins) {
        if (cid > MAX_ID) {
            atomicOr(&t.st->err, ERR_ID);
            return;
        }
        int q = atomicAdd(&t.st->n_ins, 1);
        d.ins[q] = make_float4(cx, cy, cz, __int_as_float((int)cid));
    }
}

// The fold of ds_fold_kernel for the groups it deferred, one warp per group,
// 32 members per step.  After the first member the fold's state is the
// current winner c, and a member p replaces c exactly when d(p) <= d(c) (a
// later point wins ties): c after member i is the minimum of the members so
// far and the initial c (the best stored point of the voxel when it has one)
// under (distance ascending, position descending), a warp prefix minimum.
// Member i triggers (the voxel's points are replaced) when it replaces c,
// when it coincides with c (same_point), or, for a voxel holding more than
// one stored point, when it is the first member.  The point inserted is the
// final c under its own id (the stored point's, or first_id + its index).
__global__ void __launch_bounds__(128) ds_fold_big_kernel(DevTree t, long long n, long long a, long long first_id,
                                                          DsScratch d) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    if (t.st->err & ERR_INPUT) return;
    const long long e = min(max((long long)t.st->count, a + 1), n);
    const int nb = *d.n_big;
    for (int b = warp; b < nb; b += nwarps) {
        const int g = d.big[b];
        const int j = d.groups[g];
        const int4 info = d.g_info[g];
        const float4 best = d.g_best[g];
        const uint32_t h = __ldg(d.hkey[0] + j);
        const int4 k = __ldg(d.s_key + j);
        const float4 mid = d.mid[d.hval[0][j]];
        const int n0 = info.x;
        // running c: distance, position in the run (-2: the stored best,
        // -1: none), coordinates
        float cdist = n0 > 0 ? best.w : __int_as_float(0x7f800000);
        long long cpos = n0 > 0 ? -2 : -1;
        float cx = best.x, cy = best.y, cz = best.z;
        long long cid = n0 > 0 ? (long long)info.z : -1;
        bool first_open = n0 > 1;  // the first member triggers regardless
        int triggers = 0;
        bool more = true;
        for (long long base = j; more && base < n; base += 32) {
            const long long jj = base + lane;
            const uint32_t hh = jj < n ? __ldg(d.hkey[0] + jj) : ~h;
            const unsigned off_run = __ballot_sync(0xffffffffu, hh != h);
            // entries from the first one of another hash on are not in the run
            const int run_end = off_run ? __ffs(off_run) - 1 : 32;
            bool member = false;
            float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
            long long idx = -1;
            if (lane < run_end) {
                const int4 kk = __ldg(d.s_key + jj);
                if (same_key(kk, k)) {
                    p = __ldg(d.s_pts + jj);
                    idx = __float_as_int(p.w);
                    member = idx >= a && idx < e;
                }
            }
            // members come in increasing index order: one at or past e ends the group
            const unsigned past = __ballot_sync(0xffffffffu, idx >= e);
            const int lim = past ? __ffs(past) - 1 : run_end;
            member = member && lane < lim;
            if (off_run || past) more = false;
            const float pd = member ? sq_dist(p.x, p.y, p.z, mid.x, mid.y, mid.z) : __int_as_float(0x7f800000);
            // inclusive prefix minimum over this step's members
            float md = pd;
            int mlane = member ? lane : -1;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const float od = __shfl_up_sync(0xffffffffu, md, o);
                const int ol = __shfl_up_sync(0xffffffffu, mlane, o);
                // (od, ol) is earlier: it stays the minimum only if strictly smaller
                if (lane >= o && ol >= 0 && (mlane < 0 || od < md)) {
                    md = od;
                    mlane = ol;
                }
            }
            // exclusive prefix: the inclusive one of the lane before, then the carry
            float ed = __shfl_up_sync(0xffffffffu, md, 1);
            int el = __shfl_up_sync(0xffffffffu, mlane, 1);
            if (lane == 0) el = -1;
            // c before this member: the carry unless a member of this step beat it
            const bool from_step = el >= 0 && ed <= cdist;
            const float prev_d = from_step ? ed : cdist;
            const int src = from_step ? el : lane;
            const float sx = __shfl_sync(0xffffffffu, p.x, src), sy = __shfl_sync(0xffffffffu, p.y, src),
                        sz = __shfl_sync(0xffffffffu, p.z, src);
            const float prev_x = from_step ? sx : cx, prev_y = from_step ? sy : cy, prev_z = from_step ? sz : cz;
            const bool prev_none = !from_step && cpos == -1;
            const unsigned mem = __ballot_sync(0xffffffffu, member);
            const bool is_first = first_open && mem != 0 && lane == __ffs(mem) - 1;
            const bool replaces = member && pd <= prev_d;
            const bool trig = member && (replaces || is_first ||
                                         (!prev_none && same_point(p.x, p.y, p.z, prev_x, prev_y, prev_z)));
            triggers += __popc(__ballot_sync(0xffffffffu, trig));
            if (mem) first_open = false;
            // carry: the step's minimum over everything, if it beats c
            const float sd = __shfl_sync(0xffffffffu, md, 31);
            const int sl = __shfl_sync(0xffffffffu, mlane, 31);
            if (sl >= 0 && sd <= cdist) {
                cdist = sd;
                cpos = base + sl;
                cx = __shfl_sync(0xffffffffu, p.x, sl);
                cy = __shfl_sync(0xffffffffu, p.y, sl);
                cz = __shfl_sync(0xffffffffu, p.z, sl);
                cid = first_id + __shfl_sync(0xffffffffu, idx, sl);
            }
        }
        if (lane != 0) continue;
        const bool have_ins = triggers > 0;
        d.g_out[g] = make_int4(have_ins && n0 > 0 ? 1 : 0, have_ins ? 1 : 0, triggers, 0);
        if (!have_ins) continue;
        atomicAdd((unsigned long long*)&t.st->count2, (unsigned long long)triggers);
        if (cid > MAX_ID) {
            atomicOr(&t.st->err, ERR_ID);
            continue;
        }
        const int q = atomicAdd(&t.st->n_ins, 1);
        d.ins[q] = make_float4(cx, cy, cz, __int_as_float((int)cid));
    }
}

// Deletes (with the downsample flag) the stored points ds_search_kernel found
// in the boxes of the groups whose fold decided so: one thread per listed
// (group, slot) pair, no tree walk (nothing moved since the search).
__global__ void ds_delete_pairs_kernel(DevTree t, UpdateAux a, DsScratch d) {
    const int np = *d.n_pairs;
    if (np > d.pair_cap || (t.st->err & ERR_INPUT)) return;  // the list overflowed: ds_delete_kernel walks
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const int2 pr = d.pairs[i];
        if (!d.g_out[pr.x].x) continue;
        float* w = &t.pts[pr.y].w;
        *w = __uint_as_float(__float_as_uint(*w) | F_DEL | F_DSDEL);
        mark_dirty(a, t.st, pr.y / LEAF_CAP);
    }
}

// The same deletion by walking the tree from every voxel box, when the pair
// list overflowed.
__global__ void __launch_bounds__(128) ds_delete_kernel(DevTree t, UpdateAux a, DsScratch d) {
    if (*d.n_pairs <= d.pair_cap) return;  // ds_delete_pairs_kernel did it
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool active = g < t.st->n_groups && !(t.st->err & ERR_INPUT) && d.g_out[g].x;
    const Box3 qb = active ? group_box(d, d.hval[0][d.groups[g]]) : empty_box();
    warp_box_walk(t, active, qb, [&](int src, int L, const float4& p, int nl) {
        const Box3 hb = shfl_box(qb, src);
        const uint32_t w = __float_as_uint(p.w);
        const bool in = lane < nl && !(w & F_DEL) && qbox_holds(hb, p.x, p.y, p.z);
        if (in) t.pts[(long long)L * LEAF_CAP + lane].w = __uint_as_float(w | F_DEL | F_DSDEL);
        const unsigned inb = __ballot_sync(0xffffffffu, in);
        if (inb != 0 && lane == src) mark_dirty(a, t.st, L);
    });
}

__global__ void pack_points_kernel(DevTree t, const float* __restrict__ in, int stride, long long n, long long first_id,
                                   float4* __restrict__ out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x = in[i * stride], y = in[i * stride + 1], z = in[i * stride + 2];
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) atomicOr(&t.st->err, ERR_INPUT);
    long long id = first_id + i;
    if (id > MAX_ID) atomicOr(&t.st->err, ERR_ID);
    out[i] = make_float4(x, y, z, __int_as_float((int)(id & ID_MASK)));
}

__global__ void check_finite_kernel(DevTree t, const float* __restrict__ in, long long count) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    if (!isfinite(in[i])) atomicOr(&t.st->err, ERR_INPUT);
}

inline size_t au(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

void launch_route_append(const DevTree& t, const UpdateAux& a, const float4* pts, long long n, int4* ovf_leaf,
                         float4* ovf_pts, cudaStream_t s) {
    if (n <= 0) return;
    route_append_kernel<<<blocks_for(n, 256), 256, 0, s>>>(t, a, pts, n, nullptr, ovf_leaf, ovf_pts);
}

void launch_route_append_dev_count(const DevTree& t, const UpdateAux& a, const float4* pts, long long n_bound,
                                   const int* n_dev, int4* ovf_leaf, float4* ovf_pts, cudaStream_t s) {
    if (n_bound <= 0) return;
    route_append_kernel<<<blocks_for(n_bound, 256), 256, 0, s>>>(t, a, pts, n_bound, n_dev, ovf_leaf, ovf_pts);
}

void launch_refit(const DevTree& t, const UpdateAux& a, const int* items, const int* n_items, int max_items,
                  const Criteria& c, cudaStream_t s) {
    if (max_items <= 0) return;
    refit_mark_kernel<<<blocks_for(max_items, 256), 256, 0, s>>>(t, a, items, n_items);
    refit_compute_kernel<<<blocks_for(max_items, 128), 128, 0, s>>>(t, a, items, n_items, c, c.fill);
}


void launch_select_jobs(const DevTree& t, const UpdateAux& a, int max_viol, cudaStream_t s) {
    if (max_viol <= 0) return;
    select_jobs_kernel<<<blocks_for(max_viol, 256), 256, 0, s>>>(t, a, &t.st->n_viol);
    clear_viol_kernel<<<blocks_for(max_viol, 256), 256, 0, s>>>(a, &t.st->n_viol);
}

void launch_clear_viol(const DevTree& t, const UpdateAux& a, int max_viol, cudaStream_t s) {
    if (max_viol <= 0) return;
    clear_viol_kernel<<<blocks_for(max_viol, 256), 256, 0, s>>>(a, &t.st->n_viol);
}

void launch_job_count(const DevTree& t, const UpdateAux& a, int leaf_top, int node_top, const int4* ovf_leaf,
                      int max_ovf, int max_jobs, void* scan_temp, cudaStream_t s) {
    if (leaf_top > 0) job_count_leaf_kernel<<<blocks_for(leaf_top, 256), 256, 0, s>>>(t, a, leaf_top);
    if (node_top > 1) job_count_node_kernel<<<blocks_for(node_top, 256), 256, 0, s>>>(t, a, node_top);
    if (max_ovf > 0) job_count_ovf_kernel<<<blocks_for(max_ovf, 256), 256, 0, s>>>(t, a, ovf_leaf, &t.st->n_ovf);
    // job_off = exclusive scan of job_count over max_jobs entries (unused tail
    // entries are zero); the total lands in job_count[max_jobs].
    exclusive_scan(a.job_count, a.job_off, max_jobs, a.job_off + max_jobs, scan_temp, s);
    job_max_kernel<<<blocks_for(max_jobs, 256), 256, 0, s>>>(t, a, &t.st->n_jobs, a.job_off + max_jobs);
}

void launch_select_and_count(const DevTree& t, const UpdateAux& a, int leaf_top, int node_top, const int4* ovf_leaf,
                             int max_ovf, cudaStream_t s) {
    // the violator count is only on the device: fixed grids, grid-stride loops
    select_jobs_kernel<<<SPEC_BLOCKS, 256, 0, s>>>(t, a, &t.st->n_viol);
    clear_viol_kernel<<<SPEC_BLOCKS, 256, 0, s>>>(a, &t.st->n_viol);
    if (leaf_top > 0) job_count_leaf_kernel<<<blocks_for(leaf_top, 256), 256, 0, s>>>(t, a, leaf_top);
    if (node_top > 1) job_count_node_kernel<<<blocks_for(node_top, 256), 256, 0, s>>>(t, a, node_top);
    if (max_ovf > 0) job_count_ovf_kernel<<<blocks_for(max_ovf, 256), 256, 0, s>>>(t, a, ovf_leaf, &t.st->n_ovf);
    job_scan_kernel<<<1, 1024, 0, s>>>(t, a);
}

void launch_job_gather(const DevTree& t, const UpdateAux& a, int leaf_top, int node_top, const int4* ovf_leaf,
                       const float4* ovf_pts, int max_ovf, float4* out, float4* removed, long long removed_cap,
                       cudaStream_t s) {
    if (leaf_top > 0)
        job_gather_leaf_kernel<<<blocks_for(leaf_top, 256), 256, 0, s>>>(t, a, leaf_top, out, removed, removed_cap);
    if (node_top > 1) job_gather_node_kernel<<<blocks_for(node_top, 256), 256, 0, s>>>(t, a, node_top);
    if (max_ovf > 0)
        job_gather_ovf_kernel<<<blocks_for(max_ovf, 256), 256, 0, s>>>(t, a, ovf_leaf, ovf_pts, &t.st->n_ovf, out);
}

void launch_job_finish(const DevTree& t, const UpdateAux& a, int max_jobs, cudaStream_t s) {
    job_finish_kernel<<<blocks_for(max_jobs > 0 ? max_jobs : 1, 256), 256, 0, s>>>(t, a, &t.st->n_jobs);
}

void launch_delete_boxes(const DevTree& t, const UpdateAux& a, const float* boxes, long long m, uint32_t flags,
                         long long* total, cudaStream_t s) {
    if (m <= 0) return;
    int bits = box_split_bits(m);
    box_edit_kernel<0><<<box_grid(m << bits), DB_THREADS, 0, s>>>(t, a, boxes, m, bits, flags, total);
}

void launch_add_boxes(const DevTree& t, const UpdateAux& a, const float* boxes, long long m, cudaStream_t s) {
    if (m <= 0) return;
    int bits = box_split_bits(m);
    box_edit_kernel<1><<<box_grid(m << bits), DB_THREADS, 0, s>>>(t, a, boxes, m, bits, 0u, nullptr);
}

void launch_delete_points(const DevTree& t, const UpdateAux& a, const float* pts, int stride, long long n,
                          cudaStream_t s) {
    if (n <= 0) return;
    delete_points_kernel<<<blocks_for(n, 128), 128, 0, s>>>(t, a, pts, stride, n);
}

void launch_snapshot_root(const DevTree& t, cudaStream_t s) { snapshot_root_kernel<<<1, 1, 0, s>>>(t); }

void launch_set_ll(long long* p, long long v, cudaStream_t s) { set_ll_kernel<<<1, 1, 0, s>>>(p, v); }

void launch_validate(const DevTree& t, const UpdateAux& a, bool at_rest, long long* bad, cudaStream_t s) {
    if (t.node_cap > 0)
        validate_nodes_kernel<<<blocks_for(t.node_cap, 256), 256, 0, s>>>(t, at_rest, (unsigned long long*)bad);
    if (t.leaf_cap > 0)
        validate_leaves_kernel<<<blocks_for(t.leaf_cap, 256), 256, 0, s>>>(t, (unsigned long long*)bad);
    if (t.node_cap > 0)
        validate_aux_nodes_kernel<<<blocks_for(t.node_cap, 256), 256, 0, s>>>(t, a, at_rest, (unsigned long long*)bad);
    if (t.leaf_cap > 0)
        validate_aux_leaves_kernel<<<blocks_for(t.leaf_cap, 256), 256, 0, s>>>(t, a, (unsigned long long*)bad);
}

void launch_flatten(const DevTree& t, float4* out, long long* counter, cudaStream_t s) {
    if (t.leaf_cap <= 0) return;
    flatten_kernel<<<blocks_for(t.leaf_cap, 256), 256, 0, s>>>(t, out, counter);
}

void launch_stored_ids(const DevTree& t, int* out, long long cap, long long* counter, cudaStream_t s) {
    if (t.leaf_cap <= 0) return;
    stored_ids_kernel<<<blocks_for(t.leaf_cap, 256), 256, 0, s>>>(t, out, cap, counter);
}

void launch_select_root_job(const DevTree& t, const UpdateAux& a, cudaStream_t s) {
    select_root_job_kernel<<<1, 1, 0, s>>>(t, a);
}

void launch_pack_points(const DevTree& t, const float* in, int stride, long long n, long long first_id, float4* out,
                        cudaStream_t s) {
    if (n <= 0) return;
    pack_points_kernel<<<blocks_for(n, 256), 256, 0, s>>>(t, in, stride, n, first_id, out);
}

void launch_check_finite(const DevTree& t, const float* in, long long count, cudaStream_t s) {
    if (count <= 0) return;
    check_finite_kernel<<<blocks_for(count, 256), 256, 0, s>>>(t, in, count);
}

size_t ds_scratch_bytes(long long n, long long pair_cap) {
    size_t b = 0;
    b += au(sizeof(int2) * pair_cap) + au(sizeof(int));  // pairs, n_pairs
    b += 5 * au(sizeof(float4) * n);   // pts, box_lo, box_hi, mid, ins
    b += 2 * au(sizeof(int4) * n);     // key, s_key
    b += au(sizeof(float4) * n);       // s_pts
    b += 4 * au(sizeof(uint32_t) * n); // hkey x2, hval x2
    b += au(sizeof(int) * n);          // groups
    b += 2 * au(sizeof(int4) * n);     // g_info, g_out
    b += au(sizeof(float4) * n);       // g_best
    b += au(sizeof(int) * n) + au(sizeof(int));  // big, n_big
    b += au(sort_temp_bytes(n, 1));
    return b;
}

void carve_ds_scratch(void* base, long long n, long long pair_cap, DsScratch* d) {
    char* p = (char*)base;
    auto take = [&](size_t bytes) {
        void* r = p;
        p += (bytes + 255) & ~(size_t)255;
        return r;
    };
    d->pts = (float4*)take(sizeof(float4) * n);
    d->box_lo = (float4*)take(sizeof(float4) * n);
    d->box_hi = (float4*)take(sizeof(float4) * n);
    d->mid = (float4*)take(sizeof(float4) * n);
    d->ins = (float4*)take(sizeof(float4) * n);
    d->key = (int4*)take(sizeof(int4) * n);
    d->s_key = (int4*)take(sizeof(int4) * n);
    d->s_pts = (float4*)take(sizeof(float4) * n);
    d->hkey[0] = (uint32_t*)take(sizeof(uint32_t) * n);
    d->hkey[1] = (uint32_t*)take(sizeof(uint32_t) * n);
    d->hval[0] = (uint32_t*)take(sizeof(uint32_t) * n);
    d->hval[1] = (uint32_t*)take(sizeof(uint32_t) * n);
    d->groups = (int*)take(sizeof(int) * n);
    d->g_info = (int4*)take(sizeof(int4) * n);
    d->g_out = (int4*)take(sizeof(int4) * n);
    d->g_best = (float4*)take(sizeof(float4) * n);
    d->big = (int*)take(sizeof(int) * n);
    d->n_big = (int*)take(sizeof(int));
    d->pairs = (int2*)take(sizeof(int2) * pair_cap);
    d->n_pairs = (int*)take(sizeof(int));
    d->pair_cap = (int)pair_cap;
    d->temp = (void*)p;
}

void launch_ds_prepare(const DevTree& t, const float* in, int stride, long long n, float ds, DsScratch& d,
                       cudaStream_t s) {
    if (n <= 0) return;
    ds_prepare_kernel<<<blocks_for(n, 256), 256, 0, s>>>(t, in, stride, n, ds, d);
    // 24-bit keys: three passes; the sorted pairs stay where the last pass
    // left them
    if (radix_sort_pairs(d.hkey[0], d.hval[0], d.hkey[1], d.hval[1], n, 1, n, DS_HASH_BITS, d.temp, s, false)) {
        std::swap(d.hkey[0], d.hkey[1]);
        std::swap(d.hval[0], d.hval[1]);
    }
    ds_leaders_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, d, t.st);
}

void launch_ds_search(const DevTree& t, long long n, float ds, long long a, DsScratch& d, int max_groups,
                      cudaStream_t s) {
    if (n - a > 0) ds_h1_kernel<<<blocks_for(n - a, 256), 256, 0, s>>>(n, a, d, t.st);
    if (max_groups > 0) ds_search_kernel<<<blocks_for(max_groups, 128), 128, 0, s>>>(t, n, a, d, ds);
}

void launch_ds_fold(const DevTree& t, const UpdateAux& aux, long long n, long long a, long long first_id,
                    DsScratch& d, int max_groups, cudaStream_t s) {
    if (max_groups <= 0) return;
    ds_fold_kernel<<<blocks_for(max_groups, 128), 128, 0, s>>>(t, n, a, first_id, d);
    ds_fold_big_kernel<<<DS_BIG_BLOCKS, 128, 0, s>>>(t, n, a, first_id, d);
    ds_delete_pairs_kernel<<<SPEC_BLOCKS, 256, 0, s>>>(t, aux, d);
    ds_delete_kernel<<<blocks_for(max_groups, 128), 128, 0, s>>>(t, aux, d);
}

}  // namespace ikdg
