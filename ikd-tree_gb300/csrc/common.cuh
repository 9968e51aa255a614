// Device-side layout of the incremental k-d tree and the arithmetic shared by
// every kernel.
//
// The tree replaces the reference's pointer nodes (KD_TREE_NODE,
// ikd-Tree/ikd_Tree.h:64-86) with two pools in HBM:
//
//   * internal nodes: a 64-byte record (4 x float4) per node that carries the
//     AABBs of BOTH children, the two child codes, the split value and the
//     split axis.  One record load decides which children a query visits.
//     Beside it: per-child slot / deleted counts (int4) and the parent link.
//   * leaf buckets: LEAF_CAP float4 slots per leaf, {x, y, z, id | flags}.
//
// Child code: > 0 internal node, < 0 leaf (-(leaf + 1)), 0 none.  Node 0 is a
// sentinel whose left child is the root (the role of STATIC_ROOT_NODE,
// ikd_Tree.cpp:358-363), so the root's AABB and counts live in node 0's record
// like every other child's.
//
// Deletion is a flag in the slot's id word: F_DEL marks a deleted point,
// F_DSDEL additionally marks a point removed by voxel downsampling (the
// reference's point_downsample_deleted, ikd_Tree.h:72).  AABBs always bound the
// non-deleted points of a subtree (Update, ikd_Tree.cpp:1183-1323).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ikdg {

constexpr int LEAF_CAP = 32;       // slots per leaf bucket
constexpr int MAX_STACK = 64;      // traversal stack entries (tree depth bound)
constexpr uint32_t ID_MASK = 0x3fffffffu;
constexpr uint32_t F_DEL = 0x80000000u;
constexpr uint32_t F_DSDEL = 0x40000000u;
constexpr int MAX_ID = 0x3fffffff;

// Error bits in DevStatus::err.
constexpr int ERR_STACK = 1;       // a traversal exceeded MAX_STACK
constexpr int ERR_POOL = 2;        // node or leaf pool exhausted
constexpr int ERR_OUTPUT = 4;      // an output capacity was exceeded
constexpr int ERR_ID = 8;          // point id space exhausted
constexpr int ERR_INPUT = 16;      // non-finite input coordinate
constexpr int ERR_LOOP = 32;       // a bounded device loop hit its cap
constexpr int ERR_POOL_LEAF = 64;  // leaf pool exhausted
constexpr int ERR_SEG = 128;       // builder segment list overflow
constexpr int ERR_ROUTE = 256;     // insertion into a tree without root
constexpr int ERR_OVF_JOB = 512;   // overflow point outside every rebuild job
constexpr int ERR_LIST = 1024;     // a work list would exceed its capacity
constexpr int ERR_ANY_INTERNAL = ERR_POOL | ERR_LOOP | ERR_POOL_LEAF | ERR_SEG | ERR_ROUTE | ERR_OVF_JOB | ERR_LIST;

// Caps on every device loop that follows tree links: a walk to the root takes
// at most MAX_WALK steps, a traversal at most MAX_VISITS node / leaf visits.
// Hitting a cap sets ERR_LOOP and ends the loop (never expected; it turns a
// corrupted tree into an error instead of a hung GPU).
constexpr int MAX_WALK = 4 * MAX_STACK;
constexpr int MAX_VISITS = 1 << 26;

__host__ __device__ inline bool code_is_leaf(int c) { return c < 0; }
__host__ __device__ inline int code_leaf(int c) { return -c - 1; }
__host__ __device__ inline int leaf_code(int l) { return -(l + 1); }

// Device-resident counters, read back by the host after each API call.
struct DevStatus {
    int node_top;         // bump pointer of the node pool
    int leaf_top;         // bump pointer of the leaf pool
    int free_node_n;      // entries on the node free stack
    int free_leaf_n;
    int free_node_taken;  // pops during the current build
    int free_leaf_taken;
    int err;              // ERR_* bits
    int n_items;          // refit start codes queued
    int n_jobs;           // rebuild jobs selected
    int n_viol;           // criterion violators recorded
    int n_ovf;            // points that did not fit their leaf
    int n_ins;            // downsampling winners to insert
    int n_groups;         // downsampling voxel groups
    int max_job;          // largest rebuild job (points)
    int root_code;        // snapshot of the sentinel's left child
    int root_slots;       // size(): stored slots, deleted ones included
    int root_deleted;     // deleted slots; validnum() = slots - deleted
    int root_height;
    long long count;      // generic result counter
    long long count2;
    long long removed_n;  // deleted points dropped by rebuilds, not yet drained
    long long job_total;  // points gathered for rebuild jobs
    int dbg[8];           // details of the first internal error (diagnostics)
    long long bad;        // structural violations found by the validator
};

struct DevTree {
    float4* node;        // [node_cap * 4]
    int4* ncnt;          // [node_cap] {slots L, deleted L, slots R, deleted R}
    int* nparent;        // [node_cap] parent * 2 + side, -1 when free
    int* nheight;        // [node_cap] height of the subtree (leaves: 0)
    float4* pts;         // [leaf_cap * LEAF_CAP]
    int* leaf_n;         // [leaf_cap] slots used
    int* lparent;        // [leaf_cap] parent * 2 + side, -1 when free
    int* free_node;      // [node_cap]
    int* free_leaf;      // [leaf_cap]
    int node_cap;
    int leaf_cap;
    DevStatus* st;
};

struct Box3 {
    float lo[3], hi[3];
};

// ---------------------------------------------------------------------------
// Exact float arithmetic.  Squared distances follow calc_dist
// (ikd_Tree.cpp:1374-1378): ((dx*dx + dy*dy) + dz*dz), every product and sum
// rounded separately (no FMA contraction).
__device__ __forceinline__ float sq_dist(float qx, float qy, float qz, float px, float py, float pz) {
    float dx = __fsub_rn(qx, px), dy = __fsub_rn(qy, py), dz = __fsub_rn(qz, pz);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// Lower bound of sq_dist over an AABB, in calc_box_dist's order
// (ikd_Tree.cpp:1381-1391).  Rounding is monotone, so for every point p inside
// the box box_dist <= sq_dist(q, p) holds exactly in float.
__device__ __forceinline__ float axis_gap(float q, float lo, float hi) {
    float g = 0.f;
    if (q < lo) g = __fsub_rn(q, lo);
    if (q > hi) g = __fsub_rn(q, hi);
    return __fmul_rn(g, g);
}
__device__ __forceinline__ float box_dist(float qx, float qy, float qz, float lx, float ly, float lz,
                                          float hx, float hy, float hz) {
    return __fadd_rn(__fadd_rn(axis_gap(qx, lx, hx), axis_gap(qy, ly, hy)), axis_gap(qz, lz, hz));
}
// Upper bound of sq_dist over an AABB (farthest corner, same order): every
// point p inside satisfies sq_dist(q, p) <= box_far.
__device__ __forceinline__ float axis_far(float q, float lo, float hi) {
    float a = fabsf(__fsub_rn(q, lo)), b = fabsf(__fsub_rn(q, hi));
    float g = fmaxf(a, b);
    return __fmul_rn(g, g);
}
__device__ __forceinline__ float box_far(float qx, float qy, float qz, float lx, float ly, float lz,
                                         float hx, float hy, float hz) {
    return __fadd_rn(__fadd_rn(axis_far(qx, lx, hx), axis_far(qy, ly, hy)), axis_far(qz, lz, hz));
}

// Order-preserving float -> uint32 map for radix sorting.
__host__ __device__ inline uint32_t float_key(float f) {
    uint32_t u;
#ifdef __CUDA_ARCH__
    u = __float_as_uint(f);
#else
    memcpy(&u, &f, 4);
#endif
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// ---------------------------------------------------------------------------
// Node record access.  Record n = node[4n .. 4n+3]:
//   f0 = {L.lo.x, L.lo.y, L.lo.z, L.hi.x}
//   f1 = {L.hi.y, L.hi.z, R.lo.x, R.lo.y}
//   f2 = {R.lo.z, R.hi.x, R.hi.y, R.hi.z}
//   f3 = {code L, code R, split, axis}   (codes and axis as int bits)
struct NodeRec {
    float4 f0, f1, f2, f3;
    __device__ __forceinline__ int left() const { return __float_as_int(f3.x); }
    __device__ __forceinline__ int right() const { return __float_as_int(f3.y); }
    __device__ __forceinline__ float split() const { return f3.z; }
    __device__ __forceinline__ int axis() const { return __float_as_int(f3.w); }
    __device__ __forceinline__ Box3 box(int side) const {
        Box3 b;
        if (side == 0) {
            b.lo[0] = f0.x; b.lo[1] = f0.y; b.lo[2] = f0.z;
            b.hi[0] = f0.w; b.hi[1] = f1.x; b.hi[2] = f1.y;
        } else {
            b.lo[0] = f1.z; b.lo[1] = f1.w; b.lo[2] = f2.x;
            b.hi[0] = f2.y; b.hi[1] = f2.z; b.hi[2] = f2.w;
        }
        return b;
    }
};

// Read-only node record: two 256-bit loads (records are 64-byte aligned).
__device__ __forceinline__ NodeRec load_node(const float4* __restrict__ node, int n) {
    NodeRec r;
    const float4* p = node + 4 * n;
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(r.f0.x), "=f"(r.f0.y), "=f"(r.f0.z), "=f"(r.f0.w), "=f"(r.f1.x), "=f"(r.f1.y),
                   "=f"(r.f1.z), "=f"(r.f1.w)
                 : "l"(p));
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(r.f2.x), "=f"(r.f2.y), "=f"(r.f2.z), "=f"(r.f2.w), "=f"(r.f3.x), "=f"(r.f3.y),
                   "=f"(r.f3.z), "=f"(r.f3.w)
                 : "l"(p + 2));
    return r;
}

// Coherent (L1-bypassing) record load for kernels that read records other
// threads of the same launch have just written.
__device__ __forceinline__ NodeRec load_node_cg(const float4* node, int n) {
    NodeRec r;
    r.f0 = __ldcg(node + 4 * n + 0);
    r.f1 = __ldcg(node + 4 * n + 1);
    r.f2 = __ldcg(node + 4 * n + 2);
    r.f3 = __ldcg(node + 4 * n + 3);
    return r;
}

__device__ __forceinline__ bool box_empty(const Box3& b) { return !(b.lo[0] <= b.hi[0]); }

__device__ __forceinline__ void write_child_box(float4* node, int n, int side, const Box3& b) {
    float* f = reinterpret_cast<float*>(node + 4 * n);
    int o = side == 0 ? 0 : 6;
    f[o + 0] = b.lo[0]; f[o + 1] = b.lo[1]; f[o + 2] = b.lo[2];
    f[o + 3] = b.hi[0]; f[o + 4] = b.hi[1]; f[o + 5] = b.hi[2];
}
__device__ __forceinline__ void write_child_code(float4* node, int n, int side, int code) {
    int* f = reinterpret_cast<int*>(node + 4 * n);
    f[12 + side] = code;
}
__device__ __forceinline__ void write_child_cnt(int4* ncnt, int n, int side, int slots, int deleted) {
    int* c = reinterpret_cast<int*>(ncnt + n);
    c[2 * side] = slots;
    c[2 * side + 1] = deleted;
}

__device__ __forceinline__ Box3 empty_box() {
    Box3 b;
    for (int a = 0; a < 3; ++a) {
        b.lo[a] = __int_as_float(0x7f800000);   // +inf
        b.hi[a] = __int_as_float(0xff800000);   // -inf
    }
    return b;
}

__device__ __forceinline__ void box_grow(Box3& b, float x, float y, float z) {
    b.lo[0] = fminf(b.lo[0], x); b.hi[0] = fmaxf(b.hi[0], x);
    b.lo[1] = fminf(b.lo[1], y); b.hi[1] = fmaxf(b.hi[1], y);
    b.lo[2] = fminf(b.lo[2], z); b.hi[2] = fmaxf(b.hi[2], z);
}
__device__ __forceinline__ void box_union(Box3& b, const Box3& o) {
    for (int a = 0; a < 3; ++a) {
        b.lo[a] = fminf(b.lo[a], o.lo[a]);
        b.hi[a] = fmaxf(b.hi[a], o.hi[a]);
    }
}

// Half-open box tests of Search_by_range / Delete_by_range
// (ikd_Tree.cpp:1019-1026, :653-670).  `q` is the query box {min, max}.
__device__ __forceinline__ bool qbox_disjoint(const Box3& q, const Box3& n) {
    for (int a = 0; a < 3; ++a)
        if (q.hi[a] <= n.lo[a] || q.lo[a] > n.hi[a]) return true;
    return false;
}
__device__ __forceinline__ bool qbox_covers(const Box3& q, const Box3& n) {
    for (int a = 0; a < 3; ++a)
        if (!(q.lo[a] <= n.lo[a] && q.hi[a] > n.hi[a])) return false;
    return true;
}
__device__ __forceinline__ bool qbox_holds(const Box3& q, float x, float y, float z) {
    return q.lo[0] <= x && q.hi[0] > x && q.lo[1] <= y && q.hi[1] > y && q.lo[2] <= z && q.hi[2] > z;
}

// Pool allocation: pop the free stack first, then bump.  Returns -1 and sets
// ERR_POOL when the pool is exhausted (the host sizes pools beforehand).
__device__ __forceinline__ int alloc_node(const DevTree& t) {
    int k = atomicAdd(&t.st->free_node_taken, 1);
    if (k < t.st->free_node_n) return t.free_node[t.st->free_node_n - 1 - k];
    int n = atomicAdd(&t.st->node_top, 1);
    if (n >= t.node_cap) {
        atomicOr(&t.st->err, ERR_POOL);
        return -1;
    }
    return n;
}
// Bulk form of the same allocation for `c` items at once: one reservation on
// the shared counters (free stack first, then bump), then item j of the run
// resolves to its index without further atomics.
struct PoolRun {
    int base;   // first free-stack slot taken
    int nfree;  // items served by the free stack
    int top;    // first bumped index
};
__device__ __forceinline__ PoolRun pool_reserve(int* taken, int free_n, int* top, int c) {
    PoolRun r;
    r.base = c > 0 ? atomicAdd(taken, c) : 0;
    r.nfree = min(max(free_n - r.base, 0), c);
    r.top = c - r.nfree > 0 ? atomicAdd(top, c - r.nfree) : 0;
    return r;
}
__device__ __forceinline__ int pool_pick(const PoolRun& r, const int* free_list, int free_n, int cap, int j,
                                         DevStatus* st, int err) {
    if (j < r.nfree) return free_list[free_n - 1 - (r.base + j)];
    const int x = r.top + (j - r.nfree);
    if (x >= cap) {
        atomicOr(&st->err, err);
        return -1;
    }
    return x;
}
__device__ __forceinline__ int alloc_leaf(const DevTree& t) {
    int k = atomicAdd(&t.st->free_leaf_taken, 1);
    if (k < t.st->free_leaf_n) return t.free_leaf[t.st->free_leaf_n - 1 - k];
    int n = atomicAdd(&t.st->leaf_top, 1);
    if (n >= t.leaf_cap) {
        atomicOr(&t.st->err, ERR_POOL_LEAF);
        return -1;
    }
    return n;
}

}  // namespace ikdg
