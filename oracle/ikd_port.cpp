// CPU restatement of the ikd-Tree algorithm (hku-mars/ikd-Tree,
// ikd-Tree/ikd_Tree.cpp) behind the oracle C API (oracle/oracle_capi.h).
//
// TEST INFRASTRUCTURE ONLY.  It is the oracle on machines where the reference
// sources are absent, and the timed CPU baseline there.  It is pinned against
// the unmodified reference (oracle/_ref) by tests/test_oracle.py and the
// golden fixtures in tests/golden/.
//
// What it keeps from the reference, step for step: one point per node with the
// subtree AABB, size, invalid and downsample-deleted counts and lazy labels;
// the median build on the longest AABB axis (nth_element at (l+r)>>1);
// scapegoat rebuilds on the alpha_bal / alpha_del criteria; the bounded
// max-heap kNN with its distance comparator; half-open box tests; the radius
// search with its whole-subtree shortcut; the voxel downsampling of Add_Points.
//
// One deliberate simplification: the reference hands rebuilds of subtrees
// with >= 1500 points to a background thread that replays logged operations
// afterwards (ikd_Tree.cpp:200-315, :624-633).  Here every rebuild runs inline
// at the point where the reference would enqueue it.  Once the reference's
// thread is idle both produce the same set of valid points.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>
#include <pthread.h>
#include <omp.h>

#include "oracle_capi.h"

namespace port {

constexpr double kEps = 1e-6;            // EPSS, ikd_Tree.h:13
constexpr int kMinUnbalanced = 10;       // Minimal_Unbalanced_Tree_Size, ikd_Tree.h:14

struct Pt {
    float x, y, z;
};

struct Box {
    float lo[3], hi[3];
};

inline float coord(const Pt& p, int a) { return a == 0 ? p.x : (a == 1 ? p.y : p.z); }

// calc_dist, ikd_Tree.cpp:1374-1378: ((dx*dx + dy*dy) + dz*dz), unfused.
inline float sqdist(const Pt& a, const Pt& b) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return dx * dx + dy * dy + dz * dz;
}

// same_point, ikd_Tree.cpp:1368-1371.
inline bool near_same(const Pt& a, const Pt& b) {
    return std::fabs(a.x - b.x) < kEps && std::fabs(a.y - b.y) < kEps && std::fabs(a.z - b.z) < kEps;
}

// Node record: the fields of KD_TREE_NODE (ikd_Tree.h:64-86), kept the same
// size class (a per-node mutex included) so the pointer-chasing cost is alike.
struct Node {
    Pt p{};
    uint8_t axis = 0;
    int size = 1, invalid = 0, down_del = 0;
    bool pt_del = false, sub_del = false, pt_ds = false, sub_ds = false;
    bool push_l = false, push_r = false;
    float radius_sq = 0.f;
    pthread_mutex_t lock;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    Node *l = nullptr, *r = nullptr, *parent = nullptr;
    float a_del = 0.f, a_bal = 0.5f;
    Node() { pthread_mutex_init(&lock, nullptr); }
    ~Node() { pthread_mutex_destroy(&lock); }
};

// calc_box_dist, ikd_Tree.cpp:1381-1391 (accumulated x, y, z in order).
inline float box_sqdist(const Node* n, const Pt& q) {
    if (n == nullptr) return INFINITY;
    float d = 0.0f;
    const float qv[3] = {q.x, q.y, q.z};
    for (int a = 0; a < 3; ++a) {
        if (qv[a] < n->lo[a]) d += (qv[a] - n->lo[a]) * (qv[a] - n->lo[a]);
        if (qv[a] > n->hi[a]) d += (qv[a] - n->hi[a]) * (qv[a] - n->hi[a]);
    }
    return d;
}

// PointType_CMP ordering, ikd_Tree.h:95-106.
struct Cand {
    Pt p;
    float d;
};
inline bool cand_less(const Cand& a, const Cand& b) {
    if (std::fabs(a.d - b.d) < 1e-10) return a.p.x < b.p.x;
    return a.d < b.d;
}

// Bounded max-heap with the reference's push / pop rules (MANUAL_HEAP,
// ikd_Tree.h:108-172): push is ignored when full; pop moves the last entry to
// the top and sifts it down.
struct CandHeap {
    std::vector<Cand> h;
    int cap;
    explicit CandHeap(int c) : cap(c) { h.reserve(c > 0 ? c : 1); }
    int size() const { return (int)h.size(); }
    const Cand& top() const { return h[0]; }
    void push(const Cand& c) {
        if ((int)h.size() >= cap) return;
        int i = (int)h.size();
        h.push_back(c);
        while (i > 0) {
            int up = (i - 1) / 2;
            if (!cand_less(h[up], c)) break;
            h[i] = h[up];
            i = up;
        }
        h[i] = c;
    }
    void pop() {
        if (h.empty()) return;
        Cand last = h.back();
        h.pop_back();
        int n = (int)h.size();
        if (n == 0) return;
        int i = 0, c = 1;
        while (c < n) {
            if (c + 1 < n && cand_less(h[c], h[c + 1])) ++c;
            if (!cand_less(last, h[c])) break;
            h[i] = h[c];
            i = c;
            c = 2 * i + 1;
        }
        h[i] = last;
    }
};

class Tree {
   public:
    Tree(float del, float bal, float box) : del_param_(del), bal_param_(bal), ds_(box) {}
    ~Tree() { free_subtree(&root_); delete sentinel_; }

    // Build, ikd_Tree.cpp:352-364.
    void build(std::vector<Pt> pts) {
        if (root_ != nullptr) free_subtree(&root_);
        if (pts.empty()) return;
        delete sentinel_;
        sentinel_ = new Node;
        clear_node(sentinel_);
        build_rec(&sentinel_->l, 0, (int)pts.size() - 1, pts);
        update(sentinel_);
        sentinel_->size = 0;
        root_ = sentinel_->l;
    }

    // Nearest_Search, ikd_Tree.cpp:366-397.
    int nearest(const Pt& q, int k, double max_dist, Pt* out_p, float* out_d) {
        if (k <= 0) return 0;  // the reference reads an empty heap's top here
        CandHeap heap(2 * k);
        knn_rec(root_, k, q, heap, max_dist);
        int found = std::min(k, heap.size());
        for (int i = found - 1; i >= 0; --i) {  // popped largest-first, stored from the back
            out_p[i] = heap.top().p;
            out_d[i] = heap.top().d;
            heap.pop();
        }
        return found;
    }

    void box_search(const Box& b, std::vector<Pt>& out) {
        out.clear();
        range_rec(root_, b, out);
    }

    void radius_search(const Pt& q, float r, std::vector<Pt>& out) {
        out.clear();
        radius_rec(root_, q, r, out);
    }

    // Add_Points, ikd_Tree.cpp:413-489 (the single-threaded branches).
    int add_points(const std::vector<Pt>& pts, bool downsample) {
        int inserted = 0;
        for (const Pt& p : pts) {
            if (!downsample) {
                add_rec(&root_, p, true, root_axis());
                continue;
            }
            Box vox;
            const float pv[3] = {p.x, p.y, p.z};
            for (int a = 0; a < 3; ++a) {
                vox.lo[a] = std::floor(pv[a] / ds_) * ds_;
                vox.hi[a] = vox.lo[a] + ds_;
            }
            Pt centre;
            centre.x = vox.lo[0] + (vox.hi[0] - vox.lo[0]) / 2.0;
            centre.y = vox.lo[1] + (vox.hi[1] - vox.lo[1]) / 2.0;
            centre.z = vox.lo[2] + (vox.hi[2] - vox.lo[2]) / 2.0;
            std::vector<Pt> inside;
            range_rec(root_, vox, inside);
            float best = sqdist(p, centre);
            Pt winner = p;
            for (const Pt& s : inside) {
                float d = sqdist(s, centre);
                if (d < best) {
                    best = d;
                    winner = s;
                }
            }
            if (inside.size() > 1 || near_same(p, winner)) {
                if (!inside.empty()) delete_range_rec(&root_, vox, true, true);
                add_rec(&root_, winner, true, root_axis());
                ++inserted;
            }
        }
        return inserted;
    }

    void delete_points(const std::vector<Pt>& pts) {
        for (const Pt& p : pts) delete_point_rec(&root_, p, true);
    }

    int delete_boxes(const std::vector<Box>& boxes) {
        int n = 0;
        for (const Box& b : boxes) n += delete_range_rec(&root_, b, true, false);
        return n;
    }

    void add_boxes(const std::vector<Box>& boxes) {
        for (const Box& b : boxes) add_range_rec(&root_, b, true);
    }

    void flatten_valid(std::vector<Pt>& out) { flatten(root_, out, Record::None); }

    int size() const { return root_ ? root_->size : 0; }
    int validnum() const { return root_ ? root_->size - root_->invalid : 0; }
    Node* root() const { return root_; }

    void take_removed(std::vector<Pt>& out) {
        out.insert(out.end(), removed_.begin(), removed_.end());
        removed_.clear();
    }

   private:
    enum class Record { None, Deleted };

    // The reference reads Root_Node->division_axis unguarded (ikd_Tree.cpp:447,
    // :472); a tree emptied by a rebuild would crash it.  Axis 0 stands in.
    int root_axis() const { return root_ != nullptr ? root_->axis : 0; }

    float del_param_, bal_param_, ds_;
    Node* root_ = nullptr;
    Node* sentinel_ = nullptr;
    std::vector<Pt> scratch_;
    std::vector<Pt> removed_;

    // InitTreeNode, ikd_Tree.cpp:51-76.
    static void clear_node(Node* n) {
        n->p = Pt{0.f, 0.f, 0.f};
        for (int a = 0; a < 3; ++a) n->lo[a] = n->hi[a] = 0.f;
        n->axis = 0;
        n->parent = n->l = n->r = nullptr;
        n->size = 0;
        n->invalid = n->down_del = 0;
        n->pt_del = n->sub_del = n->push_l = n->push_r = n->pt_ds = false;
    }

    // BuildTree, ikd_Tree.cpp:573-622.
    void build_rec(Node** slot, int l, int r, std::vector<Pt>& s) {
        if (l > r) return;
        Node* n = new Node;
        clear_node(n);
        *slot = n;
        int mid = (l + r) >> 1;
        float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int i = l; i <= r; ++i)
            for (int a = 0; a < 3; ++a) {
                mn[a] = std::min(mn[a], coord(s[i], a));
                mx[a] = std::max(mx[a], coord(s[i], a));
            }
        int axis = 0;
        float ext[3];
        for (int a = 0; a < 3; ++a) ext[a] = mx[a] - mn[a];
        for (int a = 1; a < 3; ++a)
            if (ext[a] > ext[axis]) axis = a;
        n->axis = (uint8_t)axis;
        auto less_on = [axis](const Pt& a, const Pt& b) { return coord(a, axis) < coord(b, axis); };
        std::nth_element(s.begin() + l, s.begin() + mid, s.begin() + r + 1, less_on);
        n->p = s[mid];
        Node *lc = nullptr, *rc = nullptr;
        build_rec(&lc, l, mid - 1, s);
        build_rec(&rc, mid + 1, r, s);
        n->l = lc;
        n->r = rc;
        update(n);
    }

    // Rebuild, ikd_Tree.cpp:624-645, always inline (see file header).
    void rebuild(Node** slot) {
        Node* parent = (*slot)->parent;
        scratch_.clear();
        flatten(*slot, scratch_, Record::Deleted);
        free_subtree(slot);
        build_rec(slot, 0, (int)scratch_.size() - 1, scratch_);
        if (*slot != nullptr) (*slot)->parent = parent;
        if (slot == &root_ && sentinel_ != nullptr) sentinel_->l = *slot;
    }

    // Applies a lazy label of `from` to child `c` (the body of Push_Down,
    // ikd_Tree.cpp:1116-1127).
    static void push_label(const Node* from, Node* c) {
        c->sub_ds |= from->sub_ds;
        c->pt_ds |= from->sub_ds;
        c->sub_del = from->sub_del || c->sub_ds;
        c->pt_del = c->sub_del || c->pt_ds;
        if (from->sub_ds) c->down_del = c->size;
        c->invalid = from->sub_del ? c->size : c->down_del;
        c->push_l = c->push_r = true;
    }

    // Push_Down, ikd_Tree.cpp:1109-1181.
    static void push_down(Node* n) {
        if (n == nullptr) return;
        if (n->push_l && n->l != nullptr) {
            push_label(n, n->l);
            n->push_l = false;
        }
        if (n->push_r && n->r != nullptr) {
            push_label(n, n->r);
            n->push_r = false;
        }
    }

    // Update, ikd_Tree.cpp:1183-1323: counts, labels and the AABB of the
    // subtree's non-deleted content (all content once everything is deleted).
    void update(Node* n) {
        Node* kids[2] = {n->l, n->r};
        n->size = 1;
        n->invalid = n->pt_del ? 1 : 0;
        n->down_del = n->pt_ds ? 1 : 0;
        bool all_ds = n->pt_ds, all_del = n->pt_del, any_del = n->pt_del;
        for (Node* c : kids) {
            if (c == nullptr) continue;
            n->size += c->size;
            n->invalid += c->invalid;
            n->down_del += c->down_del;
            all_ds = all_ds && c->sub_ds;
            all_del = all_del && c->sub_del;
            any_del = any_del || c->sub_del;
        }
        n->sub_ds = all_ds;
        n->sub_del = all_del;
        const bool take_all = all_del || !any_del;
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (Node* c : kids) {
            if (c == nullptr || (!take_all && c->sub_del)) continue;
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], c->lo[a]);
                hi[a] = std::max(hi[a], c->hi[a]);
            }
        }
        if (take_all || !n->pt_del)
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], coord(n->p, a));
                hi[a] = std::max(hi[a], coord(n->p, a));
            }
        for (int a = 0; a < 3; ++a) {
            n->lo[a] = lo[a];
            n->hi[a] = hi[a];
        }
        float hx = (n->hi[0] - n->lo[0]) * 0.5;
        float hy = (n->hi[1] - n->lo[1]) * 0.5;
        float hz = (n->hi[2] - n->lo[2]) * 0.5;
        n->radius_sq = hx * hx + hy * hy + hz * hz;
        for (Node* c : kids)
            if (c != nullptr) c->parent = n;
        if (n == root_ && n->size > 3) {
            Node* son = n->l != nullptr ? n->l : n->r;
            float bal = float(son->size) / (n->size - 1);
            n->a_del = float(n->invalid) / n->size;
            n->a_bal = (bal >= 0.5 - kEps) ? bal : 1 - bal;
        }
    }

    // Criterion_Check, ikd_Tree.cpp:1089-1107.
    bool needs_rebuild(const Node* n) const {
        if (n->size <= kMinUnbalanced) return false;
        const Node* son = n->l != nullptr ? n->l : n->r;
        float del = float(n->invalid) / n->size;
        float bal = float(son->size) / (n->size - 1);
        if (del > del_param_) return true;
        return bal > bal_param_ || bal < 1 - bal_param_;
    }

    void finish_mutation(Node** slot, bool allow_rebuild) {
        update(*slot);
        if (allow_rebuild && needs_rebuild(*slot)) rebuild(slot);
    }

    static bool box_disjoint(const Box& b, const Node* n) {
        for (int a = 0; a < 3; ++a)
            if (b.hi[a] <= n->lo[a] || b.lo[a] > n->hi[a]) return true;
        return false;
    }
    static bool box_covers(const Box& b, const Node* n) {
        for (int a = 0; a < 3; ++a)
            if (!(b.lo[a] <= n->lo[a] && b.hi[a] > n->hi[a])) return false;
        return true;
    }
    static bool box_holds(const Box& b, const Pt& p) {
        for (int a = 0; a < 3; ++a)
            if (!(b.lo[a] <= coord(p, a) && b.hi[a] > coord(p, a))) return false;
        return true;
    }

    // Delete_by_range, ikd_Tree.cpp:647-710.
    int delete_range_rec(Node** slot, const Box& b, bool allow_rebuild, bool ds) {
        Node* n = *slot;
        if (n == nullptr || n->sub_del) return 0;
        push_down(n);
        if (box_disjoint(b, n)) return 0;
        if (box_covers(b, n)) {
            n->sub_del = n->pt_del = true;
            n->push_l = n->push_r = true;
            int newly = n->size - n->invalid;
            n->invalid = n->size;
            if (ds) {
                n->sub_ds = n->pt_ds = true;
                n->down_del = n->size;
            }
            return newly;
        }
        int newly = 0;
        if (!n->pt_del && box_holds(b, n->p)) {
            n->pt_del = true;
            newly = 1;
            if (ds) n->pt_ds = true;
        }
        newly += delete_range_rec(&n->l, b, allow_rebuild, ds);
        newly += delete_range_rec(&n->r, b, allow_rebuild, ds);
        finish_mutation(slot, allow_rebuild);
        return newly;
    }

    // Delete_by_point, ikd_Tree.cpp:712-760.
    void delete_point_rec(Node** slot, const Pt& p, bool allow_rebuild) {
        Node* n = *slot;
        if (n == nullptr || n->sub_del) return;
        push_down(n);
        if (near_same(n->p, p) && !n->pt_del) {
            n->pt_del = true;
            n->invalid += 1;
            if (n->invalid == n->size) n->sub_del = true;
            return;
        }
        if (coord(p, n->axis) < coord(n->p, n->axis))
            delete_point_rec(&n->l, p, allow_rebuild);
        else
            delete_point_rec(&n->r, p, allow_rebuild);
        finish_mutation(slot, allow_rebuild);
    }

    // Add_by_range, ikd_Tree.cpp:762-815.
    void add_range_rec(Node** slot, const Box& b, bool allow_rebuild) {
        Node* n = *slot;
        if (n == nullptr) return;
        push_down(n);
        if (box_disjoint(b, n)) return;
        if (box_covers(b, n)) {
            n->sub_del = n->sub_ds;
            n->pt_del = n->pt_ds;
            n->push_l = n->push_r = true;
            n->invalid = n->down_del;
            return;
        }
        if (box_holds(b, n->p)) n->pt_del = n->pt_ds;
        add_range_rec(&n->l, b, allow_rebuild);
        add_range_rec(&n->r, b, allow_rebuild);
        finish_mutation(slot, allow_rebuild);
    }

    // Add_by_point, ikd_Tree.cpp:817-866.
    void add_rec(Node** slot, const Pt& p, bool allow_rebuild, int parent_axis) {
        Node* n = *slot;
        if (n == nullptr) {
            n = new Node;
            clear_node(n);
            n->p = p;
            n->axis = (uint8_t)((parent_axis + 1) % 3);
            *slot = n;
            update(n);
            return;
        }
        push_down(n);
        if (coord(p, n->axis) < coord(n->p, n->axis))
            add_rec(&n->l, p, allow_rebuild, n->axis);
        else
            add_rec(&n->r, p, allow_rebuild, n->axis);
        finish_mutation(slot, allow_rebuild);
    }

    // Search, ikd_Tree.cpp:868-1013 (concurrent callers share the per-node
    // trylock around Push_Down, :875-884).
    void knn_rec(Node* n, int k, const Pt& q, CandHeap& heap, double max_dist) {
        if (n == nullptr || n->sub_del) return;
        double cur = box_sqdist(n, q);
        double max_sq = max_dist * max_dist;
        if (cur > max_sq) return;
        if (n->push_l || n->push_r) {
            if (pthread_mutex_trylock(&n->lock) == 0) {
                push_down(n);
                pthread_mutex_unlock(&n->lock);
            } else {
                pthread_mutex_lock(&n->lock);
                pthread_mutex_unlock(&n->lock);
            }
        }
        if (!n->pt_del) {
            float d = sqdist(q, n->p);
            if (d <= max_sq && (heap.size() < k || d < heap.top().d)) {
                if (heap.size() >= k) heap.pop();
                heap.push(Cand{n->p, d});
            }
        }
        float dl = box_sqdist(n->l, q);
        float dr = box_sqdist(n->r, q);
        if (heap.size() < k || (dl < heap.top().d && dr < heap.top().d)) {
            Node* first = dl <= dr ? n->l : n->r;
            Node* second = dl <= dr ? n->r : n->l;
            float d2nd = dl <= dr ? dr : dl;
            knn_rec(first, k, q, heap, max_dist);
            if (heap.size() < k || d2nd < heap.top().d) knn_rec(second, k, q, heap, max_dist);
        } else {
            if (dl < heap.top().d) knn_rec(n->l, k, q, heap, max_dist);
            if (dr < heap.top().d) knn_rec(n->r, k, q, heap, max_dist);
        }
    }

    // Search_by_range, ikd_Tree.cpp:1015-1044.
    void range_rec(Node* n, const Box& b, std::vector<Pt>& out) {
        if (n == nullptr) return;
        push_down(n);
        if (box_disjoint(b, n)) return;
        if (box_covers(b, n)) {
            flatten(n, out, Record::None);
            return;
        }
        if (box_holds(b, n->p) && !n->pt_del) out.push_back(n->p);
        range_rec(n->l, b, out);
        range_rec(n->r, b, out);
    }

    // Search_by_radius, ikd_Tree.cpp:1046-1087.
    void radius_rec(Node* n, const Pt& q, float r, std::vector<Pt>& out) {
        if (n == nullptr) return;
        push_down(n);
        Pt c;
        c.x = (n->lo[0] + n->hi[0]) * 0.5;
        c.y = (n->lo[1] + n->hi[1]) * 0.5;
        c.z = (n->lo[2] + n->hi[2]) * 0.5;
        float dist = std::sqrt(sqdist(c, q));
        if (dist > r + std::sqrt(n->radius_sq)) return;
        if (dist <= r - std::sqrt(n->radius_sq)) {
            flatten(n, out, Record::None);
            return;
        }
        if (!n->pt_del && sqdist(n->p, q) <= r * r) out.push_back(n->p);
        radius_rec(n->l, q, r, out);
        radius_rec(n->r, q, r, out);
    }

    // flatten, ikd_Tree.cpp:1325-1352.
    void flatten(Node* n, std::vector<Pt>& out, Record rec) {
        if (n == nullptr) return;
        push_down(n);
        if (!n->pt_del) out.push_back(n->p);
        flatten(n->l, out, rec);
        flatten(n->r, out, rec);
        if (rec == Record::Deleted && n->pt_del && !n->pt_ds) removed_.push_back(n->p);
    }

    // delete_tree_nodes, ikd_Tree.cpp:1354-1366.
    void free_subtree(Node** slot) {
        if (*slot == nullptr) return;
        push_down(*slot);
        free_subtree(&(*slot)->l);
        free_subtree(&(*slot)->r);
        delete *slot;
        *slot = nullptr;
    }
};

struct Handle {
    Tree* tree;
    std::vector<std::vector<Pt>> results;
    std::vector<Pt> removed;
};

std::vector<Pt> to_pts(const float* xyz, int n) {
    std::vector<Pt> v((size_t)(n > 0 ? n : 0));
    for (int i = 0; i < n; ++i) v[i] = Pt{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    return v;
}

std::vector<Box> to_boxes(const float* b, int m) {
    std::vector<Box> v((size_t)(m > 0 ? m : 0));
    for (int i = 0; i < m; ++i)
        for (int a = 0; a < 3; ++a) {
            v[i].lo[a] = b[6 * i + a];
            v[i].hi[a] = b[6 * i + 3 + a];
        }
    return v;
}

}  // namespace port

using port::Handle;

extern "C" {

void* ora_create(float d, float b, float box) {
    Handle* h = new Handle;
    h->tree = new port::Tree(d, b, box);
    return h;
}

void ora_destroy(void* hp) {
    Handle* h = (Handle*)hp;
    delete h->tree;
    delete h;
}

void ora_build(void* hp, const float* xyz, int n) { ((Handle*)hp)->tree->build(port::to_pts(xyz, n)); }

int ora_add_points(void* hp, const float* xyz, int n, int ds) {
    Handle* h = (Handle*)hp;
    if (h->tree->root() == nullptr) return -1;
    return h->tree->add_points(port::to_pts(xyz, n), ds != 0);
}

void ora_delete_points(void* hp, const float* xyz, int n) {
    ((Handle*)hp)->tree->delete_points(port::to_pts(xyz, n));
}

int ora_delete_boxes(void* hp, const float* boxes, int m) {
    return ((Handle*)hp)->tree->delete_boxes(port::to_boxes(boxes, m));
}

void ora_add_boxes(void* hp, const float* boxes, int m) {
    ((Handle*)hp)->tree->add_boxes(port::to_boxes(boxes, m));
}

void ora_knn(void* hp, const float* q, int nq, int k, double max_dist, float* out_xyz, float* out_d2,
             int* out_cnt, int nthreads) {
    port::Tree* t = ((Handle*)hp)->tree;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    {
        std::vector<port::Pt> pts((size_t)(k > 0 ? k : 1));
        std::vector<float> d((size_t)(k > 0 ? k : 1));
#pragma omp for schedule(dynamic, 256)
        for (int i = 0; i < nq; ++i) {
            port::Pt p{q[3 * i], q[3 * i + 1], q[3 * i + 2]};
            int c = t->nearest(p, k, max_dist, pts.data(), d.data());
            out_cnt[i] = c;
            for (int j = 0; j < c; ++j) {
                float* o = out_xyz + ((size_t)i * k + j) * 3;
                o[0] = pts[j].x;
                o[1] = pts[j].y;
                o[2] = pts[j].z;
                out_d2[(size_t)i * k + j] = d[j];
            }
        }
    }
}

long long ora_box_search(void* hp, const float* boxes, int nb, long long* counts, int nthreads) {
    Handle* h = (Handle*)hp;
    auto bv = port::to_boxes(boxes, nb);
    h->results.assign((size_t)nb, {});
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = 0; i < nb; ++i) h->tree->box_search(bv[i], h->results[i]);
    long long tot = 0;
    for (int i = 0; i < nb; ++i) tot += (counts[i] = (long long)h->results[i].size());
    return tot;
}

long long ora_radius_search(void* hp, const float* q, const float* r, int nq, long long* counts,
                            int nthreads) {
    Handle* h = (Handle*)hp;
    h->results.assign((size_t)nq, {});
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = 0; i < nq; ++i)
        h->tree->radius_search(port::Pt{q[3 * i], q[3 * i + 1], q[3 * i + 2]}, r[i], h->results[i]);
    long long tot = 0;
    for (int i = 0; i < nq; ++i) tot += (counts[i] = (long long)h->results[i].size());
    return tot;
}

void ora_fetch(void* hp, float* out) {
    size_t o = 0;
    for (auto& v : ((Handle*)hp)->results)
        for (auto& p : v) {
            out[o++] = p.x;
            out[o++] = p.y;
            out[o++] = p.z;
        }
}

int ora_flatten(void* hp, float* out, int cap) {
    std::vector<port::Pt> v;
    ((Handle*)hp)->tree->flatten_valid(v);
    for (int i = 0; i < (int)v.size() && i < cap; ++i) {
        out[3 * i] = v[i].x;
        out[3 * i + 1] = v[i].y;
        out[3 * i + 2] = v[i].z;
    }
    return (int)v.size();
}

int ora_size(void* hp) { return ((Handle*)hp)->tree->size(); }
int ora_validnum(void* hp) { return ((Handle*)hp)->tree->validnum(); }
void ora_settle(void*) {}

void ora_set_async(void*, int) {}

int ora_acquire_removed(void* hp) {
    Handle* h = (Handle*)hp;
    h->removed.clear();
    h->tree->take_removed(h->removed);
    return (int)h->removed.size();
}

void ora_fetch_removed(void* hp, float* out) {
    Handle* h = (Handle*)hp;
    for (size_t i = 0; i < h->removed.size(); ++i) {
        out[3 * i] = h->removed[i].x;
        out[3 * i + 1] = h->removed[i].y;
        out[3 * i + 2] = h->removed[i].z;
    }
}

void ora_tree_range(void* hp, float* box6) {
    port::Node* r = ((Handle*)hp)->tree->root();
    for (int a = 0; a < 3; ++a) {
        box6[a] = r ? r->lo[a] : 0.f;
        box6[3 + a] = r ? r->hi[a] : 0.f;
    }
}

void ora_root_alpha(void* hp, float* out2) {
    port::Node* r = ((Handle*)hp)->tree->root();
    out2[0] = r ? r->a_bal : 0.f;
    out2[1] = r ? r->a_del : 0.f;
}

}  // extern "C"
