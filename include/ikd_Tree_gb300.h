// ikd_Tree_gb300.h - drop-in KD_TREE<PointType> over libikdg (include/ikdg.h).
//
// Mirrors the public interface of hku-mars/ikd-Tree's KD_TREE<PointType>
// (ikd-Tree/ikd_Tree.h:59-249): same class and method names, argument order,
// defaults and return values, so code written against the reference compiles
// unchanged after switching the include.  Every call runs on the GPU through
// the C ABI; there is no CPU code path.
//
// PointType needs public float members x, y, z (ikdTree_PointType,
// pcl::PointXYZ, pcl::PointXYZI, pcl::PointXYZINormal, ...).  Searches and
// acquire_removed_points return full PointType values: the facade keeps the
// inserted points on the host, keyed by the id the device tree assigns to
// each, so payload fields such as intensity or normals come back exactly as
// they were inserted.  Points no call can return any more (downsampling
// losers, deleted points dropped by rebuilds and already handed out) are
// dropped from that store whenever it holds more than twice the live ones, so
// host memory stays proportional to the map, not to everything ever inserted.
//
// Differences from the reference, by design:
//   * results at exactly tied distances are ordered by insertion id;
//   * searches are exact at box / radius boundaries (no tree-shape effects);
//   * Delete_Points finds a matching point wherever the split planes put it;
//   * Add_Points on an empty tree works;
//   * rebuilds run on the GPU synchronously, not on a background thread, so
//     validnum() never reports -1;
//   * the tree lives in device memory: Root_Node is an opaque handle that is
//     non-null exactly while the tree stores points (code that tests it
//     against nullptr or passes it to flatten keeps working), not a node.
// Batched forms of the searches (Nearest_Search_Batch, Box_Search_Batch,
// Radius_Search_Batch) run a whole set of queries in one kernel launch.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "ikdg.h"

#ifndef IKD_TREE_GB300_NO_BASIC_TYPES
// ikd-Tree/ikd_Tree.h:22-35.
struct ikdTree_PointType {
    float x, y, z;
    ikdTree_PointType(float px = 0.0f, float py = 0.0f, float pz = 0.0f) : x(px), y(py), z(pz) {}
};

struct BoxPointType {
    float vertex_min[3];
    float vertex_max[3];
};
#endif

// ikd-Tree/ikd_Tree.h:39.
enum delete_point_storage_set { NOT_RECORD, DELETE_POINTS_REC, MULTI_THREAD_REC };

#if defined(EIGEN_CORE_H) || defined(IKD_TREE_GB300_EIGEN_ALLOCATOR)
#define IKDG_POINT_ALLOCATOR(T) Eigen::aligned_allocator<T>
#else
#define IKDG_POINT_ALLOCATOR(T) std::allocator<T>
#endif

class IkdgError : public std::runtime_error {
   public:
    IkdgError(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
    int status() const { return status_; }

   private:
    int status_;
};

// Opaque stand-in for the reference's node type: only ever used through
// KD_TREE::Root_Node as "is there a tree" and as flatten's first argument.
struct KD_TREE_NODE;

template <typename PointType>
class KD_TREE {
   public:
    using PointVector = std::vector<PointType, IKDG_POINT_ALLOCATOR(PointType)>;
    using Ptr = std::shared_ptr<KD_TREE<PointType>>;

    // KD_TREE(delete_param, balance_param, box_length), ikd_Tree.h:226.
    explicit KD_TREE(float delete_param = 0.5, float balance_param = 0.6, float box_length = 0.2, int device = -1) {
        check(ikdg_create(delete_param, balance_param, box_length, device, &t_), "create");
    }
    ~KD_TREE() {
        if (t_ != nullptr) ikdg_destroy(t_);
    }
    KD_TREE(const KD_TREE&) = delete;
    KD_TREE& operator=(const KD_TREE&) = delete;

    // ikd_Tree.h:228-231.
    void Set_delete_criterion_param(float delete_param) {
        check(ikdg_set_delete_criterion_param(t_, delete_param), "Set_delete_criterion_param");
    }
    void Set_balance_criterion_param(float balance_param) {
        check(ikdg_set_balance_criterion_param(t_, balance_param), "Set_balance_criterion_param");
    }
    void set_downsample_param(float box_length) {
        check(ikdg_set_downsample_param(t_, box_length), "set_downsample_param");
    }
    void InitializeKDTree(float delete_param = 0.5, float balance_param = 0.7, float box_length = 0.2) {
        Set_delete_criterion_param(delete_param);
        Set_balance_criterion_param(balance_param);
        set_downsample_param(box_length);
    }

    // ikd_Tree.h:232-234, :245.
    int size() {
        int64_t n = 0;
        check(ikdg_size(t_, &n), "size");
        return (int)n;
    }
    int validnum() {
        int64_t n = 0;
        check(ikdg_validnum(t_, &n), "validnum");
        return (int)n;
    }
    void root_alpha(float& alpha_bal, float& alpha_del) { check(ikdg_root_alpha(t_, &alpha_bal, &alpha_del), "root_alpha"); }
    BoxPointType tree_range() {
        float b[6];
        check(ikdg_tree_range(t_, b), "tree_range");
        BoxPointType r;
        for (int a = 0; a < 3; ++a) {
            r.vertex_min[a] = b[a];
            r.vertex_max[a] = b[3 + a];
        }
        return r;
    }

    // Build(PointVector), ikd_Tree.h:235 (by value, as the reference).
    void Build(PointVector point_cloud) {
        std::vector<float> xyz = pack(point_cloud);
        check(ikdg_build(t_, xyz.data(), (int64_t)point_cloud.size(), 3), "Build");
        ids_.clear();
        pay_.clear();
        next_id_ = 0;
        remember(point_cloud);
        refresh_root();
    }

    // Nearest_Search, ikd_Tree.h:236.
    void Nearest_Search(PointType point, int k_nearest, PointVector& Nearest_Points, std::vector<float>& Point_Distance,
                        double max_dist = INFINITY) {
        Nearest_Points.clear();
        Point_Distance.clear();
        if (k_nearest <= 0) return;
        float q[3] = {point.x, point.y, point.z};
        std::vector<int32_t> ids(k_nearest);
        std::vector<float> d2(k_nearest);
        int32_t cnt = 0;
        check(ikdg_knn(t_, q, 1, 3, k_nearest, max_dist, ids.data(), d2.data(), nullptr, &cnt), "Nearest_Search");
        for (int j = 0; j < cnt; ++j) {
            Nearest_Points.push_back(payload(ids[j]));
            Point_Distance.push_back(d2[j]);
        }
    }

    // Batched Nearest_Search: row i of the outputs belongs to queries[i].
    void Nearest_Search_Batch(const PointVector& queries, int k_nearest, std::vector<PointVector>& Nearest_Points,
                              std::vector<std::vector<float>>& Point_Distance, double max_dist = INFINITY) {
        const size_t nq = queries.size();
        Nearest_Points.assign(nq, PointVector());
        Point_Distance.assign(nq, std::vector<float>());
        if (nq == 0 || k_nearest <= 0) return;
        std::vector<float> q = pack(queries);
        std::vector<int32_t> ids(nq * (size_t)k_nearest), cnt(nq);
        std::vector<float> d2(nq * (size_t)k_nearest);
        check(ikdg_knn(t_, q.data(), (int64_t)nq, 3, k_nearest, max_dist, ids.data(), d2.data(), nullptr, cnt.data()),
              "Nearest_Search_Batch");
        for (size_t i = 0; i < nq; ++i)
            for (int j = 0; j < cnt[i]; ++j) {
                Nearest_Points[i].push_back(payload(ids[i * k_nearest + j]));
                Point_Distance[i].push_back(d2[i * k_nearest + j]);
            }
    }

    // Box_Search, ikd_Tree.h:237.
    void Box_Search(const BoxPointType& Box_of_Point, PointVector& Storage) {
        std::vector<BoxPointType> b(1, Box_of_Point);
        std::vector<PointVector> out;
        Box_Search_Batch(b, out);
        Storage.swap(out[0]);
    }
    void Box_Search_Batch(const std::vector<BoxPointType>& boxes, std::vector<PointVector>& results) {
        std::vector<float> b = pack_boxes(boxes);
        csr_search(results, boxes.size(), [&](int64_t* offs, int32_t* ids, int64_t cap, int64_t* total) {
            return ikdg_box_search(t_, b.data(), (int64_t)boxes.size(), offs, ids, nullptr, cap, total);
        });
    }

    // Radius_Search, ikd_Tree.h:238.
    void Radius_Search(PointType point, const float radius, PointVector& Storage) {
        PointVector q(1, point);
        std::vector<float> r(1, radius);
        std::vector<PointVector> out;
        Radius_Search_Batch(q, r, out);
        Storage.swap(out[0]);
    }
    void Radius_Search_Batch(const PointVector& centres, const std::vector<float>& radii,
                             std::vector<PointVector>& results) {
        if (radii.size() != centres.size() && radii.size() != 1) throw IkdgError(IKDG_BAD_ARG, "radius count");
        std::vector<float> q = pack(centres);
        const int rstride = radii.size() == 1 ? 0 : 1;
        csr_search(results, centres.size(), [&](int64_t* offs, int32_t* ids, int64_t cap, int64_t* total) {
            return ikdg_radius_search(t_, q.data(), (int64_t)centres.size(), 3, radii.data(), rstride, offs, ids,
                                      nullptr, cap, total);
        });
    }

    // Add_Points, ikd_Tree.h:239.
    int Add_Points(PointVector& PointToAdd, bool downsample_on) {
        std::vector<float> xyz = pack(PointToAdd);
        int64_t added = 0;
        check(ikdg_add_points(t_, xyz.data(), (int64_t)PointToAdd.size(), 3, downsample_on ? 1 : 0, &added),
              "Add_Points");
        // The device assigned ids next .. next + n - 1 to the inputs.
        remember(PointToAdd);
        refresh_root();
        compact();
        return (int)added;
    }

    // Add_Point_Boxes, ikd_Tree.h:240.
    void Add_Point_Boxes(std::vector<BoxPointType>& BoxPoints) {
        std::vector<float> b = pack_boxes(BoxPoints);
        check(ikdg_add_boxes(t_, b.data(), (int64_t)BoxPoints.size()), "Add_Point_Boxes");
    }

    // Delete_Points, ikd_Tree.h:241.
    void Delete_Points(PointVector& PointToDel) {
        std::vector<float> xyz = pack(PointToDel);
        check(ikdg_delete_points(t_, xyz.data(), (int64_t)PointToDel.size(), 3), "Delete_Points");
        refresh_root();
        compact();
    }

    // Delete_Point_Boxes, ikd_Tree.h:242.
    int Delete_Point_Boxes(std::vector<BoxPointType>& BoxPoints) {
        std::vector<float> b = pack_boxes(BoxPoints);
        int64_t n = 0;
        check(ikdg_delete_boxes(t_, b.data(), (int64_t)BoxPoints.size(), &n), "Delete_Point_Boxes");
        refresh_root();
        compact();
        return (int)n;
    }

    // flatten(Root_Node, Storage, NOT_RECORD), ikd_Tree.h:243: the valid points
    // (the whole tree; the node argument can only be Root_Node here).
    void flatten(KD_TREE_NODE* root, PointVector& Storage, delete_point_storage_set storage_type) {
        Storage.clear();
        if (root == nullptr) return;
        flatten(Storage, storage_type);
    }
    void flatten(PointVector& Storage, delete_point_storage_set storage_type = NOT_RECORD) {
        (void)storage_type;
        Storage.clear();
        int64_t n = 0;
        int st = ikdg_flatten(t_, nullptr, nullptr, 0, &n);
        if (st != IKDG_OK && st != IKDG_CAPACITY) check(st, "flatten");
        if (n == 0) return;
        std::vector<int32_t> ids(n);
        check(ikdg_flatten(t_, nullptr, ids.data(), n, &n), "flatten");
        Storage.reserve(n);
        for (int64_t i = 0; i < n; ++i) Storage.push_back(payload(ids[i]));
    }

    // acquire_removed_points, ikd_Tree.h:244: the removed points as inserted
    // (payload fields included).
    void acquire_removed_points(PointVector& removed_points) {
        int64_t n = 0;
        int st = ikdg_acquire_removed_points(t_, nullptr, nullptr, 0, &n);
        if (st != IKDG_OK && st != IKDG_CAPACITY) check(st, "acquire_removed_points");
        if (n == 0) return;
        std::vector<int32_t> ids(n);
        check(ikdg_acquire_removed_points(t_, nullptr, ids.data(), n, &n), "acquire_removed_points");
        for (int64_t i = 0; i < n; ++i) removed_points.push_back(payload(ids[i]));
        compact();
    }

    // Points held by the host-side payload store (live ones plus garbage not
    // yet dropped); at most about twice the points the tree can still return.
    size_t stored_payloads() const { return pay_.size(); }

    // Public members of the reference kept for source compatibility
    // (ikd_Tree.h:246-248).  Root_Node is non-null exactly while the tree
    // stores points (size() > 0); the others are not used by the GPU tree.
    PointVector PCL_Storage;
    KD_TREE_NODE* Root_Node = nullptr;
    int max_queue_size = 0;

    ikdg_tree* handle() { return t_; }

   private:
    void refresh_root() {
        int64_t n = 0;
        check(ikdg_size(t_, &n), "size");
        Root_Node = n > 0 ? reinterpret_cast<KD_TREE_NODE*>(&root_token_) : nullptr;
    }

    ikdg_tree* t_ = nullptr;
    char root_token_ = 0;
    // Payload store: ids_ ascending (ids are handed out in increasing order)
    // with the inserted point of each id at the same position in pay_.
    std::vector<int32_t> ids_;
    std::vector<PointType> pay_;
    int64_t next_id_ = 0;

    template <class V>
    void remember(const V& pts) {
        ids_.reserve(ids_.size() + pts.size());
        pay_.reserve(pay_.size() + pts.size());
        for (size_t i = 0; i < pts.size(); ++i) {
            ids_.push_back((int32_t)(next_id_ + (int64_t)i));
            pay_.push_back(pts[i]);
        }
        next_id_ += (int64_t)pts.size();
    }
    const PointType& payload(int32_t id) const {
        auto it = std::lower_bound(ids_.begin(), ids_.end(), id);
        if (it == ids_.end() || *it != id) throw IkdgError(IKDG_INTERNAL, "ikdg: no stored point for a returned id");
        return pay_[it - ids_.begin()];
    }
    // Drops the payloads of ids the tree can no longer return, once they
    // outnumber the live ones.
    void compact() {
        int64_t live = 0;
        int st = ikdg_live_ids(t_, nullptr, 0, &live);
        if (st != IKDG_OK && st != IKDG_CAPACITY) check(st, "live_ids");
        if ((int64_t)ids_.size() <= 2 * live + 4096) return;
        std::vector<int32_t> keep(live);
        if (live > 0) check(ikdg_live_ids(t_, keep.data(), live, &live), "live_ids");
        std::sort(keep.begin(), keep.end());
        size_t w = 0, k = 0;
        for (size_t r = 0; r < ids_.size(); ++r) {
            while (k < keep.size() && keep[k] < ids_[r]) ++k;
            if (k < keep.size() && keep[k] == ids_[r]) {
                ids_[w] = ids_[r];
                pay_[w] = pay_[r];
                ++w;
            }
        }
        ids_.resize(w);
        pay_.erase(pay_.begin() + w, pay_.end());
        ids_.shrink_to_fit();
        pay_.shrink_to_fit();
    }

    void check(int st, const char* what) {
        if (st != IKDG_OK)
            throw IkdgError(st, std::string("ikdg ") + what + ": " + ikdg_status_string(st) + " (" +
                                    (t_ ? ikdg_last_error(t_) : "") + ")");
    }
    template <class V>
    static std::vector<float> pack(const V& pts) {
        std::vector<float> xyz(3 * pts.size());
        for (size_t i = 0; i < pts.size(); ++i) {
            xyz[3 * i] = pts[i].x;
            xyz[3 * i + 1] = pts[i].y;
            xyz[3 * i + 2] = pts[i].z;
        }
        return xyz;
    }
    static std::vector<float> pack_boxes(const std::vector<BoxPointType>& boxes) {
        std::vector<float> b(6 * boxes.size());
        for (size_t i = 0; i < boxes.size(); ++i)
            for (int a = 0; a < 3; ++a) {
                b[6 * i + a] = boxes[i].vertex_min[a];
                b[6 * i + 3 + a] = boxes[i].vertex_max[a];
            }
        return b;
    }
    template <class F>
    void csr_search(std::vector<PointVector>& results, size_t nq, F&& call) {
        results.assign(nq, PointVector());
        if (nq == 0) return;
        std::vector<int64_t> offs(nq + 1);
        int64_t total = 0;
        int st = call(offs.data(), nullptr, 0, &total);
        if (st != IKDG_OK && st != IKDG_CAPACITY) check(st, "range search");
        if (total == 0) return;
        std::vector<int32_t> ids(total);
        check(call(offs.data(), ids.data(), total, &total), "range search");
        for (size_t i = 0; i < nq; ++i) {
            results[i].reserve(offs[i + 1] - offs[i]);
            for (int64_t j = offs[i]; j < offs[i + 1]; ++j) results[i].push_back(payload(ids[j]));
        }
    }
};
