// C API over the UNMODIFIED ikd-Tree reference (ikd-Tree/ikd_Tree.cpp), for
// pinning the oracle and generating golden fixtures.  TEST INFRASTRUCTURE ONLY.
//
// The reference translation unit is included verbatim from its own location
// (the include path points at the reference checkout; nothing is copied).  The
// reference's private members are opened with an access-specifier macro so the
// harness can wait for the background rebuild thread to go idle
// (Rebuild_Ptr, ikd-Tree/ikd_Tree.h:184); no behaviour of the reference changes.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <queue>
#include <thread>
#include <vector>
#include <pthread.h>
#include <unistd.h>
#include <omp.h>

#include <pcl/point_types.h>

#define private public
#include "ikd_Tree.cpp"
#undef private

#include "oracle_capi.h"

using Tree = KD_TREE<ikdTree_PointType>;
using PV = Tree::PointVector;

namespace {
struct Handle {
    Tree* tree;
    std::vector<PV> results;  // last box / radius search, per query
    PV removed;
    bool async = false;       // mutations skip the settle (timing mode)
};

PV to_pv(const float* xyz, int n) {
    PV v(n);
    for (int i = 0; i < n; ++i) v[i] = ikdTree_PointType(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    return v;
}

std::vector<BoxPointType> to_boxes(const float* b, int m) {
    std::vector<BoxPointType> v(m);
    for (int i = 0; i < m; ++i)
        for (int a = 0; a < 3; ++a) {
            v[i].vertex_min[a] = b[6 * i + a];
            v[i].vertex_max[a] = b[6 * i + 3 + a];
        }
    return v;
}

// Wait until the reference's rebuild thread holds no pending or running job.
void settle(Tree* t) {
    for (int it = 0; it < 200000; ++it) {
        if (t->Rebuild_Ptr == nullptr && !t->rebuild_flag) return;
        usleep(100);
    }
}
}  // namespace

extern "C" {

void* ora_create(float d, float b, float box) {
    Handle* h = new Handle;
    h->tree = new Tree(d, b, box);
    return h;
}

void ora_destroy(void* hp) {
    Handle* h = (Handle*)hp;
    settle(h->tree);
    delete h->tree;
    delete h;
}

void ora_build(void* hp, const float* xyz, int n) {
    Handle* h = (Handle*)hp;
    settle(h->tree);
    h->tree->Build(to_pv(xyz, n));
}

int ora_add_points(void* hp, const float* xyz, int n, int ds) {
    Handle* h = (Handle*)hp;
    if (!h->async) settle(h->tree);
    if (h->tree->Root_Node == nullptr) return -1;
    PV v = to_pv(xyz, n);
    int r = h->tree->Add_Points(v, ds != 0);
    if (!h->async) settle(h->tree);
    return r;
}

void ora_delete_points(void* hp, const float* xyz, int n) {
    Handle* h = (Handle*)hp;
    if (!h->async) settle(h->tree);
    PV v = to_pv(xyz, n);
    h->tree->Delete_Points(v);
    if (!h->async) settle(h->tree);
}

int ora_delete_boxes(void* hp, const float* boxes, int m) {
    Handle* h = (Handle*)hp;
    if (!h->async) settle(h->tree);
    auto v = to_boxes(boxes, m);
    int r = h->tree->Delete_Point_Boxes(v);
    if (!h->async) settle(h->tree);
    return r;
}

void ora_add_boxes(void* hp, const float* boxes, int m) {
    Handle* h = (Handle*)hp;
    if (!h->async) settle(h->tree);
    auto v = to_boxes(boxes, m);
    h->tree->Add_Point_Boxes(v);
    if (!h->async) settle(h->tree);
}

void ora_knn(void* hp, const float* q, int nq, int k, double max_dist, float* out_xyz, float* out_d2,
             int* out_cnt, int nthreads) {
    Handle* h = (Handle*)hp;
    if (!h->async) settle(h->tree);
    Tree* t = h->tree;
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = 0; i < nq; ++i) {
        PV pts;
        std::vector<float> d2;
        ikdTree_PointType p(q[3 * i], q[3 * i + 1], q[3 * i + 2]);
        t->Nearest_Search(p, k, pts, d2, max_dist);
        int c = (int)pts.size();
        out_cnt[i] = c;
        for (int j = 0; j < c; ++j) {
            out_xyz[((size_t)i * k + j) * 3 + 0] = pts[j].x;
            out_xyz[((size_t)i * k + j) * 3 + 1] = pts[j].y;
            out_xyz[((size_t)i * k + j) * 3 + 2] = pts[j].z;
            out_d2[(size_t)i * k + j] = d2[j];
        }
    }
}

long long ora_box_search(void* hp, const float* boxes, int nb, long long* counts, int nthreads) {
    Handle* h = (Handle*)hp;
    if (!h->async) settle(h->tree);
    auto bv = to_boxes(boxes, nb);
    h->results.assign(nb, PV());
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = 0; i < nb; ++i) h->tree->Box_Search(bv[i], h->results[i]);
    long long tot = 0;
    for (int i = 0; i < nb; ++i) {
        counts[i] = (long long)h->results[i].size();
        tot += counts[i];
    }
    return tot;
}

long long ora_radius_search(void* hp, const float* q, const float* r, int nq, long long* counts,
                            int nthreads) {
    Handle* h = (Handle*)hp;
    if (!h->async) settle(h->tree);
    h->results.assign(nq, PV());
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = 0; i < nq; ++i) {
        ikdTree_PointType p(q[3 * i], q[3 * i + 1], q[3 * i + 2]);
        h->tree->Radius_Search(p, r[i], h->results[i]);
    }
    long long tot = 0;
    for (int i = 0; i < nq; ++i) {
        counts[i] = (long long)h->results[i].size();
        tot += counts[i];
    }
    return tot;
}

void ora_fetch(void* hp, float* out) {
    Handle* h = (Handle*)hp;
    size_t o = 0;
    for (auto& v : h->results)
        for (auto& p : v) {
            out[o++] = p.x;
            out[o++] = p.y;
            out[o++] = p.z;
        }
}

int ora_flatten(void* hp, float* out, int cap) {
    Handle* h = (Handle*)hp;
    settle(h->tree);
    PV v;
    if (h->tree->Root_Node != nullptr) h->tree->flatten(h->tree->Root_Node, v, NOT_RECORD);
    int n = (int)v.size();
    for (int i = 0; i < n && i < cap; ++i) {
        out[3 * i] = v[i].x;
        out[3 * i + 1] = v[i].y;
        out[3 * i + 2] = v[i].z;
    }
    return n;
}

int ora_size(void* hp) {
    Handle* h = (Handle*)hp;
    settle(h->tree);
    return h->tree->size();
}

int ora_validnum(void* hp) {
    Handle* h = (Handle*)hp;
    settle(h->tree);
    return h->tree->validnum();
}

void ora_settle(void* hp) { settle(((Handle*)hp)->tree); }

void ora_set_async(void* hp, int async) { ((Handle*)hp)->async = async != 0; }

int ora_acquire_removed(void* hp) {
    Handle* h = (Handle*)hp;
    settle(h->tree);
    h->removed.clear();
    h->tree->acquire_removed_points(h->removed);
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
    Handle* h = (Handle*)hp;
    settle(h->tree);
    BoxPointType b = h->tree->tree_range();
    for (int a = 0; a < 3; ++a) {
        box6[a] = b.vertex_min[a];
        box6[3 + a] = b.vertex_max[a];
    }
}

void ora_root_alpha(void* hp, float* out2) {
    Handle* h = (Handle*)hp;
    settle(h->tree);
    if (h->tree->Root_Node == nullptr) {
        out2[0] = out2[1] = 0.f;
        return;
    }
    h->tree->root_alpha(out2[0], out2[1]);
}

}  // extern "C"
