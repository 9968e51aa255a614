// Drives the drop-in KD_TREE<PointType> facade (include/ikd_Tree_gb300.h) the
// way reference user code does, with a payload point type, and checks every
// result against brute force.  Exit code 0 = pass.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include "ikd_Tree_gb300.h"

struct PointXYZI {  // shaped like pcl::PointXYZI: coordinates plus a payload
    float x = 0, y = 0, z = 0, pad = 1;
    float intensity = 0, pad2[3] = {0, 0, 0};
};

static float d2(const PointXYZI& a, const PointXYZI& b) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return dx * dx + dy * dy + dz * dz;
}

#define CHECK(c)                                                      \
    do {                                                              \
        if (!(c)) {                                                   \
            std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c); \
            return 1;                                                 \
        }                                                             \
    } while (0)

int main() {
    using Tree = KD_TREE<PointXYZI>;
    using PV = Tree::PointVector;
    std::mt19937 rng(3);
    std::uniform_real_distribution<float> U(-10, 10);
    PV cloud(20000);
    for (size_t i = 0; i < cloud.size(); ++i) {
        cloud[i].x = U(rng);
        cloud[i].y = U(rng);
        cloud[i].z = U(rng);
        cloud[i].intensity = (float)i;  // payload identifies the point
    }
    Tree::Ptr tree(new Tree(0.3, 0.6, 0.2));
    CHECK(tree->Root_Node == nullptr);  // FAST-LIO's "not built yet" test
    tree->Build(cloud);
    CHECK(tree->Root_Node != nullptr);
    CHECK(tree->size() == 20000 && tree->validnum() == 20000);

    // Nearest_Search: neighbours, squared distances, payloads.
    for (int t = 0; t < 50; ++t) {
        PointXYZI q;
        q.x = U(rng);
        q.y = U(rng);
        q.z = U(rng);
        PV nn;
        std::vector<float> dist;
        tree->Nearest_Search(q, 5, nn, dist);
        std::vector<std::pair<float, int>> all;
        for (size_t i = 0; i < cloud.size(); ++i) all.push_back({d2(q, cloud[i]), (int)i});
        std::sort(all.begin(), all.end());
        CHECK(nn.size() == 5 && dist.size() == 5);
        for (int j = 0; j < 5; ++j) {
            CHECK(dist[j] == all[j].first);
            CHECK(d2(q, nn[j]) == dist[j]);
            const PointXYZI& src = cloud[(int)nn[j].intensity];
            CHECK(src.x == nn[j].x && src.y == nn[j].y && src.z == nn[j].z);
        }
    }

    // Batched search equals single searches.
    PV qs(200);
    for (auto& q : qs) {
        q.x = U(rng);
        q.y = U(rng);
        q.z = U(rng);
    }
    std::vector<PV> bn;
    std::vector<std::vector<float>> bd;
    tree->Nearest_Search_Batch(qs, 8, bn, bd, 1.5);
    for (size_t i = 0; i < qs.size(); ++i) {
        PV nn;
        std::vector<float> dist;
        tree->Nearest_Search(qs[i], 8, nn, dist, 1.5);
        CHECK(nn.size() == bn[i].size());
        for (size_t j = 0; j < nn.size(); ++j) CHECK(dist[j] == bd[i][j] && nn[j].intensity == bn[i][j].intensity);
    }

    // Box_Search / Radius_Search against brute force.
    BoxPointType box;
    for (int a = 0; a < 3; ++a) {
        box.vertex_min[a] = -2;
        box.vertex_max[a] = 3;
    }
    PV inbox;
    tree->Box_Search(box, inbox);
    size_t want = 0;
    for (auto& p : cloud)
        want += (p.x >= -2 && p.x < 3 && p.y >= -2 && p.y < 3 && p.z >= -2 && p.z < 3);
    CHECK(inbox.size() == want);
    PV ball;
    PointXYZI c;
    tree->Radius_Search(c, 2.5f, ball);
    want = 0;
    for (auto& p : cloud) want += d2(p, c) <= 2.5f * 2.5f;
    CHECK(ball.size() == want);

    // Mutations keep the facade's bookkeeping in step with the device ids.
    PV add(1000);
    for (size_t i = 0; i < add.size(); ++i) {
        add[i].x = U(rng);
        add[i].y = U(rng);
        add[i].z = U(rng);
        add[i].intensity = 100000.f + (float)i;
    }
    CHECK(tree->Add_Points(add, false) == 0);
    CHECK(tree->validnum() == 21000);
    std::vector<BoxPointType> boxes(1, box);
    int deleted = tree->Delete_Point_Boxes(boxes);
    CHECK(tree->validnum() == 21000 - deleted);
    PV all;
    tree->flatten(all);
    CHECK((int)all.size() == tree->validnum());
    // the reference's call shape: flatten(Root_Node, PCL_Storage, NOT_RECORD)
    tree->flatten(tree->Root_Node, tree->PCL_Storage, NOT_RECORD);
    CHECK(tree->PCL_Storage.size() == all.size());
    for (auto& p : all) CHECK(!(p.x >= -2 && p.x < 3 && p.y >= -2 && p.y < 3 && p.z >= -2 && p.z < 3));
    PV del(all.begin(), all.begin() + 100);
    tree->Delete_Points(del);
    CHECK(tree->validnum() == 21000 - deleted - 100);
    int n_ds = tree->Add_Points(add, true);
    CHECK(n_ds > 0);
    float ab, ad;
    tree->root_alpha(ab, ad);
    CHECK(ab >= 0.5f && ab <= 1.f && ad >= 0.f && ad <= 1.f);
    BoxPointType r = tree->tree_range();
    CHECK(r.vertex_min[0] >= -10 && r.vertex_max[0] <= 10);

    // acquire_removed_points hands back the removed points as inserted,
    // payload included.  delete_param 0: every subtree holding a deleted
    // point is rebuilt, so every deleted point is dropped and recorded.
    {
        Tree t2(0.0, 0.6, 0.2);
        PV c2(3000);
        for (size_t i = 0; i < c2.size(); ++i) {
            c2[i].x = U(rng);
            c2[i].y = U(rng);
            c2[i].z = U(rng);
            c2[i].intensity = (float)i;
        }
        t2.Build(c2);
        PV gone(c2.begin() + 10, c2.begin() + 60);
        t2.Delete_Points(gone);
        std::vector<BoxPointType> b2(1, box);
        int nb = t2.Delete_Point_Boxes(b2);
        PV removed;
        t2.acquire_removed_points(removed);
        CHECK((int)removed.size() == 50 + nb);
        int from_list = 0;
        for (auto& p : removed) {
            const int i = (int)p.intensity;
            CHECK(i >= 0 && i < (int)c2.size());
            CHECK(c2[i].x == p.x && c2[i].y == p.y && c2[i].z == p.z);
            const bool in_box = p.x >= -2 && p.x < 3 && p.y >= -2 && p.y < 3 && p.z >= -2 && p.z < 3;
            from_list += (i >= 10 && i < 60 && !in_box);
            CHECK(in_box || (i >= 10 && i < 60));
        }
        CHECK(t2.validnum() == 3000 - (int)removed.size());
        PV again;
        t2.acquire_removed_points(again);
        CHECK(again.empty());
        (void)from_list;
    }

    // A long mapping stream keeps the host-side payload store bounded by the
    // points the tree can still return (plus a fixed slack), not by the
    // number of points ever inserted.
    {
        Tree t3(0.5, 0.6, 0.3);
        PV seed(20000);
        for (auto& p : seed) {
            p.x = U(rng);
            p.y = U(rng);
            p.z = U(rng);
        }
        t3.Build(seed);
        std::uniform_real_distribution<float> V(-1, 1);
        size_t inserted = seed.size();
        for (int it = 0; it < 60; ++it) {
            const float cx = -8.f + 0.25f * (float)it;
            PV scan(5000);
            for (size_t i = 0; i < scan.size(); ++i) {
                scan[i].x = cx + 2.f * V(rng);
                scan[i].y = U(rng);
                scan[i].z = U(rng);
                scan[i].intensity = (float)(inserted + i);
            }
            inserted += scan.size();
            t3.Add_Points(scan, true);
            BoxPointType behind;
            behind.vertex_min[0] = -100;
            behind.vertex_max[0] = cx - 3.f;
            for (int a = 1; a < 3; ++a) {
                behind.vertex_min[a] = -100;
                behind.vertex_max[a] = 100;
            }
            std::vector<BoxPointType> bb(1, behind);
            t3.Delete_Point_Boxes(bb);
            PV dropped;
            t3.acquire_removed_points(dropped);
            CHECK(t3.stored_payloads() <= 2 * (size_t)t3.size() + 4096);
        }
        CHECK(inserted > 2 * t3.stored_payloads());
        PV nn;
        std::vector<float> dist;
        PointXYZI q;
        q.x = 6.f;
        t3.Nearest_Search(q, 5, nn, dist);
        CHECK(nn.size() == 5);
        for (auto& p : nn) CHECK(p.intensity >= 0.f);
    }
    std::printf("facade ok: deleted %d, downsampled inserts %d, valid %d\n", deleted, n_ds, tree->validnum());
    return 0;
}
