// Host side of libikdg: the tree object that owns the device pools, the
// per-call orchestration of the kernels, and the extern "C" entry points
// declared in include/ikdg.h.
//
// Every call runs on the tree's CUDA stream.  Host-pointer calls copy their
// inputs in, run the kernels, copy the results out and synchronise; the
// reference API is synchronous (it returns counts), so are these.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <mutex>
#include <new>
#include <shared_mutex>
#include <string>
#include <vector>

#include "ikdg.h"
#include "kernels.cuh"
#include "search.cuh"
#include "update.cuh"


namespace ikdg {
namespace {

struct CudaFail {
    cudaError_t e;
    const char* what;
};
struct Internal {
    std::string what;
};
struct BadArg {
    std::string what;
};
struct CapacityFail {
    std::string what;
};

#define CK(x)                                        \
    do {                                             \
        cudaError_t _e = (x);                        \
        if (_e != cudaSuccess) throw ::ikdg::CudaFail{_e, #x}; \
    } while (0)

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Grow-only device buffer.
struct Arena {
    void* p = nullptr;
    size_t bytes = 0;
    void ensure(size_t need, cudaStream_t s) {
        if (need <= bytes) return;
        if (p != nullptr) {
            CK(cudaStreamSynchronize(s));
            CK(cudaFree(p));
            p = nullptr;
            bytes = 0;
        }
        size_t nb = std::max(need, (size_t)1 << 20);
        CK(cudaMalloc(&p, nb));
        bytes = nb;
    }
    void release() {
        if (p != nullptr) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
};

// Sequential sub-allocation inside an arena.
struct Carver {
    char* base;
    size_t off = 0;
    explicit Carver(void* b) : base((char*)b) {}
    template <class T>
    T* take(size_t count) {
        T* r = (T*)(base + off);
        off += align_up(sizeof(T) * std::max<size_t>(count, 1));
        return r;
    }
};

// Squared-distance gate of Search (ikd_Tree.cpp:872-873, :887): the reference
// compares a float distance against max_dist * max_dist in double.  For float
// d, (double)d <= m2  <=>  d <= the largest float not above m2.
float max_sq_threshold(double max_dist) {
    double m2 = max_dist * max_dist;
    if (std::isnan(m2)) return NAN;
    if (std::isinf(m2)) return INFINITY;
    float f = (float)m2;
    if ((double)f > m2) f = std::nextafter(f, -INFINITY);
    return f;
}

// SO(3) exponential (Rodrigues) and its right Jacobian, in double.
void so3_exp(const double w[3], double R[9]) {
    const double th = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    double a, b;  // R = I + a [w]x + b [w]x^2
    if (th < 1e-6) {
        a = 1.0 - th * th / 6.0;
        b = 0.5 - th * th / 24.0;
    } else {
        a = std::sin(th) / th;
        b = (1.0 - std::cos(th)) / (th * th);
    }
    const double K[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
    double K2[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            double s = 0;
            for (int m = 0; m < 3; ++m) s += K[3 * r + m] * K[3 * m + c];
            K2[3 * r + c] = s;
        }
    for (int i = 0; i < 9; ++i) R[i] = (i % 4 == 0 ? 1.0 : 0.0) + a * K[i] + b * K2[i];
}

// Right Jacobian J_r(w) = I - (1 - cos t)/t^2 [w]x + (t - sin t)/t^3 [w]x^2.
void so3_jr(const double w[3], double J[9]) {
    const double th = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    double a, b;
    if (th < 1e-4) {
        a = 0.5 - th * th / 24.0;
        b = 1.0 / 6.0 - th * th / 120.0;
    } else {
        a = (1.0 - std::cos(th)) / (th * th);
        b = (th - std::sin(th)) / (th * th * th);
    }
    const double K[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
    double K2[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            double s = 0;
            for (int m = 0; m < 3; ++m) s += K[3 * r + m] * K[3 * m + c];
            K2[3 * r + c] = s;
        }
    for (int i = 0; i < 9; ++i) J[i] = (i % 4 == 0 ? 1.0 : 0.0) - a * K[i] + b * K2[i];
}

template <class T>
void grow_array(T*& p, size_t old_n, size_t new_n, int fill_byte, cudaStream_t s) {
    T* q = nullptr;
    CK(cudaMalloc(&q, sizeof(T) * std::max<size_t>(new_n, 1)));
    if (fill_byte >= 0) CK(cudaMemsetAsync(q, fill_byte, sizeof(T) * new_n, s));
    if (p != nullptr && old_n > 0) CK(cudaMemcpyAsync(q, p, sizeof(T) * old_n, cudaMemcpyDeviceToDevice, s));
    if (p != nullptr) {
        CK(cudaStreamSynchronize(s));
        CK(cudaFree(p));
    }
    p = q;
}

template <class T>
void free_array(T*& p) {
    if (p != nullptr) cudaFree(p);
    p = nullptr;
}

}  // namespace

struct Tree {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    float del_param = 0.5f, bal_param = 0.6f, ds_size = 0.2f;
    int fill = 16;
    int min_size = 2 * LEAF_CAP;
    int knn_lanes = 1;     // threads per kNN query (1, 2 or 4)
    // Tree levels used to order a kNN batch before the search: -1 (default)
    // = QBIN_BITS for batches of at least QBIN_AUTO_QUERIES queries, none
    // below (measured on the 1M-point map: -12 % at 1M queries, +16 % at
    // 100k); 0 = never; 1..16 = always (batches of QBIN_MIN_QUERIES or more).
    int knn_bin_bits = -1;
    int bin_bits_for(long long nq) const {
        if (knn_bin_bits >= 0) return knn_bin_bits;
        return nq >= QBIN_AUTO_QUERIES ? QBIN_BITS : 0;
    }
    // On Grace-Blackwell the GPU reads and writes pageable host memory through
    // NVLink-C2C with the CPU's page tables (cudaDevAttrPageableMemoryAccess).
    // Host-pointer searches then run their kernels directly on the caller's
    // buffers instead of staging copies.  IKDG_HOST_STAGING=1 forces copies.
    int host_mode = 0;  // 0: staging copies, 1: direct reads + staged results, 2: all direct

    DevTree dt{};
    UpdateAux aux{};
    DevStatus* st_dev = nullptr;
    DevStatus* st = nullptr;  // pinned host mirror
    Arena op, bld, small;
    float4* removed = nullptr;
    long long removed_cap = 0;
    long long next_id = 0;
    int list_cap = 0;

    // Calls that change or stage through the tree's own buffers hold `mu`
    // exclusively; small host-pointer kNN calls hold it shared and run on
    // search contexts of their own (below), so concurrent Nearest_Search
    // callers (ikd_Tree.cpp:875-884) search at the same time.
    std::shared_mutex mu;
    std::mutex err_mu;
    std::string err;
    // IKDG_DEBUG_VALIDATE=1: check the whole tree's structure after every
    // mutation (slow; for tests and debugging).
    bool debug_validate = std::getenv("IKDG_DEBUG_VALIDATE") != nullptr;
    std::string dbg_note;
    int dbg_round = 0;

    // ---- lifetime -------------------------------------------------------------
    void init(int dev) {
        device = dev;
        CK(cudaSetDevice(device));
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        own_stream = true;
        CK(cudaMalloc(&st_dev, sizeof(DevStatus)));
        CK(cudaMallocHost(&st, sizeof(DevStatus)));
        std::memset(st, 0, sizeof(DevStatus));
        CK(cudaMemsetAsync(st_dev, 0, sizeof(DevStatus), stream));
        dt.st = st_dev;
        int pageable = 0;
        if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) {
            cudaGetLastError();
            pageable = 0;
        }
        host_mode = pageable != 0 ? 1 : 0;
        if (const char* m = std::getenv("IKDG_HOST_MODE")) host_mode = pageable != 0 ? std::atoi(m) : 0;
        if (std::getenv("IKDG_HOST_STAGING") != nullptr) host_mode = 0;
        ensure_pools(64, 64);
        reset_tree();
        CK(cudaStreamSynchronize(stream));
    }

    void destroy() {
        destroy_ctxs();
        if (stream != nullptr) cudaStreamSynchronize(stream);
        free_array(dt.node);
        free_array(dt.ncnt);
        free_array(dt.nparent);
        free_array(dt.nheight);
        free_array(dt.pts);
        free_array(dt.leaf_n);
        free_array(dt.lparent);
        free_array(dt.free_node);
        free_array(dt.free_leaf);
        free_array(aux.pend);
        free_array(aux.arrive);
        free_array(aux.viol_flag);
        free_array(aux.job_of_node);
        free_array(aux.node_job);
        free_array(aux.dirty_flag);
        free_array(aux.job_of_leaf);
        free_array(aux.leaf_job);
        free_array(aux.items);
        free_array(aux.viol);
        free_array(aux.jobs);
        free_array(aux.job_link);
        free_array(aux.job_count);
        free_array(aux.job_off);
        free_array(aux.job_fill);
        free_array(removed);
        op.release();
        bld.release();
        small.release();
        if (st_dev != nullptr) cudaFree(st_dev);
        if (st != nullptr) cudaFreeHost(st);
        st_dev = nullptr;
        st = nullptr;
        if (own_stream && stream != nullptr) cudaStreamDestroy(stream);
        stream = nullptr;
    }

    // ---- pools -----------------------------------------------------------------
    void ensure_pools(long long need_nodes, long long need_leaves) {
        int old_n = dt.node_cap, old_l = dt.leaf_cap;
        if (need_nodes > INT32_MAX / 2 || need_leaves > INT32_MAX / 2) throw CapacityFail{"tree too large"};
        int new_n = old_n, new_l = old_l;
        if (need_nodes > old_n) new_n = (int)std::max<long long>(need_nodes, (long long)old_n * 3 / 2);
        if (need_leaves > old_l) new_l = (int)std::max<long long>(need_leaves, (long long)old_l * 3 / 2);
        if (new_n != old_n) {
            grow_array(dt.node, (size_t)old_n * 4, (size_t)new_n * 4, -1, stream);
            grow_array(dt.ncnt, old_n, new_n, 0, stream);
            grow_array(dt.nparent, old_n, new_n, 0xff, stream);
            grow_array(dt.nheight, old_n, new_n, 0, stream);
            grow_array(dt.free_node, old_n, new_n, -1, stream);
            grow_array(aux.pend, old_n, new_n, 0, stream);
            grow_array(aux.arrive, old_n, new_n, 0, stream);
            grow_array(aux.viol_flag, old_n, new_n, 0, stream);
            grow_array(aux.job_of_node, old_n, new_n, 0xff, stream);
            grow_array(aux.node_job, old_n, new_n, 0xff, stream);
            dt.node_cap = new_n;
        }
        if (new_l != old_l) {
            grow_array(dt.pts, (size_t)old_l * LEAF_CAP, (size_t)new_l * LEAF_CAP, -1, stream);
            grow_array(dt.leaf_n, old_l, new_l, 0, stream);
            grow_array(dt.lparent, old_l, new_l, 0xff, stream);
            grow_array(dt.free_leaf, old_l, new_l, -1, stream);
            grow_array(aux.dirty_flag, old_l, new_l, 0, stream);
            grow_array(aux.job_of_leaf, old_l, new_l, 0xff, stream);
            grow_array(aux.leaf_job, old_l, new_l, 0xff, stream);
            dt.leaf_cap = new_l;
        }
        int need_list = dt.node_cap + dt.leaf_cap + 2;
        if (need_list > list_cap) {
            grow_array(aux.items, list_cap, need_list, -1, stream);
            grow_array(aux.viol, list_cap, need_list, -1, stream);
            grow_array(aux.jobs, list_cap, need_list, -1, stream);
            grow_array(aux.job_link, list_cap, need_list, -1, stream);
            grow_array(aux.job_count, list_cap, need_list, 0, stream);
            grow_array(aux.job_off, list_cap, need_list, 0, stream);
            grow_array(aux.job_fill, list_cap, need_list, 0, stream);
            list_cap = need_list;
            aux.list_cap = need_list;
        }
    }

    // Room for a build of `pts` points in `jobs` jobs on top of the current pools.
    void reserve_build(long long pts, long long jobs) {
        long long min_leaf = std::max(1, (fill + 1) / 2);
        long long leaves = pts / min_leaf + jobs + 2;
        long long nodes = leaves + 2;
        long long free_l = (long long)st->free_leaf_n + dt.leaf_cap - st->leaf_top;
        long long free_n = (long long)st->free_node_n + dt.node_cap - st->node_top;
        long long want_l = dt.leaf_cap, want_n = dt.node_cap;
        if (free_l < leaves) want_l = (long long)st->leaf_top + leaves + leaves / 4 + 64;
        if (free_n < nodes) want_n = (long long)st->node_top + nodes + nodes / 4 + 64;
        ensure_pools(want_n, want_l);
    }

    void ensure_removed(long long need) {
        if (need <= removed_cap) return;
        long long nc = std::max(need, removed_cap * 3 / 2 + 1024);
        grow_array(removed, (size_t)std::min<long long>(removed_cap, st->removed_n), (size_t)nc, -1, stream);
        removed_cap = nc;
    }

    // ---- status ------------------------------------------------------------------
    void read_status() {
        CK(cudaMemcpyAsync(st, st_dev, sizeof(DevStatus), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        if (st->err & ERR_ANY_INTERNAL) {
            int e = st->err;
            std::string m = "device error:";
            if (e & ERR_POOL) m += " node pool exhausted;";
            if (e & ERR_POOL_LEAF) m += " leaf pool exhausted;";
            if (e & ERR_SEG) m += " builder segment overflow;";
            if (e & ERR_ROUTE) m += " insertion without root;";
            if (e & ERR_OVF_JOB) {
                m += " overflow point outside rebuild jobs [leaf " + std::to_string(st->dbg[1]) + " parent " +
                     std::to_string(st->dbg[2]) + " fill " + std::to_string(st->dbg[3]) + " job_of_leaf " +
                     std::to_string(st->dbg[4]) + " dirty " + std::to_string(st->dbg[5]) + " parent_viol " +
                     std::to_string(st->dbg[6]) + " n_ovf " + std::to_string(st->dbg[7]) + " n_jobs " +
                     std::to_string(st->n_jobs) + "];";
            }
            if (e & ERR_LOOP) m += " loop cap reached;";
            if (e & ERR_LIST) m += " work list overflow;";
            throw Internal{m};
        }
    }
    void zero_fields(size_t off, size_t bytes) {
        CK(cudaMemsetAsync((char*)st_dev + off, 0, bytes, stream));
    }
    // Clears the per-call counters (everything but the pool state and removed_n).
    void reset_counters() {
        zero_fields(offsetof(DevStatus, err), offsetof(DevStatus, root_code) - offsetof(DevStatus, err));
        zero_fields(offsetof(DevStatus, count), 2 * sizeof(long long));
        zero_fields(offsetof(DevStatus, job_total), sizeof(long long) + 8 * sizeof(int));
    }
    void set_status_ll(size_t off, long long v) {
        CK(cudaMemcpyAsync((char*)st_dev + off, &v, sizeof(v), cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));  // v lives on this stack frame
    }

    // Empty tree: pools cleared, sentinel with no children.
    void reset_tree() {
        zero_fields(0, 6 * sizeof(int));
        int one = 1;
        CK(cudaMemcpyAsync(&st_dev->node_top, &one, sizeof(int), cudaMemcpyHostToDevice, stream));
        const float inf = INFINITY;
        float rec[16] = {inf, inf, inf, -inf, -inf, -inf, inf, inf, inf, -inf, -inf, -inf, 0.f, 0.f, 0.f, 0.f};
        int zero_codes[4] = {0, 0, 0, 0};
        std::memcpy(&rec[12], zero_codes, sizeof(zero_codes));
        int4 zc = make_int4(0, 0, 0, 0);
        int minus1 = -1, h0 = 0;
        CK(cudaMemcpyAsync(dt.node, rec, sizeof(rec), cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(dt.ncnt, &zc, sizeof(zc), cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(dt.nparent, &minus1, sizeof(int), cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(dt.nheight, &h0, sizeof(int), cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));  // the sources above live on this stack frame
        st->node_top = 1;
        st->leaf_top = 0;
        st->free_node_n = st->free_leaf_n = 0;
        st->root_code = 0;
        st->root_slots = st->root_deleted = 0;
    }

    // ---- rebuild jobs ---------------------------------------------------------------
    Criteria criteria() const { return Criteria{del_param, bal_param, min_size, fill}; }

    // Runs the jobs selected in aux (st->n_jobs on the device, nj here):
    // gather their valid points (plus overflow points), rebuild, relink and
    // refit their ancestors.
    // bound: an upper bound on the jobs selected (the violator count); the
    // job counts, totals and sizes come back in one status read.
    // counted: the jobs were selected and counted before the last status read
    // (launch_select_and_count), which brought their count and sizes back.
    void run_jobs(int bound, const int4* ovf_leaf, const float4* ovf_pts, int ovf_bound, bool counted = false) {
        if (!counted) {
            small.ensure(scan_temp_bytes(bound + 1) + 1024, stream);
            launch_job_count(dt, aux, st->leaf_top, st->node_top, ovf_leaf, ovf_bound, bound, small.p, stream);
            read_status();
        }
        const int nj = st->n_jobs;
        if (nj == 0) throw Internal{"violators without a topmost job"};
        if (debug_validate) {
            std::vector<int> jobs(nj), links(nj);
            CK(cudaMemcpyAsync(jobs.data(), aux.jobs, sizeof(int) * nj, cudaMemcpyDeviceToHost, stream));
            CK(cudaMemcpyAsync(links.data(), aux.job_link, sizeof(int) * nj, cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            std::vector<int> sl(links);
            std::sort(sl.begin(), sl.end());
            for (int i = 1; i < nj; ++i)
                if (sl[i] == sl[i - 1]) {
                    std::string m = "two rebuild jobs share the link " + std::to_string(sl[i]) + " (" + dbg_note +
                                    "); jobs with it:";
                    for (int j = 0; j < nj; ++j)
                        if (links[j] == sl[i]) {
                            m += " [job " + std::to_string(j) + " code " + std::to_string(jobs[j]);
                            int parent_link = -9, cnt = -9;
                            if (jobs[j] < 0) {
                                CK(cudaMemcpy(&parent_link, dt.lparent + code_leaf(jobs[j]), sizeof(int),
                                              cudaMemcpyDeviceToHost));
                                CK(cudaMemcpy(&cnt, dt.leaf_n + code_leaf(jobs[j]), sizeof(int),
                                              cudaMemcpyDeviceToHost));
                            } else {
                                CK(cudaMemcpy(&parent_link, dt.nparent + jobs[j], sizeof(int), cudaMemcpyDeviceToHost));
                            }
                            m += " parent_link " + std::to_string(parent_link) + " leaf_n " + std::to_string(cnt) + "]";
                        }
                    float rec[16];
                    CK(cudaMemcpy(rec, dt.node, sizeof(rec), cudaMemcpyDeviceToHost));
                    int root = 0;
                    std::memcpy(&root, &rec[12], sizeof(int));
                    m += " root code " + std::to_string(root) + "; round " + std::to_string(dbg_round);
                    throw Internal{m};
                }
        }
        long long total = st->job_total;
        long long max_job = st->max_job;
        reserve_build(total, nj);
        ensure_removed(st->removed_n + st->root_deleted + 1);
        size_t bytes = align_up(sizeof(float4) * std::max<long long>(total, 1)) +
                       build_scratch_bytes(std::max<long long>(total, 1), nj, fill) + 4096;
        bld.ensure(bytes, stream);
        float4* gathered = (float4*)bld.p;
        BuildScratch bs;
        carve_build_scratch((char*)bld.p + align_up(sizeof(float4) * std::max<long long>(total, 1)),
                            std::max<long long>(total, 1), nj, fill, &bs);
        launch_job_gather(dt, aux, st->leaf_top, st->node_top, ovf_leaf, ovf_pts, ovf_bound, gathered, removed,
                          removed_cap, stream);
        build_subtrees(dt, gathered, total, aux.job_off, aux.job_link, nj, std::max<long long>(max_job, 1), fill, bs,
                       stream);
        zero_fields(offsetof(DevStatus, n_items), sizeof(int));
        zero_fields(offsetof(DevStatus, n_viol), sizeof(int));
        launch_job_finish(dt, aux, nj, stream);
        zero_fields(offsetof(DevStatus, n_jobs), sizeof(int));
        launch_refit(dt, aux, aux.items, &st_dev->n_items, nj, criteria(), stream);
    }

    // After a mutation queued dirty leaves in aux.items: refit, then rebuild
    // the topmost subtrees that violate the criteria (up to three rounds).
    void finish_update(const int4* ovf_leaf, const float4* ovf_pts, int ovf_bound, bool refit_first = true) {
        int bound = list_cap;
        if (refit_first) {
            launch_refit(dt, aux, aux.items, &st_dev->n_items, bound, criteria(), stream);
            if (debug_validate) check_valid("after the refit of a mutation", /*at_rest=*/false);
        }
        // The dirty list is consumed: the next update starts a fresh one.
        zero_fields(offsetof(DevStatus, n_items), sizeof(int));
        // Rebuilding a subtree can unbalance its ancestors; each round moves
        // the violations up, so a few rounds settle the tree.  The root
        // snapshot is taken before every status read: when the read finds no
        // violators it is already the final status of the call.
        bool settled = false;
        for (int round = 0; round < 8; ++round) {
            launch_snapshot_root(dt, stream);
            // The first round selects and counts its rebuild jobs before the
            // status read (nothing happens on the device when there are no
            // violators), so one read brings the violators, the jobs and
            // their sizes.  After a mutation no build ran since the last
            // read, so the host's pool tops bound the leaf and node scans;
            // later rounds, and the call after rebuild_all's build, read
            // first.
            const bool ahead = round == 0 && refit_first;
            if (ahead) launch_select_and_count(dt, aux, st->leaf_top, st->node_top, ovf_leaf, ovf_bound, stream);
            read_status();
            int nv = st->n_viol;
            if (nv == 0) {
                settled = true;
                break;
            }
            if (round == 7) {
                // Still unsettled: clear the flags; the next call retries.
                launch_clear_viol(dt, aux, nv, stream);
                break;
            }
            if (!ahead) launch_select_jobs(dt, aux, nv, stream);
            dbg_round = round;
            // at most nv jobs: run_jobs reads the job count with its own sizes
            run_jobs(nv, round == 0 ? ovf_leaf : nullptr, round == 0 ? ovf_pts : nullptr, round == 0 ? ovf_bound : 0,
                     ahead);
            zero_fields(offsetof(DevStatus, n_items), sizeof(int));
            if (debug_validate) {
                read_status();
                if (st->n_viol == 0) check_valid("after a rebuild round");
            }
        }
        if (!settled) {
            zero_fields(offsetof(DevStatus, n_viol), sizeof(int));
            launch_snapshot_root(dt, stream);
            read_status();
        }
        if (st->err & ERR_STACK) throw Internal{"tree deeper than the traversal stack"};
        if (debug_validate) check_valid("end of update");
        if (st->err & ERR_ID) throw CapacityFail{"point id space exhausted"};
    }

    // Builds the points `pts` (device, {x,y,z,id}) as the whole tree.
    void build_root(const float4* pts, long long n) {
        long long nn = std::max<long long>(n, 1);
        reserve_build(n, 1);
        int host_job[3] = {0, (int)n, 0};
        small.ensure(4096, stream);
        int* job = (int*)small.p;
        CK(cudaMemcpyAsync(job, host_job, sizeof(host_job), cudaMemcpyHostToDevice, stream));
        bld.ensure(build_scratch_bytes(nn, 1, fill) + 4096, stream);
        BuildScratch bs;
        carve_build_scratch(bld.p, nn, 1, fill, &bs);
        build_subtrees(dt, pts, n, job, job + 2, 1, nn, fill, bs, stream);
        launch_snapshot_root(dt, stream);
        read_status();
    }

    // ---- API -----------------------------------------------------------------------
    void build(const float* xyz, long long n, int stride) {
        if (n < 0 || stride < 3 || (n > 0 && xyz == nullptr)) throw BadArg{"build: bad arguments"};
        if (n > MAX_ID) throw CapacityFail{"build: too many points"};
        reset_counters();
        float4* packed = nullptr;
        if (n > 0) {
            op.ensure(align_up(sizeof(float) * n * stride) + align_up(sizeof(float4) * n), stream);
            Carver c(op.p);
            float* raw = c.take<float>((size_t)n * stride);
            packed = c.take<float4>(n);
            CK(cudaMemcpyAsync(raw, xyz, sizeof(float) * n * stride, cudaMemcpyHostToDevice, stream));
            launch_pack_points(dt, raw, stride, n, 0, packed, stream);
            read_status();
            if (st->err & ERR_INPUT) throw BadArg{"build: non-finite coordinate"};
        }
        reset_tree();
        next_id = n;
        if (n == 0) {
            launch_snapshot_root(dt, stream);
            read_status();
            return;
        }
        build_root(packed, n);
    }

    void add_points(const float* xyz, long long n, int stride, bool downsample, long long* n_added) {
        if (n < 0 || stride < 3 || (n > 0 && xyz == nullptr)) throw BadArg{"add_points: bad arguments"};
        if (n_added) *n_added = 0;
        if (n == 0) return;
        if (next_id + n > (long long)MAX_ID + 1) throw CapacityFail{"point id space exhausted"};
        if (downsample && !(ds_size > 0.f && std::isfinite(ds_size))) throw BadArg{"downsample size must be > 0"};
        reset_counters();
        if (debug_validate) check_valid("start of Add_Points");
        if (!downsample) {
            op.ensure(align_up(sizeof(float) * n * stride) + 2 * align_up(sizeof(float4) * n) +
                          align_up(sizeof(int4) * n),
                      stream);
            Carver c(op.p);
            float* raw = c.take<float>((size_t)n * stride);
            float4* packed = c.take<float4>(n);
            int4* ovf_leaf = c.take<int4>(n);
            float4* ovf_pts = c.take<float4>(n);
            CK(cudaMemcpyAsync(raw, xyz, sizeof(float) * n * stride, cudaMemcpyHostToDevice, stream));
            launch_pack_points(dt, raw, stride, n, next_id, packed, stream);
            if (st->root_code == 0) {
                read_status();
                if (st->err & ERR_INPUT) throw BadArg{"add_points: non-finite coordinate"};
                next_id += n;
                build_root(packed, n);
                return;
            }
            // no status read before the insertion: route_append_kernel does
            // nothing once a non-finite input has set ERR_INPUT, and the read
            // that ends finish_update reports it
            launch_route_append(dt, aux, packed, n, ovf_leaf, ovf_pts, stream);
            next_id += n;  // taken even if a later step fails: ids are never reused
            finish_update(ovf_leaf, ovf_pts, (int)n);
            if (st->err & ERR_INPUT) {
                next_id -= n;  // nothing was inserted
                throw BadArg{"add_points: non-finite coordinate"};
            }
            return;
        }
        // Voxel downsampling.
        // (voxel, stored point) pairs: the stored points now plus this call's
        // insertions.  IKDG_DS_PAIR_CAP lowers the room (tests use it to run
        // the walking deletion that takes over when the list overflows).
        long long pair_cap = std::min<long long>((long long)st->root_slots + n + 65536, INT_MAX / 2);
        if (const char* e = std::getenv("IKDG_DS_PAIR_CAP")) pair_cap = std::max(1ll, std::min(pair_cap, std::atoll(e)));
        op.ensure(align_up(sizeof(float) * n * stride) + ds_scratch_bytes(n, pair_cap) + align_up(sizeof(float4) * n) +
                      align_up(sizeof(int4) * n) + 4096,
                  stream);
        Carver c(op.p);
        float* raw = c.take<float>((size_t)n * stride);
        int4* ovf_leaf = c.take<int4>(n);
        float4* ovf_pts = c.take<float4>(n);
        DsScratch d;
        carve_ds_scratch(op.p == nullptr ? nullptr : (char*)op.p + c.off, n, pair_cap, &d);
        CK(cudaMemcpyAsync(raw, xyz, sizeof(float) * n * stride, cudaMemcpyHostToDevice, stream));
        launch_ds_prepare(dt, raw, stride, n, ds_size, d, stream);
        // No status read between the phases of a sub-batch: the kernels read
        // the group count, the sub-batch end and the non-finite flag on the
        // device (n bounds the group count for their grids), and the status
        // read that ends the sub-batch brings all three back.
        const int n_bound = (int)n;
        const long long first_id = next_id;
        next_id += n;  // taken even if a later step fails: ids are never reused
        long long a = 0;
        while (a < n) {
            launch_set_ll((long long*)((char*)st_dev + offsetof(DevStatus, count)), n, stream);
            if (debug_validate) check_valid("start of a downsampling sub-batch");
            launch_ds_search(dt, n, ds_size, a, d, n_bound, stream);
            zero_fields(offsetof(DevStatus, n_ins), sizeof(int));
            launch_ds_fold(dt, aux, n, a, first_id, d, n_bound, stream);
            if (debug_validate) {
                read_status();
                std::string m = "sub-batch from " + std::to_string(a) + " to " + std::to_string(st->count) +
                                " groups " + std::to_string(st->n_groups) + " ins " + std::to_string(st->n_ins) +
                                " items " + std::to_string(st->n_items);
                dbg_note = m;
            }
            if (st->root_code == 0) {
                read_status();
                if (st->err & ERR_INPUT) {
                    next_id = first_id;  // nothing was inserted
                    throw BadArg{"add_points: non-finite coordinate"};
                }
                if (st->n_ins > 0) build_root(d.ins, st->n_ins);
            } else {
                launch_route_append_dev_count(dt, aux, d.ins, n_bound, &st_dev->n_ins, ovf_leaf, ovf_pts, stream);
                finish_update(ovf_leaf, ovf_pts, n_bound);
                // a non-finite input left the tree untouched (no kernel above
                // changed anything once ERR_INPUT was set)
                if (st->err & ERR_INPUT) {
                    next_id = first_id;
                    throw BadArg{"add_points: non-finite coordinate"};
                }
            }
            // finish_update / build_root ended with a status read: st->count
            // is the end ds_h1_kernel found for this sub-batch
            a = std::min<long long>(std::max<long long>(st->count, a + 1), n);
        }
        // Every sub-batch ended with a status read (finish_update, build_root
        // or the read before it), so count2 is current.
        if (n_added) *n_added = st->count2;
    }

    void delete_points(const float* xyz, long long n, int stride) {
        if (n < 0 || stride < 3 || (n > 0 && xyz == nullptr)) throw BadArg{"delete_points: bad arguments"};
        if (n == 0 || st->root_code == 0) return;
        reset_counters();
        op.ensure(align_up(sizeof(float) * n * stride), stream);
        float* raw = (float*)op.p;
        CK(cudaMemcpyAsync(raw, xyz, sizeof(float) * n * stride, cudaMemcpyHostToDevice, stream));
        launch_delete_points(dt, aux, raw, stride, n, stream);
        finish_update(nullptr, nullptr, 0);
    }

    long long delete_boxes(const float* boxes, long long m) {
        if (m < 0 || (m > 0 && boxes == nullptr)) throw BadArg{"delete_boxes: bad arguments"};
        if (m == 0 || st->root_code == 0) return 0;
        reset_counters();
        op.ensure(align_up(sizeof(float) * m * 6), stream);
        float* raw = (float*)op.p;
        CK(cudaMemcpyAsync(raw, boxes, sizeof(float) * m * 6, cudaMemcpyHostToDevice, stream));
        launch_delete_boxes(dt, aux, raw, m, F_DEL, (long long*)((char*)st_dev + offsetof(DevStatus, count)),
                            stream);
        // The rebuild rounds leave `count` alone: its value arrives with the
        // status reads of finish_update.
        finish_update(nullptr, nullptr, 0);
        return st->count;
    }

    void add_boxes(const float* boxes, long long m) {
        if (m < 0 || (m > 0 && boxes == nullptr)) throw BadArg{"add_boxes: bad arguments"};
        if (m == 0 || st->root_code == 0) return;
        reset_counters();
        op.ensure(align_up(sizeof(float) * m * 6), stream);
        float* raw = (float*)op.p;
        CK(cudaMemcpyAsync(raw, boxes, sizeof(float) * m * 6, cudaMemcpyHostToDevice, stream));
        launch_add_boxes(dt, aux, raw, m, stream);
        finish_update(nullptr, nullptr, 0);
    }

    // True when every non-null pointer is page-locked host memory (registered
    // with or allocated by CUDA).
    static bool all_pinned(std::initializer_list<const void*> ptrs) {
        for (const void* p : ptrs) {
            if (p == nullptr) continue;
            cudaPointerAttributes a{};
            if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
                cudaGetLastError();
                return false;
            }
            if (a.type != cudaMemoryTypeHost) return false;
        }
        return true;
    }

    // ---- concurrent small searches ------------------------------------------------
    // A search context: a stream, a device buffer (a status block for the
    // kernel's error bits, the result rows, the kNN scratch) and a pinned host
    // mirror of the status and rows, so one device-to-host copy returns
    // everything.  Contexts are pooled per tree and reused.
    struct SearchCtx {
        cudaStream_t s = nullptr;
        char* d = nullptr;
        char* h = nullptr;
        size_t dcap = 0, hcap = 0;
    };
    std::mutex ctx_mu;
    std::vector<SearchCtx*> ctx_free;
    std::vector<SearchCtx*> ctx_all;

    SearchCtx* take_ctx() {
        {
            std::lock_guard<std::mutex> l(ctx_mu);
            if (!ctx_free.empty()) {
                SearchCtx* c = ctx_free.back();
                ctx_free.pop_back();
                return c;
            }
        }
        SearchCtx* c = new SearchCtx;
        if (cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) != cudaSuccess) {
            delete c;
            throw CudaFail{cudaGetLastError(), "search stream"};
        }
        std::lock_guard<std::mutex> l(ctx_mu);
        ctx_all.push_back(c);
        return c;
    }
    void give_ctx(SearchCtx* c) {
        std::lock_guard<std::mutex> l(ctx_mu);
        ctx_free.push_back(c);
    }
    void destroy_ctxs() {
        for (SearchCtx* c : ctx_all) {
            if (c->s) cudaStreamSynchronize(c->s);
            if (c->d) cudaFree(c->d);
            if (c->h) cudaFreeHost(c->h);
            if (c->s) cudaStreamDestroy(c->s);
            delete c;
        }
        ctx_all.clear();
        ctx_free.clear();
    }
    static void ctx_reserve(SearchCtx* c, size_t dneed, size_t hneed) {
        if (dneed > c->dcap) {
            if (c->d) CK(cudaFree(c->d));
            c->d = nullptr;
            c->dcap = 0;
            CK(cudaMalloc(&c->d, dneed));
            c->dcap = dneed;
        }
        if (hneed > c->hcap) {
            if (c->h) CK(cudaFreeHost(c->h));
            c->h = nullptr;
            c->hcap = 0;
            CK(cudaMallocHost(&c->h, hneed));
            c->hcap = hneed;
        }
    }

    // Host-pointer kNN of a few queries (called with `mu` held shared).  Same
    // kernels and results as knn(); the tree is only read.
    void knn_small(const float* q, long long nq, int stride, int k, double max_dist, int* ids, float* d2, float* xyz,
                   int* cnt) {
        if (nq < 0 || stride < 3 || k < 1 || (nq > 0 && (q == nullptr || ids == nullptr || d2 == nullptr)))
            throw BadArg{"knn: bad arguments"};
        if (nq == 0) return;
        const size_t nk = (size_t)nq * k;
        const size_t o_ids = align_up(sizeof(DevStatus));
        const size_t o_d2 = o_ids + align_up(sizeof(int) * nk);
        const size_t o_xyz = o_d2 + align_up(sizeof(float) * nk);
        const size_t o_cnt = o_xyz + (xyz ? align_up(sizeof(float) * 3 * nk) : 0);
        const size_t o_end = o_cnt + (cnt ? align_up(sizeof(int) * nq) : 0);
        const size_t o_q = o_end;
        const size_t o_tmp = o_q + (host_mode == 0 ? align_up(sizeof(float) * nq * stride) : 0);
        const size_t dneed = o_tmp + align_up(knn_temp_bytes(nq, k) + 256);
        const size_t hneed = std::max(o_end, o_tmp);
        SearchCtx* c = take_ctx();
        try {
            ctx_reserve(c, dneed, hneed);
            DevTree t = dt;
            t.st = (DevStatus*)c->d;  // this call's error bits land in its own status block
            CK(cudaMemsetAsync(c->d + offsetof(DevStatus, err), 0, sizeof(int), c->s));
            const float* qsrc = q;
            if (host_mode == 0) {
                std::memcpy(c->h + o_q, q, sizeof(float) * nq * stride);
                CK(cudaMemcpyAsync(c->d + o_q, c->h + o_q, sizeof(float) * nq * stride, cudaMemcpyHostToDevice,
                                   c->s));
                qsrc = (const float*)(c->d + o_q);
            }
            launch_knn(t, qsrc, stride, nq, k, max_sq_threshold(max_dist), (int*)(c->d + o_ids),
                       (float*)(c->d + o_d2), xyz ? (float*)(c->d + o_xyz) : nullptr,
                       cnt ? (int*)(c->d + o_cnt) : nullptr, c->d + o_tmp, knn_lanes, bin_bits_for(nq), c->s);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(c->h, c->d, o_end, cudaMemcpyDeviceToHost, c->s));
            CK(cudaStreamSynchronize(c->s));
            const DevStatus* hs = (const DevStatus*)c->h;
            if (hs->err & ERR_STACK) throw Internal{"knn: traversal stack overflow"};
            if (hs->err & ERR_LOOP) throw Internal{"knn: loop cap reached"};
            std::memcpy(ids, c->h + o_ids, sizeof(int) * nk);
            std::memcpy(d2, c->h + o_d2, sizeof(float) * nk);
            if (xyz) std::memcpy(xyz, c->h + o_xyz, sizeof(float) * 3 * nk);
            if (cnt) std::memcpy(cnt, c->h + o_cnt, sizeof(int) * nq);
        } catch (...) {
            give_ctx(c);
            throw;
        }
        give_ctx(c);
    }

    void knn(const float* q, long long nq, int stride, int k, double max_dist, int* ids, float* d2, float* xyz,
             int* cnt, bool device_ptrs) {
        if (nq < 0 || stride < 3 || k < 1 || (nq > 0 && (q == nullptr || ids == nullptr || d2 == nullptr)))
            throw BadArg{"knn: bad arguments"};
        if (nq == 0) return;
        if ((long long)nq * k > (1ll << 31)) throw BadArg{"knn: nq * k too large"};
        float lim = max_sq_threshold(max_dist);
        size_t nk = (size_t)nq * k;
        if (device_ptrs) {
            small.ensure(knn_temp_bytes(nq, k) + 256, stream);
            launch_knn(dt, q, stride, nq, k, lim, ids, d2, xyz, cnt, small.p, knn_lanes, bin_bits_for(nq), stream);
            CK(cudaGetLastError());
            return;
        }
        // the search reports through the error bits alone
        zero_fields(offsetof(DevStatus, err), sizeof(int));
        if (host_mode == 2 || (host_mode == 1 && all_pinned({ids, d2, xyz, cnt}))) {
            // Kernels read the queries and write the results in host memory:
            // each warp's rows leave as coalesced 16-byte spans, so the
            // transfer over the chip link overlaps the search instead of
            // following it as one copy.
            small.ensure(knn_temp_bytes(nq, k) + 256, stream);
            launch_knn(dt, q, stride, nq, k, lim, ids, d2, xyz, cnt, small.p, knn_lanes, bin_bits_for(nq), stream,
                       /*host_out=*/true);
            read_status();
            if (st->err & ERR_STACK) throw Internal{"knn: traversal stack overflow"};
            return;
        }
        op.ensure(align_up(sizeof(float) * nq * stride) + align_up(sizeof(int) * nk) + align_up(sizeof(float) * nk) +
                      align_up(sizeof(float) * nk * 3) + align_up(sizeof(int) * nq) + align_up(knn_temp_bytes(nq, k)),
                  stream);
        Carver c(op.p);
        float* dq = c.take<float>((size_t)nq * stride);
        int* dids = c.take<int>(nk);
        float* dd2 = c.take<float>(nk);
        float* dxyz = xyz ? c.take<float>(nk * 3) : nullptr;
        int* dcnt = cnt ? c.take<int>(nq) : nullptr;
        char* temp = c.take<char>(knn_temp_bytes(nq, k));
        // Mode 1: the kernel reads the (small, in-order) queries straight from
        // host memory; the results come back by DMA.
        const float* qsrc = q;
        if (host_mode == 0) {
            CK(cudaMemcpyAsync(dq, q, sizeof(float) * nq * stride, cudaMemcpyHostToDevice, stream));
            qsrc = dq;
        }
        launch_knn(dt, qsrc, stride, nq, k, lim, dids, dd2, dxyz, dcnt, temp, knn_lanes, bin_bits_for(nq), stream);
        CK(cudaMemcpyAsync(ids, dids, sizeof(int) * nk, cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(d2, dd2, sizeof(float) * nk, cudaMemcpyDeviceToHost, stream));
        if (xyz) CK(cudaMemcpyAsync(xyz, dxyz, sizeof(float) * nk * 3, cudaMemcpyDeviceToHost, stream));
        if (cnt) CK(cudaMemcpyAsync(cnt, dcnt, sizeof(int) * nq, cudaMemcpyDeviceToHost, stream));
        read_status();
        if (st->err & ERR_STACK) throw Internal{"knn: traversal stack overflow"};
    }

    // mode 0: boxes (6 floats each), mode 1: centres + radii.
    void range(int mode, const float* q, long long nq, int stride, const float* radius, int rstride,
               long long* offsets, int* ids, float* xyz, long long capacity, long long* total) {
        if (nq < 0 || offsets == nullptr || total == nullptr || (nq > 0 && q == nullptr))
            throw BadArg{"range search: bad arguments"};
        if (mode == 1 && (stride < 3 || (nq > 0 && radius == nullptr) || rstride < 0))
            throw BadArg{"radius search: bad arguments"};
        int qs = mode == 0 ? 6 : stride;
        *total = 0;
        offsets[0] = 0;
        if (nq == 0) return;
        reset_counters();
        op.ensure(align_up(sizeof(float) * nq * qs) + align_up(sizeof(float) * nq) +
                      2 * align_up(sizeof(long long) * (nq + 1)),
                  stream);
        Carver c(op.p);
        float* dq = c.take<float>((size_t)nq * qs);
        float* dr = c.take<float>(nq);
        long long* dcounts = c.take<long long>(nq + 1);
        long long* doffs = c.take<long long>(nq + 1);
        CK(cudaMemcpyAsync(dq, q, sizeof(float) * nq * qs, cudaMemcpyHostToDevice, stream));
        std::vector<float> rr;
        if (mode == 1) {
            rr.resize(nq);
            for (long long i = 0; i < nq; ++i) rr[i] = radius[i * rstride];
            CK(cudaMemcpyAsync(dr, rr.data(), sizeof(float) * nq, cudaMemcpyHostToDevice, stream));
        }
        launch_range(dt, mode, dq, qs, dr, 1, nq, dcounts, nullptr, nullptr, nullptr, -1, stream);
        std::vector<long long> counts(nq);
        CK(cudaMemcpyAsync(counts.data(), dcounts, sizeof(long long) * nq, cudaMemcpyDeviceToHost, stream));
        read_status();
        if (st->err & ERR_STACK) throw Internal{"range search: traversal stack overflow"};
        long long acc = 0;
        for (long long i = 0; i < nq; ++i) {
            offsets[i] = acc;
            acc += counts[i];
        }
        offsets[nq] = acc;
        *total = acc;
        if (acc > capacity || (acc > 0 && ids == nullptr)) throw CapacityFail{"range search: output too small"};
        if (acc == 0) return;
        bld.ensure(align_up(sizeof(int) * acc) + align_up(sizeof(float) * acc * 3), stream);
        Carver o(bld.p);
        int* dids = o.take<int>(acc);
        float* dxyz = xyz ? o.take<float>(acc * 3) : nullptr;
        CK(cudaMemcpyAsync(doffs, offsets, sizeof(long long) * (nq + 1), cudaMemcpyHostToDevice, stream));
        launch_range(dt, mode, dq, qs, dr, 1, nq, nullptr, doffs, dids, dxyz, -1, stream);
        CK(cudaMemcpyAsync(ids, dids, sizeof(int) * acc, cudaMemcpyDeviceToHost, stream));
        if (xyz) CK(cudaMemcpyAsync(xyz, dxyz, sizeof(float) * acc * 3, cudaMemcpyDeviceToHost, stream));
        read_status();
        if (st->err & ERR_OUTPUT) throw Internal{"range search: hits differ between the count and write passes"};
    }

    // Device-pointer range search, asynchronous on the tree's stream: count
    // pass, device prefix sum into offsets (offsets[nq] = total), write pass.
    // A query whose results would end past `capacity` is not written.
    void range_device(int mode, const float* q, long long nq, int stride, const float* radius, int rstride,
                      long long* offsets, int* ids, float* xyz, long long capacity, long long* total) {
        if (nq < 0 || offsets == nullptr || capacity < 0 || (nq > 0 && q == nullptr) ||
            (capacity > 0 && ids == nullptr))
            throw BadArg{"range search (device): bad arguments"};
        if (mode == 1 && (stride < 3 || (nq > 0 && radius == nullptr) || rstride < 0))
            throw BadArg{"radius search (device): bad arguments"};
        const int qs = mode == 0 ? 6 : stride;
        if (nq == 0) {
            CK(cudaMemsetAsync(offsets, 0, sizeof(long long), stream));
            if (total) CK(cudaMemsetAsync(total, 0, sizeof(long long), stream));
            return;
        }
        small.ensure(align_up(sizeof(long long) * (nq + 1)) + align_up(scan_temp_bytes(nq + 1)) + 256, stream);
        Carver c(small.p);
        long long* counts = c.take<long long>(nq + 1);
        void* temp = c.take<char>(scan_temp_bytes(nq + 1));
        CK(cudaMemsetAsync(counts + nq, 0, sizeof(long long), stream));
        launch_range(dt, mode, q, qs, radius, rstride, nq, counts, nullptr, nullptr, nullptr, -1, stream);
        exclusive_scan(counts, offsets, nq + 1, total, temp, stream);
        if (ids != nullptr) launch_range(dt, mode, q, qs, radius, rstride, nq, counts, offsets, ids, xyz, capacity, stream);
        CK(cudaGetLastError());
    }

    // ---- point-to-plane registration (no counterpart in the reference) -----------
    void upload_pose(const double pose[6], double* Rt_dev) {
        double R[9];
        so3_exp(pose, R);
        double h[12];
        for (int i = 0; i < 9; ++i) h[i] = R[i];
        for (int i = 0; i < 3; ++i) h[9 + i] = pose[3 + i];
        CK(cudaMemcpyAsync(Rt_dev, h, sizeof(h), cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));  // h lives on this stack frame
    }

    void p2p_forward(const float* scan, long long n, const double* pose, int k, double max_dist, float thresh,
                     float* planes, float* res, int* valid, double* loss) {
        if (n < 0 || scan == nullptr || pose == nullptr || planes == nullptr || res == nullptr || valid == nullptr ||
            k < 3 || k > KNN_SMEM_MAX)
            throw BadArg{"p2p_forward: bad arguments"};
        if (loss) *loss = 0;
        if (n == 0) return;
        reset_counters();
        const int nb = reg_blocks(n);
        op.ensure(align_up(sizeof(double) * 12) + align_up(sizeof(float) * 3 * n) + align_up(sizeof(int) * n * k) +
                      align_up(sizeof(float) * n * k) + align_up(sizeof(float) * 3 * n * k) + align_up(sizeof(int) * n) +
                      align_up(sizeof(double) * nb) + align_up(knn_temp_bytes(n, k)),
                  stream);
        Carver c(op.p);
        double* Rt = c.take<double>(12);
        float* w = c.take<float>(3 * n);
        int* ids = c.take<int>((size_t)n * k);
        float* d2 = c.take<float>((size_t)n * k);
        float* nbr = c.take<float>((size_t)3 * n * k);
        int* cnt = c.take<int>(n);
        double* part = c.take<double>(nb);
        char* temp = c.take<char>(knn_temp_bytes(n, k));
        upload_pose(pose, Rt);
        launch_transform(scan, n, Rt, w, stream);
        launch_knn(dt, w, 3, n, k, max_sq_threshold(max_dist), ids, d2, nbr, cnt, temp, knn_lanes, bin_bits_for(n),
                   stream);
        launch_plane_residual(scan, Rt, n, k, nbr, cnt, thresh, (float4*)planes, res, valid, part, stream);
        std::vector<double> h(nb);
        CK(cudaMemcpyAsync(h.data(), part, sizeof(double) * nb, cudaMemcpyDeviceToHost, stream));
        read_status();
        double s = 0;
        for (double v : h) s += v;
        if (loss) *loss = s;
    }

    void p2p_adjoint(const float* scan, long long n, const double* pose, const float* planes, const float* res,
                     const int* valid, double grad_loss, float* grad_points, double* grad_pose) {
        if (n < 0 || scan == nullptr || pose == nullptr || planes == nullptr || res == nullptr || valid == nullptr ||
            grad_pose == nullptr)
            throw BadArg{"p2p_adjoint: bad arguments"};
        for (int i = 0; i < 6; ++i) grad_pose[i] = 0;
        if (n == 0) return;
        const int nb = reg_blocks(n);
        op.ensure(align_up(sizeof(double) * 12) + align_up(sizeof(double) * 6 * nb), stream);
        Carver c(op.p);
        double* Rt = c.take<double>(12);
        double* part = c.take<double>((size_t)6 * nb);
        upload_pose(pose, Rt);
        launch_adjoint(scan, n, Rt, (const float4*)planes, res, valid, (float)grad_loss, grad_points, part, stream);
        std::vector<double> h(6 * (size_t)nb);
        CK(cudaMemcpyAsync(h.data(), part, sizeof(double) * 6 * nb, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        double s[6] = {0, 0, 0, 0, 0, 0};
        for (int b = 0; b < nb; ++b)
            for (int j = 0; j < 6; ++j) s[j] += h[6 * (size_t)b + j];
        double J[9];
        so3_jr(pose, J);
        for (int r = 0; r < 3; ++r)  // dL/domega = J_r^T (sum p x R^T g)
            grad_pose[r] = J[r] * s[3] + J[3 + r] * s[4] + J[6 + r] * s[5];
        for (int r = 0; r < 3; ++r) grad_pose[3 + r] = s[r];
    }

    void flatten(float* xyz, int* ids, long long capacity, long long* n) {
        if (n == nullptr) throw BadArg{"flatten: bad arguments"};
        long long valid = (long long)st->root_slots - st->root_deleted;
        *n = valid;
        if (valid > capacity || (valid > 0 && xyz == nullptr && ids == nullptr))
            throw CapacityFail{"flatten: output too small"};
        if (valid == 0) return;
        reset_counters();
        op.ensure(align_up(sizeof(float4) * valid), stream);
        float4* out = (float4*)op.p;
        launch_flatten(dt, out, (long long*)((char*)st_dev + offsetof(DevStatus, count)), stream);
        std::vector<float4> h(valid);
        CK(cudaMemcpyAsync(h.data(), out, sizeof(float4) * valid, cudaMemcpyDeviceToHost, stream));
        read_status();
        if (st->count != valid) throw Internal{"flatten: valid count mismatch"};
        for (long long i = 0; i < valid; ++i) {
            if (xyz) {
                xyz[3 * i] = h[i].x;
                xyz[3 * i + 1] = h[i].y;
                xyz[3 * i + 2] = h[i].z;
            }
            if (ids) {
                uint32_t w;
                std::memcpy(&w, &h[i].w, 4);
                ids[i] = (int)(w & ID_MASK);
            }
        }
    }

    void acquire_removed(float* xyz, int* ids, long long capacity, long long* n) {
        if (n == nullptr) throw BadArg{"acquire_removed_points: bad arguments"};
        read_status();
        long long k = std::min<long long>(st->removed_n, removed_cap);
        *n = k;
        if (k > capacity || (k > 0 && xyz == nullptr && ids == nullptr))
            throw CapacityFail{"acquire_removed_points: output too small"};
        if (k > 0) {
            std::vector<float4> h(k);
            CK(cudaMemcpyAsync(h.data(), removed, sizeof(float4) * k, cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            for (long long i = 0; i < k; ++i) {
                if (xyz) {
                    xyz[3 * i] = h[i].x;
                    xyz[3 * i + 1] = h[i].y;
                    xyz[3 * i + 2] = h[i].z;
                }
                if (ids) {
                    uint32_t w;
                    std::memcpy(&w, &h[i].w, 4);
                    ids[i] = (int)(w & ID_MASK);
                }
            }
        }
        zero_fields(offsetof(DevStatus, removed_n), sizeof(long long));
        read_status();
    }

    // Ids the tree can still return: every stored slot (valid or deleted),
    // then the removed points not yet acquired.
    void live_ids(int* ids, long long capacity, long long* n) {
        if (n == nullptr) throw BadArg{"live_ids: bad arguments"};
        const long long stored = st->root_slots;
        const long long rem = std::min<long long>(st->removed_n, removed_cap);
        *n = stored + rem;
        if (*n > capacity || (*n > 0 && ids == nullptr)) throw CapacityFail{"live_ids: output too small"};
        if (*n == 0) return;
        reset_counters();
        op.ensure(align_up(sizeof(int) * std::max<long long>(stored, 1)), stream);
        int* out = (int*)op.p;
        if (stored > 0) launch_stored_ids(dt, out, stored, (long long*)((char*)st_dev + offsetof(DevStatus, count)),
                                          stream);
        if (stored > 0) CK(cudaMemcpyAsync(ids, out, sizeof(int) * stored, cudaMemcpyDeviceToHost, stream));
        std::vector<float4> h(rem);
        if (rem > 0) CK(cudaMemcpyAsync(h.data(), removed, sizeof(float4) * rem, cudaMemcpyDeviceToHost, stream));
        read_status();
        if (st->count != stored) throw Internal{"live_ids: stored slot count mismatch"};
        for (long long i = 0; i < rem; ++i) {
            uint32_t w;
            std::memcpy(&w, &h[i].w, 4);
            ids[stored + i] = (int)(w & ID_MASK);
        }
    }

    void rebuild_all() {
        if (st->root_code == 0) return;
        reset_counters();
        launch_select_root_job(dt, aux, stream);
        run_jobs(1, nullptr, nullptr, 0);
        // run_jobs already refit the root's parent (the sentinel: nothing to do)
        finish_update(nullptr, nullptr, 0, /*refit_first=*/false);
    }

    void check_valid(const char* stage, bool at_rest = true) {
        long long bad = validate(at_rest);
        if (bad) {
            std::string m = std::string("structural validation failed at ") + stage + " (" + dbg_note + "): " +
                            std::to_string(bad) + " violations; first:";
            for (int i = 0; i < 7; ++i) m += " " + std::to_string(st->dbg[i]);
            throw Internal{m};
        }
    }

    long long validate(bool at_rest = true) {
        zero_fields(offsetof(DevStatus, bad), sizeof(long long));
        launch_validate(dt, aux, at_rest, (long long*)((char*)st_dev + offsetof(DevStatus, bad)), stream);
        read_status();
        return st->bad;
    }

    void tree_range(float* box6) {
        float rec[6];
        CK(cudaMemcpyAsync(rec, dt.node, sizeof(rec), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        bool empty = st->root_code == 0 || !(rec[0] <= rec[3]);
        for (int a = 0; a < 6; ++a) box6[a] = empty ? 0.f : rec[a];
    }

    void root_alpha(float* bal, float* del) {
        int slots = st->root_slots;
        float b = 0.5f, d = 0.f;
        if (st->root_code > 0 && slots > 0) {
            int4 c;
            CK(cudaMemcpyAsync(&c, dt.ncnt + st->root_code, sizeof(c), cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            float fb = (float)c.x / (float)slots;
            b = fb >= 0.5f ? fb : 1.f - fb;
        }
        if (slots > 0) d = (float)st->root_deleted / (float)slots;
        if (bal) *bal = b;
        if (del) *del = d;
    }
};

// ---- multi-tree batches (no counterpart in the reference) --------------------------
// A list of search requests over several trees, run as one CUDA graph: the
// trees' device descriptors are copied in, one persistent search kernel per
// register class runs on its own graph branch, then (for box / radius
// requests) a prefix sum over the hit counts and one persistent write kernel.
struct Batch {
    struct Req {
        BatchReq d{};
        Tree* tree = nullptr;
        double max_dist = 0;
        int lanes = 0;  // 0: the tree's kNN lanes setting
    };
    struct Group {
        int kclass, lanes, r0, r1;
        long long c_begin, c_end;
        int grid;
    };

    int device = -1;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool use_graph = true;
    // Run every request's queries in spatial order (Morton code in the tree's
    // box): one key pass and one radix sort over the whole batch, then the
    // search and write kernels take a request's queries through that order,
    // so the lanes of a warp walk nearby nodes and leaves.  Results stay in
    // query order.  Off by default: on 64 maps with 1.37M queries the sort
    // cost more than the coherence saved (8.08 ms against 7.85 ms).
    bool use_order = false;
    std::vector<Req> reqs;  // in the order added
    std::mutex mu;
    std::string err;

    // plan (rebuilt when requests change)
    bool planned = false;
    std::vector<Tree*> trees;
    std::vector<int> order;          // sorted position -> request
    std::vector<int> range_reqs;     // request indices of range requests, in order added
    std::vector<Group> groups;
    long long n_range_queries = 0, c2_end = 0;
    int write_grid = 0;
    char* dev = nullptr;             // one device allocation for the plan
    DevTree* d_trees = nullptr;
    BatchReq* d_reqs = nullptr;
    long long* d_c1 = nullptr;
    long long* d_c2 = nullptr;
    int* d_ridx = nullptr;
    long long* d_counts = nullptr;
    long long* d_goff = nullptr;
    long long* d_totals = nullptr;
    unsigned long long* d_ctr = nullptr;
    void* d_scan = nullptr;
    // query order (use_order): per request first query, keys / values of the sort
    long long n_queries = 0;
    int req_bits = 0;
    bool ordered = false;
    long long* d_qstart = nullptr;
    uint32_t* d_okeys[2] = {nullptr, nullptr};
    uint32_t* d_ovals[2] = {nullptr, nullptr};
    void* d_osort = nullptr;
    DevStatus* d_st = nullptr;
    DevTree* h_trees = nullptr;      // pinned: read by the graph's first copy
    DevStatus* h_st = nullptr;       // pinned
    std::vector<long long> h_totals;
    std::vector<cudaStream_t> branch;
    std::vector<cudaEvent_t> ev_join;
    cudaEvent_t ev_fork = nullptr, ev_done = nullptr, ev_t0 = nullptr;
    std::vector<cudaEvent_t> ev_tree;
    cudaGraphExec_t exec = nullptr;
    bool launched = false;

    void init(int dev_id) {
        device = dev_id;
        CK(cudaSetDevice(device));
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        own_stream = true;
        CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ev_done, cudaEventDisableTiming));
        CK(cudaMallocHost(&h_st, sizeof(DevStatus)));
    }

    void drop_plan() {
        if (launched && ev_done != nullptr) cudaEventSynchronize(ev_done);
        if (exec != nullptr) cudaGraphExecDestroy(exec);
        exec = nullptr;
        if (dev != nullptr) cudaFree(dev);
        dev = nullptr;
        if (h_trees != nullptr) cudaFreeHost(h_trees);
        h_trees = nullptr;
        for (auto s : branch) cudaStreamDestroy(s);
        branch.clear();
        for (auto e : ev_join) cudaEventDestroy(e);
        ev_join.clear();
        for (auto e : ev_tree) cudaEventDestroy(e);
        ev_tree.clear();
        planned = false;
    }

    void destroy() {
        drop_plan();
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_done) cudaEventDestroy(ev_done);
        if (h_st) cudaFreeHost(h_st);
        if (own_stream && stream) cudaStreamDestroy(stream);
        ev_fork = ev_done = nullptr;
        h_st = nullptr;
        stream = nullptr;
    }

    int add(Req r) {
        if (r.tree == nullptr) throw BadArg{"batch: null tree"};
        if (r.tree->device != device) throw BadArg{"batch: tree lives on another device"};
        drop_plan();
        reqs.push_back(r);
        return (int)reqs.size() - 1;
    }

    void clear() {
        drop_plan();
        reqs.clear();
    }

    int req_class(const Req& r) const { return r.d.kind == BATCH_KNN ? batch_kclass(r.d.k) : BATCH_RANGE_CLASS; }
    int req_lanes(const Req& r) const {
        if (r.d.kind != BATCH_KNN) return 1;
        int l = r.lanes > 0 ? r.lanes : r.tree->knn_lanes;
        return l >= 4 ? 4 : l >= 2 ? 2 : 1;
    }

    void plan() {
        drop_plan();
        const int n = (int)reqs.size();
        trees.clear();
        range_reqs.clear();
        std::vector<int> tree_of(n);
        for (int i = 0; i < n; ++i) {
            auto it = std::find(trees.begin(), trees.end(), reqs[i].tree);
            tree_of[i] = (int)(it - trees.begin());
            if (it == trees.end()) trees.push_back(reqs[i].tree);
            if (reqs[i].d.kind != BATCH_KNN) range_reqs.push_back(i);
        }
        order.resize(n);
        for (int i = 0; i < n; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            int ka = req_class(reqs[a]) * 8 + req_lanes(reqs[a]), kb = req_class(reqs[b]) * 8 + req_lanes(reqs[b]);
            return ka < kb;
        });
        // device descriptors, sorted order
        std::vector<BatchReq> d(n);
        std::vector<long long> c1(n);
        groups.clear();
        long long chunk = 0, cbase = 0;
        for (int p = 0; p < n; ++p) {
            Req& r = reqs[order[p]];
            BatchReq b = r.d;
            b.tree = tree_of[order[p]];
            const int kc = req_class(r), lanes = req_lanes(r);
            b.kclass = kc < BATCH_RANGE_CLASS ? kc : 0;
            b.lanes = lanes;
            const long long per = kc < BATCH_RANGE_CLASS ? BATCH_CHUNK / lanes : BATCH_CHUNK;
            b.c1 = chunk;
            b.n1 = (b.nq + per - 1) / per;
            chunk += b.n1;
            if (b.kind != BATCH_KNN) {
                b.cbase = cbase;
                cbase += b.nq;
            }
            if (groups.empty() || groups.back().kclass != kc || groups.back().lanes != lanes)
                groups.push_back(Group{kc, lanes, p, p + 1, b.c1, chunk, 0});
            else {
                groups.back().r1 = p + 1;
                groups.back().c_end = chunk;
            }
            d[p] = b;
            c1[p] = b.c1;
        }
        n_range_queries = cbase;
        std::vector<long long> qstart(n + 1, 0);
        for (int p = 0; p < n; ++p) qstart[p + 1] = qstart[p] + d[p].nq;
        n_queries = qstart[n];
        req_bits = 1;
        while ((1 << req_bits) < n) ++req_bits;
        ordered = use_order && n_queries >= QBIN_MIN_QUERIES && req_bits <= 24;
        // phase 2: range requests by c2
        std::vector<int> ridx;
        std::vector<long long> c2;
        long long chunk2 = 0;
        std::vector<int> pos_of(n);
        for (int p = 0; p < n; ++p) pos_of[order[p]] = p;
        for (size_t j = 0; j < range_reqs.size(); ++j) {
            BatchReq& b = d[pos_of[range_reqs[j]]];
            b.c2 = chunk2;
            b.n2 = (b.nq + BATCH_CHUNK - 1) / BATCH_CHUNK;
            if (b.n2 > 0) {
                ridx.push_back(pos_of[range_reqs[j]]);
                c2.push_back(chunk2);
            }
            chunk2 += b.n2;
        }
        c2_end = chunk2;
        for (auto& g : groups) g.grid = batch_search_grid(g.kclass, g.lanes);
        write_grid = batch_write_grid();
        // one allocation for the plan
        const size_t nt = trees.size(), nr = range_reqs.size();
        size_t bytes = align_up(sizeof(DevTree) * nt) + align_up(sizeof(BatchReq) * n) +
                       align_up(sizeof(long long) * n) + align_up(sizeof(long long) * (ridx.size() + 1)) +
                       align_up(sizeof(int) * (ridx.size() + 1)) + 2 * align_up(sizeof(long long) * (cbase + 1)) +
                       align_up(sizeof(long long) * (nr + 1)) + align_up(sizeof(unsigned long long) * 64) +
                       align_up(scan_temp_bytes(cbase + 1)) + align_up(sizeof(DevStatus)) + 4096;
        const long long nqo = ordered ? n_queries : 0;
        bytes += align_up(sizeof(long long) * (n + 1)) + 4 * align_up(sizeof(uint32_t) * std::max<long long>(nqo, 1)) +
                 align_up(ordered ? sort_temp_bytes(nqo, 1) : 0);
        CK(cudaMalloc(&dev, bytes));
        Carver c(dev);
        d_trees = c.take<DevTree>(nt);
        d_reqs = c.take<BatchReq>(n);
        d_c1 = c.take<long long>(n);
        d_c2 = c.take<long long>(ridx.size() + 1);
        d_ridx = c.take<int>(ridx.size() + 1);
        d_counts = c.take<long long>(cbase + 1);
        d_goff = c.take<long long>(cbase + 1);
        d_totals = c.take<long long>(nr + 1);
        d_ctr = c.take<unsigned long long>(64);
        d_scan = c.take<char>(scan_temp_bytes(cbase + 1));
        d_st = c.take<DevStatus>(1);
        d_qstart = c.take<long long>(n + 1);
        for (int b2 = 0; b2 < 2; ++b2) {
            d_okeys[b2] = c.take<uint32_t>(std::max<long long>(nqo, 1));
            d_ovals[b2] = c.take<uint32_t>(std::max<long long>(nqo, 1));
        }
        d_osort = ordered ? (void*)c.take<char>(sort_temp_bytes(nqo, 1)) : nullptr;
        for (int p = 0; p < n; ++p) d[p].perm = ordered ? (const int*)(d_ovals[0] + qstart[p]) : nullptr;
        for (size_t j = 0; j < nr; ++j) d[pos_of[range_reqs[j]]].total = d_totals + j;
        CK(cudaMallocHost(&h_trees, sizeof(DevTree) * std::max<size_t>(nt, 1)));
        CK(cudaMemcpyAsync(d_reqs, d.data(), sizeof(BatchReq) * n, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(d_c1, c1.data(), sizeof(long long) * n, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(d_qstart, qstart.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice, stream));
        if (!ridx.empty()) {
            CK(cudaMemcpyAsync(d_c2, c2.data(), sizeof(long long) * c2.size(), cudaMemcpyHostToDevice, stream));
            CK(cudaMemcpyAsync(d_ridx, ridx.data(), sizeof(int) * ridx.size(), cudaMemcpyHostToDevice, stream));
        }
        CK(cudaMemsetAsync(d_counts, 0, sizeof(long long) * (cbase + 1), stream));
        CK(cudaMemsetAsync(d_totals, 0, sizeof(long long) * (nr + 1), stream));
        CK(cudaStreamSynchronize(stream));  // d and the vectors above live on this frame
        h_totals.assign(nr, 0);
        nridx = (int)ridx.size();
        for (size_t g = 1; g < groups.size(); ++g) {
            cudaStream_t bs;
            CK(cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking));
            branch.push_back(bs);
            cudaEvent_t e;
            CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            ev_join.push_back(e);
        }
        for (size_t i = 0; i < nt; ++i) {
            cudaEvent_t e;
            CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            ev_tree.push_back(e);
        }
        planned = true;
        if (use_graph) {
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            try {
                enqueue();
            } catch (...) {
                cudaStreamEndCapture(stream, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            CK(cudaStreamEndCapture(stream, &g));
            cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
            cudaGraphDestroy(g);
            CK(e);
        }
    }
    int nridx = 0;

    // The work of one run, on `stream` (captured into the graph, or issued
    // directly when graphs are off).
    void enqueue() {
        CK(cudaMemcpyAsync(d_trees, h_trees, sizeof(DevTree) * trees.size(), cudaMemcpyHostToDevice, stream));
        CK(cudaMemsetAsync(d_ctr, 0, sizeof(unsigned long long) * 64, stream));
        CK(cudaMemsetAsync(d_st, 0, sizeof(DevStatus), stream));
        if (ordered) {
            launch_batch_keys(d_trees, d_reqs, d_qstart, (int)reqs.size(), n_queries, req_bits, d_okeys[0],
                              d_ovals[0], stream);
            radix_sort_pairs(d_okeys[0], d_ovals[0], d_okeys[1], d_ovals[1], n_queries, 1, n_queries, 32, d_osort,
                             stream);
        }
        if (groups.size() > 1) CK(cudaEventRecord(ev_fork, stream));
        for (size_t g = 0; g < groups.size(); ++g) {
            const Group& G = groups[g];
            cudaStream_t s = g == 0 ? stream : branch[g - 1];
            if (g > 0) CK(cudaStreamWaitEvent(s, ev_fork, 0));
            launch_batch_search(d_trees, d_reqs, d_c1, G.r0, G.r1, G.c_begin, G.c_end, G.kclass, G.lanes, d_counts,
                                d_ctr + g, G.grid, s);
            if (g > 0) CK(cudaEventRecord(ev_join[g - 1], s));
        }
        for (size_t g = 1; g < groups.size(); ++g) CK(cudaStreamWaitEvent(stream, ev_join[g - 1], 0));
        if (nridx > 0) {
            exclusive_scan(d_counts, d_goff, n_range_queries + 1, nullptr, d_scan, stream);
            launch_batch_write(d_trees, d_reqs, d_ridx, d_c2, nridx, c2_end, d_goff, d_ctr + 63, write_grid, stream);
        }
        // range requests without queries: empty CSR
        for (int j : range_reqs)
            if (reqs[j].d.nq == 0) CK(cudaMemsetAsync(reqs[j].d.offsets, 0, sizeof(long long), stream));
        CK(cudaGetLastError());
    }

    void run() {
        if (reqs.empty()) return;
        if (!planned) plan();
        // the previous run's copy of h_trees must be done before it changes
        if (launched) CK(cudaEventSynchronize(ev_done));
        for (size_t i = 0; i < trees.size(); ++i) {
            Tree* t = trees[i];
            std::unique_lock<std::shared_mutex> lock(t->mu);
            h_trees[i] = t->dt;
            h_trees[i].st = d_st;
            CK(cudaEventRecord(ev_tree[i], t->stream));
            CK(cudaStreamWaitEvent(stream, ev_tree[i], 0));
        }
        if (use_graph)
            CK(cudaGraphLaunch(exec, stream));
        else
            enqueue();
        CK(cudaEventRecord(ev_done, stream));
        launched = true;
        // later work on each tree (mutations) waits for this run
        for (Tree* t : trees) {
            std::unique_lock<std::shared_mutex> lock(t->mu);
            CK(cudaStreamWaitEvent(t->stream, ev_done, 0));
        }
    }

    // Waits for the last run; fills totals (one per range request, in the
    // order added).  Returns false when a range request overflowed.
    bool synchronize(long long* totals) {
        CK(cudaStreamSynchronize(stream));
        if (!planned) return true;
        CK(cudaMemcpy(h_st, d_st, sizeof(DevStatus), cudaMemcpyDeviceToHost));
        if (!range_reqs.empty())
            CK(cudaMemcpy(h_totals.data(), d_totals, sizeof(long long) * range_reqs.size(), cudaMemcpyDeviceToHost));
        if (totals)
            for (size_t j = 0; j < h_totals.size(); ++j) totals[j] = h_totals[j];
        if (h_st->err & (ERR_STACK | ERR_LOOP)) throw Internal{"batch: traversal stack overflow or loop cap"};
        return !(h_st->err & ERR_OUTPUT);
    }

    // Median time (ms) of `reps` runs of this batch, on its stream.
    float time_runs(int reps) {
        cudaEvent_t a, b;
        CK(cudaEventCreate(&a));
        CK(cudaEventCreate(&b));
        std::vector<float> ts;
        run();
        synchronize(nullptr);
        for (int i = 0; i < reps; ++i) {
            CK(cudaEventRecord(a, stream));
            run();
            CK(cudaEventRecord(b, stream));
            CK(cudaEventSynchronize(b));
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, a, b));
            ts.push_back(ms);
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        synchronize(nullptr);
        std::sort(ts.begin(), ts.end());
        return ts[ts.size() / 2];
    }
};

// Per tree of the batch: the leaf fill (points per leaf when the tree is
// rebuilt, 8..32) and the lanes per kNN query (1, 2, 4) with the fastest
// median run of that tree's requests alone.  Leaves the tree rebuilt at the
// chosen fill and the requests at the chosen lanes.
void autotune_batch(Batch& b, int reps, const std::vector<int>& fills, const std::vector<int>& lanes_set,
                    int* chosen) {
    std::vector<Tree*> ts;
    for (auto& r : b.reqs)
        if (std::find(ts.begin(), ts.end(), r.tree) == ts.end()) ts.push_back(r.tree);
    for (size_t ti = 0; ti < ts.size(); ++ti) {
        Tree* t = ts[ti];
        Batch sub;
        sub.init(b.device);
        std::vector<int> map;
        for (size_t i = 0; i < b.reqs.size(); ++i)
            if (b.reqs[i].tree == t) {
                sub.reqs.push_back(b.reqs[i]);
                map.push_back((int)i);
            }
        bool has_knn = false;
        for (auto& r : sub.reqs) has_knn |= r.d.kind == BATCH_KNN;
        float best = 1e30f;
        int best_fill = t->fill, best_lanes = 1;
        try {
            for (int f : fills) {
                {
                    std::unique_lock<std::shared_mutex> lock(t->mu);
                    t->fill = f;
                    t->rebuild_all();
                }
                for (int l : lanes_set) {
                    if (!has_knn && l != lanes_set.front()) continue;
                    for (auto& r : sub.reqs) r.lanes = l;
                    sub.drop_plan();
                    float ms = sub.time_runs(reps);
                    if (ms < best) {
                        best = ms;
                        best_fill = f;
                        best_lanes = l;
                    }
                }
            }
            {
                std::unique_lock<std::shared_mutex> lock(t->mu);
                t->fill = best_fill;
                t->rebuild_all();
            }
        } catch (...) {
            sub.destroy();
            throw;
        }
        sub.destroy();
        for (int i : map)
            if (b.reqs[i].d.kind == BATCH_KNN) b.reqs[i].lanes = best_lanes;
        if (chosen != nullptr) {
            chosen[2 * ti] = best_fill;
            chosen[2 * ti + 1] = best_lanes;
        }
    }
    b.drop_plan();
}

}  // namespace ikdg

struct ikdg_tree {
    ikdg::Tree t;
};

struct ikdg_batch {
    ikdg::Batch b;
};

namespace {

int fail(ikdg_tree* h, int code, const std::string& msg) {
    if (h != nullptr) {
        std::lock_guard<std::mutex> l(h->t.err_mu);
        h->t.err = msg;
    }
    return code;
}

// Runs f with the tree's lock held (exclusively, or shared for the
// concurrent small searches) and maps exceptions to status codes.
template <bool SHARED = false, class F>
int guarded(ikdg_tree* h, F&& f) {
    if (h == nullptr) return IKDG_BAD_ARG;
    std::unique_lock<std::shared_mutex> xl(h->t.mu, std::defer_lock);
    std::shared_lock<std::shared_mutex> sl(h->t.mu, std::defer_lock);
    if (SHARED)
        sl.lock();
    else
        xl.lock();
    try {
        CK(cudaSetDevice(h->t.device));
        f(h->t);
        return IKDG_OK;
    } catch (const ikdg::CudaFail& e) {
        return fail(h, IKDG_CUDA_ERR, std::string(e.what) + ": " + cudaGetErrorString(e.e));
    } catch (const ikdg::BadArg& e) {
        return fail(h, IKDG_BAD_ARG, e.what);
    } catch (const ikdg::CapacityFail& e) {
        return fail(h, IKDG_CAPACITY, e.what);
    } catch (const ikdg::Internal& e) {
        return fail(h, IKDG_INTERNAL, e.what);
    } catch (const std::bad_alloc&) {
        return fail(h, IKDG_INTERNAL, "host allocation failed");
    }
}

template <class F>
int batch_guarded(ikdg_batch* h, F&& f) {
    if (h == nullptr) return IKDG_BAD_ARG;
    std::lock_guard<std::mutex> lock(h->b.mu);
    auto bfail = [&](int code, const std::string& msg) {
        h->b.err = msg;
        return code;
    };
    try {
        CK(cudaSetDevice(h->b.device));
        f(h->b);
        return IKDG_OK;
    } catch (const ikdg::CudaFail& e) {
        return bfail(IKDG_CUDA_ERR, std::string(e.what) + ": " + cudaGetErrorString(e.e));
    } catch (const ikdg::BadArg& e) {
        return bfail(IKDG_BAD_ARG, e.what);
    } catch (const ikdg::CapacityFail& e) {
        return bfail(IKDG_CAPACITY, e.what);
    } catch (const ikdg::Internal& e) {
        return bfail(IKDG_INTERNAL, e.what);
    } catch (const std::bad_alloc&) {
        return bfail(IKDG_INTERNAL, "host allocation failed");
    }
}

}  // namespace

extern "C" {

const char* ikdg_status_string(int s) {
    switch (s) {
        case IKDG_OK: return "ok";
        case IKDG_BAD_ARG: return "bad argument";
        case IKDG_CAPACITY: return "output capacity too small";
        case IKDG_DEVICE_TIMEOUT: return "device wait timed out";
        case IKDG_CUDA_ERR: return "CUDA error";
        case IKDG_NO_DEVICE: return "no CUDA device";
        case IKDG_INTERNAL: return "internal error";
        default: return "unknown status";
    }
}

const char* ikdg_last_error(const ikdg_tree* t) { return t ? t->t.err.c_str() : "null tree"; }

int ikdg_create(float delete_param, float balance_param, float box_length, int device, ikdg_tree** out) {
    if (out == nullptr) return IKDG_BAD_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return IKDG_NO_DEVICE;
    }
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return IKDG_NO_DEVICE;
    if (device >= ndev) return IKDG_BAD_ARG;
    ikdg_tree* h = new (std::nothrow) ikdg_tree;
    if (h == nullptr) return IKDG_INTERNAL;
    h->t.del_param = delete_param;
    h->t.bal_param = balance_param;
    h->t.ds_size = box_length;
    try {
        h->t.init(device);
    } catch (const ikdg::CudaFail& e) {
        h->t.destroy();
        delete h;
        return IKDG_CUDA_ERR;
    } catch (...) {
        h->t.destroy();
        delete h;
        return IKDG_INTERNAL;
    }
    *out = h;
    return IKDG_OK;
}

int ikdg_destroy(ikdg_tree* h) {
    if (h == nullptr) return IKDG_BAD_ARG;
    {
        std::unique_lock<std::shared_mutex> lock(h->t.mu);
        cudaSetDevice(h->t.device);
        h->t.destroy();
    }
    delete h;
    return IKDG_OK;
}

int ikdg_set_delete_criterion_param(ikdg_tree* h, float v) {
    return guarded(h, [&](ikdg::Tree& t) { t.del_param = v; });
}
int ikdg_set_balance_criterion_param(ikdg_tree* h, float v) {
    return guarded(h, [&](ikdg::Tree& t) { t.bal_param = v; });
}
int ikdg_set_downsample_param(ikdg_tree* h, float v) {
    return guarded(h, [&](ikdg::Tree& t) { t.ds_size = v; });
}
int ikdg_set_leaf_fill(ikdg_tree* h, int fill) {
    return guarded(h, [&](ikdg::Tree& t) {
        if (fill < 8 || fill > ikdg::LEAF_CAP) throw ikdg::BadArg{"leaf fill must be in [8, 32]"};
        t.fill = fill;
    });
}

int ikdg_set_knn_lanes(ikdg_tree* h, int lanes) {
    return guarded(h, [&](ikdg::Tree& t) {
        if (lanes != 1 && lanes != 2 && lanes != 4) throw ikdg::BadArg{"kNN lanes must be 1, 2 or 4"};
        t.knn_lanes = lanes;
    });
}

int ikdg_set_knn_bin_bits(ikdg_tree* h, int bits) {
    return guarded(h, [&](ikdg::Tree& t) {
        if (bits < -1 || bits > ikdg::QBIN_BITS) throw ikdg::BadArg{"kNN bin bits must be in [-1, 16]"};
        t.knn_bin_bits = bits;
    });
}

int ikdg_build(ikdg_tree* h, const float* xyz, int64_t n, int32_t stride) {
    return guarded(h, [&](ikdg::Tree& t) { t.build(xyz, n, stride); });
}

int ikdg_add_points(ikdg_tree* h, const float* xyz, int64_t n, int32_t stride, int downsample_on, int64_t* n_added) {
    return guarded(h, [&](ikdg::Tree& t) {
        long long a = 0;
        t.add_points(xyz, n, stride, downsample_on != 0, &a);
        if (n_added) *n_added = a;
    });
}

int ikdg_delete_points(ikdg_tree* h, const float* xyz, int64_t n, int32_t stride) {
    return guarded(h, [&](ikdg::Tree& t) { t.delete_points(xyz, n, stride); });
}

int ikdg_delete_boxes(ikdg_tree* h, const float* boxes, int64_t m, int64_t* n_deleted) {
    return guarded(h, [&](ikdg::Tree& t) {
        long long d = t.delete_boxes(boxes, m);
        if (n_deleted) *n_deleted = d;
    });
}

int ikdg_add_boxes(ikdg_tree* h, const float* boxes, int64_t m) {
    return guarded(h, [&](ikdg::Tree& t) { t.add_boxes(boxes, m); });
}

int ikdg_knn(ikdg_tree* h, const float* q, int64_t nq, int32_t stride, int32_t k, double max_dist, int32_t* ids,
             float* d2, float* xyz, int32_t* cnt) {
    // A few queries with a small k (the per-point Nearest_Search of a mapping
    // front end): concurrent callers search at the same time.
    if (nq <= ikdg::SMALL_KNN_QUERIES && k <= ikdg::KNN_SMEM_MAX)
        return guarded<true>(h, [&](ikdg::Tree& t) { t.knn_small(q, nq, stride, k, max_dist, ids, d2, xyz, cnt); });
    return guarded(h, [&](ikdg::Tree& t) { t.knn(q, nq, stride, k, max_dist, ids, d2, xyz, cnt, false); });
}

int ikdg_knn_device(ikdg_tree* h, const float* q, int64_t nq, int32_t stride, int32_t k, double max_dist,
                    int32_t* ids, float* d2, float* xyz, int32_t* cnt) {
    return guarded(h, [&](ikdg::Tree& t) { t.knn(q, nq, stride, k, max_dist, ids, d2, xyz, cnt, true); });
}

int ikdg_knn_device_noalloc(ikdg_tree* h, const float* q, int64_t nq, int32_t stride, int32_t k, double max_dist,
                            int32_t* ids, float* d2, float* xyz, int32_t* cnt) {
    return guarded(h, [&](ikdg::Tree& t) {
        if (nq < 0 || stride < 3 || k < 1 || (nq > 0 && (q == nullptr || ids == nullptr || d2 == nullptr)))
            throw ikdg::BadArg{"knn_device_noalloc: bad arguments"};
        if (k > ikdg::KNN_SMEM_MAX) throw ikdg::BadArg{"knn_device_noalloc: k must be <= 64"};
        if (nq > ikdg::NOALLOC_MAX_QUERIES)
            throw ikdg::BadArg{"knn_device_noalloc: at most " + std::to_string(ikdg::NOALLOC_MAX_QUERIES) +
                               " queries per call (size of the static scratch array)"};
        if (nq == 0) return;
        void* scratch = nullptr;
        CK(ikdg::noalloc_scratch(t.device, &scratch));
        if (ikdg::knn_temp_bytes(nq, k) > ikdg::noalloc_scratch_bytes())
            throw ikdg::Internal{"knn_device_noalloc: scratch array too small"};
        // Batches of QBIN_MIN_QUERIES or more are sorted (bins at QBIN_BITS
        // levels): the sort is the part that needs scratch.  Smaller batches
        // run unsorted and touch no scratch.  Nothing here allocates.
        ikdg::launch_knn(t.dt, q, stride, nq, k, ikdg::max_sq_threshold(max_dist), ids, d2, xyz, cnt, scratch,
                         t.knn_lanes, ikdg::QBIN_BITS, t.stream);
        CK(cudaGetLastError());
    });
}

int ikdg_p2p_forward(ikdg_tree* h, const float* scan, int64_t n, const double* pose, int32_t k, double max_dist,
                     float plane_thresh, float* planes, float* residuals, int32_t* valid, double* loss) {
    return guarded(h, [&](ikdg::Tree& t) {
        t.p2p_forward(scan, n, pose, k, max_dist, plane_thresh, planes, residuals, valid, loss);
    });
}

int ikdg_p2p_adjoint(ikdg_tree* h, const float* scan, int64_t n, const double* pose, const float* planes,
                     const float* residuals, const int32_t* valid, double grad_loss, float* grad_points,
                     double* grad_pose) {
    return guarded(h, [&](ikdg::Tree& t) {
        t.p2p_adjoint(scan, n, pose, planes, residuals, valid, grad_loss, grad_points, grad_pose);
    });
}

int ikdg_box_search(ikdg_tree* h, const float* boxes, int64_t nb, int64_t* offsets, int32_t* ids, float* xyz,
                    int64_t capacity, int64_t* total) {
    return guarded(h, [&](ikdg::Tree& t) {
        long long tot = 0;
        try {
            t.range(0, boxes, nb, 6, nullptr, 0, (long long*)offsets, ids, xyz, capacity, &tot);
        } catch (...) {
            if (total) *total = tot;
            throw;
        }
        if (total) *total = tot;
    });
}

int ikdg_radius_search(ikdg_tree* h, const float* centers, int64_t nq, int32_t stride, const float* radius,
                       int32_t radius_stride, int64_t* offsets, int32_t* ids, float* xyz, int64_t capacity,
                       int64_t* total) {
    return guarded(h, [&](ikdg::Tree& t) {
        long long tot = 0;
        try {
            t.range(1, centers, nq, stride, radius, radius_stride, (long long*)offsets, ids, xyz, capacity, &tot);
        } catch (...) {
            if (total) *total = tot;
            throw;
        }
        if (total) *total = tot;
    });
}

int ikdg_size(ikdg_tree* h, int64_t* out) {
    return guarded(h, [&](ikdg::Tree& t) {
        if (out == nullptr) throw ikdg::BadArg{"size: null output"};
        *out = t.st->root_slots;
    });
}

int ikdg_validnum(ikdg_tree* h, int64_t* out) {
    return guarded(h, [&](ikdg::Tree& t) {
        if (out == nullptr) throw ikdg::BadArg{"validnum: null output"};
        *out = (int64_t)t.st->root_slots - t.st->root_deleted;
    });
}

int ikdg_tree_range(ikdg_tree* h, float* box6) {
    return guarded(h, [&](ikdg::Tree& t) {
        if (box6 == nullptr) throw ikdg::BadArg{"tree_range: null output"};
        t.tree_range(box6);
    });
}

int ikdg_root_alpha(ikdg_tree* h, float* alpha_bal, float* alpha_del) {
    return guarded(h, [&](ikdg::Tree& t) { t.root_alpha(alpha_bal, alpha_del); });
}

int ikdg_flatten(ikdg_tree* h, float* xyz, int32_t* ids, int64_t capacity, int64_t* n) {
    return guarded(h, [&](ikdg::Tree& t) {
        long long k = 0;
        try {
            t.flatten(xyz, ids, capacity, &k);
        } catch (...) {
            if (n) *n = k;
            throw;
        }
        if (n) *n = k;
    });
}

int ikdg_acquire_removed_points(ikdg_tree* h, float* xyz, int32_t* ids, int64_t capacity, int64_t* n) {
    return guarded(h, [&](ikdg::Tree& t) {
        long long k = 0;
        try {
            t.acquire_removed(xyz, ids, capacity, &k);
        } catch (...) {
            if (n) *n = k;
            throw;
        }
        if (n) *n = k;
    });
}

int ikdg_live_ids(ikdg_tree* h, int32_t* ids, int64_t capacity, int64_t* n) {
    return guarded(h, [&](ikdg::Tree& t) {
        long long k = 0;
        try {
            t.live_ids(ids, capacity, &k);
        } catch (...) {
            if (n) *n = k;
            throw;
        }
        if (n) *n = k;
    });
}

int ikdg_rebuild(ikdg_tree* h) {
    return guarded(h, [&](ikdg::Tree& t) { t.rebuild_all(); });
}

int ikdg_debug_validate(ikdg_tree* h, int64_t* violations) {
    return guarded(h, [&](ikdg::Tree& t) {
        long long v = t.validate();
        if (violations) *violations = v;
    });
}

int ikdg_get_stream(ikdg_tree* h, void** stream) {
    return guarded(h, [&](ikdg::Tree& t) {
        if (stream == nullptr) throw ikdg::BadArg{"get_stream: null output"};
        *stream = (void*)t.stream;
    });
}

int ikdg_set_stream(ikdg_tree* h, void* stream) {
    return guarded(h, [&](ikdg::Tree& t) {
        CK(cudaStreamSynchronize(t.stream));
        if (t.own_stream) CK(cudaStreamDestroy(t.stream));
        t.stream = (cudaStream_t)stream;
        t.own_stream = false;
    });
}

int ikdg_synchronize(ikdg_tree* h) {
    return guarded(h, [&](ikdg::Tree& t) {
        CK(cudaStreamSynchronize(t.stream));
        CK(cudaGetLastError());
    });
}

int ikdg_box_search_device(ikdg_tree* h, const float* boxes, int64_t nb, int64_t* offsets, int32_t* ids, float* xyz,
                           int64_t capacity, int64_t* total) {
    return guarded(h, [&](ikdg::Tree& t) {
        t.range_device(0, boxes, nb, 6, nullptr, 0, (long long*)offsets, ids, xyz, capacity, (long long*)total);
    });
}

int ikdg_radius_search_device(ikdg_tree* h, const float* centers, int64_t nq, int32_t stride, const float* radius,
                              int32_t radius_stride, int64_t* offsets, int32_t* ids, float* xyz, int64_t capacity,
                              int64_t* total) {
    return guarded(h, [&](ikdg::Tree& t) {
        t.range_device(1, centers, nq, stride, radius, radius_stride, (long long*)offsets, ids, xyz, capacity,
                       (long long*)total);
    });
}

// ---- multi-tree batches ------------------------------------------------------------

const char* ikdg_batch_last_error(const ikdg_batch* b) { return b ? b->b.err.c_str() : "null batch"; }

int ikdg_batch_create(int device, ikdg_batch** out) {
    if (out == nullptr) return IKDG_BAD_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return IKDG_NO_DEVICE;
    }
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return IKDG_NO_DEVICE;
    if (device >= ndev) return IKDG_BAD_ARG;
    ikdg_batch* h = new (std::nothrow) ikdg_batch;
    if (h == nullptr) return IKDG_INTERNAL;
    try {
        h->b.init(device);
    } catch (...) {
        h->b.destroy();
        delete h;
        return IKDG_CUDA_ERR;
    }
    *out = h;
    return IKDG_OK;
}

int ikdg_batch_destroy(ikdg_batch* h) {
    if (h == nullptr) return IKDG_BAD_ARG;
    {
        std::lock_guard<std::mutex> lock(h->b.mu);
        cudaSetDevice(h->b.device);
        h->b.destroy();
    }
    delete h;
    return IKDG_OK;
}

int ikdg_batch_clear(ikdg_batch* h) {
    return batch_guarded(h, [&](ikdg::Batch& b) { b.clear(); });
}

int ikdg_batch_add_knn(ikdg_batch* h, ikdg_tree* tree, const float* queries, int64_t nq, int32_t stride, int32_t k,
                       double max_dist, int32_t* ids, float* d2, float* xyz, int32_t* counts, int32_t* request) {
    return batch_guarded(h, [&](ikdg::Batch& b) {
        if (tree == nullptr || nq < 0 || stride < 3 || k < 1 ||
            (nq > 0 && (queries == nullptr || ids == nullptr || d2 == nullptr)))
            throw ikdg::BadArg{"batch_add_knn: bad arguments"};
        if (k > ikdg::BATCH_KMAX) throw ikdg::BadArg{"batch_add_knn: k must be <= 16"};
        ikdg::Batch::Req r;
        r.tree = &tree->t;
        r.max_dist = max_dist;
        r.d.kind = ikdg::BATCH_KNN;
        r.d.q = queries;
        r.d.nq = nq;
        r.d.q_stride = stride;
        r.d.k = k;
        r.d.max_sq = ikdg::max_sq_threshold(max_dist);
        r.d.ids = ids;
        r.d.d2 = d2;
        r.d.xyz = xyz;
        r.d.cnt = counts;
        int id = b.add(r);
        if (request) *request = id;
    });
}

int ikdg_batch_add_box_search(ikdg_batch* h, ikdg_tree* tree, const float* boxes, int64_t nb, int64_t* offsets,
                              int32_t* ids, float* xyz, int64_t capacity, int32_t* request) {
    return batch_guarded(h, [&](ikdg::Batch& b) {
        if (tree == nullptr || nb < 0 || offsets == nullptr || capacity < 0 || (nb > 0 && boxes == nullptr) ||
            (capacity > 0 && ids == nullptr))
            throw ikdg::BadArg{"batch_add_box_search: bad arguments"};
        ikdg::Batch::Req r;
        r.tree = &tree->t;
        r.d.kind = ikdg::BATCH_BOX;
        r.d.q = boxes;
        r.d.nq = nb;
        r.d.q_stride = 6;
        r.d.ids = ids;
        r.d.xyz = xyz;
        r.d.offsets = (long long*)offsets;
        r.d.capacity = capacity;
        int id = b.add(r);
        if (request) *request = id;
    });
}

int ikdg_batch_add_radius_search(ikdg_batch* h, ikdg_tree* tree, const float* centers, int64_t nq, int32_t stride,
                                 const float* radius, int32_t radius_stride, int64_t* offsets, int32_t* ids,
                                 float* xyz, int64_t capacity, int32_t* request) {
    return batch_guarded(h, [&](ikdg::Batch& b) {
        if (tree == nullptr || nq < 0 || stride < 3 || radius_stride < 0 || offsets == nullptr || capacity < 0 ||
            (nq > 0 && (centers == nullptr || radius == nullptr)) || (capacity > 0 && ids == nullptr))
            throw ikdg::BadArg{"batch_add_radius_search: bad arguments"};
        ikdg::Batch::Req r;
        r.tree = &tree->t;
        r.d.kind = ikdg::BATCH_RADIUS;
        r.d.q = centers;
        r.d.nq = nq;
        r.d.q_stride = stride;
        r.d.radius = radius;
        r.d.r_stride = radius_stride;
        r.d.ids = ids;
        r.d.xyz = xyz;
        r.d.offsets = (long long*)offsets;
        r.d.capacity = capacity;
        int id = b.add(r);
        if (request) *request = id;
    });
}

int ikdg_batch_set_knn_lanes(ikdg_batch* h, int32_t request, int32_t lanes) {
    return batch_guarded(h, [&](ikdg::Batch& b) {
        if (request < 0 || request >= (int)b.reqs.size() || !(lanes == 0 || lanes == 1 || lanes == 2 || lanes == 4))
            throw ikdg::BadArg{"batch_set_knn_lanes: bad arguments"};
        b.reqs[request].lanes = lanes;
        b.drop_plan();
    });
}

int ikdg_batch_set_graph(ikdg_batch* h, int use_graph) {
    return batch_guarded(h, [&](ikdg::Batch& b) {
        b.drop_plan();
        b.use_graph = use_graph != 0;
    });
}

int ikdg_batch_set_query_order(ikdg_batch* h, int ordered) {
    return batch_guarded(h, [&](ikdg::Batch& b) {
        b.drop_plan();
        b.use_order = ordered != 0;
    });
}


int ikdg_batch_run(ikdg_batch* h) {
    return batch_guarded(h, [&](ikdg::Batch& b) { b.run(); });
}

int ikdg_batch_synchronize(ikdg_batch* h, int64_t* range_totals) {
    return batch_guarded(h, [&](ikdg::Batch& b) {
        if (!b.synchronize((long long*)range_totals))
            throw ikdg::CapacityFail{"batch: a range request's results exceed its capacity"};
    });
}

int ikdg_batch_autotune(ikdg_batch* h, int32_t reps, int32_t* chosen) {
    return batch_guarded(h, [&](ikdg::Batch& b) {
        if (reps < 1) throw ikdg::BadArg{"batch_autotune: reps must be >= 1"};
        ikdg::autotune_batch(b, reps, {8, 12, 16, 24, 32}, {1, 2, 4}, chosen);
    });
}

int ikdg_batch_num_trees(ikdg_batch* h, int32_t* n) {
    return batch_guarded(h, [&](ikdg::Batch& b) {
        if (n == nullptr) throw ikdg::BadArg{"batch_num_trees: null output"};
        std::vector<ikdg::Tree*> ts;
        for (auto& r : b.reqs)
            if (std::find(ts.begin(), ts.end(), r.tree) == ts.end()) ts.push_back(r.tree);
        *n = (int32_t)ts.size();
    });
}

int ikdg_batch_get_stream(ikdg_batch* h, void** stream) {
    return batch_guarded(h, [&](ikdg::Batch& b) {
        if (stream == nullptr) throw ikdg::BadArg{"batch_get_stream: null output"};
        *stream = (void*)b.stream;
    });
}

}  // extern "C"
