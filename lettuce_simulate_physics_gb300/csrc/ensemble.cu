// Batched ensembles: many independent systems of uneven N advanced together on one GPU. No
// counterpart in the reference; every system follows the reference's single-system physics
// (the kick-drift-kick step of src/simulation.cpp, forces as src/cpu_backend.cpp) with its own
// softening and opening angle.
//
// Layout. Systems are stored back to back, tree systems first: bodies [0, n_tree) form one forest
// tree (tree.cu in forest mode: per-system key frames, a (system, key) sort, one root per system,
// per-system opening angles), bodies [n_tree, n) are direct-sum systems. Both parts share the
// engine's body arrays, so one kick-drift pass and one kick pass cover every system.
//
// Force phase. The direct systems are cut into work items (an i-tile of one system against all of
// its bodies) and run as one batched launch per kernel shape (i-bodies per thread and j-tile, both
// chosen per size class by the autotuner), on a second stream
// that overlaps the forest's sort, build and walk; the tree walk takes each group's root and
// softening from its system. No host read is needed: the tree build takes its sizes from the
// previous build (with headroom) and a device-side check records a miss in a sticky word.
//
// Runs. A run of steps is either launched step by step or captured once as a CUDA graph and
// replayed. Before it starts, the state is copied aside; if the sticky word shows that a
// sync-free build missed, the run is redone from that copy with every build checked on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "../../include/lettuce_gb300.h"
#include "engine.cuh"

namespace lg {

namespace {

constexpr int kClasses = 3;  // direct size classes: N < 2048, N < 4096, larger
int size_class(uint32_t n) { return n < 2048 ? 0 : (n < 4096 ? 1 : 2); }
int default_ipt(int cls) { return cls == 0 ? 1 : (cls == 1 ? 2 : 4); }
constexpr int kIptCandidates[] = {1, 2, 4};
constexpr int kTileCandidates[] = {256, 128};
constexpr int kGroupCandidates[] = {64, 96, 128};
bool valid_shape(int ipt, int tile) {
    return (ipt == 1 || ipt == 2 || ipt == 4 || ipt == 8) && (tile == 256 || (tile == 128 && ipt != 8));
}

struct Segment {
    int first, count, ipt, tile;
};

}  // namespace

class Ensemble {
public:
    explicit Ensemble(int device) : e_(new Engine(device)) {
        LG_CK(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking));
        LG_CK(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
        LG_CK(cudaEventCreateWithFlags(&join_, cudaEventDisableTiming));
        LG_CK(cudaEventCreate(&t0_));
        LG_CK(cudaEventCreate(&t1_));
        cudaDeviceProp prop{};
        LG_CK(cudaGetDeviceProperties(&prop, device));
        device_name_ = prop.name;
        for (int c = 0; c < kClasses; ++c) {
            tuning_.direct_ipt[c] = default_ipt(c);
            tuning_.direct_tile[c] = 256;
        }
        tuning_.walk_group = e_->group_max;
        tuning_.tuned = 0;
        sticky_.reserve(256);
        LG_CK(cudaMemset(sticky_.as<char>(), 0, 256));
    }

    ~Ensemble() {
        cudaSetDevice(e_->dev);
        drop_graph();
        cudaStreamSynchronize(side_);
        cudaStreamSynchronize(e_->stream);
        for (cudaEvent_t ev : {fork_, join_, t0_, t1_})
            if (ev) cudaEventDestroy(ev);
        if (side_) cudaStreamDestroy(side_);
    }

    Ensemble(const Ensemble&) = delete;
    Ensemble& operator=(const Ensemble&) = delete;

    void upload(size_t nsys, const uint32_t* counts, const double* eps, const double* theta, const int* method,
                double G, const float* x, const float* y, const float* z, const float* vx, const float* vy,
                const float* vz, const float* m, const uint32_t* id) {
        Engine& e = *e_;
        LG_CK(cudaSetDevice(e.dev));
        drop_graph();
        if (nsys > 0 && (!counts || !eps || !method)) fail(kArg, "ensemble upload: null system table");
        if (nsys >= (size_t(1) << 30)) fail(kArg, "ensemble upload: too many systems");
        size_t total = 0;
        for (size_t s = 0; s < nsys; ++s) {
            if (method[s] != LG_DIRECT && method[s] != LG_TREE)
                fail(kArg, "ensemble upload: method of system " + std::to_string(s) + " is neither LG_DIRECT nor LG_TREE");
            const float e2 = static_cast<float>(eps[s] * eps[s]);
            if (!(eps[s] > 0) || !(e2 >= FLT_MIN) || !std::isfinite(e2))
                fail(kArg, "ensemble upload: system " + std::to_string(s) + " needs a softening eps > 0 (eps^2 a normal float)");
            if (method[s] == LG_TREE) {
                if (!theta || !(theta[s] >= 0) || !std::isfinite(theta[s]))
                    fail(kArg, "ensemble upload: tree system " + std::to_string(s) + " needs an opening angle theta >= 0");
            }
            total += counts[s];
        }
        if (total >= static_cast<size_t>(INT32_MAX)) fail(kRuntime, "ensemble upload: more than 2^31-1 bodies");
        if (total > 0 && (!x || !y || !z || !vx || !vy || !vz || !m || !id))
            fail(kArg, "ensemble upload: null body array");
        G_ = G;
        // Internal order: tree systems (non-empty), then the rest, each in input order.
        order_.clear();
        for (size_t s = 0; s < nsys; ++s)
            if (method[s] == LG_TREE && counts[s] > 0) order_.push_back(static_cast<int>(s));
        nsys_tree_ = static_cast<int>(order_.size());
        for (size_t s = 0; s < nsys; ++s)
            if (!(method[s] == LG_TREE && counts[s] > 0)) order_.push_back(static_cast<int>(s));
        nsys_ = static_cast<int>(nsys);
        in_off_.assign(nsys + 1, 0);
        for (size_t s = 0; s < nsys; ++s) in_off_[s + 1] = in_off_[s] + counts[s];
        off_.assign(nsys + 1, 0);
        count_.assign(nsys, 0);
        eps_.assign(nsys, 0);
        theta_.assign(nsys, 0);
        for (int k = 0; k < nsys_; ++k) {
            const int s = order_[k];
            count_[k] = counts[s];
            eps_[k] = eps[s];
            theta_[k] = method[s] == LG_TREE ? theta[s] : 0.0;
            off_[k + 1] = off_[k] + counts[s];
        }
        n_tree_ = static_cast<int>(off_[nsys_tree_]);
        n_ = static_cast<int>(total);
        // Bodies into internal order.
        std::vector<float> hx(total), hy(total), hz(total), hvx(total), hvy(total), hvz(total), hm(total);
        std::vector<uint32_t> hid(total);
        for (int k = 0; k < nsys_; ++k) {
            const size_t src = in_off_[order_[k]], dst = off_[k], c = count_[k];
            std::memcpy(&hx[dst], x + src, c * 4);
            std::memcpy(&hy[dst], y + src, c * 4);
            std::memcpy(&hz[dst], z + src, c * 4);
            std::memcpy(&hvx[dst], vx + src, c * 4);
            std::memcpy(&hvy[dst], vy + src, c * 4);
            std::memcpy(&hvz[dst], vz + src, c * 4);
            std::memcpy(&hm[dst], m + src, c * 4);
            std::memcpy(&hid[dst], id + src, c * 4);
        }
        e.upload(total, hx.data(), hy.data(), hz.data(), hvx.data(), hvy.data(), hvz.data(), hm.data(), hid.data());
        // System tables on the device.
        std::vector<uint32_t> sys(static_cast<size_t>(n_tree_) + 1), off(static_cast<size_t>(nsys_) + 1);
        std::vector<float> inv_theta(static_cast<size_t>(nsys_tree_) + 1), e2(static_cast<size_t>(nsys_tree_) + 1);
        for (int k = 0; k < nsys_tree_; ++k) {
            for (size_t i = off_[k]; i < off_[k + 1]; ++i) sys[i] = static_cast<uint32_t>(k);
            inv_theta[k] = theta_[k] > 0 ? static_cast<float>(1.0 / theta_[k]) : FLT_MAX;
            e2[k] = static_cast<float>(eps_[k] * eps_[k]);
        }
        for (int k = 0; k <= nsys_; ++k) off[k] = static_cast<uint32_t>(off_[k]);
        d_sys_.reserve(sys.size() * 4);
        d_off_.reserve(off.size() * 4);
        d_inv_theta_.reserve(inv_theta.size() * 4);
        d_e2_.reserve(e2.size() * 4);
        d_energy_.reserve(static_cast<size_t>(nsys_ + 1) * 16);
        LG_CK(cudaMemcpy(d_sys_.as<uint32_t>(), sys.data(), sys.size() * 4, cudaMemcpyHostToDevice));
        LG_CK(cudaMemcpy(d_off_.as<uint32_t>(), off.data(), off.size() * 4, cudaMemcpyHostToDevice));
        LG_CK(cudaMemcpy(d_inv_theta_.as<float>(), inv_theta.data(), inv_theta.size() * 4, cudaMemcpyHostToDevice));
        LG_CK(cudaMemcpy(d_e2_.as<float>(), e2.data(), e2.size() * 4, cudaMemcpyHostToDevice));
        tree_set_forest(e, n_tree_, nsys_tree_, d_sys_.as<uint32_t>(), d_off_.as<uint32_t>(),
                        d_inv_theta_.as<float>());
        direct_pairs_ = 0;
        for (int k = nsys_tree_; k < nsys_; ++k)
            direct_pairs_ += static_cast<unsigned long long>(count_[k]) * (count_[k] > 0 ? count_[k] - 1 : 0);
        build_work();
        acc_valid_ = false;
        stats_ = lg_ensemble_stats{};
    }

    void run(double dt, int steps, bool use_graph) {
        Engine& e = *e_;
        LG_CK(cudaSetDevice(e.dev));
        if (steps < 0) fail(kArg, "ensemble run: steps < 0");
        stats_.steps = steps;
        stats_.used_graph = 0;
        stats_.run_ms = 0;
        if (steps == 0 || n_ == 0) return;
        cudaStream_t s = e.stream;
        if (!acc_valid_) forces_verified(false);
        const bool graph = use_graph && (n_tree_ == 0 || tree_sync_free_ready(e));
        const uint64_t l0 = e.launches;
        const bool reuse = graph && exec_ && g_steps_ == steps && g_dt_ == dt && g_gen_ == tree_generation(e);
        if (graph && !reuse) capture(dt, steps);
        LG_CK(cudaEventRecord(t0_, s));
        if (graph && e.cur != g_cur0_) {
            // The graph reads the body set it was captured on; a force phase since (one sort)
            // left the state in the other one.
            copy_bodies(e.bodies(e.cur), e.bodies(g_cur0_));
            e.cur = g_cur0_;
        }
        take_snapshot();
        LG_CK(cudaMemsetAsync(sticky_.as<unsigned>(), 0, 4, s));
        if (graph) {
            LG_CK(cudaGraphLaunch(exec_, s));
            e.cur = g_cur1_;
            e.launches += g_launches_;
        } else {
            for (int k = 0; k < steps; ++k) step_async(dt);
        }
        LG_CK(cudaEventRecord(t1_, s));
        LG_CK(cudaMemcpyAsync(e.pinned_small, e.small.as<char>(), 128, cudaMemcpyDeviceToHost, s));
        LG_CK(cudaMemcpyAsync(e.pinned_small + 32, sticky_.as<unsigned>(), 4, cudaMemcpyDeviceToHost, s));
        LG_CK(cudaStreamSynchronize(s));
        float ms = 0;
        LG_CK(cudaEventElapsedTime(&ms, t0_, t1_));
        check_err("ensemble run");
        if (e.pinned_small[32]) {
            // A sync-free build exceeded the sizes it was launched with (or needed a key restart):
            // redo the run from the copy with every build checked on the host.
            restore_snapshot();
            drop_graph();
            tree_reset_guess(e);
            LG_CK(cudaEventRecord(t0_, s));
            for (int k = 0; k < steps; ++k) {
                launch_kick_drift(e.bodies(e.cur), e.acc.as<float4>(), static_cast<float>(0.5 * dt), dt, n_, s);
                ++e.launches;
                forces_verified(false);
                launch_kick(e.bodies(e.cur), e.acc.as<float4>(), static_cast<float>(0.5 * dt), n_, s);
                ++e.launches;
            }
            LG_CK(cudaEventRecord(t1_, s));
            LG_CK(cudaStreamSynchronize(s));
            LG_CK(cudaEventElapsedTime(&ms, t0_, t1_));
            ++stats_.recoveries;
        } else {
            stats_.used_graph = graph ? 1 : 0;
            record_interactions();
        }
        stats_.run_ms = ms;
        stats_.launches_per_step = (e.launches - l0) / static_cast<uint64_t>(steps);
        acc_valid_ = true;
    }

    void energy(double* E, double* ke, double* pe) {
        Engine& e = *e_;
        LG_CK(cudaSetDevice(e.dev));
        if (n_ > 0) forces_verified(true);
        std::vector<double> h(static_cast<size_t>(2 * nsys_) + 2, 0.0);
        if (nsys_ > 0 && n_ > 0) {
            launch_sys_energy(e.bodies(e.cur), e.acc.as<float4>(), d_off_.as<uint32_t>(), nsys_, d_energy_.as<double>(),
                              e.stream);
            ++e.launches;
            LG_CK(cudaMemcpyAsync(h.data(), d_energy_.as<double>(), static_cast<size_t>(2 * nsys_) * 8,
                                  cudaMemcpyDeviceToHost, e.stream));
            LG_CK(cudaStreamSynchronize(e.stream));
        }
        for (int k = 0; k < nsys_; ++k) {
            const int s = order_[k];
            if (E) E[s] = h[2 * k] + h[2 * k + 1];
            if (ke) ke[s] = h[2 * k];
            if (pe) pe[s] = h[2 * k + 1];
        }
    }

    void download(float* x, float* y, float* z, float* vx, float* vy, float* vz, float* m, uint32_t* id) {
        Engine& e = *e_;
        if (n_ == 0) return;
        std::vector<float> hx(n_), hy(n_), hz(n_), hvx(n_), hvy(n_), hvz(n_), hm(n_);
        std::vector<uint32_t> hid(n_);
        e.download(hx.data(), hy.data(), hz.data(), hvx.data(), hvy.data(), hvz.data(), hm.data(), hid.data());
        scatter(hx, x);
        scatter(hy, y);
        scatter(hz, z);
        scatter(hvx, vx);
        scatter(hvy, vy);
        scatter(hvz, vz);
        scatter(hm, m);
        scatter(hid, id);
    }

    void read_accel(float* ax, float* ay, float* az, float* pot) {
        Engine& e = *e_;
        if (n_ == 0) return;
        std::vector<float> hx(n_), hy(n_), hz(n_), hp(n_);
        e.read_accel(hx.data(), hy.data(), hz.data(), hp.data());
        scatter(hx, ax);
        scatter(hy, ay);
        scatter(hz, az);
        if (pot) scatter(hp, pot);
    }

    void tune() {
        Engine& e = *e_;
        LG_CK(cudaSetDevice(e.dev));
        if (n_ == 0) return;
        drop_graph();
        if (load_cache()) {
            apply_tuning();
            return;
        }
        cudaStream_t s = e.stream;
        // Direct classes: time each candidate shape's batched launch (i-bodies per thread, j-tile)
        // over that class's systems alone.
        for (int c = 0; c < kClasses; ++c) {
            std::vector<DirectWork> items;
            float best_ms = FLT_MAX;
            int best = tuning_.direct_ipt[c], best_tile = tuning_.direct_tile[c];
            for (int ipt : kIptCandidates) {
                items.clear();
                for (int k = nsys_tree_; k < nsys_; ++k)
                    if (count_[k] > 0 && size_class(count_[k]) == c) add_items(items, k, ipt);
                if (items.empty()) break;
                tune_work_.reserve(items.size() * sizeof(DirectWork));
                LG_CK(cudaMemcpy(tune_work_.as<DirectWork>(), items.data(), items.size() * sizeof(DirectWork),
                                 cudaMemcpyHostToDevice));
                const BodyArrays b = e.bodies(e.cur);
                const int nw = static_cast<int>(items.size());
                for (int tile : kTileCandidates) {
                    launch_direct_batch(b, tune_work_.as<DirectWork>(), nw, ipt, tile, static_cast<float>(G_), false,
                                        false, e.acc.as<float4>(), e.err_word(), s);
                    LG_CK(cudaEventRecord(t0_, s));
                    for (int r = 0; r < 5; ++r)
                        launch_direct_batch(b, tune_work_.as<DirectWork>(), nw, ipt, tile, static_cast<float>(G_),
                                            false, false, e.acc.as<float4>(), e.err_word(), s);
                    LG_CK(cudaEventRecord(t1_, s));
                    LG_CK(cudaStreamSynchronize(s));
                    float ms = 0;
                    LG_CK(cudaEventElapsedTime(&ms, t0_, t1_));
                    if (ms < best_ms) {
                        best_ms = ms;
                        best = ipt;
                        best_tile = tile;
                    }
                }
            }
            tuning_.direct_ipt[c] = best;
            tuning_.direct_tile[c] = best_tile;
        }
        build_work();
        // Forest walk group size: time the whole tree force phase (sort, build, walk).
        if (n_tree_ > 0) {
            float best_ms = FLT_MAX;
            int best = tuning_.walk_group;
            for (int g : kGroupCandidates) {
                e.group_max = g;
                tree_reset_guess(e);
                forces_verified(false);  // exact build, then sizes for the sync-free ones
                forces_verified(false);
                LG_CK(cudaEventRecord(t0_, s));
                for (int r = 0; r < 3; ++r) forces_async(false);
                LG_CK(cudaEventRecord(t1_, s));
                LG_CK(cudaStreamSynchronize(s));
                float ms = 0;
                LG_CK(cudaEventElapsedTime(&ms, t0_, t1_));
                if (ms < best_ms) {
                    best_ms = ms;
                    best = g;
                }
            }
            tuning_.walk_group = best;
        }
        tuning_.tuned = 1;
        save_cache();
        apply_tuning();
    }

    void set_tuning(const lg_ensemble_tuning& t) {
        for (int c = 0; c < kClasses; ++c)
            if (!valid_shape(t.direct_ipt[c], t.direct_tile[c]))
                fail(kArg, "ensemble tuning: direct_ipt must be 1, 2, 4 or 8 and direct_tile 256, or 128 with "
                           "direct_ipt 1, 2 or 4");
        if (t.walk_group < 1 || t.walk_group > 1024) fail(kArg, "ensemble tuning: walk_group must be in [1, 1024]");
        tuning_ = t;
        LG_CK(cudaSetDevice(e_->dev));
        drop_graph();
        apply_tuning();
    }

    lg_ensemble_tuning tuning() const { return tuning_; }

    lg_ensemble_stats stats() const {
        lg_ensemble_stats s = stats_;
        s.nsys = nsys_;
        s.nsys_tree = nsys_tree_;
        s.nsys_direct = nsys_ - nsys_tree_;
        s.n = static_cast<size_t>(n_);
        s.n_tree = static_cast<size_t>(n_tree_);
        s.n_direct = static_cast<size_t>(n_ - n_tree_);
        return s;
    }

private:
    // ---- force phase and steps (no host reads: capturable) -----------------------------------
    void forces_async(bool pot) {
        Engine& e = *e_;
        cudaStream_t s = e.stream;
        LG_CK(cudaMemsetAsync(e.small.as<char>() + 32, 0, 64, s));  // walk group counter, interaction counters
        const BodyArrays b = e.bodies(e.cur);
        const bool split = n_tree_ > 0 && n_ > n_tree_;
        if (n_ > n_tree_) {
            cudaStream_t ds = split ? side_ : s;
            if (split) {
                LG_CK(cudaEventRecord(fork_, s));
                LG_CK(cudaStreamWaitEvent(side_, fork_, 0));
            }
            // Reads the direct systems' positions from the current body set; the forest's sort
            // copies those bodies unchanged into the other set, and writes acc only below n_tree.
            for (const Segment& g : segs_) {
                launch_direct_batch(b, d_work_.as<DirectWork>() + g.first, g.count, g.ipt, g.tile,
                                    static_cast<float>(G_), pot, false, e.acc.as<float4>(), e.err_word(), ds);
                ++e.launches;
            }
            if (split) LG_CK(cudaEventRecord(join_, side_));
        }
        if (n_tree_ > 0) {
            tree_sort(e);
            tree_build(e, theta_.empty() ? 0.5 : theta_[0]);
            tree_check_async(e, sticky_.as<unsigned>());
            tree_walk(e, static_cast<float>(G_), 0.f, pot, false, d_sys_.as<uint32_t>(), d_e2_.as<float>());
        }
        if (split) LG_CK(cudaStreamWaitEvent(s, join_, 0));
    }

    void step_async(double dt) {
        Engine& e = *e_;
        const float hdt = static_cast<float>(0.5 * dt);
        launch_kick_drift(e.bodies(e.cur), e.acc.as<float4>(), hdt, dt, n_, e.stream);
        ++e.launches;
        forces_async(false);
        launch_kick(e.bodies(e.cur), e.acc.as<float4>(), hdt, n_, e.stream);
        ++e.launches;
    }

    // Force phase with the tree's sizes checked on the host (rebuilt exactly after a miss).
    void forces_verified(bool pot) {
        Engine& e = *e_;
        cudaStream_t s = e.stream;
        for (int attempt = 0;; ++attempt) {
            forces_async(pot);
            LG_CK(cudaMemcpyAsync(e.pinned_small, e.small.as<char>(), 128, cudaMemcpyDeviceToHost, s));
            if (n_tree_ > 0)
                LG_CK(cudaMemcpyAsync(e.pinned_small + 64, tree_counts_device(e), 32, cudaMemcpyDeviceToHost, s));
            LG_CK(cudaStreamSynchronize(s));
            if (n_tree_ > 0 && !tree_verify(e, e.pinned_small + 64)) {
                if (attempt >= 2) fail(kRuntime, "ensemble: tree sizes still wrong after an exact rebuild");
                LG_CK(cudaMemsetAsync(e.err_word(), 0, 4, s));
                continue;
            }
            check_err("ensemble forces");
            record_interactions();
            break;
        }
        acc_valid_ = true;
    }

    void record_interactions() {
        const unsigned long long* cnt =
            reinterpret_cast<const unsigned long long*>(reinterpret_cast<const char*>(e_->pinned_small) + 64);
        stats_.last_interactions = (n_tree_ > 0 ? cnt[0] + cnt[1] : 0ull) + direct_pairs_;
    }

    void check_err(const char* where) {
        Engine& e = *e_;
        const unsigned w = e.pinned_small[0];
        if (!w) return;
        LG_CK(cudaMemsetAsync(e.err_word(), 0, 4, e.stream));
        LG_CK(cudaStreamSynchronize(e.stream));
        std::string why;
        if (w & kErrWaitTimeout) why += " wait-timeout";
        if (w & kErrStackOverflow) why += " stack-overflow";
        if (w & kErrNodeOverflow) why += " node-overflow";
        if (w & kErrDeepKeys) why += " deep-key-restart";
        if (w & kErrListOverflow) why += " list-overflow";
        acc_valid_ = false;
        fail(kRuntime, std::string(where) + ": device error" + why + "; results are invalid");
    }

    void capture(double dt, int steps) {
        Engine& e = *e_;
        drop_graph();
        const int cur0 = e.cur;
        const uint64_t l0 = e.launches;
        LG_CK(cudaStreamBeginCapture(e.stream, cudaStreamCaptureModeThreadLocal));
        try {
            for (int k = 0; k < steps; ++k) step_async(dt);
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(e.stream, &g);
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            e.cur = cur0;
            e.launches = l0;
            throw;
        }
        cudaGraph_t g = nullptr;
        LG_CK(cudaStreamEndCapture(e.stream, &g));
        cudaGraphExec_t x = nullptr;
        const cudaError_t r = cudaGraphInstantiate(&x, g, 0);
        cudaGraphDestroy(g);
        LG_CK(r);
        exec_ = x;
        g_steps_ = steps;
        g_dt_ = dt;
        g_cur0_ = cur0;
        g_cur1_ = e.cur;
        g_launches_ = e.launches - l0;
        g_gen_ = tree_generation(e);
        e.cur = cur0;  // nothing ran yet
        e.launches = l0;
        ++stats_.captures;
    }

    void drop_graph() {
        if (exec_) cudaGraphExecDestroy(exec_);
        exec_ = nullptr;
    }

    // ---- direct work table ---------------------------------------------------------------------
    void add_items(std::vector<DirectWork>& items, int k, int ipt) const {
        const int tile = direct_block_bodies(ipt);
        const int lo = static_cast<int>(off_[k]), hi = static_cast<int>(off_[k + 1]);
        const float e2 = static_cast<float>(eps_[k] * eps_[k]);
        for (int base = lo; base < hi; base += tile) {
            DirectWork w{};
            w.base = base;
            w.iend = std::min(hi, base + tile);
            w.j0 = lo;
            w.j1 = hi;
            w.e2 = e2;
            w.sys = k;
            items.push_back(w);
        }
    }

    void build_work() {
        segs_.clear();
        std::vector<DirectWork> all;
        for (int ipt : {1, 2, 4, 8})
            for (int tile : {256, 128}) {
                std::vector<DirectWork> items;
                for (int k = nsys_tree_; k < nsys_; ++k) {
                    const int c = count_[k] > 0 ? size_class(count_[k]) : -1;
                    if (c >= 0 && tuning_.direct_ipt[c] == ipt && tuning_.direct_tile[c] == tile) add_items(items, k, ipt);
                }
                if (items.empty()) continue;
                // Longest j-loops first, so the launch's tail is made of short items.
                std::stable_sort(items.begin(), items.end(),
                                 [](const DirectWork& a, const DirectWork& b) { return a.j1 - a.j0 > b.j1 - b.j0; });
                segs_.push_back(Segment{static_cast<int>(all.size()), static_cast<int>(items.size()), ipt, tile});
                all.insert(all.end(), items.begin(), items.end());
            }
        if (!all.empty()) {
            d_work_.reserve(all.size() * sizeof(DirectWork));
            LG_CK(cudaMemcpy(d_work_.as<DirectWork>(), all.data(), all.size() * sizeof(DirectWork),
                             cudaMemcpyHostToDevice));
        }
    }

    void apply_tuning() {
        Engine& e = *e_;
        build_work();
        if (e.group_max != tuning_.walk_group) {
            e.group_max = tuning_.walk_group;
            tree_reset_guess(e);
            acc_valid_ = false;
        }
    }

    // ---- tuning cache: lines "<device>\t<key>\t<value>" ------------------------------------------
    std::string cache_key(const char* what, int cls) const {
        return device_name_ + "\t" + what + (cls >= 0 ? std::to_string(cls) : std::string()) + "\t";
    }

    bool load_cache() {
        const char* path = std::getenv("LETTUCE_GB300_TUNE_CACHE");
        if (!path || !*path) return false;
        std::ifstream f(path);
        if (!f) return false;
        lg_ensemble_tuning t = tuning_;
        int found = 0;
        std::string line;
        while (std::getline(f, line)) {
            for (int c = 0; c < kClasses; ++c) {
                const std::string k = cache_key("direct_ipt", c);
                if (line.compare(0, k.size(), k) == 0) {
                    const int v = std::atoi(line.c_str() + k.size());
                    if (v == 1 || v == 2 || v == 4 || v == 8) {
                        t.direct_ipt[c] = v;
                        found |= 1 << c;
                    }
                }
                const std::string kt = cache_key("direct_tile", c);
                if (line.compare(0, kt.size(), kt) == 0) {
                    const int v = std::atoi(line.c_str() + kt.size());
                    if (v == 256 || v == 128) {
                        t.direct_tile[c] = v;
                        found |= 1 << (kClasses + 1 + c);
                    }
                }
            }
            const std::string k = cache_key("walk_group", -1);
            if (line.compare(0, k.size(), k) == 0) {
                const int v = std::atoi(line.c_str() + k.size());
                if (v >= 1 && v <= 1024) {
                    t.walk_group = v;
                    found |= 1 << kClasses;
                }
            }
        }
        if (found != (1 << (2 * kClasses + 1)) - 1) return false;
        for (int c = 0; c < kClasses; ++c)
            if (!valid_shape(t.direct_ipt[c], t.direct_tile[c])) return false;
        t.tuned = 1;
        tuning_ = t;
        return true;
    }

    void save_cache() const {
        const char* path = std::getenv("LETTUCE_GB300_TUNE_CACHE");
        if (!path || !*path) return;
        std::vector<std::string> keep;
        {
            std::ifstream f(path);
            std::string line;
            while (f && std::getline(f, line))
                if (line.compare(0, device_name_.size() + 1, device_name_ + "\t") != 0) keep.push_back(line);
        }
        std::ofstream f(path, std::ios::trunc);
        if (!f) return;  // the cache is an optimisation: an unwritable path is not an error
        for (const auto& l : keep) f << l << "\n";
        for (int c = 0; c < kClasses; ++c) {
            f << cache_key("direct_ipt", c) << tuning_.direct_ipt[c] << "\n";
            f << cache_key("direct_tile", c) << tuning_.direct_tile[c] << "\n";
        }
        f << cache_key("walk_group", -1) << tuning_.walk_group << "\n";
    }

    // ---- state copy for recovery -----------------------------------------------------------------
    void take_snapshot() {
        Engine& e = *e_;
        const size_t n = static_cast<size_t>(n_);
        const BodyArrays b = e.bodies(e.cur);
        snap_cur_ = e.cur;
        copy_set(b, snap_, n, true);
    }

    void restore_snapshot() {
        Engine& e = *e_;
        e.cur = snap_cur_;
        copy_set(e.bodies(e.cur), snap_, static_cast<size_t>(n_), false);
    }

    void copy_set(const BodyArrays& b, BodySet& sn, size_t n, bool save) {
        Engine& e = *e_;
        struct Item {
            void* body;
            DevBuf* snap;
            size_t bytes;
        } items[] = {{b.x, &sn.x, 8}, {b.y, &sn.y, 8}, {b.z, &sn.z, 8},     {b.hm, &sn.hm, 16}, {b.lo, &sn.lo, 16},
                     {b.vx, &sn.vx, 4}, {b.vy, &sn.vy, 4}, {b.vz, &sn.vz, 4}, {b.m, &sn.m, 4},     {b.id, &sn.id, 4},
                     {e.acc.as<float4>(), &snap_acc_, 16}};
        for (Item& it : items) {
            if (save) it.snap->reserve(it.bytes * n);
            if (save)
                LG_CK(cudaMemcpyAsync(it.snap->as<char>(), it.body, it.bytes * n, cudaMemcpyDeviceToDevice, e.stream));
            else
                LG_CK(cudaMemcpyAsync(it.body, it.snap->as<char>(), it.bytes * n, cudaMemcpyDeviceToDevice, e.stream));
        }
    }

    void copy_bodies(const BodyArrays& from, const BodyArrays& to) {
        Engine& e = *e_;
        const size_t n = static_cast<size_t>(n_);
        const std::pair<const void*, void*> p8[] = {{from.x, to.x}, {from.y, to.y}, {from.z, to.z}};
        const std::pair<const void*, void*> p16[] = {{from.hm, to.hm}, {from.lo, to.lo}};
        const std::pair<const void*, void*> p4[] = {{from.vx, to.vx}, {from.vy, to.vy}, {from.vz, to.vz},
                                                    {from.m, to.m},   {from.id, to.id}, {from.cost, to.cost}};
        for (const auto& q : p8) LG_CK(cudaMemcpyAsync(q.second, q.first, 8 * n, cudaMemcpyDeviceToDevice, e.stream));
        for (const auto& q : p16) LG_CK(cudaMemcpyAsync(q.second, q.first, 16 * n, cudaMemcpyDeviceToDevice, e.stream));
        for (const auto& q : p4) LG_CK(cudaMemcpyAsync(q.second, q.first, 4 * n, cudaMemcpyDeviceToDevice, e.stream));
    }

    template <class T>
    void scatter(const std::vector<T>& internal, T* out) const {
        if (!out) return;
        for (int k = 0; k < nsys_; ++k)
            std::memcpy(out + in_off_[order_[k]], internal.data() + off_[k], count_[k] * sizeof(T));
    }

    std::unique_ptr<Engine> e_;
    cudaStream_t side_ = nullptr;
    cudaEvent_t fork_ = nullptr, join_ = nullptr, t0_ = nullptr, t1_ = nullptr;
    std::string device_name_;
    double G_ = 1.0;
    int nsys_ = 0, nsys_tree_ = 0, n_ = 0, n_tree_ = 0;
    std::vector<int> order_;  // internal system -> input system
    std::vector<size_t> in_off_, off_;
    std::vector<uint32_t> count_;
    std::vector<double> eps_, theta_;
    unsigned long long direct_pairs_ = 0;
    DevBuf d_sys_, d_off_, d_inv_theta_, d_e2_, d_energy_, d_work_, tune_work_, sticky_;
    std::vector<Segment> segs_;
    lg_ensemble_tuning tuning_{};
    lg_ensemble_stats stats_{};
    bool acc_valid_ = false;
    // graph
    cudaGraphExec_t exec_ = nullptr;
    int g_steps_ = 0, g_cur0_ = 0, g_cur1_ = 0;
    double g_dt_ = 0;
    uint64_t g_launches_ = 0, g_gen_ = 0;
    // recovery copy
    BodySet snap_;
    DevBuf snap_acc_;
    int snap_cur_ = 0;
};

}  // namespace lg

// ---- C ABI -----------------------------------------------------------------------------------
struct lg_ensemble {
    std::unique_ptr<lg::Ensemble> p;
};

namespace {

template <class F>
lg_status eguard(F&& f) {
    try {
        f();
        lg::g_last_error.clear();
        return LG_OK;
    } catch (const lg::Error& ex) {
        lg::g_last_error = ex.what();
        return static_cast<lg_status>(ex.status);
    } catch (const std::bad_alloc&) {
        lg::g_last_error = "host allocation failed";
        return LG_ERR_RUNTIME;
    } catch (const std::exception& ex) {
        lg::g_last_error = ex.what();
        return LG_ERR_RUNTIME;
    }
}

lg::Ensemble& ens(lg_ensemble* en) {
    if (!en || !en->p) lg::fail(lg::kArg, "null ensemble");
    return *en->p;
}

}  // namespace

extern "C" {

lg_status lg_ensemble_create(int device, lg_ensemble** out) {
    return eguard([&] {
        if (!out) lg::fail(lg::kArg, "null pointer: out");
        *out = nullptr;
        int count = 0;
        const cudaError_t e = cudaGetDeviceCount(&count);
        if (e != cudaSuccess || count == 0) {
            cudaGetLastError();
            lg::fail(lg::kUnavailable, "no CUDA device available");
        }
        if (device < 0 || device >= count) lg::fail(lg::kArg, "device index out of range");
        auto h = std::make_unique<lg_ensemble>();
        h->p = std::make_unique<lg::Ensemble>(device);
        *out = h.release();
    });
}

lg_status lg_ensemble_destroy(lg_ensemble* en) {
    delete en;
    return LG_OK;
}

lg_status lg_ensemble_upload(lg_ensemble* en, size_t nsys, const uint32_t* counts, const double* eps,
                             const double* theta, const int* method, double G, const float* x, const float* y,
                             const float* z, const float* vx, const float* vy, const float* vz, const float* m,
                             const uint32_t* id) {
    return eguard([&] { ens(en).upload(nsys, counts, eps, theta, method, G, x, y, z, vx, vy, vz, m, id); });
}

lg_status lg_ensemble_run(lg_ensemble* en, double dt, int steps, int use_graph) {
    return eguard([&] { ens(en).run(dt, steps, use_graph != 0); });
}

lg_status lg_ensemble_energy(lg_ensemble* en, double* energy, double* ke, double* pe) {
    return eguard([&] { ens(en).energy(energy, ke, pe); });
}

lg_status lg_ensemble_download(lg_ensemble* en, float* x, float* y, float* z, float* vx, float* vy, float* vz,
                               float* m, uint32_t* id) {
    return eguard([&] { ens(en).download(x, y, z, vx, vy, vz, m, id); });
}

lg_status lg_ensemble_read_accel(lg_ensemble* en, float* ax, float* ay, float* az, float* pot) {
    return eguard([&] { ens(en).read_accel(ax, ay, az, pot); });
}

lg_status lg_ensemble_tune(lg_ensemble* en) {
    return eguard([&] { ens(en).tune(); });
}

lg_status lg_ensemble_get_tuning(lg_ensemble* en, lg_ensemble_tuning* out) {
    return eguard([&] {
        if (!out) lg::fail(lg::kArg, "null pointer: out");
        *out = ens(en).tuning();
    });
}

lg_status lg_ensemble_set_tuning(lg_ensemble* en, const lg_ensemble_tuning* t) {
    return eguard([&] {
        if (!t) lg::fail(lg::kArg, "null pointer: tuning");
        ens(en).set_tuning(*t);
    });
}

lg_status lg_ensemble_get_stats(lg_ensemble* en, lg_ensemble_stats* out) {
    return eguard([&] {
        if (!out) lg::fail(lg::kArg, "null pointer: out");
        *out = ens(en).stats();
    });
}

}  // extern "C"
