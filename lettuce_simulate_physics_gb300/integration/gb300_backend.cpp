// gb300_backend.cpp -- the reference's `class Backend` (src/backend.hpp:89-141) over the GB300
// engine's C ABI (include/lettuce_gb300.h). It replaces src/cuda_backend.cu (or src/cuda_stub.cpp)
// at the reference's link-time seam (CMakeLists.txt:94-108): it defines make_cuda_backend,
// cuda_compiled and cuda_device_count, so simulation.cpp, bench.cpp, parallel.cpp and the tests
// use the engine unchanged.
//
// Errors follow the reference: LG_ERR_LOGIC -> std::logic_error, any other failure ->
// std::runtime_error; make_cuda_backend returns nullptr and sets `why` when the engine is
// unavailable.
//
// Locally-essential trees (the MPI layer's export_let / compute_forces_with(remote)) are outside
// the engine. export_let is answered here on the host from the engine's tree, which is in the
// reference CPU backend's node layout, with the receiver contract of src/backend.hpp:58-77;
// compute_forces_with with remote trees throws.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "backend.hpp"
#include "lettuce_gb300.h"

namespace {

[[noreturn]] void raise(lg_status s) {
    const std::string msg = lg_last_error();
    if (s == LG_ERR_LOGIC) throw std::logic_error(msg);
    throw std::runtime_error(msg);
}

inline void ck(lg_status s) {
    if (s != LG_OK) raise(s);
}

lg_force_params cparams(const ForceParams& p) {
    lg_force_params c{};
    c.G = p.G;
    c.eps = p.eps;
    c.theta = p.theta;
    c.method = p.method == ForceMethod::tree ? LG_TREE : LG_DIRECT;
    return c;
}

class Gb300Backend final : public Backend {
public:
    explicit Gb300Backend(lg_engine* e) : e_(e) {}
    ~Gb300Backend() override { lg_destroy(e_); }
    Gb300Backend(const Gb300Backend&) = delete;
    Gb300Backend& operator=(const Gb300Backend&) = delete;

    std::string name() const override {
        char buf[512];
        ck(lg_name(e_, buf, sizeof buf));
        return buf;
    }

    void upload(const Bodies& b) override {
        ck(lg_upload(e_, b.size(), b.x.data(), b.y.data(), b.z.data(), b.vx.data(), b.vy.data(), b.vz.data(),
                     b.m.data(), b.id.data()));
        tree_cache_ok_ = false;
    }

    void download(Bodies& b) override {
        size_t n = 0;
        ck(lg_size(e_, &n));
        b.resize(n);
        ck(lg_download(e_, b.x.data(), b.y.data(), b.z.data(), b.vx.data(), b.vy.data(), b.vz.data(), b.m.data(),
                       b.id.data()));
    }

    void compute_forces(const ForceParams& p, bool potential) override {
        const lg_force_params c = cparams(p);
        ck(lg_compute_forces(e_, &c, potential ? 1 : 0));
        tree_cache_ok_ = false;
    }

    void kick(double dt) override { ck(lg_kick(e_, dt)); }

    void drift(double dt) override {
        ck(lg_drift(e_, dt));
        tree_cache_ok_ = false;
    }

    Diag diagnostics() override {
        lg_diag d{};
        ck(lg_diagnostics(e_, &d));
        Diag o;
        o.mass = d.mass; o.ke = d.ke; o.pe = d.pe; o.has_pe = d.has_pe != 0;
        o.px = d.px; o.py = d.py; o.pz = d.pz;
        o.lx = d.lx; o.ly = d.ly; o.lz = d.lz;
        o.cx = d.cx; o.cy = d.cy; o.cz = d.cz;
        return o;
    }

    double exact_potential_energy(double G, double eps) override {
        double v = 0;
        ck(lg_exact_potential_energy(e_, G, eps, &v));
        return v;
    }

    PhaseTimes times() const override {
        lg_phase_times t{};
        ck(lg_times(e_, &t));
        PhaseTimes o;
        o.force_ms = t.force_ms; o.sort_ms = t.sort_ms; o.build_ms = t.build_ms; o.walk_ms = t.walk_ms;
        o.step_ms = t.step_ms; o.interactions = t.interactions; o.comm_ms = t.comm_ms; o.balance_ms = t.balance_ms;
        return o;
    }

    Box3 local_bounds() override {
        Box3 b;
        ck(lg_local_bounds(e_, b.lo, b.hi));
        return b;
    }

    void build_tree(const ForceParams& p) override {
        const lg_force_params c = cparams(p);
        ck(lg_build_tree(e_, &c));
        tree_cache_ok_ = false;
        built_method_ = p.method;
    }

    LetTree export_let(const Box3& target, const ForceParams& p) override {
        LetTree out;
        size_t n = 0;
        ck(lg_size(e_, &n));
        if (n == 0) return out;
        if (p.method == ForceMethod::direct) return export_direct();
        load_tree();
        if (nodes_.empty() || mom_[3] <= 0) return out;
        const float bcx = 0.5f * (target.lo[0] + target.hi[0]), bhx = 0.5f * (target.hi[0] - target.lo[0]);
        const float bcy = 0.5f * (target.lo[1] + target.hi[1]), bhy = 0.5f * (target.hi[1] - target.lo[1]);
        const float bcz = 0.5f * (target.lo[2] + target.hi[2]), bhz = 0.5f * (target.hi[2] - target.lo[2]);
        // Breadth-first: the output doubles as the queue, so each sibling set stays contiguous.
        std::vector<uint32_t> src;
        auto emit = [&](uint32_t ni) {
            const float* m = &mom_[11 * ni];
            LetNode l{};
            l.cx = m[0]; l.cy = m[1]; l.cz = m[2]; l.mass = m[3];
            l.qxx = m[4]; l.qxy = m[5]; l.qxz = m[6]; l.qyy = m[7]; l.qyz = m[8]; l.qzz = m[9];
            l.rcrit2 = m[10];
            l.first_child = -1; l.child_count = 0; l.body_first = -1; l.body_count = 0;
            out.nodes.push_back(l);
            src.push_back(ni);
        };
        emit(0);
        for (size_t k = 0; k < out.nodes.size(); ++k) {
            const uint32_t ni = src[k];
            const float* m = &mom_[11 * ni];
            const uint32_t* r = &range_[4 * ni];  // lo, hi, first, nchild
            const float dx = std::max(std::fabs(m[0] - bcx) - bhx, 0.f);
            const float dy = std::max(std::fabs(m[1] - bcy) - bhy, 0.f);
            const float dz = std::max(std::fabs(m[2] - bcz) - bhz, 0.f);
            if (dx * dx + dy * dy + dz * dz >= m[10]) continue;  // terminal
            if (r[3] == 0) {
                out.nodes[k].body_first = static_cast<int32_t>(out.bx.size());
                out.nodes[k].body_count = static_cast<int32_t>(r[1] - r[0]);
                for (uint32_t i = r[0]; i < r[1]; ++i) {
                    out.bx.push_back(bodies_.x[i]); out.by.push_back(bodies_.y[i]);
                    out.bz.push_back(bodies_.z[i]); out.bm.push_back(bodies_.m[i]);
                }
                continue;
            }
            const int32_t first = static_cast<int32_t>(out.nodes.size());
            for (uint32_t c = r[2]; c < r[2] + r[3]; ++c)
                if (mom_[11 * c + 3] > 0) emit(c);
            out.nodes[k].first_child = first;
            out.nodes[k].child_count = static_cast<int32_t>(out.nodes.size()) - first;
        }
        return out;
    }

    void compute_forces_with(const ForceParams& p, bool potential,
                             const std::vector<const LetTree*>& remote) override {
        const lg_force_params c = cparams(p);
        ck(lg_compute_forces_with(e_, &c, potential ? 1 : 0, remote.size()));
    }

    MemoryNeed memory_need(uint64_t n, ForceMethod m) const override {
        lg_memory_estimate e{};
        ck(lg_memory_need(n, m == ForceMethod::tree ? LG_TREE : LG_DIRECT, &e));
        MemoryNeed o;
        o.device = e.device;
        o.host = e.host;
        return o;
    }

    bool device_memory(uint64_t& free_bytes, uint64_t& total_bytes) override {
        ck(lg_device_memory(e_, &free_bytes, &total_bytes));
        return true;
    }

    bool body_costs(std::vector<float>& cost) override {
        size_t n = 0;
        ck(lg_size(e_, &n));
        cost.resize(n);
        int valid = 0;
        ck(lg_body_costs(e_, cost.data(), n, &valid));
        if (!valid) cost.clear();
        return valid != 0;
    }

private:
    // One always-open root holding every body (the reference's direct-method LET).
    LetTree export_direct() {
        LetTree out;
        download(bodies_);
        out.bx = bodies_.x; out.by = bodies_.y; out.bz = bodies_.z; out.bm = bodies_.m;
        double M = 0, sx = 0, sy = 0, sz = 0;
        for (size_t i = 0; i < bodies_.size(); ++i) {
            const double m = bodies_.m[i];
            M += m; sx += m * bodies_.x[i]; sy += m * bodies_.y[i]; sz += m * bodies_.z[i];
        }
        LetNode r{};
        if (M > 0) { r.cx = float(sx / M); r.cy = float(sy / M); r.cz = float(sz / M); }
        r.mass = float(M);
        r.rcrit2 = 3.0e38f;
        r.first_child = -1; r.child_count = 0;
        r.body_first = 0; r.body_count = static_cast<int32_t>(bodies_.size());
        out.nodes.push_back(r);
        return out;
    }

    // The engine's tree after build_tree (reference node layout), cached until the next change.
    void load_tree() {
        if (tree_cache_ok_) return;
        size_t nodes = 0, leaves = 0, groups = 0;
        int depth = 0;
        ck(lg_tree_counts(e_, &nodes, &leaves, &groups, &depth));
        range_.resize(4 * nodes);
        mom_.resize(11 * nodes);
        ck(lg_tree_nodes(e_, range_.data(), mom_.data(), nullptr, nodes));
        nodes_.assign(nodes, 0);
        download(bodies_);
        tree_cache_ok_ = true;
    }

    lg_engine* e_;
    bool tree_cache_ok_ = false;
    ForceMethod built_method_ = ForceMethod::direct;
    std::vector<uint32_t> range_;
    std::vector<float> mom_;
    std::vector<char> nodes_;
    Bodies bodies_;
};

}  // namespace

std::unique_ptr<Backend> make_cuda_backend(int device, std::string& why) {
    lg_engine* e = nullptr;
    const lg_status s = lg_create(device, &e);
    if (s != LG_OK) {
        why = lg_last_error();
        return nullptr;
    }
    return std::make_unique<Gb300Backend>(e);
}

bool cuda_compiled() { return lg_compiled() != 0; }

int cuda_device_count() { return lg_device_count(); }
