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
// Locally-essential trees (the MPI layer's export_let / compute_forces_with(remote)) are built and
// walked on the device (lg_export_let, lg_compute_forces_with): LetNode and lg_let_node share one
// layout, so the trees cross the boundary without conversion.
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
    }

    void kick(double dt) override { ck(lg_kick(e_, dt)); }

    void drift(double dt) override {
        ck(lg_drift(e_, dt));
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
    }

    LetTree export_let(const Box3& target, const ForceParams& p) override {
        LetTree out;
        const lg_force_params c = cparams(p);
        size_t nn = 0, nb = 0;
        ck(lg_export_let(e_, target.lo, target.hi, &c, &nn, &nb));
        out.nodes.resize(nn);
        out.bx.resize(nb); out.by.resize(nb); out.bz.resize(nb); out.bm.resize(nb);
        ck(lg_export_let_read(e_, reinterpret_cast<lg_let_node*>(out.nodes.data()), out.bx.data(), out.by.data(),
                              out.bz.data(), out.bm.data()));
        return out;
    }

    void compute_forces_with(const ForceParams& p, bool potential,
                             const std::vector<const LetTree*>& remote) override {
        const lg_force_params c = cparams(p);
        std::vector<lg_let_tree> trees(remote.size());
        for (size_t k = 0; k < remote.size(); ++k) {
            const LetTree& t = *remote[k];
            lg_let_tree& d = trees[k];
            d.nodes = reinterpret_cast<const lg_let_node*>(t.nodes.data());
            d.nnodes = t.nodes.size();
            d.bx = t.bx.data(); d.by = t.by.data(); d.bz = t.bz.data(); d.bm = t.bm.data();
            d.nbodies = t.bx.size();
        }
        ck(lg_compute_forces_with(e_, &c, potential ? 1 : 0, trees.data(), trees.size()));
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
    lg_engine* e_;
};

static_assert(sizeof(LetNode) == sizeof(lg_let_node), "LetNode and lg_let_node share one layout");

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
