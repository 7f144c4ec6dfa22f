// ref_shim.cpp -- C entry points over the reference's own OpenMP backend.
//
// TEST INFRASTRUCTURE. oracle/Makefile compiles this file with the reference's source directory on
// the include path, so the reference's src/cpu_backend.cpp is compiled unmodified, from where it
// lies, into oracle/_ref/libref_cpu.so. Nothing is copied. The library pins the C restatement in
// lettuce_oracle.c and generates the golden vectors under tests/golden/.
//
// The reference keeps its tree in private members of a class in an anonymous namespace
// (src/cpu_backend.cpp:884-906). Including the .cpp in this translation unit, with `private`
// widened, lets the shim read the sorted keys, nodes and groups for the bit-exact topology checks.
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#define private public
#include "cpu_backend.cpp"
#undef private

#include "render.hpp"

namespace {
CpuBackend* as_cpu(void* h) { return static_cast<CpuBackend*>(h); }
}  // namespace

extern "C" {

void* ref_create(int threads) { return new CpuBackend(threads); }
void ref_destroy(void* h) { delete as_cpu(h); }

void ref_upload(void* h, size_t n, const float* x, const float* y, const float* z, const float* vx, const float* vy,
                const float* vz, const float* m, const uint32_t* id) {
    Bodies b;
    b.x.assign(x, x + n); b.y.assign(y, y + n); b.z.assign(z, z + n);
    b.vx.assign(vx, vx + n); b.vy.assign(vy, vy + n); b.vz.assign(vz, vz + n);
    b.m.assign(m, m + n); b.id.assign(id, id + n);
    as_cpu(h)->upload(b);
}

size_t ref_size(void* h) { return as_cpu(h)->n_; }

void ref_download(void* h, float* x, float* y, float* z, float* vx, float* vy, float* vz, float* m, uint32_t* id) {
    Bodies b;
    as_cpu(h)->download(b);
    const size_t n = b.size();
    std::memcpy(x, b.x.data(), n * 4); std::memcpy(y, b.y.data(), n * 4); std::memcpy(z, b.z.data(), n * 4);
    std::memcpy(vx, b.vx.data(), n * 4); std::memcpy(vy, b.vy.data(), n * 4); std::memcpy(vz, b.vz.data(), n * 4);
    std::memcpy(m, b.m.data(), n * 4); std::memcpy(id, b.id.data(), n * 4);
}

void ref_accel(void* h, float* ax, float* ay, float* az, float* pot) {
    CpuBackend* c = as_cpu(h);
    const size_t n = c->n_;
    std::memcpy(ax, c->ax_.data(), n * 4); std::memcpy(ay, c->ay_.data(), n * 4); std::memcpy(az, c->az_.data(), n * 4);
    if (pot) std::memcpy(pot, c->pot_.data(), n * 4);
}

static ForceParams params(int method, double G, double eps, double theta) {
    ForceParams p;
    p.G = G; p.eps = eps; p.theta = theta;
    p.method = method == 1 ? ForceMethod::tree : ForceMethod::direct;
    return p;
}

void ref_build_tree(void* h, int method, double theta) { as_cpu(h)->build_tree(params(method, 1, 0.01, theta)); }

void ref_compute_forces(void* h, int method, double G, double eps, double theta, int potential) {
    as_cpu(h)->compute_forces(params(method, G, eps, theta), potential != 0);
}

void ref_kick(void* h, double dt) { as_cpu(h)->kick(dt); }
void ref_drift(void* h, double dt) { as_cpu(h)->drift(dt); }

int ref_diagnostics(void* h, double* out) {
    Diag d = as_cpu(h)->diagnostics();
    double v[12] = {d.mass, d.ke, d.pe, d.px, d.py, d.pz, d.lx, d.ly, d.lz, d.cx, d.cy, d.cz};
    std::memcpy(out, v, sizeof v);
    return d.has_pe ? 1 : 0;
}

double ref_exact_potential_energy(void* h, double G, double eps) { return as_cpu(h)->exact_potential_energy(G, eps); }

uint64_t ref_times(void* h, double* out) {
    PhaseTimes t = as_cpu(h)->times();
    out[0] = t.force_ms; out[1] = t.sort_ms; out[2] = t.build_ms; out[3] = t.walk_ms; out[4] = t.step_ms;
    return t.interactions;
}

int ref_body_costs(void* h, float* cost) {
    std::vector<float> c;
    if (!as_cpu(h)->body_costs(c)) return 0;
    std::memcpy(cost, c.data(), c.size() * 4);
    return 1;
}

// Locally-essential trees through the reference's own export_let / compute_forces_with. The last
// export is kept in the shim until the next one; LetNode is copied out as its 60 raw bytes.
static LetTree g_last_let;

void ref_export_let(void* h, const float* lo, const float* hi, int method, double theta, size_t* nnodes,
                    size_t* nbodies) {
    Box3 box;
    for (int c = 0; c < 3; ++c) { box.lo[c] = lo[c]; box.hi[c] = hi[c]; }
    g_last_let = as_cpu(h)->export_let(box, params(method, 1, 0.01, theta));
    *nnodes = g_last_let.nodes.size();
    *nbodies = g_last_let.bx.size();
}

void ref_export_let_read(void* nodes60, float* bx, float* by, float* bz, float* bm) {
    std::memcpy(nodes60, g_last_let.nodes.data(), g_last_let.nodes.size() * sizeof(LetNode));
    const size_t nb = g_last_let.bx.size();
    std::memcpy(bx, g_last_let.bx.data(), nb * 4); std::memcpy(by, g_last_let.by.data(), nb * 4);
    std::memcpy(bz, g_last_let.bz.data(), nb * 4); std::memcpy(bm, g_last_let.bm.data(), nb * 4);
}

// compute_forces_with(p, potential, {one remote tree given as raw arrays}).
void ref_compute_forces_remote(void* h, int method, double G, double eps, double theta, int potential,
                               const void* nodes60, size_t nnodes, const float* bx, const float* by, const float* bz,
                               const float* bm, size_t nbodies) {
    LetTree t;
    t.nodes.resize(nnodes);
    std::memcpy(t.nodes.data(), nodes60, nnodes * sizeof(LetNode));
    t.bx.assign(bx, bx + nbodies); t.by.assign(by, by + nbodies); t.bz.assign(bz, bz + nbodies);
    t.bm.assign(bm, bm + nbodies);
    as_cpu(h)->compute_forces_with(params(method, G, eps, theta), potential != 0, {&t});
}

// The reference's render_image (src/render.cpp) on the given bodies; rgb: w * h * 3 bytes.
void ref_render(size_t n, const float* x, const float* y, const float* z, const float* vx, const float* vy,
                const float* vz, const float* m, int w, int h, const char* view, double extent, int color,
                unsigned char* rgb, double* extent_used) {
    Bodies b;
    b.x.assign(x, x + n); b.y.assign(y, y + n); b.z.assign(z, z + n);
    b.vx.assign(vx, vx + n); b.vy.assign(vy, vy + n); b.vz.assign(vz, vz + n);
    b.m.assign(m, m + n); b.id.resize(n);
    RenderOptions o;
    o.width = w; o.height = h; o.view = view; o.extent = extent;
    o.color = color == 1 ? ColorMode::speed : ColorMode::density;
    Image img = render_image(b, o);
    std::memcpy(rgb, img.rgb.data(), img.rgb.size());
    *extent_used = img.extent;
}

size_t ref_num_nodes(void* h) { return as_cpu(h)->nodes_.size(); }
size_t ref_num_groups(void* h) { return as_cpu(h)->groups_.size(); }
size_t ref_num_leaves(void* h) { return as_cpu(h)->leaves_.size(); }
int ref_max_depth(void* h) { return as_cpu(h)->max_depth_; }

// Same 64-byte layout as or_node: 11 floats, then first, nchild, lo, hi.
void ref_get_nodes(void* h, void* out) {
    const auto& v = as_cpu(h)->nodes_;
    char* o = static_cast<char*>(out);
    for (size_t k = 0; k < v.size(); ++k) {
        const Node& nd = v[k];
        float f[11] = {nd.cx, nd.cy, nd.cz, nd.m, nd.qxx, nd.qxy, nd.qxz, nd.qyy, nd.qyz, nd.qzz, nd.rcrit2};
        uint32_t u[4] = {nd.first, nd.nchild, nd.lo, nd.hi};
        std::memcpy(o + 60 * k, f, 44);
        std::memcpy(o + 60 * k + 44, u, 16);
    }
}

void ref_get_geo(void* h, float* out) {
    const auto& v = as_cpu(h)->geo_;
    for (size_t k = 0; k < v.size(); ++k) {
        out[4 * k] = v[k].gx; out[4 * k + 1] = v[k].gy; out[4 * k + 2] = v[k].gz; out[4 * k + 3] = v[k].half;
    }
}

void ref_get_groups(void* h, void* out) {
    const auto& v = as_cpu(h)->groups_;
    char* o = static_cast<char*>(out);
    for (size_t k = 0; k < v.size(); ++k) {
        float f[6] = {v[k].bx, v[k].by, v[k].bz, v[k].hx, v[k].hy, v[k].hz};
        uint32_t u[2] = {v[k].lo, v[k].hi};
        std::memcpy(o + 32 * k, f, 24);
        std::memcpy(o + 32 * k + 24, u, 8);
    }
}

void ref_get_leaves(void* h, uint32_t* out) {
    const auto& v = as_cpu(h)->leaves_;
    std::memcpy(out, v.data(), v.size() * 4);
}

void ref_get_keys(void* h, uint64_t* out) {
    CpuBackend* c = as_cpu(h);
    std::memcpy(out, c->key_.data(), c->n_ * 8);
}

void ref_get_frame(void* h, double* out) {
    CpuBackend* c = as_cpu(h);
    out[0] = c->ox_; out[1] = c->oy_; out[2] = c->oz_; out[3] = c->side_;
}

}  // extern "C"
