// ref_cuda_shim.cpp -- C entry points over the reference's own CUDA backend.
//
// baseline/Makefile compiles the reference's src/cuda_backend.cu unmodified (nvcc, sm_103a, the
// reference's own CUDA flags) and links it with this file into baseline/_ref/build/libref_cuda.so.
// The library lets the benchmark time the reference's GPU path on the same GPU and on the same
// bodies as the engine, through the reference's public Backend interface (src/backend.hpp:89-141).
// Every entry point returns 0, or -1 with the exception's text in refgpu_error().
#include <cstdint>
#include <cstring>
#include <exception>
#include <memory>
#include <string>

#include "backend.hpp"

namespace {
thread_local std::string g_err;

Backend* as_be(void* h) { return static_cast<Backend*>(h); }

template <class F>
int guard(F&& f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
    } catch (...) {
        g_err = "unknown exception";
    }
    return -1;
}
}  // namespace

extern "C" {

const char* refgpu_error() { return g_err.c_str(); }

void* refgpu_create(int device) {
    std::string why;
    std::unique_ptr<Backend> be = make_cuda_backend(device, why);
    if (!be) {
        g_err = why;
        return nullptr;
    }
    return be.release();
}

void refgpu_destroy(void* h) { delete as_be(h); }

int refgpu_name(void* h, char* out, size_t cap) {
    return guard([&] {
        const std::string s = as_be(h)->name();
        std::strncpy(out, s.c_str(), cap);
        if (cap) out[cap - 1] = 0;
    });
}

int refgpu_upload(void* h, size_t n, const float* x, const float* y, const float* z, const float* vx,
                  const float* vy, const float* vz, const float* m, const uint32_t* id) {
    return guard([&] {
        Bodies b;
        b.x.assign(x, x + n); b.y.assign(y, y + n); b.z.assign(z, z + n);
        b.vx.assign(vx, vx + n); b.vy.assign(vy, vy + n); b.vz.assign(vz, vz + n);
        b.m.assign(m, m + n); b.id.assign(id, id + n);
        as_be(h)->upload(b);
    });
}

int refgpu_download(void* h, float* x, float* y, float* z, float* vx, float* vy, float* vz, float* m,
                    uint32_t* id) {
    return guard([&] {
        Bodies b;
        as_be(h)->download(b);
        const size_t n = b.size();
        std::memcpy(x, b.x.data(), n * 4); std::memcpy(y, b.y.data(), n * 4); std::memcpy(z, b.z.data(), n * 4);
        std::memcpy(vx, b.vx.data(), n * 4); std::memcpy(vy, b.vy.data(), n * 4);
        std::memcpy(vz, b.vz.data(), n * 4); std::memcpy(m, b.m.data(), n * 4);
        std::memcpy(id, b.id.data(), n * 4);
    });
}

int refgpu_compute_forces(void* h, int method, double G, double eps, double theta, int potential) {
    return guard([&] {
        ForceParams p;
        p.G = G;
        p.eps = eps;
        p.theta = theta;
        p.method = method ? ForceMethod::tree : ForceMethod::direct;
        as_be(h)->compute_forces(p, potential != 0);
    });
}

int refgpu_kick(void* h, double dt) { return guard([&] { as_be(h)->kick(dt); }); }
int refgpu_drift(void* h, double dt) { return guard([&] { as_be(h)->drift(dt); }); }

// out: force, sort, build, walk, step (ms); *inter: interactions of the last force call.
int refgpu_times(void* h, double* out, uint64_t* inter) {
    return guard([&] {
        const PhaseTimes t = as_be(h)->times();
        out[0] = t.force_ms; out[1] = t.sort_ms; out[2] = t.build_ms; out[3] = t.walk_ms; out[4] = t.step_ms;
        *inter = t.interactions;
    });
}

// Diagnostics (13 values: mass, ke, pe, px, py, pz, lx, ly, lz, cx, cy, cz, has_pe); synchronises.
int refgpu_diagnostics(void* h, double* out) {
    return guard([&] {
        const Diag d = as_be(h)->diagnostics();
        const double v[13] = {d.mass, d.ke, d.pe, d.px, d.py, d.pz, d.lx, d.ly, d.lz, d.cx, d.cy, d.cz,
                              d.has_pe ? 1.0 : 0.0};
        std::memcpy(out, v, sizeof v);
    });
}

}  // extern "C"
