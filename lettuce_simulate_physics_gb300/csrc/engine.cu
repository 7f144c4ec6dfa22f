// The engine behind the C ABI (include/lettuce_gb300.h): resident state, the Backend semantics of
// the reference (src/backend.hpp:89-141, behaviour as in src/cuda_backend.cu:1213-1660), and the
// extern "C" entry points. Host C++ only; kernels live in integrate.cu, direct.cu, tree.cu, walk.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/lettuce_gb300.h"
#include "engine.cuh"

namespace lg {

thread_local std::string g_last_error;

Engine::Engine(int device) : dev(device) {
    LG_CK(cudaSetDevice(dev));
    cudaDeviceProp prop{};
    LG_CK(cudaGetDeviceProperties(&prop, dev));
    // Fail here, with a clear message, when this build has no image for the device.
    cudaFuncAttributes fa{};
    cudaError_t e = cudaFuncGetAttributes(&fa, probe_kernel());
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(kUnavailable, std::string("device ") + prop.name + " (sm_" + std::to_string(prop.major) +
                               std::to_string(prop.minor) + ") has no kernel image in this build (" +
                               cudaGetErrorString(e) + "); the engine is built for sm_103a");
    }
    sms = prop.multiProcessorCount;
    l2_bytes = prop.l2CacheSize;
    char buf[512];
    std::snprintf(buf, sizeof buf, "cuda: %s (sm_%d%d, %d SMs, %.0f GB)", prop.name, prop.major, prop.minor,
                  prop.multiProcessorCount, prop.totalGlobalMem / 1073741824.0);
    name = buf;
    // Walk settings, read at construction as the reference does (src/cuda_backend.cu:1239-1254).
    if (const char* w = std::getenv("LETTUCE_CUDA_WALK")) {
        std::string v = w;
        if (v != "body" && v != "group") fail(kRuntime, "LETTUCE_CUDA_WALK must be body or group, not '" + v + "'");
        walk_body = v == "body";
    }
    if (const char* g = std::getenv("LETTUCE_CUDA_GROUP")) {
        char* end = nullptr;
        long v = std::strtol(g, &end, 10);
        if (!end || *end || v < 1 || v > 1024)
            fail(kRuntime, std::string("LETTUCE_CUDA_GROUP must be an integer in [1, 1024], not '") + g + "'");
        group_max = static_cast<int>(v);
    }
    if (walk_body) group_max = 1;
    if (const char* m = std::getenv("LETTUCE_GB300_WALK_GROUPS")) {
        const std::string v = m;
        if (v != "merged" && v != "reference")
            fail(kRuntime, "LETTUCE_GB300_WALK_GROUPS must be merged or reference, not '" + v + "'");
        walk_merge = v == "merged";
    }
    if (const char* c = std::getenv("LETTUCE_GB300_WALK_MERGE_CAP")) {
        const int v = std::atoi(c);
        if (v < 1 || v > 1024) fail(kRuntime, "LETTUCE_GB300_WALK_MERGE_CAP must be in [1, 1024]");
        merge_cap = v;
    }
    // Direct launch shape override "ipt,slices[,tile]" (tuning; otherwise chosen per size).
    if (const char* d = std::getenv("LETTUCE_GB300_DIRECT")) {
        int ipt = 0, slices = 0, tile = 256;
        const int got = std::sscanf(d, "%d,%d,%d", &ipt, &slices, &tile);
        if (got < 2 || (ipt != 1 && ipt != 2 && ipt != 4 && ipt != 8) || slices < 1 || (tile != 256 && tile != 128) ||
            (tile == 128 && ipt == 8))
            fail(kRuntime, std::string("LETTUCE_GB300_DIRECT must be 'ipt,slices[,tile]' with ipt in {1,2,4,8} and "
                                       "tile 256, or 128 with ipt in {1,2,4}, not '") + d + "'");
        direct_shape_override = DirectShape{ipt, tile, slices};
    }
    name += walk_body ? ", per-body walk" : ", group walk " + std::to_string(group_max);
    if (!walk_body) name += walk_merge ? " (packed)" : " (reference groups)";
    LG_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    LG_CK(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    LG_CK(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
    LG_CK(cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming));
    for (auto& ev : events) LG_CK(cudaEventCreate(&ev));
    for (auto& ev : user_events) LG_CK(cudaEventCreate(&ev));
    small.reserve(4096);
    LG_CK(cudaMemset(small.as<char>(), 0, 4096));
    pinned_small = nullptr;
    LG_CK(cudaMallocHost(&pinned_small, 4096));
    tree = make_tree_state();
    adjoint = make_adjoint_state();
    lets = make_let_store();
}

Engine::~Engine() {
    cudaSetDevice(dev);
    if (stream) cudaStreamSynchronize(stream);
    if (side) cudaStreamSynchronize(side);
    tree.reset();
    adjoint.reset();
    lets.reset();
    for (auto& ev : events) if (ev) cudaEventDestroy(ev);
    for (auto& ev : user_events) if (ev) cudaEventDestroy(ev);
    if (pinned_small) cudaFreeHost(pinned_small);
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (join_ev) cudaEventDestroy(join_ev);
    if (side) cudaStreamDestroy(side);
    if (stream) cudaStreamDestroy(stream);
}

BodyArrays Engine::bodies(int which) const {
    const BodySet& s = set[which];
    BodyArrays b;
    b.x = s.x.as<double>(); b.y = s.y.as<double>(); b.z = s.z.as<double>();
    b.hm = s.hm.as<float4>(); b.lo = s.lo.as<float4>();
    b.vx = s.vx.as<float>(); b.vy = s.vy.as<float>(); b.vz = s.vz.as<float>(); b.m = s.m.as<float>();
    b.cost = s.cost.as<float>(); b.id = s.id.as<uint32_t>(); b.level = s.level.as<uint8_t>();
    return b;
}

void Engine::reserve_bodies(size_t count) {
    for (auto& s : set) {
        s.x.reserve(count * 8); s.y.reserve(count * 8); s.z.reserve(count * 8);
        s.hm.reserve(count * 16); s.lo.reserve(count * 16);
        s.vx.reserve(count * 4); s.vy.reserve(count * 4); s.vz.reserve(count * 4); s.m.reserve(count * 4);
        s.cost.reserve(count * 4); s.id.reserve(count * 4); s.level.reserve(count + 16);
    }
    acc.reserve(count * 16);
    staging.reserve(count * 4 * 4);
}

void Engine::upload(size_t count, const float* x, const float* y, const float* z, const float* vx, const float* vy,
                    const float* vz, const float* m, const uint32_t* id) {
    LG_CK(cudaSetDevice(dev));
    if (count >= static_cast<size_t>(INT32_MAX))
        fail(kRuntime, "cuda backend: n = " + std::to_string(count) + " exceeds the 2^31-1 body limit");
    reserve_bodies(count);
    n = static_cast<int>(count);
    cur = 0;
    has_pe = false;
    acc_ok = true;
    tree_ok = false;
    costs_ok = false;
    kick_rec = drift_rec = false;
    block_ready = false;
    times = lg_phase_times{};
    tree_reset_guess(*this);
    if (n == 0) return;
    const size_t fb = count * 4;
    BodyArrays b = bodies(0);
    float* st = staging.as<float>();
    LG_CK(cudaMemcpyAsync(st, x, fb, cudaMemcpyHostToDevice, stream));
    LG_CK(cudaMemcpyAsync(st + count, y, fb, cudaMemcpyHostToDevice, stream));
    LG_CK(cudaMemcpyAsync(st + 2 * count, z, fb, cudaMemcpyHostToDevice, stream));
    LG_CK(cudaMemcpyAsync(b.vx, vx, fb, cudaMemcpyHostToDevice, stream));
    LG_CK(cudaMemcpyAsync(b.vy, vy, fb, cudaMemcpyHostToDevice, stream));
    LG_CK(cudaMemcpyAsync(b.vz, vz, fb, cudaMemcpyHostToDevice, stream));
    LG_CK(cudaMemcpyAsync(b.m, m, fb, cudaMemcpyHostToDevice, stream));
    LG_CK(cudaMemcpyAsync(b.id, id, fb, cudaMemcpyHostToDevice, stream));
    launch_widen(st, st + count, st + 2 * count, b.m, b, n, stream);
    ++launches;
    // A kick before the first force call adds zero rather than garbage.
    LG_CK(cudaMemsetAsync(acc.as<float4>(), 0, count * 16, stream));
    LG_CK(cudaMemsetAsync(b.cost, 0, fb, stream));
    LG_CK(cudaStreamSynchronize(stream));
}

void Engine::upload64(size_t count, const double* x, const double* y, const double* z, const float* vx,
                      const float* vy, const float* vz, const float* m, const uint32_t* id) {
    std::vector<float> f(count * 3);
    for (size_t i = 0; i < count; ++i) {
        f[i] = static_cast<float>(x[i]);
        f[count + i] = static_cast<float>(y[i]);
        f[2 * count + i] = static_cast<float>(z[i]);
    }
    upload(count, f.data(), f.data() + count, f.data() + 2 * count, vx, vy, vz, m, id);
    if (n == 0) return;
    const BodyArrays b = bodies(cur);
    const size_t db = count * 8;
    LG_CK(cudaMemcpyAsync(b.x, x, db, cudaMemcpyHostToDevice, stream));
    LG_CK(cudaMemcpyAsync(b.y, y, db, cudaMemcpyHostToDevice, stream));
    LG_CK(cudaMemcpyAsync(b.z, z, db, cudaMemcpyHostToDevice, stream));
    launch_refresh_hilo(b, n, stream);
    ++launches;
    LG_CK(cudaStreamSynchronize(stream));
}

void Engine::download(float* x, float* y, float* z, float* vx, float* vy, float* vz, float* m, uint32_t* id) {
    LG_CK(cudaSetDevice(dev));
    if (n == 0) return;
    const size_t count = static_cast<size_t>(n), fb = count * 4;
    BodyArrays b = bodies(cur);
    float* st = staging.as<float>();
    launch_round_pos(b, st, st + count, st + 2 * count, n, stream);
    ++launches;
    LG_CK(cudaMemcpyAsync(x, st, fb, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaMemcpyAsync(y, st + count, fb, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaMemcpyAsync(z, st + 2 * count, fb, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaMemcpyAsync(vx, b.vx, fb, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaMemcpyAsync(vy, b.vy, fb, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaMemcpyAsync(vz, b.vz, fb, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaMemcpyAsync(m, b.m, fb, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaMemcpyAsync(id, b.id, fb, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaStreamSynchronize(stream));
}

unsigned* Engine::err_word() const { return small.as<unsigned>(); }
unsigned* Engine::ticket() const { return small.as<unsigned>() + 4; }
unsigned long long* Engine::inter_counter() const { return reinterpret_cast<unsigned long long*>(small.as<char>() + 64); }
double* Engine::dscratch() const { return reinterpret_cast<double*>(small.as<char>() + 128); }

float Engine::elapsed(int a, int b) const {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, events[a], events[b]) != cudaSuccess) {
        cudaGetLastError();
        return 0.f;
    }
    return ms;
}

void Engine::check_device_errors(const char* where) {
    unsigned e = pinned_small[0];
    if (e & (kErrWaitTimeout | kErrStackOverflow | kErrNodeOverflow | kErrListOverflow)) {
        LG_CK(cudaMemsetAsync(err_word(), 0, 4, stream));
        std::string what;
        if (e & kErrWaitTimeout) what += " device wait timed out;";
        if (e & kErrStackOverflow) what += " traversal stack overflow;";
        if (e & kErrNodeOverflow) what += " tree node capacity exceeded;";
        if (e & kErrListOverflow) what += " interaction list overflow;";
        fail(kRuntime, std::string(where) + ":" + what + " accelerations are invalid");
    }
}

void Engine::ensure_tree_valid() {
    if (!tree_ok) return;
    LG_CK(cudaMemcpyAsync(pinned_small + 64, tree_counts_device(*this), 32, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaStreamSynchronize(stream));
    if (tree_verify(*this, pinned_small + 64)) return;
    lg_force_params p{};
    p.method = LG_TREE;
    p.theta = tree_theta(*this);
    build_tree(p);  // exact sizes now; invalidates the accelerations as any build does
}

void Engine::build_tree(const lg_force_params& p) {
    LG_CK(cudaSetDevice(dev));
    tree_ok = false;
    times.sort_ms = times.build_ms = 0;
    pend_tree_times = false;
    if (p.method != LG_TREE || n == 0) return;
    // The sort reorders the bodies but not acc or the costs: stale until the next force call.
    costs_ok = false;
    has_pe = false;
    acc_ok = false;
    LG_CK(cudaEventRecord(events[EV_BUILD0], stream));
    {
        NvtxRange r("lettuce sort");
        tree_sort(*this);
    }
    LG_CK(cudaEventRecord(events[EV_SORTED], stream));
    {
        NvtxRange r("lettuce build");
        tree_build(*this, p.theta);
    }
    LG_CK(cudaEventRecord(events[EV_BUILT], stream));
    tree_ok = true;
    pend_tree_times = true;
}

void Engine::compute_forces_with(const lg_force_params& p, bool potential, const lg_let_tree* remote,
                                 size_t nremote) {
    LG_CK(cudaSetDevice(dev));
    if (nremote > 0 && !remote) fail(kArg, "compute_forces_with: null remote tree array");
    times.walk_ms = times.force_ms = 0;
    times.interactions = 0;
    costs_ok = false;
    const bool tree_m = p.method == LG_TREE;
    if (n == 0) {
        times.sort_ms = times.build_ms = 0;
        has_pe = potential;
        acc_ok = true;
        return;
    }
    if (tree_m && !tree_ok)
        fail(kLogic, "cuda compute_forces_with: call build_tree after the last upload/drift first");
    const float G = static_cast<float>(p.G);
    const float e2 = static_cast<float>(p.eps * p.eps);
    const bool eps0 = !(e2 >= 1.17549435e-38f);  // zero or denormal: guarded pair kernel
    LG_CK(cudaMemsetAsync(small.as<char>(), 0, 128, stream));
    // Remote trees (other ranks' locally-essential trees) go to the device before the timed part.
    const LetView let = nremote > 0 ? let_upload(*this, remote, nremote) : LetView{};
    const bool have_let = let.ntrees > 0;
    LG_CK(cudaEventRecord(events[EV_WALK0], stream));
    BodyArrays b = bodies(cur);
    NvtxRange walk_range(tree_m ? "lettuce walk" : "lettuce direct");
    if (!tree_m) {
        DirectShape sh = direct_shape_override.ipt ? direct_shape_override : default_direct_shape(n, sms);
        int slices = std::max(1, sh.slices);
        if (slices > 1) partial.reserve(static_cast<size_t>(slices) * n * 16 + 16 * 1024);
        launch_direct(b, n, G, e2, potential, eps0, sh, acc.as<float4>(), partial.as<float4>(), err_word(), stream,
                      b.cost);
        launches += slices > 1 ? 2 : 1;
        // Remote trees per block of 128 consecutive bodies (src/cpu_backend.cpp:695-717).
        if (have_let) tree_walk_remote_blocks(*this, G, e2, potential, eps0, let, let_body_blocks(*this, 128));
    } else {
        tree_walk(*this, G, e2, potential, eps0, nullptr, nullptr, have_let ? &let : nullptr);
    }
    LG_CK(cudaEventRecord(events[EV_WALK1], stream));
    LG_CK(cudaMemcpyAsync(pinned_small, small.as<char>(), 128, cudaMemcpyDeviceToHost, stream));
    if (tree_m) LG_CK(cudaMemcpyAsync(pinned_small + 64, tree_counts_device(*this), 32, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaStreamSynchronize(stream));
    if (tree_m && !tree_verify(*this, pinned_small + 64)) {
        // A sync-free build guessed its sizes wrong (or missed a key restart): rebuild exactly and
        // walk again. The bodies are already sorted, so the stable re-sort keeps their order.
        LG_CK(cudaMemsetAsync(err_word(), 0, 4, stream));
        build_tree(p);
        compute_forces_with(p, potential, remote, nremote);
        return;
    }
    check_device_errors(tree_m ? "cuda tree walk" : "cuda direct");
    times.sort_ms = tree_m && pend_tree_times ? elapsed(EV_BUILD0, EV_SORTED) : 0.0;
    times.build_ms = tree_m && pend_tree_times ? elapsed(EV_SORTED, EV_BUILT) : 0.0;
    pend_tree_times = false;
    times.walk_ms = elapsed(EV_WALK0, EV_WALK1);
    times.force_ms = times.sort_ms + times.build_ms + times.walk_ms;
    const unsigned long long* cnt = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(pinned_small) + 64);
    // Walk: [0] body pairs (own entry excluded), [1] cell terms; the direct method adds its
    // remote walk's entries to its n (n - 1) pairs.
    last_body_pairs = tree_m ? cnt[0] : static_cast<uint64_t>(n) * static_cast<uint64_t>(n - 1) + cnt[0];
    last_cell_terms = cnt[1];
    times.interactions = last_body_pairs + last_cell_terms;
    has_pe = potential;
    acc_ok = true;
    costs_ok = true;
}

void Engine::kick(double dt) {
    LG_CK(cudaSetDevice(dev));
    if (n == 0) return;
    if (!acc_ok) fail(kLogic, "cuda kick: accelerations are stale (build_tree since the last force call)");
    NvtxRange r("lettuce kick");
    LG_CK(cudaEventRecord(events[EV_KICK0], stream));
    launch_kick(bodies(cur), acc.as<float4>(), static_cast<float>(dt), n, stream);
    ++launches;
    LG_CK(cudaEventRecord(events[EV_KICK1], stream));
    kick_rec = true;
}

void Engine::drift(double dt) {
    LG_CK(cudaSetDevice(dev));
    if (n == 0) return;
    NvtxRange r("lettuce drift");
    LG_CK(cudaEventRecord(events[EV_DRIFT0], stream));
    launch_drift(bodies(cur), dt, n, stream);
    ++launches;
    LG_CK(cudaEventRecord(events[EV_DRIFT1], stream));
    drift_rec = true;
    tree_ok = false;
    has_pe = false;
}

lg_diag Engine::diagnostics() {
    LG_CK(cudaSetDevice(dev));
    lg_diag d{};
    d.has_pe = has_pe ? 1 : 0;
    if (n == 0) return d;
    const int blocks = std::min(2 * sms, (n + 255) / 256);
    diag_partial.reserve(static_cast<size_t>(blocks) * 12 * 8);
    double* out = dscratch();
    launch_diag(bodies(cur), acc.as<float4>(), n, diag_partial.as<double>(), ticket(), out, blocks, stream);
    ++launches;
    LG_CK(cudaMemcpyAsync(pinned_small, out, 12 * 8, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaStreamSynchronize(stream));
    const double* v = reinterpret_cast<const double*>(pinned_small);
    d.mass = v[0];
    d.ke = v[1];
    d.pe = has_pe ? 0.5 * v[2] : 0.0;
    d.px = v[3]; d.py = v[4]; d.pz = v[5];
    d.lx = v[6]; d.ly = v[7]; d.lz = v[8];
    if (v[0] > 0) { d.cx = v[9] / v[0]; d.cy = v[10] / v[0]; d.cz = v[11] / v[0]; }
    return d;
}

double Engine::exact_potential_energy(double G, double eps) {
    LG_CK(cudaSetDevice(dev));
    if (n < 2) return 0.0;
    double* out = dscratch();
    LG_CK(cudaMemsetAsync(out, 0, 8, stream));
    launch_exact_pe(bodies(cur), n, eps * eps, out, stream);
    ++launches;
    LG_CK(cudaMemcpyAsync(pinned_small, out, 8, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaStreamSynchronize(stream));
    return -G * reinterpret_cast<const double*>(pinned_small)[0];
}

lg_phase_times Engine::get_times() {
    lg_phase_times t = times;
    double ms = 0;
    if (kick_rec || drift_rec) LG_CK(cudaStreamSynchronize(stream));
    if (kick_rec) ms += elapsed(EV_KICK0, EV_KICK1);
    if (drift_rec) ms += elapsed(EV_DRIFT0, EV_DRIFT1);
    t.step_ms = ms;
    return t;
}

void Engine::local_bounds(float lo[3], float hi[3]) {
    LG_CK(cudaSetDevice(dev));
    for (int c = 0; c < 3; ++c) lo[c] = hi[c] = 0.f;
    if (n == 0) return;
    const int blocks = std::min(2 * sms, (n + 255) / 256);
    diag_partial.reserve(static_cast<size_t>(blocks) * 12 * 8);
    double* out = dscratch();
    launch_bounds(bodies(cur), n, diag_partial.as<double>(), ticket(), out, blocks, stream);
    ++launches;
    LG_CK(cudaMemcpyAsync(pinned_small, out, 6 * 8, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaStreamSynchronize(stream));
    const double* v = reinterpret_cast<const double*>(pinned_small);
    // Rounded to nearest, so the box equals the min/max of the downloaded float positions.
    for (int c = 0; c < 3; ++c) {
        lo[c] = static_cast<float>(v[c]);
        hi[c] = static_cast<float>(v[3 + c]);
    }
}

bool Engine::body_costs(float* cost, size_t count) {
    LG_CK(cudaSetDevice(dev));
    if (!costs_ok || n == 0) return false;
    if (count < static_cast<size_t>(n)) fail(kArg, "body_costs: output holds fewer than n values");
    LG_CK(cudaMemcpyAsync(cost, bodies(cur).cost, static_cast<size_t>(n) * 4, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaStreamSynchronize(stream));
    return true;
}

void Engine::read_accel(float* ax, float* ay, float* az, float* pot) {
    LG_CK(cudaSetDevice(dev));
    if (n == 0) return;
    std::vector<float4> h(static_cast<size_t>(n));
    LG_CK(cudaMemcpyAsync(h.data(), acc.as<float4>(), h.size() * 16, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaStreamSynchronize(stream));
    for (size_t i = 0; i < h.size(); ++i) {
        ax[i] = h[i].x; ay[i] = h[i].y; az[i] = h[i].z;
        if (pot) pot[i] = h[i].w;
    }
}

void Engine::read_pos64(double* x, double* y, double* z) {
    LG_CK(cudaSetDevice(dev));
    if (n == 0) return;
    BodyArrays b = bodies(cur);
    const size_t db = static_cast<size_t>(n) * 8;
    LG_CK(cudaMemcpyAsync(x, b.x, db, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaMemcpyAsync(y, b.y, db, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaMemcpyAsync(z, b.z, db, cudaMemcpyDeviceToHost, stream));
    LG_CK(cudaStreamSynchronize(stream));
}

void Engine::flush_l2() {
    const size_t bytes = std::max<size_t>(static_cast<size_t>(l2_bytes) * 2, size_t(256) << 20);
    flush_buf.reserve(bytes);
    launch_flush(flush_buf.as<float>(), bytes / 4, stream);
}

size_t Engine::held_bytes() const {
    size_t held = 0;
    for (const auto& s : set)
        for (const DevBuf* d : {&s.x, &s.y, &s.z, &s.hm, &s.lo, &s.vx, &s.vy, &s.vz, &s.m, &s.cost, &s.id})
            held += d->capacity();
    for (const DevBuf* d : {&acc, &staging, &partial, &diag_partial, &flush_buf, &walk_stack}) held += d->capacity();
    return held + tree_held_bytes(*this);
}

}  // namespace lg

// ---- C ABI -----------------------------------------------------------------------------------
using lg::Engine;

struct lg_engine {
    std::unique_ptr<Engine> e;
};

namespace {

template <class F>
lg_status guard(F&& f) {
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

Engine& eng(lg_engine* e) {
    if (!e || !e->e) lg::fail(lg::kArg, "null engine");
    return *e->e;
}

void need(const void* p, const char* what) {
    if (!p) lg::fail(lg::kArg, std::string("null pointer: ") + what);
}

}  // namespace

extern "C" {

const char* lg_last_error(void) { return lg::g_last_error.c_str(); }

int lg_compiled(void) { return 1; }

int lg_device_count(void) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return count;
}

lg_status lg_create(int device, lg_engine** out) {
    return guard([&] {
        need(out, "out");
        *out = nullptr;
        int count = 0;
        cudaError_t e = cudaGetDeviceCount(&count);
        if (e != cudaSuccess) {
            cudaGetLastError();
            lg::fail(lg::kUnavailable, std::string("no usable CUDA device: ") + cudaGetErrorString(e));
        }
        if (count == 0) lg::fail(lg::kUnavailable, "no CUDA device found");
        if (device < 0 || device >= count)
            lg::fail(lg::kUnavailable, "CUDA device " + std::to_string(device) + " out of range (" +
                                           std::to_string(count) + " devices)");
        auto h = std::make_unique<lg_engine>();
        try {
            h->e = std::make_unique<Engine>(device);
        } catch (const lg::Error& ex) {
            lg::fail(ex.status == lg::kRuntime ? lg::kUnavailable : ex.status, ex.what());
        }
        *out = h.release();
    });
}

void lg_destroy(lg_engine* e) { delete e; }

lg_status lg_name(const lg_engine* e, char* buf, size_t cap) {
    return guard([&] {
        need(buf, "buf");
        const std::string& s = eng(const_cast<lg_engine*>(e)).name;
        if (cap == 0) lg::fail(lg::kArg, "empty buffer");
        size_t k = std::min(cap - 1, s.size());
        std::memcpy(buf, s.data(), k);
        buf[k] = 0;
    });
}

lg_status lg_upload(lg_engine* e, size_t n, const float* x, const float* y, const float* z, const float* vx,
                    const float* vy, const float* vz, const float* m, const uint32_t* id) {
    return guard([&] {
        if (n) { need(x, "x"); need(y, "y"); need(z, "z"); need(vx, "vx"); need(vy, "vy"); need(vz, "vz");
                 need(m, "m"); need(id, "id"); }
        eng(e).upload(n, x, y, z, vx, vy, vz, m, id);
    });
}

lg_status lg_upload64(lg_engine* e, size_t n, const double* x, const double* y, const double* z, const float* vx,
                      const float* vy, const float* vz, const float* m, const uint32_t* id) {
    return guard([&] {
        if (n) { need(x, "x"); need(y, "y"); need(z, "z"); need(vx, "vx"); need(vy, "vy"); need(vz, "vz");
                 need(m, "m"); need(id, "id"); }
        eng(e).upload64(n, x, y, z, vx, vy, vz, m, id);
    });
}

// ---- FP64 sidecar of a float snapshot --------------------------------------------------------
// Layout (little-endian): "LGF64LO1", u64 n, u64 step, u64 reserved, then u32 id[n] padded to 8
// bytes, then f64 lo_x[n], lo_y[n], lo_z[n] with lo = x - (double)(float)x, exact in FP64, so
// float + lo restores the position bit for bit. Written to <path>.tmp and renamed into place.
lg_status lg_write_fp64_sidecar(lg_engine* e, const char* path, uint64_t step) {
    return guard([&] {
        need(path, "path");
        Engine& E = eng(e);
        const size_t n = static_cast<size_t>(E.n);
        std::vector<double> p(3 * n);
        std::vector<float> f(8 * n + 8);
        std::vector<uint32_t> id(n + 2, 0);
        if (n) {
            E.read_pos64(p.data(), p.data() + n, p.data() + 2 * n);
            E.download(f.data(), f.data() + n, f.data() + 2 * n, f.data() + 3 * n, f.data() + 4 * n, f.data() + 5 * n,
                       f.data() + 6 * n, id.data());
        }
        for (size_t k = 0; k < 3 * n; ++k) p[k] -= static_cast<double>(static_cast<float>(p[k]));
        const std::string tmp = std::string(path) + ".tmp";
        FILE* fp = std::fopen(tmp.c_str(), "wb");
        if (!fp) lg::fail(lg::kRuntime, std::string("cannot write ") + tmp);
        const uint64_t hdr[3] = {n, step, 0};
        bool ok = std::fwrite("LGF64LO1", 1, 8, fp) == 8 && std::fwrite(hdr, 8, 3, fp) == 3;
        const size_t nid = (n + 1) & ~size_t(1);
        ok = ok && std::fwrite(id.data(), 4, nid, fp) == nid;
        ok = ok && (n == 0 || std::fwrite(p.data(), 8, 3 * n, fp) == 3 * n);
        ok = (std::fclose(fp) == 0) && ok;
        if (!ok || std::rename(tmp.c_str(), path) != 0) {
            std::remove(tmp.c_str());
            lg::fail(lg::kRuntime, std::string("writing ") + path + " failed");
        }
    });
}

lg_status lg_read_fp64_sidecar(const char* path, size_t n, const uint32_t* id, const float* x, const float* y,
                               const float* z, double* x64, double* y64, double* z64, uint64_t* step) {
    return guard([&] {
        need(path, "path");
        if (n) { need(id, "id"); need(x, "x"); need(y, "y"); need(z, "z"); need(x64, "x64"); need(y64, "y64");
                 need(z64, "z64"); }
        FILE* fp = std::fopen(path, "rb");
        if (!fp) lg::fail(lg::kRuntime, std::string("cannot read ") + path);
        char magic[8];
        uint64_t hdr[3];
        bool ok = std::fread(magic, 1, 8, fp) == 8 && std::memcmp(magic, "LGF64LO1", 8) == 0 &&
                  std::fread(hdr, 8, 3, fp) == 3 && hdr[0] == n;
        std::vector<uint32_t> fid(((n + 1) & ~size_t(1)) + 2);
        std::vector<double> lo(3 * n);
        const size_t nid = (n + 1) & ~size_t(1);
        ok = ok && std::fread(fid.data(), 4, nid, fp) == nid && (n == 0 || std::fread(lo.data(), 8, 3 * n, fp) == 3 * n);
        std::fclose(fp);
        if (!ok) lg::fail(lg::kRuntime, std::string(path) + ": not an FP64 sidecar for " + std::to_string(n) + " bodies");
        for (size_t i = 0; i < n; ++i)
            if (fid[i] != id[i]) lg::fail(lg::kRuntime, std::string(path) + ": body order differs from the snapshot's");
        for (size_t i = 0; i < n; ++i) {
            x64[i] = static_cast<double>(x[i]) + lo[i];
            y64[i] = static_cast<double>(y[i]) + lo[n + i];
            z64[i] = static_cast<double>(z[i]) + lo[2 * n + i];
        }
        if (step) *step = hdr[1];
    });
}

lg_status lg_size(const lg_engine* e, size_t* n) {
    return guard([&] {
        need(n, "n");
        *n = static_cast<size_t>(eng(const_cast<lg_engine*>(e)).n);
    });
}

lg_status lg_download(lg_engine* e, float* x, float* y, float* z, float* vx, float* vy, float* vz, float* m,
                      uint32_t* id) {
    return guard([&] {
        Engine& E = eng(e);
        if (E.n) { need(x, "x"); need(y, "y"); need(z, "z"); need(vx, "vx"); need(vy, "vy"); need(vz, "vz");
                   need(m, "m"); need(id, "id"); }
        E.download(x, y, z, vx, vy, vz, m, id);
    });
}

lg_status lg_compute_forces(lg_engine* e, const lg_force_params* p, int potential) {
    return guard([&] {
        need(p, "params");
        Engine& E = eng(e);
        E.build_tree(*p);
        E.compute_forces_with(*p, potential != 0, nullptr, 0);
    });
}

lg_status lg_kick(lg_engine* e, double dt) { return guard([&] { eng(e).kick(dt); }); }
lg_status lg_drift(lg_engine* e, double dt) { return guard([&] { eng(e).drift(dt); }); }

lg_status lg_diagnostics(lg_engine* e, lg_diag* out) {
    return guard([&] {
        need(out, "out");
        *out = eng(e).diagnostics();
    });
}

lg_status lg_exact_potential_energy(lg_engine* e, double G, double eps, double* out) {
    return guard([&] {
        need(out, "out");
        *out = eng(e).exact_potential_energy(G, eps);
    });
}

lg_status lg_times(lg_engine* e, lg_phase_times* out) {
    return guard([&] {
        need(out, "out");
        *out = eng(e).get_times();
    });
}

lg_status lg_local_bounds(lg_engine* e, float lo[3], float hi[3]) {
    return guard([&] {
        need(lo, "lo");
        need(hi, "hi");
        eng(e).local_bounds(lo, hi);
    });
}

lg_status lg_build_tree(lg_engine* e, const lg_force_params* p) {
    return guard([&] {
        need(p, "params");
        eng(e).build_tree(*p);
    });
}

lg_status lg_compute_forces_with(lg_engine* e, const lg_force_params* p, int potential, const lg_let_tree* remote,
                                 size_t nremote) {
    return guard([&] {
        need(p, "params");
        eng(e).compute_forces_with(*p, potential != 0, remote, nremote);
    });
}

lg_status lg_export_let(lg_engine* e, const float lo[3], const float hi[3], const lg_force_params* p, size_t* nnodes,
                        size_t* nbodies) {
    return guard([&] {
        need(lo, "lo");
        need(hi, "hi");
        need(p, "params");
        need(nnodes, "nnodes");
        need(nbodies, "nbodies");
        Engine& E = eng(e);
        LG_CK(cudaSetDevice(E.dev));
        lg::let_export(E, lo, hi, *p, nnodes, nbodies);
    });
}

lg_status lg_export_let_read(lg_engine* e, lg_let_node* nodes, float* bx, float* by, float* bz, float* bm) {
    return guard([&] {
        Engine& E = eng(e);
        LG_CK(cudaSetDevice(E.dev));
        lg::let_export_read(E, nodes, bx, by, bz, bm);
    });
}

lg_status lg_block_step(lg_engine* e, const lg_force_params* p, double dt, int max_level, double eta, int steps) {
    return guard([&] {
        need(p, "params");
        eng(e).block_step(*p, dt, max_level, eta, steps);
    });
}

lg_status lg_block_levels(lg_engine* e, uint8_t* levels, size_t n) {
    return guard([&] {
        Engine& E = eng(e);
        LG_CK(cudaSetDevice(E.dev));
        if (n < static_cast<size_t>(E.n)) lg::fail(lg::kArg, "block_levels: output holds fewer than n values");
        if (!E.block_ready) lg::fail(lg::kLogic, "block_levels: no block step since the last upload");
        if (E.n == 0) return;
        LG_CK(cudaMemcpyAsync(levels, E.bodies(E.cur).level, static_cast<size_t>(E.n), cudaMemcpyDeviceToHost, E.stream));
        LG_CK(cudaStreamSynchronize(E.stream));
    });
}

lg_status lg_render(lg_engine* e, const lg_render_options* o, unsigned char* rgb, double* extent_used) {
    return guard([&] {
        need(o, "options");
        need(rgb, "rgb");
        Engine& E = eng(e);
        LG_CK(cudaSetDevice(E.dev));
        lg::render(E, *o, rgb, extent_used);
    });
}

lg_status lg_memory_need(uint64_t n, int method, lg_memory_estimate* out) {
    return guard([&] {
        need(out, "out");
        *out = lg::memory_need(n, method);
    });
}

lg_status lg_device_memory(lg_engine* e, uint64_t* free_bytes, uint64_t* total_bytes) {
    return guard([&] {
        need(free_bytes, "free");
        need(total_bytes, "total");
        Engine& E = eng(e);
        LG_CK(cudaSetDevice(E.dev));
        size_t f = 0, t = 0;
        LG_CK(cudaMemGetInfo(&f, &t));
        *free_bytes = f + E.held_bytes();
        *total_bytes = t;
    });
}

lg_status lg_body_costs(lg_engine* e, float* cost, size_t n, int* valid) {
    return guard([&] {
        need(valid, "valid");
        Engine& E = eng(e);
        if (E.n) need(cost, "cost");
        *valid = E.body_costs(cost, n) ? 1 : 0;
    });
}

lg_status lg_read_accel(lg_engine* e, float* ax, float* ay, float* az, float* pot) {
    return guard([&] {
        Engine& E = eng(e);
        if (E.n) { need(ax, "ax"); need(ay, "ay"); need(az, "az"); }
        E.read_accel(ax, ay, az, pot);
    });
}

lg_status lg_read_pos64(lg_engine* e, double* x, double* y, double* z) {
    return guard([&] {
        Engine& E = eng(e);
        if (E.n) { need(x, "x"); need(y, "y"); need(z, "z"); }
        E.read_pos64(x, y, z);
    });
}

lg_status lg_tree_counts(lg_engine* e, size_t* nodes, size_t* leaves, size_t* groups, int* max_depth) {
    return guard([&] { lg::tree_counts(eng(e), nodes, leaves, groups, max_depth); });
}

lg_status lg_tree_keys(lg_engine* e, uint64_t* keys, size_t n) {
    return guard([&] {
        need(keys, "keys");
        lg::tree_keys(eng(e), keys, n);
    });
}

lg_status lg_tree_nodes(lg_engine* e, uint32_t* lohi_first_nchild, float* moments11, float* geo4, size_t nodes) {
    return guard([&] { lg::tree_nodes(eng(e), lohi_first_nchild, moments11, geo4, nodes); });
}

lg_status lg_tree_groups(lg_engine* e, float* box6, uint32_t* lohi, size_t groups) {
    return guard([&] { lg::tree_groups(eng(e), box6, lohi, groups); });
}

lg_status lg_event_record(lg_engine* e, int slot) {
    return guard([&] {
        Engine& E = eng(e);
        if (slot < 0 || slot >= Engine::kUserEvents) lg::fail(lg::kArg, "event slot out of range");
        LG_CK(cudaEventRecord(E.user_events[slot], E.stream));
    });
}

lg_status lg_event_elapsed(lg_engine* e, int a, int b, float* ms) {
    return guard([&] {
        need(ms, "ms");
        Engine& E = eng(e);
        if (a < 0 || b < 0 || a >= Engine::kUserEvents || b >= Engine::kUserEvents)
            lg::fail(lg::kArg, "event slot out of range");
        LG_CK(cudaEventSynchronize(E.user_events[b]));
        LG_CK(cudaEventElapsedTime(ms, E.user_events[a], E.user_events[b]));
    });
}

lg_status lg_synchronize(lg_engine* e) {
    return guard([&] { LG_CK(cudaStreamSynchronize(eng(e).stream)); });
}

lg_status lg_flush_l2(lg_engine* e) { return guard([&] { eng(e).flush_l2(); }); }

lg_status lg_interaction_split(lg_engine* e, uint64_t* body_pairs, uint64_t* cell_terms) {
    return guard([&] {
        need(body_pairs, "body_pairs");
        need(cell_terms, "cell_terms");
        Engine& E = eng(e);
        *body_pairs = E.last_body_pairs;
        *cell_terms = E.last_cell_terms;
    });
}

lg_status lg_probe_fp32_peak(lg_engine* e, double* tflops) {
    return guard([&] {
        need(tflops, "tflops");
        Engine& E = eng(e);
        LG_CK(cudaSetDevice(E.dev));
        *tflops = lg::probe_fp32_peak(E.stream, E.sms, E.err_word() + 12);
    });
}

lg_status lg_probe_wait_timeout(lg_engine* e, unsigned polls) {
    return guard([&] {
        Engine& E = eng(e);
        if (polls < 1 || polls > (1u << 20)) lg::fail(lg::kArg, "probe_wait_timeout: polls must be in [1, 2^20]");
        LG_CK(cudaSetDevice(E.dev));
        // small[16..19] stays zero here: the flag no one sets.
        LG_CK(cudaMemsetAsync(E.small.as<char>(), 0, 32, E.stream));
        lg::probe_waits(E.stream, polls, E.small.as<unsigned>() + 4 + 0, E.err_word());
        ++E.launches;
        LG_CK(cudaMemcpyAsync(E.pinned_small, E.small.as<char>(), 4, cudaMemcpyDeviceToHost, E.stream));
        LG_CK(cudaStreamSynchronize(E.stream));
        E.check_device_errors("wait probe");
    });
}

lg_status lg_adjoint_forward(lg_engine* e, const lg_force_params* p, double dt, int steps, int checkpoint_every) {
    return guard([&] {
        need(p, "params");
        Engine& E = eng(e);
        lg::adjoint_forward(E, *E.adjoint, *p, dt, steps, checkpoint_every);
    });
}

lg_status lg_adjoint_backward(lg_engine* e, const double* tx, const double* ty, const double* tz, double* loss,
                              double* gx, double* gy, double* gz, double* gvx, double* gvy, double* gvz, double* gm) {
    return guard([&] {
        need(tx, "target_x");
        need(ty, "target_y");
        need(tz, "target_z");
        Engine& E = eng(e);
        const double L = lg::adjoint_backward(E, *E.adjoint, tx, ty, tz, gx, gy, gz, gvx, gvy, gvz, gm, false);
        if (loss) *loss = L;
    });
}

lg_status lg_adjoint_backward_seeded(lg_engine* e, const double* dldx, const double* dldy, const double* dldz,
                                     double* gx, double* gy, double* gz, double* gvx, double* gvy, double* gvz,
                                     double* gm) {
    return guard([&] {
        need(dldx, "dldx");
        need(dldy, "dldy");
        need(dldz, "dldz");
        Engine& E = eng(e);
        lg::adjoint_backward(E, *E.adjoint, dldx, dldy, dldz, gx, gy, gz, gvx, gvy, gvz, gm, true);
    });
}

lg_status lg_host_alloc(size_t bytes, void** out) {
    return guard([&] {
        need(out, "out");
        *out = nullptr;
        LG_CK(cudaMallocHost(out, bytes ? bytes : 1));
    });
}

lg_status lg_host_free(void* p) {
    return guard([&] {
        if (p) LG_CK(cudaFreeHost(p));
    });
}

lg_status lg_launch_count(const lg_engine* e, uint64_t* count) {
    return guard([&] {
        need(count, "count");
        *count = eng(const_cast<lg_engine*>(e)).launches;
    });
}

}  // extern "C"
