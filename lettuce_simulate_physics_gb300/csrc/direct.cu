// Direct summation (the reference's direct<POT>, src/cpu_backend.cpp:353-392, and direct_kernel,
// src/cuda_backend.cu:301-350), GB300 form:
//  - each thread keeps IPT i-bodies in registers;
//  - j-bodies stream through shared memory in tiles of TL (256, or 128) float4 (hi x, hi y, hi z, m) plus the
//    float4 low parts, fetched by the TMA engine (cp.async.bulk, mbarrier completion) into two
//    stages, so the copy of tile t+2 overlaps the arithmetic on tile t;
//  - each tile is converted once per block to coordinates relative to the block origin o (the
//    first i-body): (x_hi - o_hi) + (x_lo - o_lo) in FP32, so close pairs keep the FP64
//    separation; the converted tile is struct-of-arrays, so j-bodies k, k+1 load as one float2
//    and the inner loop evaluates both with packed f32x2 instructions (per two pairs: 3 FADD2,
//    3 FFMA2, 2 MUFU.RSQ, 3 FMUL2, 3 FFMA2 -- half the issue slots of the scalar loop);
//  - per-tile partial sums are added to the running sums with Kahan compensation;
//  - small N splits the j range over blockIdx.y (split-j); the slices' partials are summed in a
//    fixed order by a second kernel, so results do not depend on scheduling.
// Self interaction: with eps > 0 the self pair has d = 0 exactly (same relative coordinates), so
// it adds nothing to a; for the potential it is excluded by index (its mass taken as zero in the
// tiles that hold the block's own bodies). With eps == 0 the r2 > 0 guard drops self and
// coincident pairs, as the reference does.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "engine.cuh"

namespace lg {

namespace {

#ifndef LG_DIRECT_UNROLL
#define LG_DIRECT_UNROLL 2  // j-pair iterations unrolled in the inner loop (measured best on GB300)
#endif
#ifndef LG_DIRECT_MINB
#define LG_DIRECT_MINB 1    // resident blocks per SM the register budget is sized for
#endif
constexpr int DUNROLL = LG_DIRECT_UNROLL;
constexpr int DBS = 256;   // threads per block
constexpr int TILE = 256;  // j-bodies per stage (default; 128 is the other compiled shape)

template <int TL>
struct alignas(16) DirectSmem {
    float4 raw_hm[2][TL];
    float4 raw_lo[2][TL];
    float rx[2][TL], ry[2][TL], rz[2][TL], rm[2][TL];
    uint64_t bar[2];
};

// One block's work: i-bodies [base, base + DBS * IPT) clipped to iend, against j-bodies [j0, j1).
// write_final: out[i] = G-scaled sums; otherwise out[i] = unscaled partial sums (out points at the
// slice's row).
template <int IPT, int TL, bool POT, bool EPS0>
__device__ __forceinline__ void direct_block(DirectSmem<TL>& sm, const float4* __restrict__ hm,
                                             const float4* __restrict__ lo, int base, int iend, int j0, int j1,
                                             float G, float e2, float4* __restrict__ out, bool write_final,
                                             unsigned* err, float* __restrict__ cost = nullptr) {
    const int tid = threadIdx.x;
    const int ntiles = (j1 - j0 + TL - 1) / TL;
    const int n = iend;

    // Block origin: the first i-body of the block.
    const float4 oh = hm[base];
    const float4 ol = lo[base];

    float xi[IPT], yi[IPT], zi[IPT];
    float sx[IPT], sy[IPT], sz[IPT], sp[IPT], cx[IPT], cy[IPT], cz[IPT], cp[IPT];
#pragma unroll
    for (int u = 0; u < IPT; ++u) {
        const int i = min(base + u * DBS + tid, n - 1);
        const float4 h = hm[i], l = lo[i];
        xi[u] = (h.x - oh.x) + (l.x - ol.x);
        yi[u] = (h.y - oh.y) + (l.y - ol.y);
        zi[u] = (h.z - oh.z) + (l.z - ol.z);
        sx[u] = sy[u] = sz[u] = sp[u] = 0.f;
        cx[u] = cy[u] = cz[u] = cp[u] = 0.f;
    }

    f2x XI[IPT], YI[IPT], ZI[IPT];
#pragma unroll
    for (int u = 0; u < IPT; ++u) {
        XI[u] = f2_bcast(xi[u]);
        YI[u] = f2_bcast(yi[u]);
        ZI[u] = f2_bcast(zi[u]);
    }
    const f2x E2 = f2_bcast(e2);

    if (tid == 0) {
        mbar_init(&sm.bar[0], 1);
        mbar_init(&sm.bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    auto issue = [&](int t) {
        const int jt = j0 + t * TL;
        const unsigned cnt = static_cast<unsigned>(min(TL, j1 - jt));
        const int buf = t & 1;
        mbar_arrive_expect_tx(&sm.bar[buf], 2u * cnt * 16u);
        bulk_g2s(sm.raw_hm[buf], hm + jt, cnt * 16u, &sm.bar[buf]);
        bulk_g2s(sm.raw_lo[buf], lo + jt, cnt * 16u, &sm.bar[buf]);
    };
    if (tid == 0) {
        if (ntiles > 0) issue(0);
        if (ntiles > 1) issue(1);
    }

    bool failed = false;
    int t = 0;
    for (; t < ntiles; ++t) {
        const int buf = t & 1;
        const unsigned parity = (t >> 1) & 1;
        const bool ok = mbar_wait_bounded(&sm.bar[buf], parity);
        const int cnt = min(TL, j1 - (j0 + t * TL));
        const int cnt8 = (cnt + 7) & ~7;
        if (ok) {
            for (int k = tid; k < cnt8; k += DBS) {
                if (k < cnt) {
                    const float4 h = sm.raw_hm[buf][k], l = sm.raw_lo[buf][k];
                    sm.rx[buf][k] = (h.x - oh.x) + (l.x - ol.x);
                    sm.ry[buf][k] = (h.y - oh.y) + (l.y - ol.y);
                    sm.rz[buf][k] = (h.z - oh.z) + (l.z - ol.z);
                    sm.rm[buf][k] = h.w;
                } else {
                    // A far, massless body: pads the tile and adds exactly zero.
                    sm.rx[buf][k] = 1e18f;
                    sm.ry[buf][k] = 1e18f;
                    sm.rz[buf][k] = 1e18f;
                    sm.rm[buf][k] = 0.f;
                }
            }
        }
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        if (tid == 0 && t + 2 < ntiles) {
            fence_proxy_async_smem();
            issue(t + 2);
        }
        f2x px[IPT], py[IPT], pz[IPT], pp[IPT];
#pragma unroll
        for (int u = 0; u < IPT; ++u) px[u] = py[u] = pz[u] = pp[u] = 0ull;
        const float* rx = sm.rx[buf];
        const float* ry = sm.ry[buf];
        const float* rz = sm.rz[buf];
        const float* rm = sm.rm[buf];
        // Pairs k, k + 1 of the tile. With the potential, the tiles that hold the block's own
        // bodies take the self pair out by index (its mass half set to zero), as the reference's
        // direct kernel does: no m/eps is added and subtracted, so phi keeps its low bits.
        const int jt0 = j0 + t * TL;
        auto tile_pairs = [&](auto masked) {
            constexpr bool MASK = decltype(masked)::value;
#pragma unroll DUNROLL
            for (int k = 0; k < cnt8; k += 2) {
                const f2x X = *reinterpret_cast<const f2x*>(rx + k), Y = *reinterpret_cast<const f2x*>(ry + k);
                const f2x Z = *reinterpret_cast<const f2x*>(rz + k), M = *reinterpret_cast<const f2x*>(rm + k);
#pragma unroll
                for (int u = 0; u < IPT; ++u) {
                    f2x Mu = M;
                    if (MASK) {
                        const unsigned off = static_cast<unsigned>(base + u * DBS + tid - (jt0 + k));
                        if (off <= 1u) Mu = f2_mul(M, off == 0 ? f2_pack(0.f, 1.f) : f2_pack(1.f, 0.f));
                    }
                    const f2x dx = f2_sub(X, XI[u]), dy = f2_sub(Y, YI[u]), dz = f2_sub(Z, ZI[u]);
                    const f2x r2 = f2_fma(dx, dx, f2_fma(dy, dy, f2_fma(dz, dz, E2)));
                    float r2a, r2b;
                    f2_unpack(r2, r2a, r2b);
                    float ia = rsqrt_mufu(r2a), ib = rsqrt_mufu(r2b);
                    if (EPS0) {
                        ia = r2a > 0.f ? ia : 0.f;
                        ib = r2b > 0.f ? ib : 0.f;
                    }
                    const f2x inv = f2_pack(ia, ib);
                    const f2x mi = f2_mul(Mu, inv);  // the self pair (d = 0) adds nothing to a
                    const f2x f = f2_mul(mi, f2_mul(inv, inv));
                    px[u] = f2_fma(f, dx, px[u]);
                    py[u] = f2_fma(f, dy, py[u]);
                    pz[u] = f2_fma(f, dz, pz[u]);
                    if (POT) pp[u] = f2_add(pp[u], mi);
                }
            }
        };
        if (POT && jt0 < base + DBS * IPT && jt0 + cnt > base) tile_pairs(std::true_type{});
        else tile_pairs(std::false_type{});
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            kahan_add(sx[u], cx[u], f2_sum(px[u]));
            kahan_add(sy[u], cy[u], f2_sum(py[u]));
            kahan_add(sz[u], cz[u], f2_sum(pz[u]));
            if (POT) kahan_add(sp[u], cp[u], f2_sum(pp[u]));
        }
    }
    if (failed) {
        if (tid == 0) {
            atomicOr(err, kErrWaitTimeout);
            // Let any copy still in flight land before the block's shared memory is released.
            for (int u = t; u < min(ntiles, t + 2); ++u) mbar_wait_bounded(&sm.bar[u & 1], (u >> 1) & 1);
        }
        return;
    }
#pragma unroll
    for (int u = 0; u < IPT; ++u) {
        const int i = base + u * DBS + tid;
        if (i >= n) continue;
        const float p = sp[u] - cp[u];
        if (write_final) {
            out[i] = make_float4(G * (sx[u] - cx[u]), G * (sy[u] - cy[u]), G * (sz[u] - cz[u]), POT ? -G * p : 0.f);
            if (cost) cost[i] = static_cast<float>(n - 1);  // interactions: every other body
        } else
            out[i] = make_float4(sx[u] - cx[u], sy[u] - cy[u], sz[u] - cz[u], POT ? p : 0.f);
    }
}

template <int IPT, int TL, bool POT, bool EPS0>
__global__ void __launch_bounds__(DBS, LG_DIRECT_MINB) k_direct(const float4* __restrict__ hm, const float4* __restrict__ lo, int n,
                                                int jslice, float G, float e2, float4* __restrict__ out, int write_final,
                                                unsigned* err, float* cost) {
    __shared__ DirectSmem<TL> sm;
    const int j0 = blockIdx.y * jslice;
    direct_block<IPT, TL, POT, EPS0>(sm, hm, lo, blockIdx.x * (DBS * IPT), n, j0, min(n, j0 + jslice), G, e2,
                                 write_final ? out : out + static_cast<size_t>(blockIdx.y) * n, write_final != 0, err,
                                 cost);
}

// Many independent systems in one launch: block b takes work item b (an i-tile of one system
// against all of that system's bodies), with the system's own softening.
template <int IPT, int TL, bool POT, bool EPS0>
__global__ void __launch_bounds__(DBS, LG_DIRECT_MINB) k_direct_batch(const float4* __restrict__ hm, const float4* __restrict__ lo,
                                                      const DirectWork* __restrict__ work, float G,
                                                      float4* __restrict__ acc, unsigned* err) {
    __shared__ DirectSmem<TL> sm;
    const DirectWork w = work[blockIdx.x];
    direct_block<IPT, TL, POT, EPS0>(sm, hm, lo, w.base, w.iend, w.j0, w.j1, G, w.e2, acc, true, err);
}

// Sums the split-j partials in slice order (Kahan) and scales by G.
__global__ void k_direct_reduce(const float4* __restrict__ partial, int n, int slices, float G, float4* __restrict__ acc,
                                float* __restrict__ cost) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (cost) cost[i] = static_cast<float>(n - 1);
    float s[4] = {0, 0, 0, 0}, c[4] = {0, 0, 0, 0};
    for (int k = 0; k < slices; ++k) {
        const float4 p = partial[static_cast<size_t>(k) * n + i];
        kahan_add(s[0], c[0], p.x);
        kahan_add(s[1], c[1], p.y);
        kahan_add(s[2], c[2], p.z);
        kahan_add(s[3], c[3], p.w);
    }
    acc[i] = make_float4(G * (s[0] - c[0]), G * (s[1] - c[1]), G * (s[2] - c[2]), -G * (s[3] - c[3]));
}

template <int IPT, int TL>
void launch_ipt(const BodyArrays b, int n, float G, float e2, bool pot, bool eps0, int jslice, int slices, float4* out,
                int write_final, unsigned* err, float* cost, cudaStream_t s) {
    dim3 grid((n + DBS * IPT - 1) / (DBS * IPT), slices);
    if (pot) {
        if (eps0) k_direct<IPT, TL, true, true><<<grid, DBS, 0, s>>>(b.hm, b.lo, n, jslice, G, e2, out, write_final, err, cost);
        else k_direct<IPT, TL, true, false><<<grid, DBS, 0, s>>>(b.hm, b.lo, n, jslice, G, e2, out, write_final, err, cost);
    } else {
        if (eps0) k_direct<IPT, TL, false, true><<<grid, DBS, 0, s>>>(b.hm, b.lo, n, jslice, G, e2, out, write_final, err, cost);
        else k_direct<IPT, TL, false, false><<<grid, DBS, 0, s>>>(b.hm, b.lo, n, jslice, G, e2, out, write_final, err, cost);
    }
    LG_LAUNCHED();
}

// Resident blocks per SM of the i-bodies-per-thread variant (no potential), from the occupancy
// calculator; cached per variant.
int blocks_per_sm(int ipt) {
    static int cache[9] = {};
    const int k = ipt == 1 ? 1 : (ipt == 2 ? 2 : (ipt == 8 ? 8 : 4));
    if (!cache[k]) {
        int per = 0;
        cudaError_t e = cudaSuccess;
        switch (k) {
            case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_direct<1, TILE, false, false>, DBS, 0); break;
            case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_direct<2, TILE, false, false>, DBS, 0); break;
            case 8: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_direct<8, TILE, false, false>, DBS, 0); break;
            default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_direct<4, TILE, false, false>, DBS, 0); break;
        }
        if (e != cudaSuccess) {
            cudaGetLastError();
            per = 2;
        }
        cache[k] = per < 1 ? 1 : per;
    }
    return cache[k];
}

}  // namespace

// Default shape: i-bodies per thread by size, and a split-j count that makes the grid a whole
// number of waves (blocks resident at once = SMs x blocks per SM), so no partial wave idles SMs.
DirectShape default_direct_shape(int n, int sms) {
    DirectShape sh;
    sh.ipt = n >= 8 * 1024 ? 4 : (n >= 2048 ? 2 : 1);
    sh.tile = TILE;
    const int iblocks = (n + DBS * sh.ipt - 1) / (DBS * sh.ipt);
    const int wave = blocks_per_sm(sh.ipt) * sms;
    const int max_slices = std::max(1, n / 128);
    int best = 1;
    double best_eff = 0;
    for (int waves = 1; waves <= 8; ++waves) {
        const int slices = std::min(max_slices, std::max(1, (waves * wave + iblocks / 2) / iblocks));
        const int blocks = iblocks * slices;
        const double eff = static_cast<double>(blocks) / (static_cast<double>((blocks + wave - 1) / wave) * wave);
        // Prefer full waves; among equals, fewer slices (less partial-sum traffic).
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = slices;
        }
        if (eff > 0.97) break;
    }
    sh.slices = iblocks * 1 >= wave ? 1 : best;
    return sh;
}

void launch_direct(const BodyArrays b, int n, float G, float e2, bool potential, bool eps0, const DirectShape& shape,
                   float4* acc, float4* partial, unsigned* err, cudaStream_t s, float* cost) {
    if (n <= 0) return;
    int slices = shape.slices < 1 ? 1 : shape.slices;
    // Slices are whole 16-byte bodies of any length; tiles inside a slice may be partial.
    int jslice = (n + slices - 1) / slices;
    slices = (n + jslice - 1) / jslice;
    const bool final_out = slices == 1;
    float4* out = final_out ? acc : partial;
    float* c = final_out ? cost : nullptr;
    if (shape.tile == 128) {  // the other compiled tile shape (1, 2 or 4 i-bodies per thread)
        switch (shape.ipt) {
            case 1: launch_ipt<1, 128>(b, n, G, e2, potential, eps0, jslice, slices, out, final_out, err, c, s); break;
            case 2: launch_ipt<2, 128>(b, n, G, e2, potential, eps0, jslice, slices, out, final_out, err, c, s); break;
            default: launch_ipt<4, 128>(b, n, G, e2, potential, eps0, jslice, slices, out, final_out, err, c, s); break;
        }
    } else {
        switch (shape.ipt) {
            case 1: launch_ipt<1, TILE>(b, n, G, e2, potential, eps0, jslice, slices, out, final_out, err, c, s); break;
            case 2: launch_ipt<2, TILE>(b, n, G, e2, potential, eps0, jslice, slices, out, final_out, err, c, s); break;
            case 8: launch_ipt<8, TILE>(b, n, G, e2, potential, eps0, jslice, slices, out, final_out, err, c, s); break;
            default: launch_ipt<4, TILE>(b, n, G, e2, potential, eps0, jslice, slices, out, final_out, err, c, s); break;
        }
    }
    if (!final_out) {
        k_direct_reduce<<<(n + 255) / 256, 256, 0, s>>>(partial, n, slices, G, acc, cost);
        LG_LAUNCHED();
    }
}

namespace {
template <int IPT, int TL>
void launch_batch_ipt(const BodyArrays b, const DirectWork* work, int nwork, float G, bool pot, bool eps0, float4* acc,
                      unsigned* err, cudaStream_t s) {
    if (pot) {
        if (eps0) k_direct_batch<IPT, TL, true, true><<<nwork, DBS, 0, s>>>(b.hm, b.lo, work, G, acc, err);
        else k_direct_batch<IPT, TL, true, false><<<nwork, DBS, 0, s>>>(b.hm, b.lo, work, G, acc, err);
    } else {
        if (eps0) k_direct_batch<IPT, TL, false, true><<<nwork, DBS, 0, s>>>(b.hm, b.lo, work, G, acc, err);
        else k_direct_batch<IPT, TL, false, false><<<nwork, DBS, 0, s>>>(b.hm, b.lo, work, G, acc, err);
    }
    LG_LAUNCHED();
}
}  // namespace

int direct_block_bodies(int ipt) { return DBS * ipt; }

void launch_direct_batch(const BodyArrays b, const DirectWork* work, int nwork, int ipt, int tile, float G,
                         bool potential, bool eps0, float4* acc, unsigned* err, cudaStream_t s) {
    if (nwork <= 0) return;
    if (tile == 128) {
        switch (ipt) {
            case 1: launch_batch_ipt<1, 128>(b, work, nwork, G, potential, eps0, acc, err, s); break;
            case 2: launch_batch_ipt<2, 128>(b, work, nwork, G, potential, eps0, acc, err, s); break;
            default: launch_batch_ipt<4, 128>(b, work, nwork, G, potential, eps0, acc, err, s); break;
        }
    } else {
        switch (ipt) {
            case 1: launch_batch_ipt<1, TILE>(b, work, nwork, G, potential, eps0, acc, err, s); break;
            case 2: launch_batch_ipt<2, TILE>(b, work, nwork, G, potential, eps0, acc, err, s); break;
            case 8: launch_batch_ipt<8, TILE>(b, work, nwork, G, potential, eps0, acc, err, s); break;
            default: launch_batch_ipt<4, TILE>(b, work, nwork, G, potential, eps0, acc, err, s); break;
        }
    }
}


// ---- Entry point without device allocation ---------------------------------------------------
// Some callers cannot call cudaMalloc at the point where they need forces: a code that owns all
// device memory through its own fixed arena, or a time-stepping loop that must not hit
// cudaMalloc's implicit device synchronisation between steps. lg_direct_forces_noalloc serves
// them: the caller passes device inputs and outputs, and the split-j scratch lives in the static
// array below instead of an engine buffer.
namespace {

constexpr size_t kNoAllocStatusBytes = 256;
constexpr size_t kNoAllocPartials = size_t(1) << 20;  // float4 entries (16 MiB)
constexpr int kNoAllocMaxN = 1 << 20;

// Status words, then split-j partial sums. Part of the library image: every GPU that loads the
// library holds these 16 MiB until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocStatusBytes + kNoAllocPartials * 16];

// Device address of g_noalloc_scratch in the current context. The host-side name is only a
// stand-in; kernels must be given this address. It is looked up on every call (a table lookup once
// the module is loaded), so a context torn down and recreated (cudaDeviceReset) gets the new address.
unsigned char* noalloc_scratch() {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(kRuntime, std::string("lg_direct_forces_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
    }
    return static_cast<unsigned char*>(p);
}

// The kernels stage positions with bulk copies, which need 16-byte-aligned global addresses on
// this device: reject anything else on the host, before any launch.
void noalloc_check_pointer(const void* p, const char* what, int dev) {
    if (reinterpret_cast<uintptr_t>(p) & 15u)
        fail(kArg, std::string("lg_direct_forces_noalloc: ") + what + " is not 16-byte aligned");
    cudaPointerAttributes a{};
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(kArg, std::string("lg_direct_forces_noalloc: ") + what + " is not a CUDA pointer: " + cudaGetErrorString(e));
    }
    if ((a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) || a.device != dev)
        fail(kArg, std::string("lg_direct_forces_noalloc: ") + what + " is not device memory of the current device " +
                       std::to_string(dev));
}

}  // namespace

}  // namespace lg

extern "C" lg_status lg_direct_forces_noalloc(const void* posm, const void* poslo, int n, double G, double eps,
                                              int potential, void* acc, void* stream) {
    try {
        if (n < 0 || n > lg::kNoAllocMaxN)
            lg::fail(lg::kArg, "lg_direct_forces_noalloc: n = " + std::to_string(n) + " is outside [0, " +
                                   std::to_string(lg::kNoAllocMaxN) + "], the size its static scratch serves");
        if (n > 0 && (!posm || !poslo || !acc)) lg::fail(lg::kArg, "lg_direct_forces_noalloc: null device pointer");
        if (n == 0) {
            lg::g_last_error.clear();
            return LG_OK;
        }
        int dev = 0;
        LG_CK(cudaGetDevice(&dev));
        lg::noalloc_check_pointer(posm, "posm", dev);
        lg::noalloc_check_pointer(poslo, "poslo", dev);
        lg::noalloc_check_pointer(acc, "acc", dev);
        int sms = 0;
        LG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        unsigned char* base = lg::noalloc_scratch();
        unsigned* err = reinterpret_cast<unsigned*>(base);
        float4* partial = reinterpret_cast<float4*>(base + lg::kNoAllocStatusBytes);
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        lg::DirectShape sh = lg::default_direct_shape(n, sms);
        // The engine's launch-shape override "ipt,slices" applies here too.
        if (const char* d = std::getenv("LETTUCE_GB300_DIRECT")) {
            int ipt = 0, slices = 0;
            if (std::sscanf(d, "%d,%d", &ipt, &slices) != 2 || (ipt != 1 && ipt != 2 && ipt != 4 && ipt != 8) ||
                slices < 1)
                lg::fail(lg::kArg, std::string("LETTUCE_GB300_DIRECT must be 'ipt,slices' with ipt in {1,2,4,8}, not '") +
                                       d + "'");
            sh.ipt = ipt;
            sh.slices = slices;
        }
        // Split-j partial sums beyond the static array's size: fewer slices.
        const long long cap = static_cast<long long>(lg::kNoAllocPartials) / n;
        if (sh.slices > cap) sh.slices = static_cast<int>(cap < 1 ? 1 : cap);
        lg::BodyArrays b;
        b.hm = const_cast<float4*>(static_cast<const float4*>(posm));
        b.lo = const_cast<float4*>(static_cast<const float4*>(poslo));
        const float e2 = static_cast<float>(eps * eps);
        const bool eps0 = !(e2 >= 1.17549435e-38f);
        // The array keeps the previous call's contents: the status word must start at zero; the
        // partial sums are overwritten before they are read.
        LG_CK(cudaMemsetAsync(err, 0, sizeof(unsigned), s));
        lg::launch_direct(b, n, static_cast<float>(G), e2, potential != 0, eps0, sh, static_cast<float4*>(acc), partial,
                          err, s);
        unsigned h_err = 0;
        LG_CK(cudaMemcpyAsync(&h_err, err, sizeof h_err, cudaMemcpyDeviceToHost, s));
        LG_CK(cudaStreamSynchronize(s));
        if (h_err) lg::fail(lg::kRuntime, "lg_direct_forces_noalloc: device wait timed out; accelerations are invalid");
        lg::g_last_error.clear();
        return LG_OK;
    } catch (const lg::Error& ex) {
        lg::g_last_error = ex.what();
        return static_cast<lg_status>(ex.status);
    } catch (const std::exception& ex) {
        lg::g_last_error = ex.what();
        return LG_ERR_RUNTIME;
    }
}

