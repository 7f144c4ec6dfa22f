// Block (hierarchical) time steps: every body advances with its own power-of-two step
// dt_k = dt / 2^k, k = 0 .. max_level, so that close encounters take small steps without forcing
// them on every body. No counterpart in the reference (it lists block time steps as not done yet,
// docs/design.md:70-71); this is the next physics capability on the engine's own kernels.
//
// Scheme (kick-drift-kick with synchronised drifts). One step dt is 2^K substeps of dt / 2^K. At
// substep boundary s the bodies whose step starts there (level k with s a multiple of 2^(K-k))
// receive the opening half kick dt_k / 2 with the acceleration of their last force evaluation;
// every body drifts by dt / 2^K (FP64); at boundary s + 1 the forces of the bodies whose step ends
// there are evaluated (the tree is rebuilt over all bodies; walk passes with no such body are
// skipped) and those bodies receive the closing half kick and a new level:
//   dt_i = eta sqrt(eps / |a_i|),  k_i = the smallest k with dt / 2^k <= dt_i, within [kmin, K],
// where kmin is the coarsest level whose step boundary falls on this time (a body may always move
// to a finer level; to a coarser one only where the coarser step starts). The acceleration of a
// body is used only at its own step boundaries, where it has just been evaluated.
#include <cmath>

#include "engine.cuh"

namespace lg {

namespace {

constexpr int BBS = 256;
inline int grid_for(long long n, int bs) { return static_cast<int>((n + bs - 1) / bs); }

// v += a dt_level / 2 for the bodies whose level is >= kmin.
__global__ void k_block_kick(BodyArrays b, const float4* __restrict__ acc, double dt, int kmin, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = b.level[i];
    if (k < kmin) return;
    const float h = static_cast<float>(0.5 * ldexp(dt, -k));
    const float4 a = acc[i];
    b.vx[i] = __fmaf_rn(a.x, h, b.vx[i]);
    b.vy[i] = __fmaf_rn(a.y, h, b.vy[i]);
    b.vz[i] = __fmaf_rn(a.z, h, b.vz[i]);
}

// The smallest k with dt / 2^k <= eta sqrt(eps / |a|), within [kmin, kmax]. Computed exactly from
// r = (dt / eta) sqrt(|a| / eps) by frexp: k = ceil(log2 r).
__device__ __forceinline__ int level_for(float4 a, double dt, double eta, double eps, int kmin, int kmax) {
    const double ax = a.x, ay = a.y, az = a.z;
    const double am = sqrt(ax * ax + ay * ay + az * az);
    if (!(am > 0)) return kmin;
    const double r = dt / eta * sqrt(am / eps);
    if (!(r > 1)) return kmin;
    int e = 0;
    const double f = frexp(r, &e);  // r = f 2^e, f in [0.5, 1)
    int k = f == 0.5 ? e - 1 : e;
    return k < kmin ? kmin : (k > kmax ? kmax : k);
}

__global__ void k_block_levels(BodyArrays b, const float4* __restrict__ acc, double dt, double eta, double eps,
                               int kmin, int kmax, int all, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!all && b.level[i] < kmin) return;
    b.level[i] = static_cast<uint8_t>(level_for(acc[i], dt, eta, eps, kmin, kmax));
}

int trailing_zeros(unsigned v) {
    int t = 0;
    while (v && !(v & 1u)) {
        v >>= 1;
        ++t;
    }
    return t;
}

}  // namespace

void Engine::block_step(const lg_force_params& p, double dt, int K, double eta, int steps) {
    LG_CK(cudaSetDevice(dev));
    if (!(dt > 0) || !(eta > 0)) fail(kArg, "block_step: dt and eta must be positive");
    if (K < 0 || K > 20) fail(kArg, "block_step: max_level must be in [0, 20]");
    if (steps < 0) fail(kArg, "block_step: steps < 0");
    if (n == 0 || steps == 0) return;
    const double eps = p.eps > 0 ? p.eps : 1e-30;
    auto forces = [&](int kmin) {
        walk_kmin = p.method == LG_TREE ? kmin : -1;
        try {
            build_tree(p);
            compute_forces_with(p, false, nullptr, 0);
        } catch (...) {
            walk_kmin = -1;
            throw;
        }
        walk_kmin = -1;
    };
    if (!block_ready) {
        // Forces of every body, then every body's level.
        forces(0);
        k_block_levels<<<grid_for(n, BBS), BBS, 0, stream>>>(bodies(cur), acc.as<float4>(), dt, eta, eps, 0, K, 1, n);
        LG_LAUNCHED();
        ++launches;
        block_ready = true;
    }
    const unsigned sub = 1u << K;
    const double ds = ldexp(dt, -K);
    for (int st = 0; st < steps; ++st) {
        for (unsigned s = 0; s < sub; ++s) {
            const int kopen = s == 0 ? 0 : K - trailing_zeros(s);
            k_block_kick<<<grid_for(n, BBS), BBS, 0, stream>>>(bodies(cur), acc.as<float4>(), dt, kopen, n);
            LG_LAUNCHED();
            ++launches;
            drift(ds);
            const unsigned s1 = s + 1;
            const int kclose = s1 == sub ? 0 : K - trailing_zeros(s1);
            forces(kclose);
            k_block_kick<<<grid_for(n, BBS), BBS, 0, stream>>>(bodies(cur), acc.as<float4>(), dt, kclose, n);
            LG_LAUNCHED();
            k_block_levels<<<grid_for(n, BBS), BBS, 0, stream>>>(bodies(cur), acc.as<float4>(), dt, eta, eps, kclose, K,
                                                                0, n);
            LG_LAUNCHED();
            launches += 2;
        }
    }
    LG_CK(cudaStreamSynchronize(stream));
    // The accelerations are those of each body's last evaluation, not one common time.
    has_pe = false;
    acc_ok = true;
}

}  // namespace lg
