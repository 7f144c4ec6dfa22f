// Integration and reduction kernels: upload widening, download rounding, FP32 kick, FP64 drift,
// FP64 diagnostics and bounds, the exact FP64 potential energy, and utility kernels.
#include <algorithm>

#include "lg_engine.cuh"

namespace lg {

namespace {

constexpr int BS = 256;

inline int grid_for(long long n, int bs) { return static_cast<int>((n + bs - 1) / bs); }

// hi = nearest float, lo = nearest float to the remainder (exact in double).
__device__ __forceinline__ void split_hilo(double v, float& hi, float& lo) {
    hi = __double2float_rn(v);
    lo = __double2float_rn(__dsub_rn(v, static_cast<double>(hi)));
}

__device__ __forceinline__ void store_hilo(BodyArrays b, int i, double x, double y, double z, float m) {
    float hx, hy, hz, lx, ly, lz;
    split_hilo(x, hx, lx);
    split_hilo(y, hy, ly);
    split_hilo(z, hz, lz);
    b.hm[i] = make_float4(hx, hy, hz, m);
    b.lo[i] = make_float4(lx, ly, lz, 0.f);
}

// upload: float positions widen exactly to double (src/backend.hpp:95 semantics, FP64 inside).
__global__ void k_widen(const float* __restrict__ x, const float* __restrict__ y, const float* __restrict__ z,
                        const float* __restrict__ m, BodyArrays b, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double px = x[i], py = y[i], pz = z[i];
    b.x[i] = px;
    b.y[i] = py;
    b.z[i] = pz;
    store_hilo(b, i, px, py, pz, m[i]);
}

// hi/lo split and masses into hm from the FP64 positions already in b (FP64 upload).
__global__ void k_refresh_hilo(BodyArrays b, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    store_hilo(b, i, b.x[i], b.y[i], b.z[i], b.m[i]);
}

__global__ void k_round_pos(const BodyArrays b, float* __restrict__ x, float* __restrict__ y, float* __restrict__ z,
                            int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = __double2float_rn(b.x[i]);
    y[i] = __double2float_rn(b.y[i]);
    z[i] = __double2float_rn(b.z[i]);
}

// v += a dt in FP32 (src/cpu_backend.cpp:279-290).
__global__ void k_kick(BodyArrays b, const float4* __restrict__ acc, float dt, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = acc[i];
    b.vx[i] = __fmaf_rn(a.x, dt, b.vx[i]);
    b.vy[i] = __fmaf_rn(a.y, dt, b.vy[i]);
    b.vz[i] = __fmaf_rn(a.z, dt, b.vz[i]);
}

// x += v dt in FP64, then the hi/lo split the force kernels read.
__global__ void k_drift(BodyArrays b, double dt, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double px = __fma_rn(static_cast<double>(b.vx[i]), dt, b.x[i]);
    double py = __fma_rn(static_cast<double>(b.vy[i]), dt, b.y[i]);
    double pz = __fma_rn(static_cast<double>(b.vz[i]), dt, b.z[i]);
    b.x[i] = px;
    b.y[i] = py;
    b.z[i] = pz;
    store_hilo(b, i, px, py, pz, b.m[i]);
}

// Ensemble step opening: v += a (dt/2), then x += v dt -- the kick and drift kernels' arithmetic in
// one pass over the bodies.
__global__ void k_kick_drift(BodyArrays b, const float4* __restrict__ acc, float hdt, double dt, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = acc[i];
    const float vx = __fmaf_rn(a.x, hdt, b.vx[i]);
    const float vy = __fmaf_rn(a.y, hdt, b.vy[i]);
    const float vz = __fmaf_rn(a.z, hdt, b.vz[i]);
    b.vx[i] = vx;
    b.vy[i] = vy;
    b.vz[i] = vz;
    const double px = __fma_rn(static_cast<double>(vx), dt, b.x[i]);
    const double py = __fma_rn(static_cast<double>(vy), dt, b.y[i]);
    const double pz = __fma_rn(static_cast<double>(vz), dt, b.z[i]);
    b.x[i] = px;
    b.y[i] = py;
    b.z[i] = pz;
    store_hilo(b, i, px, py, pz, b.m[i]);
}

constexpr int NDIAG = 12;

// Block-level FP64 sum of NDIAG values in a fixed order (warp shuffles, then warps in order).
__device__ void block_sum(double (&v)[NDIAG], double* sh /* [BS/32][NDIAG] */) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NDIAG; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NDIAG; ++k) sh[w * NDIAG + k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < NDIAG; ++k) {
            double s = 0;
            for (int u = 0; u < BS / 32; ++u) s += sh[u * NDIAG + k];
            v[k] = s;
        }
    }
}

// Diagnostics (src/cpu_backend.cpp:307-329) over the FP64 state: per-block partials, the last
// block to finish sums them in block order (deterministic).
__global__ void k_diag(const BodyArrays b, const float4* __restrict__ acc, int n, double* partial, unsigned* ticket,
                       double* out) {
    __shared__ double sh[(BS / 32) * NDIAG];
    __shared__ bool last;
    double v[NDIAG] = {};
    for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) {
        double m = b.m[i], x = b.x[i], y = b.y[i], z = b.z[i];
        double vx = b.vx[i], vy = b.vy[i], vz = b.vz[i];
        v[0] += m;
        v[1] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        v[2] += m * static_cast<double>(acc[i].w);
        v[3] += m * vx;
        v[4] += m * vy;
        v[5] += m * vz;
        v[6] += m * (y * vz - z * vy);
        v[7] += m * (z * vx - x * vz);
        v[8] += m * (x * vy - y * vx);
        v[9] += m * x;
        v[10] += m * y;
        v[11] += m * z;
    }
    block_sum(v, sh);
    if (threadIdx.x == 0) {
        for (int k = 0; k < NDIAG; ++k) partial[blockIdx.x * NDIAG + k] = v[k];
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    // The last block sums the partials: every thread a strided subset, then the block in a fixed
    // order, so the result does not depend on which block finished last.
    __threadfence();
    double t[NDIAG] = {};
    for (int blk = threadIdx.x; blk < static_cast<int>(gridDim.x); blk += BS)
#pragma unroll
        for (int k = 0; k < NDIAG; ++k) t[k] += __ldcg(&partial[blk * NDIAG + k]);
    __syncthreads();
    block_sum(t, sh);
    if (threadIdx.x == 0) {
        for (int k = 0; k < NDIAG; ++k) out[k] = t[k];
        *ticket = 0;
    }
}

// Bounding box of the FP64 positions: out6 = min xyz, max xyz.
// Per-system energies of an ensemble: block s sums kinetic energy (1/2) m v^2 and potential
// energy (1/2) m phi over the body range [off[s], off[s + 1]) in FP64, in a fixed order.
__global__ void k_sys_energy(const BodyArrays b, const float4* __restrict__ acc, const uint32_t* __restrict__ off,
                             double* __restrict__ out) {
    __shared__ double sh[(BS / 32) * NDIAG];
    const uint32_t lo = off[blockIdx.x], hi = off[blockIdx.x + 1];
    double v[NDIAG] = {};
    for (uint32_t i = lo + threadIdx.x; i < hi; i += BS) {
        const double m = b.m[i];
        const double vx = b.vx[i], vy = b.vy[i], vz = b.vz[i];
        v[0] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        v[1] += 0.5 * m * static_cast<double>(acc[i].w);
    }
    block_sum(v, sh);
    if (threadIdx.x == 0) {
        out[2 * blockIdx.x] = v[0];
        out[2 * blockIdx.x + 1] = v[1];
    }
}

__global__ void k_bounds(const BodyArrays b, int n, double* partial, unsigned* ticket, double* out6) {
    __shared__ double sh[6][BS / 32];
    __shared__ bool last;
    double v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) {
        double p[3] = {b.x[i], b.y[i], b.z[i]};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            v[c] = fmin(v[c], p[c]);
            v[3 + c] = fmax(v[3 + c], p[c]);
        }
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        for (int o = 16; o > 0; o >>= 1) {
            double t = __shfl_down_sync(0xffffffffu, v[c], o);
            v[c] = c < 3 ? fmin(v[c], t) : fmax(v[c], t);
        }
        if (lane == 0) sh[c][w] = v[c];
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int c = threadIdx.x;
        double r = sh[c][0];
        for (int u = 1; u < BS / 32; ++u) r = c < 3 ? fmin(r, sh[c][u]) : fmax(r, sh[c][u]);
        partial[blockIdx.x * 6 + c] = r;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double r[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int blk = threadIdx.x; blk < static_cast<int>(gridDim.x); blk += BS)
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const double t = __ldcg(&partial[blk * 6 + c]);
            r[c] = c < 3 ? fmin(r[c], t) : fmax(r[c], t);
        }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        for (int o = 16; o > 0; o >>= 1) {
            const double t = __shfl_down_sync(0xffffffffu, r[c], o);
            r[c] = c < 3 ? fmin(r[c], t) : fmax(r[c], t);
        }
    }
    __syncthreads();
    if (lane == 0)
        for (int c = 0; c < 6; ++c) sh[c][w] = r[c];
    __syncthreads();
    if (threadIdx.x < 6) {
        const int c = threadIdx.x;
        double q = sh[c][0];
        for (int u = 1; u < BS / 32; ++u) q = c < 3 ? fmin(q, sh[c][u]) : fmax(q, sh[c][u]);
        out6[c] = q;
        if (c == 0) *ticket = 0;
    }
}

// Exact potential energy (src/cpu_backend.cpp:331-347): sum over i<j of m_i m_j / sqrt(r^2+eps^2)
// in FP64 from the FP64 positions; one block per 256 i-bodies, j tiled through shared memory.
__global__ void k_exact_pe(const BodyArrays b, int n, double e2, double* out) {
    __shared__ double sx[BS], sy[BS], sz[BS], sm[BS];
    __shared__ double red[BS / 32];
    const int i = blockIdx.x * BS + threadIdx.x;
    double xi = 0, yi = 0, zi = 0, mi = 0;
    if (i < n) { xi = b.x[i]; yi = b.y[i]; zi = b.z[i]; mi = b.m[i]; }
    double s = 0;
    // Only tiles that can hold j > i for some i of this block.
    for (int j0 = blockIdx.x * BS; j0 < n; j0 += BS) {
        const int j = j0 + threadIdx.x;
        __syncthreads();
        if (j < n) { sx[threadIdx.x] = b.x[j]; sy[threadIdx.x] = b.y[j]; sz[threadIdx.x] = b.z[j]; sm[threadIdx.x] = b.m[j]; }
        __syncthreads();
        const int cnt = min(BS, n - j0);
        if (i < n) {
            for (int k = 0; k < cnt; ++k) {
                if (j0 + k <= i) continue;
                double dx = sx[k] - xi, dy = sy[k] - yi, dz = sz[k] - zi;
                double r2 = dx * dx + dy * dy + dz * dz + e2;
                if (r2 > 0) s += sm[k] / sqrt(r2);
            }
        }
    }
    s *= mi;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int u = 0; u < BS / 32; ++u) t += red[u];
        atomicAdd(out, t);
    }
}

__global__ void k_fill(float* __restrict__ a, float v, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

__global__ void k_flush(float* __restrict__ a, size_t count) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        a[i] = a[i] * 0.5f + 1.f;
}

// FP32 FMA throughput probe: 8 independent FFMA chains per thread, no memory traffic in the loop.
__global__ void k_ffma_probe(int iters, float seed, unsigned* sink) {
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seed + threadIdx.x * 1e-7f + k;
    const float b = 0.999999f, c = 1e-7f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = __fmaf_rn(a[k], b, c);
    }
    float s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == 12345.678f) atomicAdd(sink, 1u);  // keeps the chains live
}

// Self-test of the bounded waits: an mbarrier no one arrives on and a flag no one sets, each
// waited on with `polls` polls by the primitives the kernels use (mbar_wait_bounded as in the
// direct kernels' TMA pipeline, a volatile flag poll as in the sort and scan look-backs). Both give
// up, record kErrWaitTimeout in the error word and return; nothing is left in flight.
__global__ void k_probe_waits(unsigned polls, const unsigned* never_set, unsigned* err) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    if (!mbar_wait_bounded(&bar, 0, polls)) atomicOr(err, kErrWaitTimeout);
    unsigned it = 0;
    while (*reinterpret_cast<volatile const unsigned*>(never_set) == 0u && ++it < polls) {
    }
    if (it >= polls) atomicOr(err, kErrWaitTimeout);
}

}  // namespace

void probe_waits(cudaStream_t s, unsigned polls, const unsigned* never_set, unsigned* err) {
    k_probe_waits<<<1, 32, 0, s>>>(polls, never_set, err);
    LG_LAUNCHED();
}

double probe_fp32_peak(cudaStream_t s, int sms, unsigned* sink) {
    const int blocks = sms * 8, threads = 256, iters = 1 << 14;
    cudaEvent_t a, b;
    LG_CK(cudaEventCreate(&a));
    LG_CK(cudaEventCreate(&b));
    k_ffma_probe<<<blocks, threads, 0, s>>>(iters, 1.f, sink);  // warm-up
    LG_LAUNCHED();
    double best = 0;
    for (int rep = 0; rep < 3; ++rep) {
        LG_CK(cudaEventRecord(a, s));
        k_ffma_probe<<<blocks, threads, 0, s>>>(iters, 1.f + rep, sink);
        LG_LAUNCHED();
        LG_CK(cudaEventRecord(b, s));
        LG_CK(cudaEventSynchronize(b));
        float ms = 0;
        LG_CK(cudaEventElapsedTime(&ms, a, b));
        const double flops = 2.0 * 8.0 * iters * static_cast<double>(blocks) * threads;
        best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return best;
}

void launch_widen(const float* x, const float* y, const float* z, const float* m, BodyArrays b, int n, cudaStream_t s) {
    if (n <= 0) return;
    k_widen<<<grid_for(n, BS), BS, 0, s>>>(x, y, z, m, b, n);
    LG_LAUNCHED();
}

void launch_refresh_hilo(BodyArrays b, int n, cudaStream_t s) {
    if (n <= 0) return;
    k_refresh_hilo<<<grid_for(n, BS), BS, 0, s>>>(b, n);
    LG_LAUNCHED();
}

void launch_round_pos(const BodyArrays b, float* x, float* y, float* z, int n, cudaStream_t s) {
    if (n <= 0) return;
    k_round_pos<<<grid_for(n, BS), BS, 0, s>>>(b, x, y, z, n);
    LG_LAUNCHED();
}

void launch_kick(BodyArrays b, const float4* acc, float dt, int n, cudaStream_t s) {
    if (n <= 0) return;
    k_kick<<<grid_for(n, BS), BS, 0, s>>>(b, acc, dt, n);
    LG_LAUNCHED();
}

void launch_drift(BodyArrays b, double dt, int n, cudaStream_t s) {
    if (n <= 0) return;
    k_drift<<<grid_for(n, BS), BS, 0, s>>>(b, dt, n);
    LG_LAUNCHED();
}

void launch_kick_drift(BodyArrays b, const float4* acc, float hdt, double dt, int n, cudaStream_t s) {
    if (n <= 0) return;
    k_kick_drift<<<grid_for(n, BS), BS, 0, s>>>(b, acc, hdt, dt, n);
    LG_LAUNCHED();
}

void launch_sys_energy(const BodyArrays b, const float4* acc, const uint32_t* off, int nsys, double* out,
                       cudaStream_t s) {
    if (nsys <= 0) return;
    k_sys_energy<<<nsys, BS, 0, s>>>(b, acc, off, out);
    LG_LAUNCHED();
}

void launch_diag(const BodyArrays b, const float4* acc, int n, double* partial, unsigned* ticket, double* out,
                 int blocks, cudaStream_t s) {
    k_diag<<<blocks, BS, 0, s>>>(b, acc, n, partial, ticket, out);
    LG_LAUNCHED();
}

void launch_bounds(const BodyArrays b, int n, double* partial, unsigned* ticket, double* out6, int blocks,
                   cudaStream_t s) {
    k_bounds<<<blocks, BS, 0, s>>>(b, n, partial, ticket, out6);
    LG_LAUNCHED();
}

void launch_exact_pe(const BodyArrays b, int n, double e2, double* out, cudaStream_t s) {
    if (n <= 0) return;
    k_exact_pe<<<grid_for(n, BS), BS, 0, s>>>(b, n, e2, out);
    LG_LAUNCHED();
}

void launch_fill_cost(float* cost, float v, int n, cudaStream_t s) {
    if (n <= 0) return;
    k_fill<<<grid_for(n, BS), BS, 0, s>>>(cost, v, n);
    LG_LAUNCHED();
}

void launch_flush(float* buf, size_t count, cudaStream_t s) {
    k_flush<<<1024, BS, 0, s>>>(buf, count);
    LG_LAUNCHED();
}

}  // namespace lg
