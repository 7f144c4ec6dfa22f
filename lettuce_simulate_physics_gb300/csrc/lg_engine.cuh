// Internal declarations of the GB300 engine: the resident state and the kernel launchers.
//
// HBM layout (n bodies, struct of arrays, every array 256-byte aligned by cudaMalloc):
//   body state, two copies (a sort gathers from one into the other):
//     x, y, z            double   24 B  FP64 positions (drift is FP64)
//     hm                 float4   16 B  (hi(x), hi(y), hi(z), m), hi = round-to-nearest float
//     lo                 float4   16 B  (x - hi(x), y - hi(y), z - hi(z), 0) rounded to float
//     vx, vy, vz, m      float    16 B
//     id                 uint32    4 B
//     cost               float     4 B  interactions of the last force call
//   acc                  float4   16 B  (ax, ay, az, phi) of the last force call, current order
// The force kernels read positions only through hm and lo: pair arithmetic is FP32 on relative
// coordinates (x_hi - o_hi) + (x_lo - o_lo) formed against a per-block (direct) or per-group
// (tree) origin o, so close pairs keep the FP64 separation.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "lg_common.cuh"

namespace lg {

struct BodyArrays {
    double *x = nullptr, *y = nullptr, *z = nullptr;
    float4 *hm = nullptr, *lo = nullptr;
    float *vx = nullptr, *vy = nullptr, *vz = nullptr, *m = nullptr, *cost = nullptr;
    uint32_t* id = nullptr;
    uint8_t* level = nullptr;  // block time-step level (dt = dt_base / 2^level)
};

// Direct-sum launch shape, chosen by the host (autotuned or defaults).
struct DirectShape {
    int ipt = 4;        // i-bodies per thread: 1, 2, 4 or 8
    int tile = 256;     // j-bodies per shared-memory stage: 256, or 128 (ipt 1, 2 or 4)
    int slices = 1;     // j-range splits (split-j); partial sums reduced in a second kernel
};

// ---- kernel launchers (each file owns its kernels) ------------------------------------------
// integrate.cu
void launch_widen(const float* x, const float* y, const float* z, const float* m, BodyArrays b, int n,
                  cudaStream_t s);
// hm/lo from the FP64 positions and masses already stored in b.
void launch_refresh_hilo(BodyArrays b, int n, cudaStream_t s);
void launch_round_pos(const BodyArrays b, float* x, float* y, float* z, int n, cudaStream_t s);
void launch_kick(BodyArrays b, const float4* acc, float dt, int n, cudaStream_t s);
void launch_drift(BodyArrays b, double dt, int n, cudaStream_t s);
// Ensemble step opening (kick by hdt, then drift by dt; the same arithmetic as the two kernels).
void launch_kick_drift(BodyArrays b, const float4* acc, float hdt, double dt, int n, cudaStream_t s);
// out[2 s], out[2 s + 1] = kinetic and potential energy of system s (bodies [off[s], off[s + 1])).
void launch_sys_energy(const BodyArrays b, const float4* acc, const uint32_t* off, int nsys, double* out,
                       cudaStream_t s);
// Diagnostics: out[13] = mass, ke, sum m phi, px, py, pz, lx, ly, lz, mx, my, mz, (unused).
void launch_diag(const BodyArrays b, const float4* acc, int n, double* partial, unsigned* ticket, double* out,
                 int blocks, cudaStream_t s);
void launch_exact_pe(const BodyArrays b, int n, double e2, double* out, cudaStream_t s);
void launch_bounds(const BodyArrays b, int n, double* partial, unsigned* ticket, double* out6, int blocks,
                   cudaStream_t s);
void launch_fill_cost(float* cost, float v, int n, cudaStream_t s);
void launch_flush(float* buf, size_t count, cudaStream_t s);

// direct.cu
// Accelerations (G-scaled) and potential of every body from all bodies; partial: slices * n float4
// of scratch when shape.slices > 1.
// cost (optional): per-body interaction counts n - 1, written by the same launches.
void launch_direct(const BodyArrays b, int n, float G, float e2, bool potential, bool eps0, const DirectShape& shape,
                   float4* acc, float4* partial, unsigned* err, cudaStream_t s, float* cost = nullptr);
DirectShape default_direct_shape(int n, int sms);
// Batched direct sums over independent systems: one block per work item, i-bodies [base, iend)
// (at most direct_block_bodies(ipt) of them) against j-bodies [j0, j1) of the same system, with
// that system's squared softening e2. Writes G-scaled accelerations and potentials.
struct alignas(32) DirectWork {
    int base, iend, j0, j1;
    float e2;
    int sys, pad0, pad1;
};
int direct_block_bodies(int ipt);
// tile: j-bodies per shared-memory stage, 256 or 128 (with 1, 2 or 4 i-bodies per thread).
void launch_direct_batch(const BodyArrays b, const DirectWork* work, int nwork, int ipt, int tile, float G,
                         bool potential, bool eps0, float4* acc, unsigned* err, cudaStream_t s);

}  // namespace lg
