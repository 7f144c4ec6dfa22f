// Adjoint (reverse mode) of the kick-drift-kick leapfrog with direct-summation or tree forces. The
// reference has no adjoint; this is the engine's own, checked against FP64 central finite
// differences and the FP64 CPU adjoint in oracle/lettuce_oracle.c.
//
// Forward map (the reference's step order, src/simulation.cpp:416-419): forces at x0, then per step
// kick(dt/2), drift(dt), forces, kick(dt/2). Loss L = sum_i m_i |x_i(T) - x*_i|^2.
//
// Reverse sweep. With h = dt/2 the adjoint of one step is
//   lv_h = lv';  lx' += J(x')^T (h lv');  lx = lx';  lv_h += dt lx';  lv = lv_h;  lx += J(x)^T (h lv_h)
// and the two products at a shared position x_s (closing kick of step s-1, opening kick of step s)
// carry the same vector, so the sweep needs one vector-Jacobian product per step:
//   lx = dL/dx_T, lv = 0, lm = |x_T - x*|^2;  for s = T-1 .. 0:  lv += dt lx;
//   (lx, lm) += VJP at x_s with weight c lv, c = dt (s > 0) or h (s = 0).
// The closing-kick product at x_T carries lv_T = 0 and drops out.
//
// Pairwise VJP. a_k = G sum_j m_j K(d_kj), K(d) = d / s^3, s^2 = |d|^2 + eps^2, d_kj = x_j - x_k:
//   dL/dx_k += G sum_j M(d_kj) (m_k w_j - m_j w_k),  M(d) u = u / s^3 - 3 d (d . u) / s^5
//   dL/dm_k -= G sum_j (w_j . d_kj) / s^3
// The self pair contributes exactly zero (d = 0, u = 0). Pair arithmetic is FP32 on block-relative
// coordinates from the FP64 hi/lo split, packed f32x2; the adjoint state is accumulated in FP64.
// Two kernels: k_vjp evaluates every ordered pair (split-j, Kahan across tiles) and serves small
// systems; k_vjp_sym evaluates every unordered pair once for both bodies (tile-pair units, partial
// sums added in FP64) and serves systems of about 26k bodies and more.
//
// Checkpoints: FP64 positions and FP32 velocities every k steps; the backward pass restores each
// segment, recomputes its positions with the same deterministic kernels (so they are bit-identical
// to the forward pass), and stores them as hi/lo float4 pairs for the VJP.
//
// Tree forces (Barnes-Hut with quadrupoles): the same sweep with the tree walk's VJP (walk_vjp.cu)
// over frozen interaction lists. The tree sorts the bodies every step, so the adjoint state is
// indexed by body id (ids 0..n-1), checkpoints also keep masses and ids, and the segment store
// keeps each step's FP64 positions in the order its force call sorted them. For the VJP of step s
// the backward pass loads those positions and rebuilds the tree: the sort of already sorted bodies
// is the identity, so the tree, its moments and its lists are bit-identical to the forward pass's.
#include <algorithm>
#include <type_traits>
#include <vector>

#include "engine.cuh"

namespace lg {

namespace {

// Launch shape of the pairwise VJP (measured best on GB300: 128 threads, one i-body per thread,
// four j-pairs unrolled).
#ifndef LG_VJP_BS
#define LG_VJP_BS 128
#endif
#ifndef LG_VJP_IPT
#define LG_VJP_IPT 1
#endif
#ifndef LG_VJP_UNROLL
#define LG_VJP_UNROLL 4
#endif
#ifndef LG_VJP_MINB
#define LG_VJP_MINB 1
#endif
constexpr int VBS = LG_VJP_BS;  // threads per block
constexpr int VTILE = 256;      // j-bodies per shared-memory tile
constexpr int VIPT = LG_VJP_IPT; // i-bodies per thread
constexpr int VUNROLL = LG_VJP_UNROLL;  // j-pair iterations unrolled

struct __align__(16) VjpSmem {
    float rx[VTILE], ry[VTILE], rz[VTILE], rm[VTILE], wx[VTILE], wy[VTILE], wz[VTILE];
};

inline int grid_for(long long n, int bs) { return static_cast<int>((n + bs - 1) / bs); }

__device__ __forceinline__ f2x ld2(const float* p) { return *reinterpret_cast<const f2x*>(p); }

// partial[slice][i] = (gx, gy, gz, h) for the i-bodies of this block and the j of this slice.
//
// Factored pair sum. With c_j = (m_k (w_j . d) - m_j (w_k . d)) / s^5,
//   sum_j M(d)(m_k w_j - m_j w_k) = m_k S1 - w_k S2 - 3 S3,
//   S1 = sum_j w_j / s^3,  S2 = sum_j m_j / s^3,  S3 = sum_j c_j d,
// so a pair costs 26 FP32 operations (packed two pairs at a time) instead of forming
// m_k w_j - m_j w_k per pair. The self pair (d = 0) adds w_k / eps^3 to S1 and m_k / eps^3 to S2,
// which are taken out again, exactly as the loop formed them, in the slice that holds it.
template <bool EPS0>
__global__ void __launch_bounds__(VBS, LG_VJP_MINB) k_vjp(const float4* __restrict__ hm, const float4* __restrict__ lo,
                                             const float4* __restrict__ wv, int n, int jslice, float e2,
                                             float4* __restrict__ partial) {
    __shared__ VjpSmem sm;
    const int tid = threadIdx.x;
    const int base = blockIdx.x * (VBS * VIPT);
    const int j0 = blockIdx.y * jslice;
    const int j1 = min(n, j0 + jslice);
    const float4 oh = hm[base], ol = lo[base];
    float mk[VIPT], wkx[VIPT], wky[VIPT], wkz[VIPT];
    float s[VIPT][8], c[VIPT][8];  // S1 (3), S2 (negated), S3 (3), h: Kahan sums and compensations
    f2x XI[VIPT], YI[VIPT], ZI[VIPT], MK[VIPT], WKX[VIPT], WKY[VIPT], WKZ[VIPT];
#pragma unroll
    for (int u = 0; u < VIPT; ++u) {
        const int i = min(base + u * VBS + tid, n - 1);
        const float4 h = hm[i], l = lo[i], w = wv[i];
        XI[u] = f2_bcast((h.x - oh.x) + (l.x - ol.x));
        YI[u] = f2_bcast((h.y - oh.y) + (l.y - ol.y));
        ZI[u] = f2_bcast((h.z - oh.z) + (l.z - ol.z));
        mk[u] = h.w;
        wkx[u] = w.x; wky[u] = w.y; wkz[u] = w.z;
        MK[u] = f2_bcast(h.w);
        WKX[u] = f2_bcast(w.x); WKY[u] = f2_bcast(w.y); WKZ[u] = f2_bcast(w.z);
#pragma unroll
        for (int q = 0; q < 8; ++q) s[u][q] = c[u][q] = 0.f;
    }
    const f2x E2 = f2_bcast(e2);
    for (int jt = j0; jt < j1; jt += VTILE) {
        const int cnt = min(VTILE, j1 - jt);
        const int cnt2 = (cnt + 1) & ~1;
        __syncthreads();
        for (int k = tid; k < cnt2; k += VBS) {
            if (k < cnt) {
                const float4 h = hm[jt + k], l = lo[jt + k], w = wv[jt + k];
                sm.rx[k] = (h.x - oh.x) + (l.x - ol.x);
                sm.ry[k] = (h.y - oh.y) + (l.y - ol.y);
                sm.rz[k] = (h.z - oh.z) + (l.z - ol.z);
                sm.rm[k] = -h.w;  // negated mass
                sm.wx[k] = w.x; sm.wy[k] = w.y; sm.wz[k] = w.z;
            } else {
                sm.rx[k] = sm.ry[k] = sm.rz[k] = 1e18f;  // far, massless, zero weight: adds nothing
                sm.rm[k] = 0.f;
                sm.wx[k] = sm.wy[k] = sm.wz[k] = 0.f;
            }
        }
        __syncthreads();
        f2x a[VIPT][8];
#pragma unroll
        for (int u = 0; u < VIPT; ++u)
#pragma unroll
            for (int q = 0; q < 8; ++q) a[u][q] = 0ull;
#pragma unroll VUNROLL
        for (int k = 0; k < cnt2; k += 2) {
            const f2x X = ld2(sm.rx + k), Y = ld2(sm.ry + k), Z = ld2(sm.rz + k), NM = ld2(sm.rm + k);
            const f2x WX = ld2(sm.wx + k), WY = ld2(sm.wy + k), WZ = ld2(sm.wz + k);
#pragma unroll
            for (int u = 0; u < VIPT; ++u) {
                const f2x dx = f2_sub(X, XI[u]), dy = f2_sub(Y, YI[u]), dz = f2_sub(Z, ZI[u]);
                const f2x r2 = f2_fma(dx, dx, f2_fma(dy, dy, f2_fma(dz, dz, E2)));
                float ra, rb;
                f2_unpack(r2, ra, rb);
                float ia = rsqrt_mufu(ra), ib = rsqrt_mufu(rb);
                if (EPS0) {
                    ia = ra > 0.f ? ia : 0.f;
                    ib = rb > 0.f ? ib : 0.f;
                }
                const f2x inv = f2_pack(ia, ib);
                const f2x inv2 = f2_mul(inv, inv), inv3 = f2_mul(inv2, inv), inv5 = f2_mul(inv3, inv2);
                const f2x dwj = f2_fma(dx, WX, f2_fma(dy, WY, f2_mul(dz, WZ)));
                const f2x dwk = f2_fma(dx, WKX[u], f2_fma(dy, WKY[u], f2_mul(dz, WKZ[u])));
                const f2x cc = f2_mul(f2_fma(MK[u], dwj, f2_mul(NM, dwk)), inv5);
                a[u][0] = f2_fma(WX, inv3, a[u][0]);
                a[u][1] = f2_fma(WY, inv3, a[u][1]);
                a[u][2] = f2_fma(WZ, inv3, a[u][2]);
                a[u][3] = f2_fma(NM, inv3, a[u][3]);
                a[u][4] = f2_fma(cc, dx, a[u][4]);
                a[u][5] = f2_fma(cc, dy, a[u][5]);
                a[u][6] = f2_fma(cc, dz, a[u][6]);
                a[u][7] = f2_fma(dwj, inv3, a[u][7]);
            }
        }
#pragma unroll
        for (int u = 0; u < VIPT; ++u)
#pragma unroll
            for (int q = 0; q < 8; ++q) kahan_add(s[u][q], c[u][q], f2_sum(a[u][q]));
    }
    // The self pair's S1 and S2 terms, formed as the loop formed them (r2 == e2).
    float self3 = 0.f;
    if (!EPS0) {
        const float inv = rsqrt_mufu(e2), inv2 = inv * inv;
        self3 = inv2 * inv;
    }
#pragma unroll
    for (int u = 0; u < VIPT; ++u) {
        const int i = base + u * VBS + tid;
        if (i >= n) continue;
        float S[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) S[q] = s[u][q] - c[u][q];
        if (!EPS0 && i >= j0 && i < j1) {
            S[0] = __fsub_rn(S[0], __fmul_rn(wkx[u], self3));
            S[1] = __fsub_rn(S[1], __fmul_rn(wky[u], self3));
            S[2] = __fsub_rn(S[2], __fmul_rn(wkz[u], self3));
            S[3] = __fadd_rn(S[3], __fmul_rn(mk[u], self3));
        }
        // m_k S1 - w_k S2 - 3 S3 (S[3] holds -S2)
        const float gx = mk[u] * S[0] + wkx[u] * S[3] - 3.f * S[4];
        const float gy = mk[u] * S[1] + wky[u] * S[3] - 3.f * S[5];
        const float gz = mk[u] * S[2] + wkz[u] * S[3] - 3.f * S[6];
        partial[static_cast<size_t>(blockIdx.y) * n + i] = make_float4(gx, gy, gz, S[7]);
    }
}

// lx += G sum_slices g, lm -= G sum_slices h (slice order, FP64).
__global__ void k_vjp_apply(const float4* __restrict__ partial, int n, int slices, double G, double* lx,
                            double* ly, double* lz, double* lm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double g0 = 0, g1 = 0, g2 = 0, h = 0;
    for (int k = 0; k < slices; ++k) {
        const float4 p = partial[static_cast<size_t>(k) * n + i];
        g0 += p.x; g1 += p.y; g2 += p.z; h += p.w;
    }
    lx[i] += G * g0;
    ly[i] += G * g1;
    lz[i] += G * g2;
    lm[i] -= G * h;
}

// ---- symmetric pairwise VJP ------------------------------------------------------------------
// Each unordered pair (k, j), k < j, is evaluated once. With d = x_j - x_k, s^2 = |d|^2 + eps^2 and
// cc = (m_k (w_j . d) - m_j (w_k . d)) / s^5, the pair adds to body k (the i side)
//   S1 += w_j / s^3,  -S2 += -m_j / s^3,  S3 += cc d,  h += (w_j . d) / s^3
// and to body j (the j side: d_jk = -d and the same cc)
//   S1 += w_k / s^3,  S2 += m_k / s^3,  S3 -= cc d,  h -= (w_k . d) / s^3,
// which is 34 FP32 operations for two ordered pairs instead of 52. Work units are pairs of
// STILE-body tiles (I, J), J >= I; a block takes a strip of SSTRIP J tiles (or fewer) for one I tile,
// its threads holding SIPT i-bodies each. The i side sums in registers over the strip. The j side
// of each pair of j-bodies is summed over a warp's lanes by a transposed butterfly (16 values over
// 32 lanes: each exchange sends half of what a lane holds), over the block's warps in shared
// memory (warp order), and stored per unit. A diagonal unit (J == I) masks the pairs j <= k. All
// sums run in a fixed order, so results do not depend on scheduling; k_vjp_sym_apply adds the
// strips' and units' partial sums per body in FP64.
#ifndef LG_VJPS_BS
#define LG_VJPS_BS 128
#endif
#ifndef LG_VJPS_IPT
#define LG_VJPS_IPT 4
#endif
#ifndef LG_VJPS_MINB
#define LG_VJPS_MINB 3
#endif
constexpr int SBS = LG_VJPS_BS;        // threads per block
constexpr int SIPT = LG_VJPS_IPT;      // i-bodies per thread
constexpr int STILE = SBS * SIPT;      // bodies per tile
#ifndef LG_VJPS_STRIP
#define LG_VJPS_STRIP 2
#endif
#ifndef LG_VJPS_SUB
#define LG_VJPS_SUB 128
#endif
constexpr int SSUB = LG_VJPS_SUB;      // j-bodies between cross-warp reductions
constexpr int SSTRIP = LG_VJPS_STRIP;  // J tiles per block
constexpr int SWARPS = SBS / 32;
static_assert(STILE % SSUB == 0 && SSUB % 2 == 0, "sub-tiles hold whole j pairs");

struct __align__(16) SymSmem {
    float jx[STILE], jy[STILE], jz[STILE], jnm[STILE], jwx[STILE], jwy[STILE], jwz[STILE];
    float red[SWARPS][SSUB][8];
};

// One exchange of the transposed butterfly: lanes with bit O keep the upper H of their 2H values
// and send the lower H, the others the reverse; each kept value adds the partner's sent one.
template <int O, int H>
__device__ __forceinline__ void tr_level(float (&v)[16], int lane) {
    const bool up = (lane & O) != 0;
#pragma unroll
    for (int t = 0; t < H; ++t) {
        const float send = up ? v[t] : v[t + H];
        const float keep = up ? v[t + H] : v[t];
        v[t] = keep + __shfl_xor_sync(0xffffffffu, send, O);
    }
}

constexpr float kFarV = 1e18f;  // a far, massless, zero-weight body: adds nothing to either side

// Row I of the j sums holds bodies [I STILE, npad) (the tiles J >= I), rows back to back.
__device__ __forceinline__ size_t jrow(int I, int npad) {
    return static_cast<size_t>(I) * npad - static_cast<size_t>(STILE) * (static_cast<size_t>(I) * (I - 1) / 2);
}

// units[b] = (I, J0, J1, strip): block b evaluates tile I against tiles [J0, J1) and writes its i
// sums to row `strip` of ipart (the tile's STILE bodies); the j sums of unit (I, J) go to row I of
// jpart. Entries are 8 floats: S1 (3), -S2, S3 (3), h, where jpart holds the j side's -S2, S3 and
// h with the opposite sign.
template <bool EPS0>
__global__ void __launch_bounds__(SBS, LG_VJPS_MINB) k_vjp_sym(const float4* __restrict__ hm, const float4* __restrict__ lo,
                                                   const float4* __restrict__ wv, int n, int npad, float e2,
                                                   const int4* __restrict__ units, float* __restrict__ ipart,
                                                   float* __restrict__ jpart) {
    __shared__ SymSmem sm;
    const int4 un = units[blockIdx.x];
    const int I = un.x, J0 = un.y, J1 = un.z, strip = un.w;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ib = I * STILE;
    const float4 oh = hm[ib], ol = lo[ib];  // the block origin: the tile's first body (ib < n)
    f2x XI[SIPT], YI[SIPT], ZI[SIPT], MK[SIPT], WKX[SIPT], WKY[SIPT], WKZ[SIPT];
    f2x a[SIPT][8];
    int iidx[SIPT];
#pragma unroll
    for (int u = 0; u < SIPT; ++u) {
        const int i = ib + u * SBS + tid;
        iidx[u] = i;
        float x = kFarV, y = kFarV, z = kFarV, m = 0.f;
        float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
        if (i < n) {  // past n: far, massless, zero weight, so it adds nothing to either side
            const float4 h = hm[i], l = lo[i];
            w = wv[i];
            x = (h.x - oh.x) + (l.x - ol.x);
            y = (h.y - oh.y) + (l.y - ol.y);
            z = (h.z - oh.z) + (l.z - ol.z);
            m = h.w;
        }
        XI[u] = f2_bcast(x); YI[u] = f2_bcast(y); ZI[u] = f2_bcast(z);
        MK[u] = f2_bcast(m);
        WKX[u] = f2_bcast(w.x); WKY[u] = f2_bcast(w.y); WKZ[u] = f2_bcast(w.z);
#pragma unroll
        for (int q = 0; q < 8; ++q) a[u][q] = 0ull;
    }
    const f2x E2 = f2_bcast(e2);
    // The (j, component) a lane holds after the butterfly: lane bits 4..1 select halves in turn.
    const int qsel = ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
    for (int J = J0; J < J1; ++J) {
        const int jb = J * STILE;
        __syncthreads();  // the previous tile's readers are done
        for (int k = tid; k < STILE; k += SBS) {
            const int j = jb + k;
            if (j < n) {
                const float4 h = hm[j], l = lo[j], w = wv[j];
                sm.jx[k] = (h.x - oh.x) + (l.x - ol.x);
                sm.jy[k] = (h.y - oh.y) + (l.y - ol.y);
                sm.jz[k] = (h.z - oh.z) + (l.z - ol.z);
                sm.jnm[k] = -h.w;
                sm.jwx[k] = w.x; sm.jwy[k] = w.y; sm.jwz[k] = w.z;
            } else {
                sm.jx[k] = sm.jy[k] = sm.jz[k] = kFarV;
                sm.jnm[k] = 0.f;
                sm.jwx[k] = sm.jwy[k] = sm.jwz[k] = 0.f;
            }
        }
        __syncthreads();
        // The tile's sub-tiles, compiled twice: with the diagonal mask (J == I) and without.
        auto tile = [&](auto diag_tag) {
        constexpr bool DIAG = decltype(diag_tag)::value;
        for (int s0 = 0; s0 < STILE; s0 += SSUB) {
            for (int jp = s0; jp < s0 + SSUB; jp += 2) {
                const f2x X = ld2(sm.jx + jp), Y = ld2(sm.jy + jp), Z = ld2(sm.jz + jp), NM = ld2(sm.jnm + jp);
                const f2x WX = ld2(sm.jwx + jp), WY = ld2(sm.jwy + jp), WZ = ld2(sm.jwz + jp);
                f2x b[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) b[q] = 0ull;
#pragma unroll
                for (int u = 0; u < SIPT; ++u) {
                    const f2x dx = f2_sub(X, XI[u]), dy = f2_sub(Y, YI[u]), dz = f2_sub(Z, ZI[u]);
                    const f2x r2 = f2_fma(dx, dx, f2_fma(dy, dy, f2_fma(dz, dz, E2)));
                    float ra, rb;
                    f2_unpack(r2, ra, rb);
                    float ia = rsqrt_mufu(ra), ibb = rsqrt_mufu(rb);
                    if (EPS0) {
                        ia = ra > 0.f ? ia : 0.f;
                        ibb = rb > 0.f ? ibb : 0.f;
                    }
                    if constexpr (DIAG) {  // only pairs j > k: the tile's lower triangle and self pairs add nothing
                        const int jg = jb + jp;
                        ia = jg > iidx[u] ? ia : 0.f;
                        ibb = jg + 1 > iidx[u] ? ibb : 0.f;
                    }
                    const f2x inv = f2_pack(ia, ibb);
                    const f2x inv2 = f2_mul(inv, inv), inv3 = f2_mul(inv2, inv), inv5 = f2_mul(inv3, inv2);
                    const f2x dwj = f2_fma(dx, WX, f2_fma(dy, WY, f2_mul(dz, WZ)));
                    const f2x dwk = f2_fma(dx, WKX[u], f2_fma(dy, WKY[u], f2_mul(dz, WKZ[u])));
                    const f2x cc = f2_mul(f2_fma(MK[u], dwj, f2_mul(NM, dwk)), inv5);
                    a[u][0] = f2_fma(WX, inv3, a[u][0]);
                    a[u][1] = f2_fma(WY, inv3, a[u][1]);
                    a[u][2] = f2_fma(WZ, inv3, a[u][2]);
                    a[u][3] = f2_fma(NM, inv3, a[u][3]);
                    a[u][4] = f2_fma(cc, dx, a[u][4]);
                    a[u][5] = f2_fma(cc, dy, a[u][5]);
                    a[u][6] = f2_fma(cc, dz, a[u][6]);
                    a[u][7] = f2_fma(dwj, inv3, a[u][7]);
                    b[0] = f2_fma(WKX[u], inv3, b[0]);
                    b[1] = f2_fma(WKY[u], inv3, b[1]);
                    b[2] = f2_fma(WKZ[u], inv3, b[2]);
                    b[3] = f2_fma(MK[u], inv3, b[3]);
                    b[4] = f2_fma(cc, dx, b[4]);
                    b[5] = f2_fma(cc, dy, b[5]);
                    b[6] = f2_fma(cc, dz, b[6]);
                    b[7] = f2_fma(dwk, inv3, b[7]);
                }
                // v[2c + h] = component c of j-body jp + h, summed over the lane's i-bodies.
                float v[16];
#pragma unroll
                for (int c = 0; c < 8; ++c) f2_unpack(b[c], v[2 * c], v[2 * c + 1]);
                tr_level<16, 8>(v, lane);
                tr_level<8, 4>(v, lane);
                tr_level<4, 2>(v, lane);
                tr_level<2, 1>(v, lane);
                v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
                if (!(lane & 1)) sm.red[warp][jp - s0 + (qsel & 1)][qsel >> 1] = v[0];
            }
            __syncthreads();
            // The sub-tile's j sums over the block's warps, in warp order.
            for (int t = tid; t < SSUB * 8; t += SBS) {
                const int jj = t >> 3, c = t & 7;
                float sum = sm.red[0][jj][c];
#pragma unroll
                for (int w = 1; w < SWARPS; ++w) sum += sm.red[w][jj][c];
                const int j = jb + s0 + jj;
                if (j < n) jpart[(jrow(I, npad) + (j - ib)) * 8 + c] = sum;
            }
            __syncthreads();  // red is rewritten by the next sub-tile
        }
        };
        if (J == I) tile(std::true_type{});
        else tile(std::false_type{});
    }
#pragma unroll
    for (int u = 0; u < SIPT; ++u) {
        if (iidx[u] >= n) continue;
        float* o = ipart + (static_cast<size_t>(strip) * STILE + (iidx[u] - ib)) * 8;
        const float4 p0 = make_float4(f2_sum(a[u][0]), f2_sum(a[u][1]), f2_sum(a[u][2]), f2_sum(a[u][3]));
        const float4 p1 = make_float4(f2_sum(a[u][4]), f2_sum(a[u][5]), f2_sum(a[u][6]), f2_sum(a[u][7]));
        reinterpret_cast<float4*>(o)[0] = p0;
        reinterpret_cast<float4*>(o)[1] = p1;
    }
}

// Per body k of tile K: the i sums of K's strips and the j sums of units (I, K), I <= K, in that
// order in FP64; then lx += G (m_k S1 - w_k S2 - 3 S3), lm -= G h.
__global__ void k_vjp_sym_apply(const float* __restrict__ ipart, const float* __restrict__ jpart,
                                const int* __restrict__ strip_base, const float4* __restrict__ hm,
                                const float4* __restrict__ wv, int n, int npad, double G, double* lx, double* ly,
                                double* lz, double* lm) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int K = k / STILE;
    double S[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int st = strip_base[K]; st < strip_base[K + 1]; ++st) {
        const float4* p = reinterpret_cast<const float4*>(ipart + (static_cast<size_t>(st) * STILE + (k - K * STILE)) * 8);
        const float4 p0 = p[0], p1 = p[1];
        S[0] += p0.x; S[1] += p0.y; S[2] += p0.z; S[3] += p0.w;
        S[4] += p1.x; S[5] += p1.y; S[6] += p1.z; S[7] += p1.w;
    }
    for (int I = 0; I <= K; ++I) {
        const float4* p = reinterpret_cast<const float4*>(jpart + (jrow(I, npad) + (k - I * STILE)) * 8);
        const float4 p0 = p[0], p1 = p[1];
        S[0] += p0.x; S[1] += p0.y; S[2] += p0.z; S[3] -= p0.w;
        S[4] -= p1.x; S[5] -= p1.y; S[6] -= p1.z; S[7] -= p1.w;
    }
    const double m = hm[k].w;
    const float4 w = wv[k];
    // m_k S1 - w_k S2 - 3 S3 (S[3] holds -S2)
    lx[k] += G * (m * S[0] + w.x * S[3] - 3.0 * S[4]);
    ly[k] += G * (m * S[1] + w.y * S[3] - 3.0 * S[5]);
    lz[k] += G * (m * S[2] + w.z * S[3] - 3.0 * S[6]);
    lm[k] -= G * S[7];
}

// lv += dt lx; w = c lv (FP32 for the VJP), with the body's mass alongside.
__global__ void k_adj_kick(const double* lx, const double* ly, const double* lz, double* lvx, double* lvy,
                           double* lvz, double dt, double c, float4* w, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double vx = lvx[i] + dt * lx[i], vy = lvy[i] + dt * ly[i], vz = lvz[i] + dt * lz[i];
    lvx[i] = vx; lvy[i] = vy; lvz[i] = vz;
    w[i] = make_float4(static_cast<float>(c * vx), static_cast<float>(c * vy), static_cast<float>(c * vz), 0.f);
}

// Terminal adjoints from the final FP64 positions and the target (target indexed by id).
__global__ void k_adj_init(const BodyArrays b, const double* tx, const double* ty, const double* tz, double* lx,
                           double* ly, double* lz, double* lvx, double* lvy, double* lvz, double* lm, double* loss_terms,
                           int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = b.id[i];
    const double m = b.m[i];
    const double dx = b.x[i] - tx[id], dy = b.y[i] - ty[id], dz = b.z[i] - tz[id];
    lx[i] = 2 * m * dx; ly[i] = 2 * m * dy; lz[i] = 2 * m * dz;
    lvx[i] = lvy[i] = lvz[i] = 0;
    const double d2 = dx * dx + dy * dy + dz * dz;
    lm[i] = d2;
    loss_terms[i] = m * d2;
}

// Checkpoint copy of the state: FP64 positions, FP32 velocities, masses and ids (the tree
// reorders the bodies).
__global__ void k_save(const BodyArrays b, double* x, double* y, double* z, float* vx, float* vy, float* vz, float* m,
                       uint32_t* id, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = b.x[i]; y[i] = b.y[i]; z[i] = b.z[i];
    vx[i] = b.vx[i]; vy[i] = b.vy[i]; vz[i] = b.vz[i];
    m[i] = b.m[i]; id[i] = b.id[i];
}

__device__ __forceinline__ void set_pos(BodyArrays b, int i, double px, double py, double pz, float m) {
    b.x[i] = px; b.y[i] = py; b.z[i] = pz;
    const float hx = __double2float_rn(px), hy = __double2float_rn(py), hz = __double2float_rn(pz);
    b.hm[i] = make_float4(hx, hy, hz, m);
    b.lo[i] = make_float4(__double2float_rn(px - hx), __double2float_rn(py - hy), __double2float_rn(pz - hz), 0.f);
}

__global__ void k_restore(BodyArrays b, const double* x, const double* y, const double* z, const float* vx,
                          const float* vy, const float* vz, const float* m, const uint32_t* id, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    b.vx[i] = vx[i]; b.vy[i] = vy[i]; b.vz[i] = vz[i];
    b.m[i] = m[i]; b.id[i] = id[i];
    set_pos(b, i, x[i], y[i], z[i], m[i]);
}

// Tree path: one step's positions (in its sorted order) and ids, and back.
__global__ void k_store_step(const BodyArrays b, double* x, double* y, double* z, uint32_t* id, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = b.x[i]; y[i] = b.y[i]; z[i] = b.z[i]; id[i] = b.id[i];
}

__global__ void k_load_step(BodyArrays b, const double* x, const double* y, const double* z, const uint32_t* id,
                            const float* m_by_id, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = id[i];
    const float m = m_by_id[k];
    b.id[i] = k;
    b.m[i] = m;
    set_pos(b, i, x[i], y[i], z[i], m);
}

__global__ void k_mass_by_id(const BodyArrays b, float* m_by_id, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) m_by_id[b.id[i]] = b.m[i];
}

// Weights in the current body order from the id-indexed ones.
__global__ void k_gather_w(const BodyArrays b, const float4* w_by_id, float4* w, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) w[i] = w_by_id[b.id[i]];
}

// lx[id] += G g_x, ..., lm[id] += G g_m (g in the current body order).
__global__ void k_tree_vjp_apply(const BodyArrays b, const double* g, int n, double G, double* lx, double* ly,
                                 double* lz, double* lm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = b.id[i];
    lx[k] += G * g[i];
    ly[k] += G * g[n + i];
    lz[k] += G * g[2 * static_cast<size_t>(n) + i];
    lm[k] += G * g[3 * static_cast<size_t>(n) + i];
}

// Terminal adjoints supplied by the caller (dL/dx_T by id): lx = seed, lv = 0, lm = 0. by_id selects
// the tree path's id indexing; the direct path indexes by body position.
__global__ void k_adj_seed(const BodyArrays b, const double* sx, const double* sy, const double* sz, double* lx,
                           double* ly, double* lz, double* lvx, double* lvy, double* lvz, double* lm, double* loss_terms,
                           int n, int by_id) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = b.id[i];
    const uint32_t k = by_id ? id : static_cast<uint32_t>(i);
    lx[k] = sx[id]; ly[k] = sy[id]; lz[k] = sz[id];
    lvx[k] = lvy[k] = lvz[k] = 0;
    lm[k] = 0;
    loss_terms[k] = 0;
}

// Terminal adjoints indexed by id.
__global__ void k_adj_init_id(const BodyArrays b, const double* tx, const double* ty, const double* tz, double* lx,
                              double* ly, double* lz, double* lvx, double* lvy, double* lvz, double* lm,
                              double* loss_terms, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = b.id[i];
    const double m = b.m[i];
    const double dx = b.x[i] - tx[id], dy = b.y[i] - ty[id], dz = b.z[i] - tz[id];
    lx[id] = 2 * m * dx; ly[id] = 2 * m * dy; lz[id] = 2 * m * dz;
    lvx[id] = lvy[id] = lvz[id] = 0;
    const double d2 = dx * dx + dy * dy + dz * dz;
    lm[id] = d2;
    loss_terms[id] = m * d2;
}

__global__ void k_copy_hilo(const BodyArrays b, float4* hm, float4* lo, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    hm[i] = b.hm[i];
    lo[i] = b.lo[i];
}

}  // namespace

// ---- host orchestration ------------------------------------------------------------------------
struct AdjointState {
    int n = 0, steps = 0, every = 0, nck = 0;
    double dt = 0;
    lg_force_params p{};
    DevBuf ck_x, ck_y, ck_z, ck_vx, ck_vy, ck_vz, ck_m, ck_id;  // checkpoints, nck * n each
    DevBuf seg_hm[2], seg_lo[2];                   // direct: two segments' positions, every * n float4 each
    DevBuf seg_x, seg_y, seg_z, seg_id;            // tree: one segment's sorted FP64 positions and ids
    DevBuf m_by_id, w_sorted, gbuf;                // tree: masses by id, weights in body order, VJP output
    DevBuf lx, ly, lz, lvx, lvy, lvz, lm, loss_terms, w, partial;
    DevBuf sym_units, sym_sbase, ipart, jpart;     // direct: the symmetric VJP's schedule and partial sums
    std::vector<int4> sym_units_h;                 // (host copies, alive while their uploads run)
    std::vector<int> sym_sbase_h;
    DevBuf tx, ty, tz;
    bool have_forward = false;
};

namespace {
void destroy_adjoint(AdjointState* a) { delete a; }
}  // namespace

std::unique_ptr<AdjointState, void (*)(AdjointState*)> make_adjoint_state() {
    return std::unique_ptr<AdjointState, void (*)(AdjointState*)>(new AdjointState, destroy_adjoint);
}

namespace {

void save_ck(Engine& e, AdjointState& a, int slot) {
    const size_t off = static_cast<size_t>(slot) * a.n;
    k_save<<<grid_for(a.n, 256), 256, 0, e.stream>>>(e.bodies(e.cur), a.ck_x.as<double>() + off, a.ck_y.as<double>() + off,
                                                   a.ck_z.as<double>() + off, a.ck_vx.as<float>() + off,
                                                   a.ck_vy.as<float>() + off, a.ck_vz.as<float>() + off,
                                                   a.ck_m.as<float>() + off, a.ck_id.as<uint32_t>() + off, a.n);
    LG_LAUNCHED();
    ++e.launches;
}

void restore_ck(Engine& e, AdjointState& a, int slot) {
    const size_t off = static_cast<size_t>(slot) * a.n;
    k_restore<<<grid_for(a.n, 256), 256, 0, e.stream>>>(e.bodies(e.cur), a.ck_x.as<double>() + off,
                                                      a.ck_y.as<double>() + off, a.ck_z.as<double>() + off,
                                                      a.ck_vx.as<float>() + off, a.ck_vy.as<float>() + off,
                                                      a.ck_vz.as<float>() + off, a.ck_m.as<float>() + off,
                                                      a.ck_id.as<uint32_t>() + off, a.n);
    LG_LAUNCHED();
    ++e.launches;
}

// Tree forces through the engine's own build and walk (sizes checked, as every force call).
void tree_forces(Engine& e, const lg_force_params& p) {
    e.build_tree(p);
    e.compute_forces_with(p, false, nullptr, 0);
}

void kdk_step_tree(Engine& e, const lg_force_params& p, double dt) {
    e.kick(0.5 * dt);
    e.drift(dt);
    tree_forces(e, p);
    e.kick(0.5 * dt);
}

void store_step(Engine& e, AdjointState& a, int slot) {
    const size_t so = static_cast<size_t>(slot) * a.n;
    k_store_step<<<grid_for(a.n, 256), 256, 0, e.stream>>>(e.bodies(e.cur), a.seg_x.as<double>() + so,
                                                         a.seg_y.as<double>() + so, a.seg_z.as<double>() + so,
                                                         a.seg_id.as<uint32_t>() + so, a.n);
    LG_LAUNCHED();
    ++e.launches;
}

void direct_forces(Engine& e, const lg_force_params& p) {
    const float G = static_cast<float>(p.G), e2 = static_cast<float>(p.eps * p.eps);
    const bool eps0 = !(e2 >= 1.17549435e-38f);
    DirectShape sh = e.direct_shape_override.ipt ? e.direct_shape_override : default_direct_shape(e.n, e.sms);
    if (sh.slices > 1) e.partial.reserve(static_cast<size_t>(sh.slices) * e.n * 16 + 16 * 1024);
    launch_direct(e.bodies(e.cur), e.n, G, e2, false, eps0, sh, e.acc.as<float4>(), e.partial.as<float4>(), e.err_word(),
                  e.stream);
    e.launches += sh.slices > 1 ? 2 : 1;
}

void kdk_step(Engine& e, const lg_force_params& p, double dt) {
    launch_kick(e.bodies(e.cur), e.acc.as<float4>(), static_cast<float>(0.5 * dt), e.n, e.stream);
    launch_drift(e.bodies(e.cur), dt, e.n, e.stream);
    direct_forces(e, p);
    launch_kick(e.bodies(e.cur), e.acc.as<float4>(), static_cast<float>(0.5 * dt), e.n, e.stream);
    e.launches += 3;
}

}  // namespace

void adjoint_forward(Engine& e, AdjointState& a, const lg_force_params& p, double dt, int steps, int every) {
    if (p.method != LG_DIRECT && p.method != LG_TREE) fail(kArg, "adjoint: unknown force method");
    const bool tree = p.method == LG_TREE;
    if (steps < 1 || every < 1) fail(kArg, "adjoint: steps and checkpoint interval must be positive");
    LG_CK(cudaSetDevice(e.dev));
    const int n = e.n;
    if (n < 1) fail(kArg, "adjoint: no bodies");
    a.n = n;
    a.steps = steps;
    a.every = every;
    a.dt = dt;
    a.p = p;
    a.nck = (steps + every - 1) / every + 1;
    const size_t cn = static_cast<size_t>(a.nck) * n;
    a.ck_x.reserve(cn * 8); a.ck_y.reserve(cn * 8); a.ck_z.reserve(cn * 8);
    a.ck_vx.reserve(cn * 4); a.ck_vy.reserve(cn * 4); a.ck_vz.reserve(cn * 4);
    a.ck_m.reserve(cn * 4); a.ck_id.reserve(cn * 4);
    if (tree) {
        // Ids index the adjoint state: they must be a permutation of 0..n-1.
        std::vector<uint32_t> ids(static_cast<size_t>(n));
        LG_CK(cudaMemcpyAsync(ids.data(), e.bodies(e.cur).id, static_cast<size_t>(n) * 4, cudaMemcpyDeviceToHost,
                              e.stream));
        LG_CK(cudaStreamSynchronize(e.stream));
        std::vector<char> seen(static_cast<size_t>(n), 0);
        for (uint32_t k : ids) {
            if (k >= static_cast<uint32_t>(n) || seen[k]) fail(kArg, "adjoint (tree): body ids must be 0..n-1");
            seen[k] = 1;
        }
        tree_forces(e, p);
    } else {
        direct_forces(e, p);
    }
    save_ck(e, a, 0);
    for (int s = 0; s < steps; ++s) {
        if (tree) kdk_step_tree(e, p, dt);
        else kdk_step(e, p, dt);
        if ((s + 1) % every == 0 && s + 1 < steps) save_ck(e, a, (s + 1) / every);
    }
    e.acc_ok = true;
    e.has_pe = false;
    e.tree_ok = tree;
    e.costs_ok = tree;
    a.have_forward = true;
    LG_CK(cudaStreamSynchronize(e.stream));
    e.check_device_errors("adjoint forward");
}

double adjoint_backward(Engine& e, AdjointState& a, const double* tx, const double* ty, const double* tz, double* gx,
                        double* gy, double* gz, double* gvx, double* gvy, double* gvz, double* gm, bool seeded) {
    if (!a.have_forward || a.n != e.n) fail(kLogic, "adjoint backward: run the adjoint forward pass first");
    LG_CK(cudaSetDevice(e.dev));
    const int n = a.n;
    const bool tree = a.p.method == LG_TREE;
    cudaStream_t s = e.stream;
    const size_t nb8 = static_cast<size_t>(n) * 8;
    for (DevBuf* d : {&a.lx, &a.ly, &a.lz, &a.lvx, &a.lvy, &a.lvz, &a.lm, &a.loss_terms, &a.tx, &a.ty, &a.tz})
        d->reserve(nb8);
    a.w.reserve(static_cast<size_t>(n) * 16);
    const size_t seg_n = static_cast<size_t>(a.every) * n;
    if (tree) {
        a.seg_x.reserve(seg_n * 8); a.seg_y.reserve(seg_n * 8); a.seg_z.reserve(seg_n * 8);
        a.seg_id.reserve(seg_n * 4);
        a.m_by_id.reserve(static_cast<size_t>(n) * 4);
        a.w_sorted.reserve(static_cast<size_t>(n) * 16);
        a.gbuf.reserve(static_cast<size_t>(n) * 32);
    } else {
        for (int b = 0; b < 2; ++b) {
            a.seg_hm[b].reserve(seg_n * 16);
            a.seg_lo[b].reserve(seg_n * 16);
        }
    }
    LG_CK(cudaMemcpyAsync(a.tx.as<double>(), tx, nb8, cudaMemcpyHostToDevice, s));
    LG_CK(cudaMemcpyAsync(a.ty.as<double>(), ty, nb8, cudaMemcpyHostToDevice, s));
    LG_CK(cudaMemcpyAsync(a.tz.as<double>(), tz, nb8, cudaMemcpyHostToDevice, s));
    const int gb = grid_for(n, 256);
    // The forward pass left the final state resident: terminal adjoints from it (by body index for
    // the direct path, whose order never changes; by id for the tree path).
    if (seeded) {
        k_adj_seed<<<gb, 256, 0, s>>>(e.bodies(e.cur), a.tx.as<double>(), a.ty.as<double>(), a.tz.as<double>(),
                                      a.lx.as<double>(), a.ly.as<double>(), a.lz.as<double>(), a.lvx.as<double>(),
                                      a.lvy.as<double>(), a.lvz.as<double>(), a.lm.as<double>(), a.loss_terms.as<double>(),
                                      n, tree ? 1 : 0);
        LG_LAUNCHED();
        if (tree) {
            k_mass_by_id<<<gb, 256, 0, s>>>(e.bodies(e.cur), a.m_by_id.as<float>(), n);
            LG_LAUNCHED();
        }
    } else if (tree) {
        k_adj_init_id<<<gb, 256, 0, s>>>(e.bodies(e.cur), a.tx.as<double>(), a.ty.as<double>(), a.tz.as<double>(),
                                         a.lx.as<double>(), a.ly.as<double>(), a.lz.as<double>(), a.lvx.as<double>(),
                                         a.lvy.as<double>(), a.lvz.as<double>(), a.lm.as<double>(),
                                         a.loss_terms.as<double>(), n);
        LG_LAUNCHED();
        k_mass_by_id<<<gb, 256, 0, s>>>(e.bodies(e.cur), a.m_by_id.as<float>(), n);
        LG_LAUNCHED();
    } else {
        k_adj_init<<<gb, 256, 0, s>>>(e.bodies(e.cur), a.tx.as<double>(), a.ty.as<double>(), a.tz.as<double>(),
                                      a.lx.as<double>(), a.ly.as<double>(), a.lz.as<double>(), a.lvx.as<double>(),
                                      a.lvy.as<double>(), a.lvz.as<double>(), a.lm.as<double>(), a.loss_terms.as<double>(),
                                      n);
        LG_LAUNCHED();
    }
    std::vector<double> terms(static_cast<size_t>(n));
    LG_CK(cudaMemcpyAsync(terms.data(), a.loss_terms.as<double>(), nb8, cudaMemcpyDeviceToHost, s));
    // Direct VJP launch shape: whole waves over split-j slices.
    const int iblocks = (n + VBS * VIPT - 1) / (VBS * VIPT);
    static int vjp_per_sm = 0;
    if (!vjp_per_sm) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&vjp_per_sm, k_vjp<false>, VBS, 0) != cudaSuccess) {
            cudaGetLastError();
            vjp_per_sm = 2;
        }
        if (vjp_per_sm < 1) vjp_per_sm = 1;
    }
    int slices = std::max(1, std::min(n / 128 + 1, (vjp_per_sm * e.sms + iblocks - 1) / iblocks));
    int jslice = (n + slices - 1) / slices;
    slices = (n + jslice - 1) / jslice;
    // Symmetric VJP (each unordered pair once) when there are enough tile units to fill the GPU
    // (at least four per SM: about 26k bodies and up; below that the one-sided kernel's split-j
    // grid fills it better) and its partial sums stay within 4 GB (about 250k bodies).
    // LETTUCE_GB300_VJP=pairs or =symmetric overrides the size rule (not the memory bound).
    const int T = (n + STILE - 1) / STILE;
    const int npad = T * STILE;
    const size_t jbytes = static_cast<size_t>(STILE) * T * (T + 1) / 2 * 32;
    long long units_needed = 0;  // one block per strip of up to SSTRIP tiles: sum over I of ceil((T - I) / SSTRIP)
    for (int I = 0; I < T; ++I) units_needed += (T - I + SSTRIP - 1) / SSTRIP;
    const bool fits = jbytes + static_cast<size_t>(units_needed) * STILE * 32 <= (size_t(4) << 30);
    bool sym = !tree && fits && units_needed >= 4LL * e.sms;
    if (const char* v = std::getenv("LETTUCE_GB300_VJP")) {
        const std::string m = v;
        if (m != "pairs" && m != "symmetric") fail(kRuntime, "LETTUCE_GB300_VJP must be pairs or symmetric, not '" + m + "'");
        sym = !tree && fits && m == "symmetric";
    }
    int nunits = 0;
    if (sym) {
        a.sym_units_h.clear();
        a.sym_sbase_h.assign(static_cast<size_t>(T) + 1, 0);
        int strip = 0;
        for (int I = 0; I < T; ++I) {
            a.sym_sbase_h[I] = strip;
            for (int J0 = I; J0 < T; J0 += SSTRIP) a.sym_units_h.push_back(make_int4(I, J0, std::min(T, J0 + SSTRIP), strip++));
        }
        a.sym_sbase_h[T] = strip;
        // Whole strips first, the shorter ones last: the grid's last wave holds the smallest blocks.
        std::stable_sort(a.sym_units_h.begin(), a.sym_units_h.end(),
                         [](const int4& p, const int4& q) { return p.z - p.y > q.z - q.y; });
        nunits = static_cast<int>(a.sym_units_h.size());
        a.sym_units.reserve(a.sym_units_h.size() * sizeof(int4));
        a.sym_sbase.reserve(a.sym_sbase_h.size() * sizeof(int));
        LG_CK(cudaMemcpyAsync(a.sym_units.as<int4>(), a.sym_units_h.data(), a.sym_units_h.size() * sizeof(int4),
                              cudaMemcpyHostToDevice, s));
        LG_CK(cudaMemcpyAsync(a.sym_sbase.as<int>(), a.sym_sbase_h.data(), a.sym_sbase_h.size() * sizeof(int),
                              cudaMemcpyHostToDevice, s));
        a.ipart.reserve(static_cast<size_t>(strip) * STILE * 32);
        a.jpart.reserve(jbytes);
    } else if (!tree) {
        a.partial.reserve(static_cast<size_t>(slices) * n * 16);
    }
    const float e2 = static_cast<float>(a.p.eps * a.p.eps);
    const bool eps0 = !(e2 >= 1.17549435e-38f);
    const double h = 0.5 * a.dt;
    // Recomputes segment seg (checkpoint restore, then the segment's positions; the forces at the
    // segment's last position and the closing kick after them are skipped, so a segment of k steps
    // costs k - 1 force evaluations). Direct: into segment buffer seg & 1.
    auto recompute = [&](int seg) {
        const int s0 = seg * a.every, s1 = std::min(a.steps, s0 + a.every);
        restore_ck(e, a, seg);
        const bool more = s1 - s0 >= 2;
        if (tree) {
            if (more) tree_forces(e, a.p);
            store_step(e, a, 0);
            for (int st = s0; st < s1 - 1; ++st) {
                e.kick(0.5 * a.dt);
                e.drift(a.dt);
                if (st + 1 < s1 - 1) {
                    tree_forces(e, a.p);
                    e.kick(0.5 * a.dt);
                }
                // Unsorted at the last step: the VJP's rebuild sorts it as the forward pass did.
                store_step(e, a, st - s0 + 1);
            }
        } else {
            float4* hm = a.seg_hm[seg & 1].as<float4>();
            float4* lo = a.seg_lo[seg & 1].as<float4>();
            if (more) direct_forces(e, a.p);
            k_copy_hilo<<<gb, 256, 0, s>>>(e.bodies(e.cur), hm, lo, n);
            LG_LAUNCHED();
            for (int st = s0; st < s1 - 1; ++st) {
                launch_kick(e.bodies(e.cur), e.acc.as<float4>(), static_cast<float>(0.5 * a.dt), n, s);
                launch_drift(e.bodies(e.cur), a.dt, n, s);
                e.launches += 2;
                if (st + 1 < s1 - 1) {
                    direct_forces(e, a.p);
                    launch_kick(e.bodies(e.cur), e.acc.as<float4>(), static_cast<float>(0.5 * a.dt), n, s);
                    ++e.launches;
                }
                const size_t so = static_cast<size_t>(st - s0 + 1) * n;
                k_copy_hilo<<<gb, 256, 0, s>>>(e.bodies(e.cur), hm + so, lo + so, n);
                LG_LAUNCHED();
            }
            e.launches += 1 + (s1 - 1 - s0);
        }
    };
    // Reverse sweep through segment seg on stream vs (direct: from segment buffer seg & 1).
    auto sweep = [&](int seg, cudaStream_t vs) {
        const int s0 = seg * a.every, s1 = std::min(a.steps, s0 + a.every);
        for (int st = s1 - 1; st >= s0; --st) {
            const double c = st > 0 ? a.dt : h;
            k_adj_kick<<<gb, 256, 0, vs>>>(a.lx.as<double>(), a.ly.as<double>(), a.lz.as<double>(), a.lvx.as<double>(),
                                           a.lvy.as<double>(), a.lvz.as<double>(), a.dt, c, a.w.as<float4>(), n);
            LG_LAUNCHED();
            const size_t so = static_cast<size_t>(st - s0) * n;
            if (tree) {
                // The step's sorted positions, then an exact rebuild of its tree.
                k_load_step<<<gb, 256, 0, s>>>(e.bodies(e.cur), a.seg_x.as<double>() + so, a.seg_y.as<double>() + so,
                                               a.seg_z.as<double>() + so, a.seg_id.as<uint32_t>() + so,
                                               a.m_by_id.as<float>(), n);
                LG_LAUNCHED();
                tree_reset_guess(e);
                e.build_tree(a.p);
                k_gather_w<<<gb, 256, 0, s>>>(e.bodies(e.cur), a.w.as<float4>(), a.w_sorted.as<float4>(), n);
                LG_LAUNCHED();
                LG_CK(cudaMemsetAsync(a.gbuf.as<double>(), 0, static_cast<size_t>(n) * 32, s));
                tree_walk_vjp(e, a.w_sorted.as<float4>(), e2, eps0, a.gbuf.as<double>());
                k_tree_vjp_apply<<<gb, 256, 0, s>>>(e.bodies(e.cur), a.gbuf.as<double>(), n, a.p.G, a.lx.as<double>(),
                                                    a.ly.as<double>(), a.lz.as<double>(), a.lm.as<double>());
                LG_LAUNCHED();
                e.launches += 4;
                LG_CK(cudaMemcpyAsync(e.pinned_small, e.err_word(), 4, cudaMemcpyDeviceToHost, s));
                LG_CK(cudaStreamSynchronize(s));
                e.check_device_errors("adjoint backward (tree VJP)");
            } else {
                const float4* hm = a.seg_hm[seg & 1].as<float4>() + so;
                const float4* lo = a.seg_lo[seg & 1].as<float4>() + so;
                if (sym) {
                    if (eps0)
                        k_vjp_sym<true><<<nunits, SBS, 0, vs>>>(hm, lo, a.w.as<float4>(), n, npad, e2,
                                                                a.sym_units.as<int4>(), a.ipart.as<float>(),
                                                                a.jpart.as<float>());
                    else
                        k_vjp_sym<false><<<nunits, SBS, 0, vs>>>(hm, lo, a.w.as<float4>(), n, npad, e2,
                                                                 a.sym_units.as<int4>(), a.ipart.as<float>(),
                                                                 a.jpart.as<float>());
                    LG_LAUNCHED();
                    k_vjp_sym_apply<<<gb, 256, 0, vs>>>(a.ipart.as<float>(), a.jpart.as<float>(), a.sym_sbase.as<int>(),
                                                        hm, a.w.as<float4>(), n, npad, a.p.G, a.lx.as<double>(),
                                                        a.ly.as<double>(), a.lz.as<double>(), a.lm.as<double>());
                    LG_LAUNCHED();
                    e.launches += 3;
                    continue;
                }
                dim3 grid(iblocks, slices);
                if (eps0)
                    k_vjp<true><<<grid, VBS, 0, vs>>>(hm, lo, a.w.as<float4>(), n, jslice, e2, a.partial.as<float4>());
                else
                    k_vjp<false><<<grid, VBS, 0, vs>>>(hm, lo, a.w.as<float4>(), n, jslice, e2, a.partial.as<float4>());
                LG_LAUNCHED();
                k_vjp_apply<<<gb, 256, 0, vs>>>(a.partial.as<float4>(), n, slices, a.p.G, a.lx.as<double>(),
                                                a.ly.as<double>(), a.lz.as<double>(), a.lm.as<double>());
                LG_LAUNCHED();
                e.launches += 3;
            }
        }
    };
    const int last = (a.steps - 1) / a.every;
    if (tree) {
        // The tree VJP rebuilds trees through the engine: one stream, segment after segment.
        for (int seg = last; seg >= 0; --seg) {
            recompute(seg);
            sweep(seg, s);
        }
    } else {
        // Direct: the sweep of segment seg runs on the side stream while the main stream recomputes
        // segment seg - 1 into the other buffer (the two are independent; the GPU takes both at
        // once). A sweep waits for its segment's recompute; a recompute waits for the sweep that
        // last read its buffer. The operations and their order per stream are unchanged, so the
        // gradients are those of the one-stream sweep bit for bit.
        cudaEvent_t ev[5];
        for (auto& x : ev) LG_CK(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
        cudaEvent_t* rec_done = ev;        // [buffer]
        cudaEvent_t* sweep_done = ev + 2;  // [buffer]
        LG_CK(cudaEventRecord(ev[4], s));  // the adjoint state's initialisation
        LG_CK(cudaStreamWaitEvent(e.side, ev[4], 0));
        bool used[2] = {false, false};
        recompute(last);
        LG_CK(cudaEventRecord(rec_done[last & 1], s));
        for (int seg = last; seg >= 0; --seg) {
            LG_CK(cudaStreamWaitEvent(e.side, rec_done[seg & 1], 0));
            sweep(seg, e.side);
            LG_CK(cudaEventRecord(sweep_done[seg & 1], e.side));
            used[seg & 1] = true;
            if (seg > 0) {
                const int b = (seg - 1) & 1;
                if (used[b]) LG_CK(cudaStreamWaitEvent(s, sweep_done[b], 0));
                recompute(seg - 1);
                LG_CK(cudaEventRecord(rec_done[b], s));
            }
        }
        LG_CK(cudaEventRecord(ev[4], e.side));
        LG_CK(cudaStreamWaitEvent(s, ev[4], 0));
        LG_CK(cudaStreamSynchronize(s));
        for (auto& x : ev) cudaEventDestroy(x);
    }
    // Gradients in id order.
    std::vector<uint32_t> ids(static_cast<size_t>(n));
    LG_CK(cudaMemcpyAsync(ids.data(), e.bodies(e.cur).id, static_cast<size_t>(n) * 4, cudaMemcpyDeviceToHost, s));
    std::vector<double> buf(static_cast<size_t>(n) * 7);
    DevBuf* outs[7] = {&a.lx, &a.ly, &a.lz, &a.lvx, &a.lvy, &a.lvz, &a.lm};
    for (int k = 0; k < 7; ++k)
        LG_CK(cudaMemcpyAsync(buf.data() + static_cast<size_t>(k) * n, outs[k]->as<double>(), nb8, cudaMemcpyDeviceToHost, s));
    LG_CK(cudaStreamSynchronize(s));
    e.check_device_errors("adjoint backward");
    double* dst[7] = {gx, gy, gz, gvx, gvy, gvz, gm};
    for (int k = 0; k < 7; ++k)
        if (dst[k])
            for (int i = 0; i < n; ++i) dst[k][tree ? static_cast<uint32_t>(i) : ids[i]] = buf[static_cast<size_t>(k) * n + i];
    double L = 0;
    for (double t : terms) L += t;
    // The backward pass replayed the segments: the forward's final state is no longer resident.
    a.have_forward = false;
    e.acc_ok = false;
    e.tree_ok = false;
    return L;
}

}  // namespace lg
