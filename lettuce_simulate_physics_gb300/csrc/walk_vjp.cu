// Vector-Jacobian product of the tree forces (the adjoint's tree step). No counterpart in the
// reference.
//
// The forces of a tree step are a_i = G [sum over the cells c of i's group list A_c(d) + sum over
// the bodies j of its body ranges m_j K(d)], d = (cell centre of mass or x_j) - x_i,
//   A_c(d) = M d / r^3 - Q d / r^5 + 5/2 (d.Q.d) d / r^7,  K(d) = d / r^3,  r^2 = |d|^2 + eps^2,
// with the lists fixed by the tree (walk.cu, the reference's opening rule) and the cell moments
// M = sum m_b, com = sum m_b x_b / M, Q = sum m_b (3 e e^T - |e|^2 I), e = x_b - com, functions of
// the bodies below the cell. With the lists held fixed ("frozen": the backward pass rebuilds the
// same tree from bit-identical positions), this file computes, for weights w_i,
//   g = d(sum_i w_i . a_i / G) / d(x, m).
//
// Per (i, entry) with u = w_i . d, q = d.Q.d, Qd = Q d, Qw = Q w_i:
//   body j:  gd = m_j (w_i / r^3 - 3 u d / r^5);  dm_j += u / r^3
//   cell c:  gd = (M/r^3 + 5/2 q/r^7) w_i + (-3 M u/r^5 + 5 (w_i.Qd)/r^7 - 35/2 q u/r^9) d
//                 - Qw/r^5 + 5 u Qd / r^7
//            dM_c += u / r^3;  dQ_kl += -(w_k d_l + w_l d_k)/r^5 + 5 u d_k d_l / r^7 (k != l),
//            dQ_kk += -w_k d_k / r^5 + 5/2 u d_k^2 / r^7
//   and dx_i -= gd, dX_entry += gd (X = x_j or the cell's centre of mass).
// The self pair (j == i) is skipped: d is identically zero, so it has no derivative.
// The cell adjoints (dM, dcom, dQ) then reach the bodies through the moment definitions
// (k_moment_chain): for every ancestor cell c of body b, with e = x_b - com_c,
//   dx_b += (m_b/M) dcom + m_b [6 dQ_diag e - 2 tr(dQ) e + 3 offdiag terms]
//   dm_b += dM + e . dcom / M + sum_kl dQ_kl (3 e_k e_l - |e|^2 delta_kl)  (stored components)
// (the derivative of Q through com vanishes because sum_b m_b e_b = 0).
//
// Kernel shape: one warp per walk group, the force walk's traversal (walk_common.cuh). Each list
// chunk is converted once to group-relative FP32 coordinates in shared memory and evaluated twice:
// lanes over i-bodies for the i side (Kahan sums in shared memory), and lanes over entries, looping
// over the group's i-bodies, for the entry side (sums per entry added to FP64 adjoint arrays with
// atomics). Both evaluate two pairs per packed f32x2 instruction.
#include "engine.cuh"
#include "walk_common.cuh"

namespace lg {

namespace {

using namespace walk;

constexpr int VWBS = 64;  // 2 warps per block
constexpr int VWARPS = VWBS / 32;
#ifndef LG_VJP_CCH
#define LG_VJP_CCH 128
#endif
#ifndef LG_VJP_BCH
#define LG_VJP_BCH 256
#endif
constexpr int VCCH = LG_VJP_CCH;  // cells per chunk (even)
constexpr int VBCH = LG_VJP_BCH;  // bodies per chunk (even)
static_assert(VCCH % 2 == 0 && VBCH % 2 == 0, "odd chunks are padded to whole pairs");
constexpr int VPASS = 128;
constexpr int VIPT = VPASS / 32;
constexpr int NADJ = 10;  // per node: dM, dcom (3), dQ (xx, xy, xz, yy, yz, zz)

struct __align__(16) VjpSmem {
    union {  // a flush converts its cells, then its bodies: the two chunks share the space
        struct {
            float cx[VCCH], cy[VCCH], cz[VCCH], cm[VCCH], qxx[VCCH], qxy[VCCH], qxz[VCCH], qyy[VCCH], qyz[VCCH],
                qzz[VCCH];
        };
        struct {
            float bx[VBCH], by[VBCH], bz[VBCH], bm[VBCH];
            uint32_t bj[VBCH];
        };
    };
    float ix[VPASS], iy[VPASS], iz[VPASS], iwx[VPASS], iwy[VPASS], iwz[VPASS];
    int kself[VPASS];  // per i-body: its position in the current body chunk, or -2
    float ks[VIPT][6][32];  // i-side Kahan sums of gd (x, y, z) and compensations
    uint32_t clist[CL_CAP];
    uint2 rlist[RL_CAP];
    uint32_t rpre[RL_CAP + 1];
    uint32_t sstk[SSTK];  // traversal stack (shared part)
};

struct VjpArgs {
    TreeView tv;
    const float4* hm;
    const float4* lo;
    const float4* w;
    double* gx;
    double* gy;
    double* gz;
    double* gm;
    double* nadj;  // NADJ arrays of T doubles
    uint32_t* stack;
    unsigned* group_ctr;
    unsigned* err;
    float e2;
};

template <bool EPS0>
__device__ __forceinline__ float inv_r(float r2) {
    const float v = rsqrt_mufu(r2);
    return EPS0 ? (r2 > 0.f ? v : 0.f) : v;
}

// Adds (x, y, z) to the Kahan sums of i-body i (slot lane i % 32 of pass i / 32).
__device__ __forceinline__ void kahan3(VjpSmem& s, int i, float x, float y, float z) {
    float* k = &s.ks[i >> 5][0][i & 31];
    float sx = k[0], sy = k[32], sz = k[64], cx = k[96], cy = k[128], cz = k[160];
    kahan_add(sx, cx, x);
    kahan_add(sy, cy, y);
    kahan_add(sz, cz, z);
    k[0] = sx; k[32] = sy; k[64] = sz; k[96] = cx; k[128] = cy; k[160] = cz;
}

// Entry partitions of the i-side loops: the warp's lanes form P groups of 32 / P lanes, each
// holding every i-body and taking every P-th entry pair; P (1, 2 or 4) is the one with the least
// lane work for np i-bodies (ties to the smaller P). Warp-uniform.
__device__ __forceinline__ int vjp_parts(int np) {
    const int w1 = 4 * ((np + 31) >> 5), w2 = 2 * ((np + 15) >> 4), w4 = (np + 7) >> 3;  // quarter sweeps
    return w4 < w2 && w4 < w1 ? 4 : (w2 < w1 ? 2 : 1);
}

// Sum of v over the P partitions (lanes lane, lane ^ Lw, ...); every lane takes part.
__device__ __forceinline__ float part_sum(float v, int P) {
    if (P >= 4) v += __shfl_xor_sync(0xffffffffu, v, 8);
    if (P >= 2) v += __shfl_xor_sync(0xffffffffu, v, 16);
    return v;
}

// Two adjacent floats of a shared-memory array as one packed pair (k even).
__device__ __forceinline__ f2x ld2(const float* p, int k) { return *reinterpret_cast<const f2x*>(p + k); }

template <bool EPS0>
__device__ __forceinline__ f2x inv_r2(f2x r2) {
    float lo, hi;
    f2_unpack(r2, lo, hi);
    return f2_pack(inv_r<EPS0>(lo), inv_r<EPS0>(hi));
}

// Cell term for two (body, cell) pairs at once: gd for weight w at offset d (cell minus body); also
// u = w.d, u / r^3, D = 5 u / r^7 and n5 = -1 / r^5, which the entry side reuses.
struct CellJ2 {
    f2x gdx, gdy, gdz, u, inv3, D, n5;
};

__device__ __forceinline__ CellJ2 cell_j2(f2x dx, f2x dy, f2x dz, f2x inv, f2x M, f2x qxx, f2x qxy, f2x qxz, f2x qyy,
                                          f2x qyz, f2x qzz, f2x wx, f2x wy, f2x wz) {
    const f2x C25 = f2_bcast(2.5f), C5 = f2_bcast(5.f), CN3 = f2_bcast(-3.f), CN175 = f2_bcast(-17.5f);
    const f2x CN1 = f2_bcast(-1.f);
    CellJ2 c;
    const f2x inv2 = f2_mul(inv, inv), inv3 = f2_mul(inv, inv2), inv5 = f2_mul(inv3, inv2);
    const f2x inv7 = f2_mul(inv5, inv2), inv9 = f2_mul(inv7, inv2);
    const f2x qx = f2_fma(qxx, dx, f2_fma(qxy, dy, f2_mul(qxz, dz)));
    const f2x qy = f2_fma(qxy, dx, f2_fma(qyy, dy, f2_mul(qyz, dz)));
    const f2x qz = f2_fma(qxz, dx, f2_fma(qyz, dy, f2_mul(qzz, dz)));
    const f2x q = f2_fma(dx, qx, f2_fma(dy, qy, f2_mul(dz, qz)));
    const f2x u = f2_fma(wx, dx, f2_fma(wy, dy, f2_mul(wz, dz)));
    const f2x qwx = f2_fma(qxx, wx, f2_fma(qxy, wy, f2_mul(qxz, wz)));
    const f2x qwy = f2_fma(qxy, wx, f2_fma(qyy, wy, f2_mul(qyz, wz)));
    const f2x qwz = f2_fma(qxz, wx, f2_fma(qyz, wy, f2_mul(qzz, wz)));
    const f2x wqd = f2_fma(wx, qx, f2_fma(wy, qy, f2_mul(wz, qz)));
    // A = M / r^3 + 5/2 q / r^7;  B = -3 M u / r^5 + 5 (w.Qd) / r^7 - 35/2 q u / r^9;  D = 5 u / r^7
    const f2x A = f2_fma(M, inv3, f2_mul(f2_mul(C25, q), inv7));
    const f2x B = f2_fma(f2_mul(CN3, f2_mul(M, u)), inv5,
                         f2_fma(f2_mul(C5, wqd), inv7, f2_mul(f2_mul(CN175, f2_mul(q, u)), inv9)));
    const f2x D = f2_mul(f2_mul(C5, u), inv7);
    const f2x n5 = f2_mul(CN1, inv5);
    c.gdx = f2_fma(A, wx, f2_fma(B, dx, f2_fma(D, qx, f2_mul(qwx, n5))));
    c.gdy = f2_fma(A, wy, f2_fma(B, dy, f2_fma(D, qy, f2_mul(qwy, n5))));
    c.gdz = f2_fma(A, wz, f2_fma(B, dz, f2_fma(D, qz, f2_mul(qwz, n5))));
    c.u = u;
    c.inv3 = inv3;
    c.D = D;
    c.n5 = n5;
    return c;
}

// One flush of the pending list: nc cells (s.clist) and nr body ranges (s.rlist) against the
// group's np i-bodies of this pass. Every loop evaluates two pairs per packed instruction: the
// i-side loops (lanes over i-bodies) take the entries two at a time, the entry-side loops (lanes
// over entries) take the i-bodies two at a time. Odd counts are padded with one zero-weight copy
// of the last element (cells: M = Q = 0; bodies: m = 0; i-bodies: w = 0), whose terms are exactly
// zero. The self pair (body j == body i) is removed by zeroing its half of the mass (i side) or of
// the weight (entry side).
template <bool EPS0>
__device__ void vjp_flush(const VjpArgs& a, VjpSmem& s, int lane, int np, uint32_t plo, int nc, int nr, float ox,
                          float oy, float oz, float e2) {
    const size_t T = a.tv.T;
    const f2x E2 = f2_bcast(e2), C05 = f2_bcast(0.5f), CN3 = f2_bcast(-3.f);
    const int P = vjp_parts(np), Lw = 32 / P, part = lane / Lw, lp = lane % Lw;
    const int nuP = (np + Lw - 1) / Lw;  // i-body rounds of the i-side loops (warp-uniform)
    const int npe = (np + 1) & ~1;
    // ---- cells
    for (int c0 = 0; c0 < nc; c0 += VCCH) {
        const int cc = min(VCCH, nc - c0);
        for (int k = lane; k < cc; k += 32) {
            const uint32_t nd = s.clist[c0 + k];
            const float4 com = a.tv.nd_com[nd], cl = a.tv.nd_comlo[nd], q0 = a.tv.nd_q0[nd], q1 = a.tv.nd_q1[nd];
            const float X = (com.x - ox) + cl.x, Y = (com.y - oy) + cl.y, Z = (com.z - oz) + cl.z;
            s.cx[k] = X; s.cy[k] = Y; s.cz[k] = Z;
            s.cm[k] = com.w;
            s.qxx[k] = q0.x; s.qxy[k] = q0.y; s.qxz[k] = q0.z; s.qyy[k] = q0.w; s.qyz[k] = q1.x; s.qzz[k] = q1.y;
            if (k == cc - 1 && (cc & 1)) {
                s.cx[cc] = X; s.cy[cc] = Y; s.cz[cc] = Z;
                s.cm[cc] = 0.f;
                s.qxx[cc] = 0.f; s.qxy[cc] = 0.f; s.qxz[cc] = 0.f; s.qyy[cc] = 0.f; s.qyz[cc] = 0.f; s.qzz[cc] = 0.f;
            }
        }
        __syncwarp();
        // i side: lanes over i-bodies, cells two at a time (every P-th pair per partition).
        for (int u = 0; u < nuP; ++u) {
            const int i = lp + Lw * u;
            const f2x xi = f2_bcast(s.ix[i]), yi = f2_bcast(s.iy[i]), zi = f2_bcast(s.iz[i]);
            const f2x wx = f2_bcast(s.iwx[i]), wy = f2_bcast(s.iwy[i]), wz = f2_bcast(s.iwz[i]);
            f2x ax = f2_bcast(0.f), ay = ax, az = ax;
#pragma unroll 2
            for (int k = 2 * part; k < cc; k += 2 * P) {
                const f2x dx = f2_sub(ld2(s.cx, k), xi), dy = f2_sub(ld2(s.cy, k), yi), dz = f2_sub(ld2(s.cz, k), zi);
                const f2x inv = inv_r2<EPS0>(f2_fma(dx, dx, f2_fma(dy, dy, f2_fma(dz, dz, E2))));
                const CellJ2 j = cell_j2(dx, dy, dz, inv, ld2(s.cm, k), ld2(s.qxx, k), ld2(s.qxy, k), ld2(s.qxz, k),
                                         ld2(s.qyy, k), ld2(s.qyz, k), ld2(s.qzz, k), wx, wy, wz);
                ax = f2_add(ax, j.gdx);
                ay = f2_add(ay, j.gdy);
                az = f2_add(az, j.gdz);
            }
            const float sx = part_sum(f2_sum(ax), P), sy = part_sum(f2_sum(ay), P), sz = part_sum(f2_sum(az), P);
            if (part == 0 && i < np) kahan3(s, i, sx, sy, sz);
        }
        // Entry side: lanes over cells, the group's i-bodies two at a time.
        for (int k = lane; k < cc; k += 32) {
            const f2x X = f2_bcast(s.cx[k]), Y = f2_bcast(s.cy[k]), Z = f2_bcast(s.cz[k]), M = f2_bcast(s.cm[k]);
            const f2x qxx = f2_bcast(s.qxx[k]), qxy = f2_bcast(s.qxy[k]), qxz = f2_bcast(s.qxz[k]);
            const f2x qyy = f2_bcast(s.qyy[k]), qyz = f2_bcast(s.qyz[k]), qzz = f2_bcast(s.qzz[k]);
            f2x G[NADJ];
#pragma unroll
            for (int f = 0; f < NADJ; ++f) G[f] = f2_bcast(0.f);
#pragma unroll 2
            for (int i = 0; i < npe; i += 2) {
                const f2x wx = ld2(s.iwx, i), wy = ld2(s.iwy, i), wz = ld2(s.iwz, i);
                const f2x dx = f2_sub(X, ld2(s.ix, i)), dy = f2_sub(Y, ld2(s.iy, i)), dz = f2_sub(Z, ld2(s.iz, i));
                const f2x inv = inv_r2<EPS0>(f2_fma(dx, dx, f2_fma(dy, dy, f2_fma(dz, dz, E2))));
                const CellJ2 j = cell_j2(dx, dy, dz, inv, M, qxx, qxy, qxz, qyy, qyz, qzz, wx, wy, wz);
                G[0] = f2_fma(j.u, j.inv3, G[0]);
                G[1] = f2_add(G[1], j.gdx);
                G[2] = f2_add(G[2], j.gdy);
                G[3] = f2_add(G[3], j.gdz);
                // dQ: with E = 5/2 u / r^7 = D / 2 and p = -w / r^5,
                //   dQ_kk += d_k (E d_k + p_k),  dQ_kl += d_l (D d_k + p_k) + p_l d_k  (k < l).
                const f2x E = f2_mul(C05, j.D);
                const f2x px = f2_mul(wx, j.n5), py = f2_mul(wy, j.n5), pz = f2_mul(wz, j.n5);
                const f2x Dx = f2_fma(j.D, dx, px), Dy = f2_fma(j.D, dy, py);
                G[4] = f2_fma(f2_fma(E, dx, px), dx, G[4]);
                G[5] = f2_fma(Dx, dy, f2_fma(py, dx, G[5]));
                G[6] = f2_fma(Dx, dz, f2_fma(pz, dx, G[6]));
                G[7] = f2_fma(f2_fma(E, dy, py), dy, G[7]);
                G[8] = f2_fma(Dy, dz, f2_fma(pz, dy, G[8]));
                G[9] = f2_fma(f2_fma(E, dz, pz), dz, G[9]);
            }
            const uint32_t nd = s.clist[c0 + k];
#pragma unroll
            for (int f = 0; f < NADJ; ++f) {
                const float g = f2_sum(G[f]);
                if (g != 0.f) atomicAdd(a.nadj + f * T + nd, static_cast<double>(g));
            }
        }
        __syncwarp();
    }
    if (nr == 0) return;
    // ---- bodies
    const int total = range_prefix(s, nr, lane);
    for (int b0 = 0; b0 < total; b0 += VBCH) {
        const int bc = min(VBCH, total - b0);
        for (int i = lane; i < np; i += 32) s.kself[i] = -2;
        __syncwarp();
        for (int k = lane; k < bc; k += 32) {
            const uint32_t j = range_body(s, nr, b0 + k);
            const float4 h = a.hm[j], l = a.lo[j];
            const float X = (h.x - ox) + l.x, Y = (h.y - oy) + l.y, Z = (h.z - oz) + l.z;
            s.bx[k] = X; s.by[k] = Y; s.bz[k] = Z;
            s.bm[k] = h.w;
            s.bj[k] = j;
            if (j - plo < static_cast<uint32_t>(np)) s.kself[j - plo] = k;
            if (k == bc - 1 && (bc & 1)) {
                s.bx[bc] = X; s.by[bc] = Y; s.bz[bc] = Z;
                s.bm[bc] = 0.f;
                s.bj[bc] = 0xffffffffu;
            }
        }
        __syncwarp();
        // i side: lanes over i-bodies, bodies two at a time (every P-th pair per partition). Per pair
        //   gd = m_j (w_i / r^3 - 3 u d / r^5)  is summed as  w_i sum m_j / r^3 + sum (-3 m_j u / r^5) d.
        for (int u = 0; u < nuP; ++u) {
            const int i = lp + Lw * u;
            const f2x xi = f2_bcast(s.ix[i]), yi = f2_bcast(s.iy[i]), zi = f2_bcast(s.iz[i]);
            const f2x wx = f2_bcast(s.iwx[i]), wy = f2_bcast(s.iwy[i]), wz = f2_bcast(s.iwz[i]);
            const int ks = i < np ? s.kself[i] : -2;
            f2x ax = f2_bcast(0.f), ay = ax, az = ax, s3 = ax;
#pragma unroll 2
            for (int k = 2 * part; k < bc; k += 2 * P) {
                f2x m = ld2(s.bm, k);
                if (static_cast<unsigned>(ks - k) <= 1u) m = f2_mul(m, ks == k ? f2_pack(0.f, 1.f) : f2_pack(1.f, 0.f));
                const f2x dx = f2_sub(ld2(s.bx, k), xi), dy = f2_sub(ld2(s.by, k), yi), dz = f2_sub(ld2(s.bz, k), zi);
                const f2x inv = inv_r2<EPS0>(f2_fma(dx, dx, f2_fma(dy, dy, f2_fma(dz, dz, E2))));
                const f2x inv2 = f2_mul(inv, inv), inv3 = f2_mul(inv, inv2), inv5 = f2_mul(inv3, inv2);
                const f2x uw = f2_fma(wx, dx, f2_fma(wy, dy, f2_mul(wz, dz)));
                const f2x t = f2_mul(f2_mul(CN3, f2_mul(m, uw)), inv5);
                s3 = f2_fma(m, inv3, s3);
                ax = f2_fma(t, dx, ax);
                ay = f2_fma(t, dy, ay);
                az = f2_fma(t, dz, az);
            }
            const float S = part_sum(f2_sum(s3), P);
            const float sx = part_sum(f2_sum(ax), P), sy = part_sum(f2_sum(ay), P), sz = part_sum(f2_sum(az), P);
            if (part == 0 && i < np) {
                const float wxs = s.iwx[i], wys = s.iwy[i], wzs = s.iwz[i];
                kahan3(s, i, fmaf(wxs, S, sx), fmaf(wys, S, sy), fmaf(wzs, S, sz));
            }
        }
        // Entry side: lanes over bodies, the group's i-bodies two at a time. Per pair
        //   dx_j += m_j (w_i / r^3 - 3 u d / r^5),  dm_j += u / r^3  (m_j applied after the sum).
        for (int k = lane; k < bc; k += 32) {
            const uint32_t j = s.bj[k];
            const int js = j - plo < static_cast<uint32_t>(np) ? static_cast<int>(j - plo) : -2;
            const f2x X = f2_bcast(s.bx[k]), Y = f2_bcast(s.by[k]), Z = f2_bcast(s.bz[k]);
            f2x GX = f2_bcast(0.f), GY = GX, GZ = GX, GM = GX;
#pragma unroll 2
            for (int i = 0; i < npe; i += 2) {
                f2x wx = ld2(s.iwx, i), wy = ld2(s.iwy, i), wz = ld2(s.iwz, i);
                if (static_cast<unsigned>(js - i) <= 1u) {
                    const f2x msk = js == i ? f2_pack(0.f, 1.f) : f2_pack(1.f, 0.f);
                    wx = f2_mul(wx, msk);
                    wy = f2_mul(wy, msk);
                    wz = f2_mul(wz, msk);
                }
                const f2x dx = f2_sub(X, ld2(s.ix, i)), dy = f2_sub(Y, ld2(s.iy, i)), dz = f2_sub(Z, ld2(s.iz, i));
                const f2x inv = inv_r2<EPS0>(f2_fma(dx, dx, f2_fma(dy, dy, f2_fma(dz, dz, E2))));
                const f2x inv2 = f2_mul(inv, inv), inv3 = f2_mul(inv, inv2), inv5 = f2_mul(inv3, inv2);
                const f2x uw = f2_fma(wx, dx, f2_fma(wy, dy, f2_mul(wz, dz)));
                const f2x t = f2_mul(f2_mul(CN3, uw), inv5);
                GX = f2_fma(wx, inv3, f2_fma(t, dx, GX));
                GY = f2_fma(wy, inv3, f2_fma(t, dy, GY));
                GZ = f2_fma(wz, inv3, f2_fma(t, dz, GZ));
                GM = f2_fma(uw, inv3, GM);
            }
            const float m = s.bm[k];
            atomicAdd(a.gx + j, static_cast<double>(m * f2_sum(GX)));
            atomicAdd(a.gy + j, static_cast<double>(m * f2_sum(GY)));
            atomicAdd(a.gz + j, static_cast<double>(m * f2_sum(GZ)));
            atomicAdd(a.gm + j, static_cast<double>(f2_sum(GM)));
        }
        __syncwarp();
    }
}

template <bool EPS0>
__global__ void __launch_bounds__(VWBS) k_walk_vjp(VjpArgs a) {
    __shared__ VjpSmem sm[VWARPS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    VjpSmem& s = sm[wid];
    uint32_t* stack = a.stack + (static_cast<size_t>(blockIdx.x) * VWARPS + wid) * SCAP;
    const unsigned ngroups = *a.tv.ngroups;
    for (;;) {
        unsigned g = 0;
        if (lane == 0) g = atomicAdd(a.group_ctr, 1u);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g >= ngroups) break;
        const uint2 gr = a.tv.grp_range[g];
        const float4 bc = a.tv.grp_box[2 * g], bh = a.tv.grp_box[2 * g + 1];
        for (uint32_t plo = gr.x; plo < gr.y; plo += VPASS) {
            const int np = static_cast<int>(min(static_cast<uint32_t>(VPASS), gr.y - plo));
            for (int i = lane; i < np; i += 32) {
                const float4 h = a.hm[plo + i], l = a.lo[plo + i], w = a.w[plo + i];
                const float x = (h.x - bc.x) + l.x, y = (h.y - bc.y) + l.y, z = (h.z - bc.z) + l.z;
                s.ix[i] = x;
                s.iy[i] = y;
                s.iz[i] = z;
                s.iwx[i] = w.x;
                s.iwy[i] = w.y;
                s.iwz[i] = w.z;
                if (i == np - 1 && (np & 1)) {  // zero-weight pad for the pairwise entry-side loops
                    s.ix[np] = x;
                    s.iy[np] = y;
                    s.iz[np] = z;
                    s.iwx[np] = 0.f;
                    s.iwy[np] = 0.f;
                    s.iwz[np] = 0.f;
                }
            }
#pragma unroll
            for (int u = 0; u < VIPT; ++u)
#pragma unroll
                for (int f = 0; f < 6; ++f) s.ks[u][f][lane] = 0.f;
            __syncwarp();
            uint32_t list_len = 0, cells_len = 0;
            traverse(a.tv, s, stack, lane, gr, bc, bh, 0u, a.err, list_len, cells_len,
                     [&](int nc, int nr) { vjp_flush<EPS0>(a, s, lane, np, plo, nc, nr, bc.x, bc.y, bc.z, a.e2); });
#pragma unroll
            for (int u = 0; u < VIPT; ++u) {
                const int i = lane + 32 * u;
                if (i >= np) continue;
                const float* k = &s.ks[u][0][lane];
                atomicAdd(a.gx + plo + i, -static_cast<double>(k[0] - k[96]));
                atomicAdd(a.gy + plo + i, -static_cast<double>(k[32] - k[128]));
                atomicAdd(a.gz + plo + i, -static_cast<double>(k[64] - k[160]));
            }
            __syncwarp();
        }
    }
}

// Cell adjoints to bodies through the moment definitions (every ancestor of the body's leaf).
__global__ void k_moment_chain(TreeView tv, const BodyArrays b, int n, const double* __restrict__ nadj, double* gx,
                               double* gy, double* gz, double* gm, unsigned* err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t T = tv.T;
    const uint32_t leaf = tv.body_leaf[i];
    if (leaf >= min(static_cast<size_t>(*tv.nleaves), tv.K)) {
        atomicOr(err, kErrNodeOverflow);
        return;
    }
    uint32_t node = tv.leaf_node[leaf];
    const double xb = b.x[i], yb = b.y[i], zb = b.z[i], mb = b.m[i];
    double ax = 0, ay = 0, az = 0, am = 0;
    for (int guard = 0; node < T && guard < 128; ++guard) {
        const double dM = nadj[node], dcx = nadj[T + node], dcy = nadj[2 * T + node], dcz = nadj[3 * T + node];
        const double qxx = nadj[4 * T + node], qxy = nadj[5 * T + node], qxz = nadj[6 * T + node];
        const double qyy = nadj[7 * T + node], qyz = nadj[8 * T + node], qzz = nadj[9 * T + node];
        const float4 c = tv.nd_com[node], cl = tv.nd_comlo[node];
        const double M = c.w;
        const double ex = xb - (static_cast<double>(c.x) + cl.x);
        const double ey = yb - (static_cast<double>(c.y) + cl.y);
        const double ez = zb - (static_cast<double>(c.z) + cl.z);
        if (M > 0) {
            ax += mb / M * dcx;
            ay += mb / M * dcy;
            az += mb / M * dcz;
            am += (ex * dcx + ey * dcy + ez * dcz) / M;
        }
        const double tr = qxx + qyy + qzz, e2 = ex * ex + ey * ey + ez * ez;
        ax += mb * (6 * qxx * ex - 2 * tr * ex + 3 * qxy * ey + 3 * qxz * ez);
        ay += mb * (6 * qyy * ey - 2 * tr * ey + 3 * qxy * ex + 3 * qyz * ez);
        az += mb * (6 * qzz * ez - 2 * tr * ez + 3 * qxz * ex + 3 * qyz * ey);
        am += dM + qxx * (3 * ex * ex - e2) + qyy * (3 * ey * ey - e2) + qzz * (3 * ez * ez - e2) +
              3 * (qxy * ex * ey + qxz * ex * ez + qyz * ey * ez);
        node = tv.nd_parent[node];
    }
    gx[i] += ax;
    gy[i] += ay;
    gz[i] += az;
    gm[i] += am;
}

template <bool EPS0>
int vjp_blocks(int sms) {
    static int per_sm = 0;
    if (!per_sm) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk_vjp<EPS0>, VWBS, 0) != cudaSuccess) {
            cudaGetLastError();
            per_sm = 1;
        }
        if (per_sm < 1) per_sm = 1;
    }
    return per_sm * sms;
}

}  // namespace

void tree_walk_vjp(Engine& e, const float4* w, float e2, bool eps0, double* g) {
    const int n = e.n;
    if (n == 0) return;
    TreeView tv = tree_view(e);
    const size_t T = tv.T;
    e.vjp_scratch.reserve(T * NADJ * 8);
    double* nadj = e.vjp_scratch.as<double>();
    LG_CK(cudaMemsetAsync(nadj, 0, T * NADJ * 8, e.stream));
    LG_CK(cudaMemsetAsync(e.small.as<char>() + 32, 0, 4, e.stream));
    const int blocks = eps0 ? vjp_blocks<true>(e.sms) : vjp_blocks<false>(e.sms);
    e.walk_stack.reserve(static_cast<size_t>(blocks) * VWARPS * SCAP * 4);
    BodyArrays b = e.bodies(e.cur);
    VjpArgs a;
    a.tv = tv;
    a.hm = b.hm;
    a.lo = b.lo;
    a.w = w;
    a.gx = g;
    a.gy = g + n;
    a.gz = g + 2 * static_cast<size_t>(n);
    a.gm = g + 3 * static_cast<size_t>(n);
    a.nadj = nadj;
    a.stack = e.walk_stack.as<uint32_t>();
    a.group_ctr = reinterpret_cast<unsigned*>(e.small.as<char>() + 32);
    a.err = e.err_word();
    a.e2 = e2;
    if (eps0) k_walk_vjp<true><<<blocks, VWBS, 0, e.stream>>>(a);
    else k_walk_vjp<false><<<blocks, VWBS, 0, e.stream>>>(a);
    LG_LAUNCHED();
    k_moment_chain<<<(n + 255) / 256, 256, 0, e.stream>>>(tv, b, n, nadj, a.gx, a.gy, a.gz, a.gm, e.err_word());
    LG_LAUNCHED();
    e.launches += 2;
}

}  // namespace lg
