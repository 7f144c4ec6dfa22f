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
// atomics).
#include "engine.cuh"
#include "walk_common.cuh"

namespace lg {

namespace {

using namespace walk;

constexpr int VWBS = 64;  // 2 warps per block
constexpr int VWARPS = VWBS / 32;
constexpr int VCCH = 64;
constexpr int VBCH = 128;
constexpr int VPASS = 128;
constexpr int VIPT = VPASS / 32;
constexpr int NADJ = 10;  // per node: dM, dcom (3), dQ (xx, xy, xz, yy, yz, zz)

struct __align__(16) VjpSmem {
    float cx[VCCH], cy[VCCH], cz[VCCH], cm[VCCH], qxx[VCCH], qxy[VCCH], qxz[VCCH], qyy[VCCH], qyz[VCCH], qzz[VCCH];
    float bx[VBCH], by[VBCH], bz[VBCH], bm[VBCH];
    uint32_t bj[VBCH];
    float ix[VPASS], iy[VPASS], iz[VPASS], iwx[VPASS], iwy[VPASS], iwz[VPASS];
    float ks[VIPT][6][32];  // i-side Kahan sums of gd (x, y, z) and compensations
    uint32_t clist[CL_CAP];
    uint2 rlist[RL_CAP];
    uint32_t rpre[RL_CAP + 1];
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

__device__ __forceinline__ void kahan3(VjpSmem& s, int u, int lane, float x, float y, float z) {
    float* k = &s.ks[u][0][lane];
    float sx = k[0], sy = k[32], sz = k[64], cx = k[96], cy = k[128], cz = k[160];
    kahan_add(sx, cx, x);
    kahan_add(sy, cy, y);
    kahan_add(sz, cz, z);
    k[0] = sx; k[32] = sy; k[64] = sz; k[96] = cx; k[128] = cy; k[160] = cz;
}

// Cell term: gd for weight w at offset d (cell minus body); also returns u / r^3, u / r^5 and
// u / r^7 pieces through the out parameters the entry side needs.
struct CellJ {
    float gdx, gdy, gdz, u, inv3, inv5, inv7;
};

__device__ __forceinline__ CellJ cell_j(float dx, float dy, float dz, float inv, float M, float qxx, float qxy,
                                        float qxz, float qyy, float qyz, float qzz, float wx, float wy, float wz) {
    CellJ c;
    const float inv2 = inv * inv, inv3 = inv * inv2, inv5 = inv3 * inv2, inv7 = inv5 * inv2, inv9 = inv7 * inv2;
    const float qx = qxx * dx + qxy * dy + qxz * dz;
    const float qy = qxy * dx + qyy * dy + qyz * dz;
    const float qz = qxz * dx + qyz * dy + qzz * dz;
    const float q = dx * qx + dy * qy + dz * qz;
    const float u = wx * dx + wy * dy + wz * dz;
    const float qwx = qxx * wx + qxy * wy + qxz * wz;
    const float qwy = qxy * wx + qyy * wy + qyz * wz;
    const float qwz = qxz * wx + qyz * wy + qzz * wz;
    const float wqd = wx * qx + wy * qy + wz * qz;
    const float A = M * inv3 + 2.5f * q * inv7;
    const float B = -3.f * M * u * inv5 + 5.f * wqd * inv7 - 17.5f * q * u * inv9;
    const float D = 5.f * u * inv7;
    c.gdx = A * wx + B * dx - qwx * inv5 + D * qx;
    c.gdy = A * wy + B * dy - qwy * inv5 + D * qy;
    c.gdz = A * wz + B * dz - qwz * inv5 + D * qz;
    c.u = u;
    c.inv3 = inv3;
    c.inv5 = inv5;
    c.inv7 = inv7;
    return c;
}

template <bool EPS0>
__device__ void vjp_flush(const VjpArgs& a, VjpSmem& s, int lane, int np, uint32_t plo, int nc, int nr, float ox,
                          float oy, float oz, float e2) {
    const size_t T = a.tv.T;
    // ---- cells
    for (int c0 = 0; c0 < nc; c0 += VCCH) {
        const int cc = min(VCCH, nc - c0);
        for (int k = lane; k < cc; k += 32) {
            const uint32_t nd = s.clist[c0 + k];
            const float4 com = a.tv.nd_com[nd], cl = a.tv.nd_comlo[nd], q0 = a.tv.nd_q0[nd], q1 = a.tv.nd_q1[nd];
            s.cx[k] = (com.x - ox) + cl.x;
            s.cy[k] = (com.y - oy) + cl.y;
            s.cz[k] = (com.z - oz) + cl.z;
            s.cm[k] = com.w;
            s.qxx[k] = q0.x; s.qxy[k] = q0.y; s.qxz[k] = q0.z; s.qyy[k] = q0.w; s.qyz[k] = q1.x; s.qzz[k] = q1.y;
        }
        __syncwarp();
        // i side: lanes over i-bodies.
#pragma unroll
        for (int u = 0; u < VIPT; ++u) {
            const int i = lane + 32 * u;
            if (i >= np) continue;
            const float xi = s.ix[i], yi = s.iy[i], zi = s.iz[i], wx = s.iwx[i], wy = s.iwy[i], wz = s.iwz[i];
            float ax = 0.f, ay = 0.f, az = 0.f;
            for (int k = 0; k < cc; ++k) {
                const float dx = s.cx[k] - xi, dy = s.cy[k] - yi, dz = s.cz[k] - zi;
                const float inv = inv_r<EPS0>(dx * dx + dy * dy + dz * dz + e2);
                const CellJ j = cell_j(dx, dy, dz, inv, s.cm[k], s.qxx[k], s.qxy[k], s.qxz[k], s.qyy[k], s.qyz[k],
                                       s.qzz[k], wx, wy, wz);
                ax += j.gdx;
                ay += j.gdy;
                az += j.gdz;
            }
            kahan3(s, u, lane, ax, ay, az);
        }
        // Entry side: lanes over cells, looping over the group's i-bodies.
        for (int k = lane; k < cc; k += 32) {
            const float X = s.cx[k], Y = s.cy[k], Z = s.cz[k], M = s.cm[k];
            const float qxx = s.qxx[k], qxy = s.qxy[k], qxz = s.qxz[k], qyy = s.qyy[k], qyz = s.qyz[k], qzz = s.qzz[k];
            float g[NADJ] = {};
            for (int i = 0; i < np; ++i) {
                const float wx = s.iwx[i], wy = s.iwy[i], wz = s.iwz[i];
                const float dx = X - s.ix[i], dy = Y - s.iy[i], dz = Z - s.iz[i];
                const float inv = inv_r<EPS0>(dx * dx + dy * dy + dz * dz + e2);
                const CellJ j = cell_j(dx, dy, dz, inv, M, qxx, qxy, qxz, qyy, qyz, qzz, wx, wy, wz);
                const float E = 2.5f * j.u * j.inv7;
                g[0] += j.u * j.inv3;
                g[1] += j.gdx;
                g[2] += j.gdy;
                g[3] += j.gdz;
                g[4] += E * dx * dx - wx * dx * j.inv5;
                g[5] += 2.f * E * dx * dy - (wx * dy + wy * dx) * j.inv5;
                g[6] += 2.f * E * dx * dz - (wx * dz + wz * dx) * j.inv5;
                g[7] += E * dy * dy - wy * dy * j.inv5;
                g[8] += 2.f * E * dy * dz - (wy * dz + wz * dy) * j.inv5;
                g[9] += E * dz * dz - wz * dz * j.inv5;
            }
            const uint32_t nd = s.clist[c0 + k];
#pragma unroll
            for (int f = 0; f < NADJ; ++f)
                if (g[f] != 0.f) atomicAdd(a.nadj + f * T + nd, static_cast<double>(g[f]));
        }
        __syncwarp();
    }
    if (nr == 0) return;
    // ---- bodies
    const int total = range_prefix(s, nr, lane);
    for (int b0 = 0; b0 < total; b0 += VBCH) {
        const int bc = min(VBCH, total - b0);
        for (int k = lane; k < bc; k += 32) {
            const uint32_t j = range_body(s, nr, b0 + k);
            const float4 h = a.hm[j], l = a.lo[j];
            s.bx[k] = (h.x - ox) + l.x;
            s.by[k] = (h.y - oy) + l.y;
            s.bz[k] = (h.z - oz) + l.z;
            s.bm[k] = h.w;
            s.bj[k] = j;
        }
        __syncwarp();
#pragma unroll
        for (int u = 0; u < VIPT; ++u) {
            const int i = lane + 32 * u;
            if (i >= np) continue;
            const uint32_t me = plo + i;
            const float xi = s.ix[i], yi = s.iy[i], zi = s.iz[i], wx = s.iwx[i], wy = s.iwy[i], wz = s.iwz[i];
            float ax = 0.f, ay = 0.f, az = 0.f;
            for (int k = 0; k < bc; ++k) {
                const float dx = s.bx[k] - xi, dy = s.by[k] - yi, dz = s.bz[k] - zi;
                const float inv = inv_r<EPS0>(dx * dx + dy * dy + dz * dz + e2);
                const float inv2 = inv * inv, inv3 = inv * inv2, inv5 = inv3 * inv2;
                const float m = s.bj[k] == me ? 0.f : s.bm[k];
                const float uw = wx * dx + wy * dy + wz * dz;
                const float t = 3.f * uw * inv5;
                ax += m * (wx * inv3 - t * dx);
                ay += m * (wy * inv3 - t * dy);
                az += m * (wz * inv3 - t * dz);
            }
            kahan3(s, u, lane, ax, ay, az);
        }
        for (int k = lane; k < bc; k += 32) {
            const uint32_t j = s.bj[k];
            const float X = s.bx[k], Y = s.by[k], Z = s.bz[k], m = s.bm[k];
            float gx = 0.f, gy = 0.f, gz = 0.f, gm = 0.f;
            for (int i = 0; i < np; ++i) {
                if (plo + i == j) continue;
                const float wx = s.iwx[i], wy = s.iwy[i], wz = s.iwz[i];
                const float dx = X - s.ix[i], dy = Y - s.iy[i], dz = Z - s.iz[i];
                const float inv = inv_r<EPS0>(dx * dx + dy * dy + dz * dz + e2);
                const float inv2 = inv * inv, inv3 = inv * inv2, inv5 = inv3 * inv2;
                const float uw = wx * dx + wy * dy + wz * dz;
                const float t = 3.f * uw * inv5;
                gx += m * (wx * inv3 - t * dx);
                gy += m * (wy * inv3 - t * dy);
                gz += m * (wz * inv3 - t * dz);
                gm += uw * inv3;
            }
            atomicAdd(a.gx + j, static_cast<double>(gx));
            atomicAdd(a.gy + j, static_cast<double>(gy));
            atomicAdd(a.gz + j, static_cast<double>(gz));
            atomicAdd(a.gm + j, static_cast<double>(gm));
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
                s.ix[i] = (h.x - bc.x) + l.x;
                s.iy[i] = (h.y - bc.y) + l.y;
                s.iz[i] = (h.z - bc.z) + l.z;
                s.iwx[i] = w.x;
                s.iwy[i] = w.y;
                s.iwz[i] = w.z;
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
