// Tree walk: the reference CPU backend's group walk (src/cpu_backend.cpp:667-689 walk,
// :816-838 build_list, :841-882 eval_group), GB300 form.
//
// One warp per walk group (persistent warps pull groups from an atomic counter):
//  - List build: a warp-cooperative depth-first traversal. Each step pops up to 32 nodes, one per
//    lane, and applies the reference's opening rule against the group's bounding box: a node that
//    contains the group, or whose box distance d satisfies d^2 < rcrit2, is opened; an accepted
//    leaf of <= 4 bodies is taken as bodies, other accepted nodes as cells; opened leaves give
//    bodies, opened internal nodes push their children. Appends are warp-compacted with ballots.
//    The traversal stack lives in global memory (one slice per warp).
//  - Evaluation in chunks: when the lists fill up, the warp converts the entries once to
//    coordinates relative to the group's box centre o, (x_hi - o) + x_lo in FP32, into
//    struct-of-arrays chunks in shared memory, and every lane evaluates them for its IPT i-bodies
//    (IPT = ceil(group size / 32)): quadrupole cell terms (cuda_backend.cu:783-800 /
//    cpu_backend.cpp:858-871 math) and softened body terms. Two consecutive entries are loaded
//    as one float2 and evaluated together with packed f32x2 instructions (one issue slot for two
//    FP32 operations). Chunk sums are added to running sums kept in shared memory with Kahan
//    compensation.
// The interaction count per body is the list length minus its own entry; the reference CPU
// backend counts that self entry, so its count exceeds this one by exactly N.
#include "engine.cuh"

namespace lg {

namespace {

constexpr int WBS = 128;  // 4 warps per block
#ifndef LG_WALK_MINB
#define LG_WALK_MINB 4  // resident blocks per SM the register budget is sized for
#endif
constexpr int WARPS = WBS / 32;
constexpr int SMALL_LEAF = 4;   // src/cpu_backend.cpp:29
constexpr int SCAP = 16384;     // traversal stack entries per warp (global memory)
constexpr int CL_CAP = 160, CL_FLUSH = 128;
constexpr int RL_CAP = 96, RL_FLUSH = 64;
constexpr int BR_FLUSH = 256;
constexpr int CCH = 64;   // cells converted per chunk
constexpr int BCH = 128;  // bodies converted per chunk
constexpr int PASS = 128; // i-bodies per pass (4 per lane)

constexpr int IPT_MAX = 4;

// Per-warp shared memory. Chunks are struct-of-arrays so that entries k, k+1 load as one float2.
struct __align__(16) WarpSmem {
    float cx[CCH], cy[CCH], cz[CCH], cm[CCH], qxx[CCH], qxy[CCH], qxz[CCH], qyy[CCH], qyz[CCH], qzz[CCH];
    float bx[BCH], by[BCH], bz[BCH], bm[BCH];
    float ks[IPT_MAX][8][32];  // Kahan sums sx sy sz sp and compensations cx cy cz cp, per slot and lane
    uint32_t clist[CL_CAP];
    uint2 rlist[RL_CAP];
    uint32_t rpre[RL_CAP + 1];
};

struct WalkArgs {
    TreeView tv;
    const float4* hm;
    const float4* lo;
    float4* acc;
    float* cost;
    uint32_t* stack;
    unsigned* group_ctr;
    unsigned long long* inter;
    unsigned* err;
    float G, e2;
    // Forest (ensemble) walk: body -> system (nullptr: one tree rooted at node 0) and the
    // per-system squared softening; system s's tree is rooted at node s.
    const uint32_t* sys;
    const float* e2_sys;
};

__device__ __forceinline__ int warp_excl_scan(int v, int lane, int& total) {
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
    }
    total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

__device__ __forceinline__ f2x ld2(const float* p) { return *reinterpret_cast<const f2x*>(p); }

// Adds one chunk's partial sums (packed halves) of slot u into the lane's Kahan sums.
template <bool POT>
__device__ __forceinline__ void merge_slot(WarpSmem& s, int u, int lane, f2x ax, f2x ay, f2x az, f2x ap) {
    float* k = &s.ks[u][0][lane];
    float sx = k[0], sy = k[32], sz = k[64], cx = k[128], cy = k[160], cz = k[192];
    kahan_add(sx, cx, f2_sum(ax));
    kahan_add(sy, cy, f2_sum(ay));
    kahan_add(sz, cz, f2_sum(az));
    k[0] = sx; k[32] = sy; k[64] = sz; k[128] = cx; k[160] = cy; k[192] = cz;
    if (POT) {
        float sp = k[96], cp = k[224];
        kahan_add(sp, cp, f2_sum(ap));
        k[96] = sp; k[224] = cp;
    }
}

template <bool EPS0>
__device__ __forceinline__ f2x pair_rsqrt(f2x r2) {
    float lo, hi;
    f2_unpack(r2, lo, hi);
    float a = rsqrt_mufu(lo), b = rsqrt_mufu(hi);
    if (EPS0) {
        a = lo > 0.f ? a : 0.f;
        b = hi > 0.f ? b : 0.f;
    }
    return f2_pack(a, b);
}

// Quadrupole cell terms: d points from the body to the cell,
// a = G [M d/r^3 - Q d/r^5 + 5/2 (dQd) d/r^7], phi = -G [M/r + 1/2 dQd/r^5]. cc is even.
template <int IPT, bool POT, bool EPS0>
__device__ __forceinline__ void eval_cells(WarpSmem& s, int cc, int lane, const float (&xi)[IPT_MAX],
                                           const float (&yi)[IPT_MAX], const float (&zi)[IPT_MAX], float e2) {
    f2x XI[IPT], YI[IPT], ZI[IPT], ax[IPT], ay[IPT], az[IPT], ap[IPT];
#pragma unroll
    for (int u = 0; u < IPT; ++u) {
        XI[u] = f2_bcast(xi[u]);
        YI[u] = f2_bcast(yi[u]);
        ZI[u] = f2_bcast(zi[u]);
        ax[u] = ay[u] = az[u] = ap[u] = 0ull;
    }
    const f2x E2 = f2_bcast(e2), C25 = f2_bcast(2.5f), NEG1 = f2_bcast(-1.f), C05 = f2_bcast(0.5f);
    // Few i-bodies per lane leave little independent work per entry: unroll over entries then.
#pragma unroll 1
    for (int k = 0; k < cc; k += 2) {
        const f2x X = ld2(s.cx + k), Y = ld2(s.cy + k), Z = ld2(s.cz + k), M = ld2(s.cm + k);
        const f2x QXX = ld2(s.qxx + k), QXY = ld2(s.qxy + k), QXZ = ld2(s.qxz + k);
        const f2x QYY = ld2(s.qyy + k), QYZ = ld2(s.qyz + k), QZZ = ld2(s.qzz + k);
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            const f2x dx = f2_sub(X, XI[u]), dy = f2_sub(Y, YI[u]), dz = f2_sub(Z, ZI[u]);
            const f2x r2 = f2_fma(dx, dx, f2_fma(dy, dy, f2_fma(dz, dz, E2)));
            const f2x inv = pair_rsqrt<EPS0>(r2);
            const f2x inv2 = f2_mul(inv, inv), inv3 = f2_mul(inv, inv2), inv5 = f2_mul(inv3, inv2);
            const f2x qx = f2_fma(QXX, dx, f2_fma(QXY, dy, f2_mul(QXZ, dz)));
            const f2x qy = f2_fma(QXY, dx, f2_fma(QYY, dy, f2_mul(QYZ, dz)));
            const f2x qz = f2_fma(QXZ, dx, f2_fma(QYZ, dy, f2_mul(QZZ, dz)));
            const f2x dqd = f2_fma(dx, qx, f2_fma(dy, qy, f2_mul(dz, qz)));
            const f2x t5 = f2_mul(dqd, inv5);
            const f2x f = f2_fma(M, inv3, f2_mul(f2_mul(C25, t5), inv2));
            const f2x n5 = f2_mul(inv5, NEG1);
            ax[u] = f2_fma(qx, n5, f2_fma(f, dx, ax[u]));
            ay[u] = f2_fma(qy, n5, f2_fma(f, dy, ay[u]));
            az[u] = f2_fma(qz, n5, f2_fma(f, dz, az[u]));
            if (POT) ap[u] = f2_add(ap[u], f2_fma(M, inv, f2_mul(C05, t5)));
        }
    }
#pragma unroll
    for (int u = 0; u < IPT; ++u) merge_slot<POT>(s, u, lane, ax[u], ay[u], az[u], ap[u]);
}

// Softened body terms a = G m d / r^3, phi = -G m / r. bc is even.
template <int IPT, bool POT, bool EPS0>
__device__ __forceinline__ void eval_bodies(WarpSmem& s, int bc, int lane, const float (&xi)[IPT_MAX],
                                            const float (&yi)[IPT_MAX], const float (&zi)[IPT_MAX], float e2) {
    f2x XI[IPT], YI[IPT], ZI[IPT], ax[IPT], ay[IPT], az[IPT], ap[IPT];
#pragma unroll
    for (int u = 0; u < IPT; ++u) {
        XI[u] = f2_bcast(xi[u]);
        YI[u] = f2_bcast(yi[u]);
        ZI[u] = f2_bcast(zi[u]);
        ax[u] = ay[u] = az[u] = ap[u] = 0ull;
    }
    const f2x E2 = f2_bcast(e2);
#pragma unroll 2
    for (int k = 0; k < bc; k += 2) {
        const f2x X = ld2(s.bx + k), Y = ld2(s.by + k), Z = ld2(s.bz + k), M = ld2(s.bm + k);
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            const f2x dx = f2_sub(X, XI[u]), dy = f2_sub(Y, YI[u]), dz = f2_sub(Z, ZI[u]);
            const f2x r2 = f2_fma(dx, dx, f2_fma(dy, dy, f2_fma(dz, dz, E2)));
            const f2x inv = pair_rsqrt<EPS0>(r2);
            const f2x mi = f2_mul(M, inv);  // rounded: the self term cancels exactly
            const f2x f = f2_mul(mi, f2_mul(inv, inv));
            ax[u] = f2_fma(f, dx, ax[u]);
            ay[u] = f2_fma(f, dy, ay[u]);
            az[u] = f2_fma(f, dz, az[u]);
            if (POT) ap[u] = f2_add(ap[u], mi);
        }
    }
#pragma unroll
    for (int u = 0; u < IPT; ++u) merge_slot<POT>(s, u, lane, ax[u], ay[u], az[u], ap[u]);
}

template <bool POT, bool EPS0>
__device__ __forceinline__ void eval_cells_n(int ipt, WarpSmem& s, int cc, int lane, const float (&xi)[IPT_MAX],
                                             const float (&yi)[IPT_MAX], const float (&zi)[IPT_MAX], float e2) {
    switch (ipt) {
        case 1: eval_cells<1, POT, EPS0>(s, cc, lane, xi, yi, zi, e2); break;
        case 2: eval_cells<2, POT, EPS0>(s, cc, lane, xi, yi, zi, e2); break;
        case 3: eval_cells<3, POT, EPS0>(s, cc, lane, xi, yi, zi, e2); break;
        default: eval_cells<4, POT, EPS0>(s, cc, lane, xi, yi, zi, e2); break;
    }
}

template <bool POT, bool EPS0>
__device__ __forceinline__ void eval_bodies_n(int ipt, WarpSmem& s, int bc, int lane, const float (&xi)[IPT_MAX],
                                              const float (&yi)[IPT_MAX], const float (&zi)[IPT_MAX], float e2) {
    switch (ipt) {
        case 1: eval_bodies<1, POT, EPS0>(s, bc, lane, xi, yi, zi, e2); break;
        case 2: eval_bodies<2, POT, EPS0>(s, bc, lane, xi, yi, zi, e2); break;
        case 3: eval_bodies<3, POT, EPS0>(s, bc, lane, xi, yi, zi, e2); break;
        default: eval_bodies<4, POT, EPS0>(s, bc, lane, xi, yi, zi, e2); break;
    }
}

// A far, massless entry: pads a chunk to an even count and contributes exactly zero.
constexpr float kFar = 1e18f;

// Evaluates the pending lists for the pass's i-bodies and empties them.
template <bool POT, bool EPS0>
__device__ __forceinline__ void flush(const WalkArgs& w, WarpSmem& s, int lane, int ipt, int nc, int nr, float ox,
                                      float oy, float oz, const float (&xi)[IPT_MAX], const float (&yi)[IPT_MAX],
                                      const float (&zi)[IPT_MAX], float e2) {
    for (int c0 = 0; c0 < nc; c0 += CCH) {
        const int cc = min(CCH, nc - c0);
        const int cc2 = (cc + 1) & ~1;
        for (int k = lane; k < cc2; k += 32) {
            if (k < cc) {
                const uint32_t nd = s.clist[c0 + k];
                const float4 com = w.tv.nd_com[nd], cl = w.tv.nd_comlo[nd], q0 = w.tv.nd_q0[nd], q1 = w.tv.nd_q1[nd];
                s.cx[k] = (com.x - ox) + cl.x;
                s.cy[k] = (com.y - oy) + cl.y;
                s.cz[k] = (com.z - oz) + cl.z;
                s.cm[k] = com.w;
                s.qxx[k] = q0.x; s.qxy[k] = q0.y; s.qxz[k] = q0.z; s.qyy[k] = q0.w; s.qyz[k] = q1.x; s.qzz[k] = q1.y;
            } else {
                s.cx[k] = kFar; s.cy[k] = kFar; s.cz[k] = kFar; s.cm[k] = 0.f;
                s.qxx[k] = s.qxy[k] = s.qxz[k] = s.qyy[k] = s.qyz[k] = s.qzz[k] = 0.f;
            }
        }
        __syncwarp();
        eval_cells_n<POT, EPS0>(ipt, s, cc2, lane, xi, yi, zi, e2);
        __syncwarp();
    }
    if (nr == 0) return;
    // Prefix of range lengths (nr <= RL_CAP).
    for (int r0 = 0; r0 < nr; r0 += 32) {
        const int r = r0 + lane;
        const int len = r < nr ? static_cast<int>(s.rlist[r].y) : 0;
        int tot;
        const int ex = warp_excl_scan(len, lane, tot);
        const uint32_t base = r0 == 0 ? 0u : s.rpre[r0];
        __syncwarp();
        if (r < nr) s.rpre[r] = base + ex;
        if (lane == 31) s.rpre[min(r0 + 32, nr)] = base + tot;
        __syncwarp();
    }
    const int total = static_cast<int>(s.rpre[nr]);
    for (int b0 = 0; b0 < total; b0 += BCH) {
        const int bc = min(BCH, total - b0);
        const int bc2 = (bc + 1) & ~1;
        for (int k = lane; k < bc2; k += 32) {
            if (k < bc) {
                const uint32_t p = b0 + k;
                int lo = 0, hi = nr;  // last r with rpre[r] <= p
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (s.rpre[mid] <= p) lo = mid;
                    else hi = mid;
                }
                const uint32_t j = s.rlist[lo].x + (p - s.rpre[lo]);
                const float4 h = w.hm[j], l = w.lo[j];
                s.bx[k] = (h.x - ox) + l.x;
                s.by[k] = (h.y - oy) + l.y;
                s.bz[k] = (h.z - oz) + l.z;
                s.bm[k] = h.w;
            } else {
                s.bx[k] = kFar; s.by[k] = kFar; s.bz[k] = kFar; s.bm[k] = 0.f;
            }
        }
        __syncwarp();
        eval_bodies_n<POT, EPS0>(ipt, s, bc2, lane, xi, yi, zi, e2);
        __syncwarp();
    }
}

template <bool POT, bool EPS0>
__device__ void walk_pass(const WalkArgs& w, WarpSmem& s, uint32_t* stack, int lane, uint2 gr, float4 bc, float4 bh,
                          uint32_t plo, int np, unsigned long long& inter_b, unsigned long long& inter_c) {
    const float ox = bc.x, oy = bc.y, oz = bc.z;
    const int ipt = (np + 31) >> 5;
    float xi[IPT_MAX], yi[IPT_MAX], zi[IPT_MAX], mi[IPT_MAX];
#pragma unroll
    for (int u = 0; u < IPT_MAX; ++u) {
        const int k = min(lane + 32 * u, np - 1);
        const float4 h = w.hm[plo + k], l = w.lo[plo + k];
        xi[u] = (h.x - ox) + l.x;
        yi[u] = (h.y - oy) + l.y;
        zi[u] = (h.z - oz) + l.z;
        mi[u] = h.w;
    }
#pragma unroll
    for (int u = 0; u < IPT_MAX; ++u)
#pragma unroll
        for (int f = 0; f < 8; ++f) s.ks[u][f][lane] = 0.f;
    const unsigned lt = (1u << lane) - 1u;
    const uint32_t root = w.sys ? w.sys[gr.x] : 0u;
    const float e2 = w.e2_sys ? w.e2_sys[root] : w.e2;
    int sp = 1;
    if (lane == 0) stack[0] = root;
    __syncwarp();
    int nc = 0, nr = 0, nbr = 0;
    uint32_t list_len = 0, cells_len = 0;
    bool overflow = false;
    // Each node is visited at most once per pass; the cap stops a malformed tree.
    const uint32_t max_iter = static_cast<uint32_t>(w.tv.T) + 64u;
    uint32_t iter = 0;
    for (;;) {
        const bool done = sp == 0;
        // One evaluation site: when the lists fill up, and once at the end.
        if (done || nc >= CL_FLUSH || nr >= RL_FLUSH || nbr >= BR_FLUSH) {
            flush<POT, EPS0>(w, s, lane, ipt, nc, nr, ox, oy, oz, xi, yi, zi, e2);
            list_len += nc + nbr;
            cells_len += nc;
            nc = nr = nbr = 0;
            if (done) break;
        }
        if (++iter > max_iter) {
            overflow = true;
            break;
        }
        const int take = min(32, sp);
        sp -= take;
        const bool have = lane < take;
        const uint32_t node = have ? stack[sp + lane] : 0u;
        __syncwarp();
        int kind = 0;  // 1 cell, 2 bodies, 3 children
        uint32_t a0 = 0, a1 = 0;
        if (have && node >= w.tv.T) {
            atomicOr(w.err, kErrNodeOverflow);
        } else if (have) {
            const uint4 r = w.tv.nd_range[node];
            const float4 com = w.tv.nd_com[node];
            const float rc2 = w.tv.nd_q1[node].z;
            const float dx = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.x, bc.x)), bh.x), 0.f);
            const float dy = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.y, bc.y)), bh.y), 0.f);
            const float dz = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.z, bc.z)), bh.z), 0.f);
            const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            // A node containing the group is always opened (src/cpu_backend.cpp:826-828).
            const bool contains = r.x <= gr.x && gr.y <= r.y;
            const bool leaf = r.w == 0;
            if (!contains && d2 >= rc2) {
                if (leaf && r.y - r.x <= static_cast<unsigned>(SMALL_LEAF)) { kind = 2; a0 = r.x; a1 = r.y - r.x; }
                else { kind = 1; a0 = node; }
            } else if (leaf) {
                kind = 2; a0 = r.x; a1 = r.y - r.x;
            } else {
                kind = 3; a0 = r.z; a1 = r.w;
            }
        }
        const unsigned cm = __ballot_sync(0xffffffffu, kind == 1);
        if (kind == 1) s.clist[nc + __popc(cm & lt)] = a0;
        nc += __popc(cm);
        const unsigned rm = __ballot_sync(0xffffffffu, kind == 2);
        if (kind == 2) s.rlist[nr + __popc(rm & lt)] = make_uint2(a0, a1);
        nr += __popc(rm);
        int btot;
        warp_excl_scan(kind == 2 ? static_cast<int>(a1) : 0, lane, btot);
        nbr += btot;
        int ctot;
        const int coff = warp_excl_scan(kind == 3 ? static_cast<int>(a1) : 0, lane, ctot);
        if (sp + ctot > SCAP) {
            overflow = true;
            break;
        }
        if (kind == 3)
            for (uint32_t k = 0; k < a1; ++k) stack[sp + coff + k] = a0 + (a1 - 1 - k);  // first child on top
        sp += ctot;
        __syncwarp();
    }
    if (overflow && lane == 0) atomicOr(w.err, iter > max_iter ? kErrNodeOverflow : kErrStackOverflow);
    const float self_inv = (POT && !EPS0) ? rsqrt_mufu(e2) : 0.f;
#pragma unroll
    for (int u = 0; u < IPT_MAX; ++u) {
        const int k = lane + 32 * u;
        if (k >= np) continue;
        const uint32_t i = plo + k;
        const float* ks = &s.ks[u][0][lane];
        float p = ks[96] - ks[224];
        // The own body is always in the list (its leaf is inside the group, so it is opened);
        // with eps > 0 its pair has d = 0 and only adds m_i/eps to the potential.
        if (POT && !EPS0) p = __fsub_rn(p, __fmul_rn(mi[u], self_inv));
        w.acc[i] = make_float4(w.G * (ks[0] - ks[128]), w.G * (ks[32] - ks[160]), w.G * (ks[64] - ks[192]),
                               POT ? -w.G * p : 0.f);
        w.cost[i] = static_cast<float>(list_len - 1);
    }
    inter_b += static_cast<unsigned long long>(list_len - cells_len - 1) * static_cast<unsigned long long>(np);
    inter_c += static_cast<unsigned long long>(cells_len) * static_cast<unsigned long long>(np);
}

template <bool POT, bool EPS0>
__global__ void __launch_bounds__(WBS, LG_WALK_MINB) k_walk(WalkArgs w) {
    __shared__ WarpSmem sm[WARPS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    WarpSmem& s = sm[wid];
    uint32_t* stack = w.stack + (static_cast<size_t>(blockIdx.x) * WARPS + wid) * SCAP;
    const unsigned ngroups = *w.tv.ngroups;
    unsigned long long inter_b = 0, inter_c = 0;
    for (;;) {
        unsigned g = 0;
        if (lane == 0) g = atomicAdd(w.group_ctr, 1u);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g >= ngroups) break;
        const uint2 gr = w.tv.grp_range[g];
        const float4 bc = w.tv.grp_box[2 * g], bh = w.tv.grp_box[2 * g + 1];
        for (uint32_t plo = gr.x; plo < gr.y; plo += PASS) {
            const int np = static_cast<int>(min(static_cast<uint32_t>(PASS), gr.y - plo));
            walk_pass<POT, EPS0>(w, s, stack, lane, gr, bc, bh, plo, np, inter_b, inter_c);
        }
    }
    if (lane == 0) {
        if (inter_b) atomicAdd(w.inter, inter_b);
        if (inter_c) atomicAdd(w.inter + 1, inter_c);
    }
}

template <bool POT, bool EPS0>
int walk_blocks(int sms) {
    static int per_sm = 0;
    if (!per_sm) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk<POT, EPS0>, WBS, 0) != cudaSuccess) {
            cudaGetLastError();
            per_sm = 1;
        }
        if (per_sm < 1) per_sm = 1;
    }
    return per_sm * sms;
}

}  // namespace

void tree_walk(Engine& e, float G, float e2, bool potential, bool eps0, const uint32_t* sys, const float* e2_sys) {
    WalkArgs w;
    w.sys = sys;
    w.e2_sys = e2_sys;
    w.tv = tree_view(e);
    BodyArrays b = e.bodies(e.cur);
    w.hm = b.hm;
    w.lo = b.lo;
    w.acc = e.acc.as<float4>();
    w.cost = b.cost;
    w.group_ctr = reinterpret_cast<unsigned*>(e.small.as<char>() + 32);
    w.inter = e.inter_counter();
    w.err = e.err_word();
    w.G = G;
    w.e2 = e2;
    int blocks;
    if (potential) blocks = eps0 ? walk_blocks<true, true>(e.sms) : walk_blocks<true, false>(e.sms);
    else blocks = eps0 ? walk_blocks<false, true>(e.sms) : walk_blocks<false, false>(e.sms);
    e.walk_stack.reserve(static_cast<size_t>(blocks) * WARPS * SCAP * 4);
    w.stack = e.walk_stack.as<uint32_t>();
    if (potential) {
        if (eps0) k_walk<true, true><<<blocks, WBS, 0, e.stream>>>(w);
        else k_walk<true, false><<<blocks, WBS, 0, e.stream>>>(w);
    } else {
        if (eps0) k_walk<false, true><<<blocks, WBS, 0, e.stream>>>(w);
        else k_walk<false, false><<<blocks, WBS, 0, e.stream>>>(w);
    }
    LG_LAUNCHED();
    ++e.launches;
}

}  // namespace lg
