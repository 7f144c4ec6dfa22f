// Tree walk: the reference CPU backend's group walk (src/cpu_backend.cpp:667-689 walk,
// :816-838 build_list, :841-882 eval_group), GB300 form.
//
// One warp per walk group (persistent warps pull groups from an atomic counter):
//  - List build: a warp-cooperative depth-first traversal. Each step pops up to 32 nodes, one per
//    lane, and applies the reference's opening rule against the group's bounding box: a node that
//    contains the group, or whose box distance d satisfies d^2 < rcrit2, is opened; an accepted
//    leaf of <= 4 bodies is taken as bodies, other accepted nodes as cells; opened leaves give
//    bodies, opened internal nodes push their children. Appends are warp-compacted with ballots.
//    The traversal stack lives in shared memory as child blocks (one entry per opened node), with
//    a global overflow slice per warp.
//  - Evaluation in chunks: when the lists fill up, the warp converts the entries once to
//    coordinates relative to the group's box centre o, (x_hi - o) + x_lo in FP32, into
//    struct-of-arrays chunks in shared memory (a flush's cells, then its bodies, in one shared
//    buffer), and every lane evaluates them for its IPT i-bodies, small groups splitting the
//    entries across lane partitions: quadrupole cell terms (cuda_backend.cu:783-800 /
//    cpu_backend.cpp:858-871 math) and softened body terms. Two consecutive entries are loaded
//    as one float2 and evaluated together with packed f32x2 instructions (one issue slot for two
//    FP32 operations). Chunk sums are added to running sums kept in shared memory with Kahan
//    compensation.
// The interaction count per body is the list length minus its own entry; the reference CPU
// backend counts that self entry, so its count exceeds this one by exactly N. The own entry adds
// nothing to the acceleration (d = 0) and is excluded from the potential by index.
#include "engine.cuh"
#include "walk_common.cuh"

namespace lg {

namespace {

using namespace walk;

constexpr int WBS = 128;  // 4 warps per block
#ifndef LG_WALK_MINB
#define LG_WALK_MINB 4  // resident blocks per SM the register budget is sized for
#endif
#ifndef LG_WALK_CUNROLL
#define LG_WALK_CUNROLL 1  // cell-entry pairs unrolled in the evaluation loop
#endif
#ifndef LG_WALK_BUNROLL
#define LG_WALK_BUNROLL 2  // body-entry pairs unrolled in the evaluation loop
#endif
constexpr int CUNROLL = LG_WALK_CUNROLL;
constexpr int BUNROLL = LG_WALK_BUNROLL;
constexpr int WARPS = WBS / 32;
#ifndef LG_WALK_CCH
#define LG_WALK_CCH 160  // a whole flush of cells (CL_CAP) in one chunk
#endif
#ifndef LG_WALK_BCH
#define LG_WALK_BCH 256
#endif
constexpr int CCH = LG_WALK_CCH;  // cells converted per chunk (a multiple of 8)
constexpr int BCH = LG_WALK_BCH;  // bodies converted per chunk (a multiple of 8)
static_assert(CCH % 8 == 0 && BCH % 8 == 0, "chunks hold whole pairs of every partition");
#ifndef LG_WALK_IPT
#define LG_WALK_IPT 4
#endif
constexpr int IPT_MAX = LG_WALK_IPT;  // i-bodies per lane at most
static_assert(IPT_MAX >= 1 && IPT_MAX <= 4, "1 to 4 i-bodies per lane");
constexpr int PASS = 32 * IPT_MAX;  // i-bodies per pass


// Per-warp shared memory. Chunks are struct-of-arrays so that entries k, k+1 load as one float2.
struct __align__(16) WarpSmem {
    union {  // a flush converts its cells, then its bodies: the two chunks share the space
        struct {
            float cx[CCH], cy[CCH], cz[CCH], cm[CCH], qxx[CCH], qxy[CCH], qxz[CCH], qyy[CCH], qyz[CCH], qzz[CCH];
        };
        struct {
            float bx[BCH], by[BCH], bz[BCH], bm[BCH];
        };
    };
    float ks[IPT_MAX][8][32];  // Kahan sums sx sy sz sp and compensations cx cy cz cp, per slot and lane
    int kself[PASS];           // with the potential: each i-body's position in the body chunk, or -2
    uint32_t clist[CL_CAP];
    uint2 rlist[RL_CAP];
    uint32_t rpre[RL_CAP + 1];
    uint32_t sstk[SSTK];  // traversal stack (shared part)
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
    // Remote trees walked after the local tree (or alone: local == 0, for the direct method's
    // blocks of consecutive bodies); accumulate adds to acc and cost instead of overwriting.
    LetView let;
    int local;
    int accumulate;
    // Block time steps: passes whose bodies all have level < kmin are skipped (level == nullptr: none).
    const uint8_t* level;
    int kmin;
};

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
// a = G [M d/r^3 - Q d/r^5 + 5/2 (dQd) d/r^7], phi = -G [M/r + 1/2 dQd/r^5]. cc is even. The
// chunk holds -Q (negated when converted), which spares one negation per pair; sign changes are
// exact, so the sums are those of the plain form bit for bit.
template <int IPT, bool POT, bool EPS0>
__device__ __forceinline__ void eval_cells(WarpSmem& s, int cc, int k0, int kstep, int lane, const float (&xi)[IPT_MAX],
                                           const float (&yi)[IPT_MAX], const float (&zi)[IPT_MAX], float e2) {
    f2x XI[IPT], YI[IPT], ZI[IPT], ax[IPT], ay[IPT], az[IPT], ap[IPT];
#pragma unroll
    for (int u = 0; u < IPT; ++u) {
        XI[u] = f2_bcast(xi[u]);
        YI[u] = f2_bcast(yi[u]);
        ZI[u] = f2_bcast(zi[u]);
        ax[u] = ay[u] = az[u] = ap[u] = 0ull;
    }
    const f2x E2 = f2_bcast(e2), CN25 = f2_bcast(-2.5f), CN05 = f2_bcast(-0.5f);
#pragma unroll CUNROLL
    for (int k = k0; k < cc; k += kstep) {
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
            // qx, qy, qz = -(Q d); s5 = -(dQd) / r^5
            const f2x s5 = f2_mul(f2_fma(dx, qx, f2_fma(dy, qy, f2_mul(dz, qz))), inv5);
            const f2x f = f2_fma(M, inv3, f2_mul(f2_mul(CN25, s5), inv2));
            ax[u] = f2_fma(qx, inv5, f2_fma(f, dx, ax[u]));
            ay[u] = f2_fma(qy, inv5, f2_fma(f, dy, ay[u]));
            az[u] = f2_fma(qz, inv5, f2_fma(f, dz, az[u]));
            if (POT) ap[u] = f2_add(ap[u], f2_fma(M, inv, f2_mul(CN05, s5)));
        }
    }
#pragma unroll
    for (int u = 0; u < IPT; ++u) merge_slot<POT>(s, u, lane, ax[u], ay[u], az[u], ap[u]);
}

// Softened body terms a = G m d / r^3, phi = -G m / r. bc is even.
// With the potential, the own body's pair is taken out by index (its mass half set to zero):
// kself[u] is the chunk position of the lane's u-th i-body (-2: not in this chunk).
template <int IPT, bool POT, bool EPS0>
__device__ __forceinline__ void eval_bodies(WarpSmem& s, int bc, int k0, int kstep, int lane,
                                            const float (&xi)[IPT_MAX], const float (&yi)[IPT_MAX],
                                            const float (&zi)[IPT_MAX], const int (&kself)[IPT_MAX], float e2) {
    f2x XI[IPT], YI[IPT], ZI[IPT], ax[IPT], ay[IPT], az[IPT], ap[IPT];
#pragma unroll
    for (int u = 0; u < IPT; ++u) {
        XI[u] = f2_bcast(xi[u]);
        YI[u] = f2_bcast(yi[u]);
        ZI[u] = f2_bcast(zi[u]);
        ax[u] = ay[u] = az[u] = ap[u] = 0ull;
    }
    const f2x E2 = f2_bcast(e2);
#pragma unroll BUNROLL
    for (int k = k0; k < bc; k += kstep) {
        const f2x X = ld2(s.bx + k), Y = ld2(s.by + k), Z = ld2(s.bz + k), M = ld2(s.bm + k);
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            f2x Mu = M;
            if (POT) {
                const unsigned off = static_cast<unsigned>(kself[u] - k);
                if (off <= 1u) Mu = f2_mul(M, off == 0 ? f2_pack(0.f, 1.f) : f2_pack(1.f, 0.f));
            }
            const f2x dx = f2_sub(X, XI[u]), dy = f2_sub(Y, YI[u]), dz = f2_sub(Z, ZI[u]);
            const f2x r2 = f2_fma(dx, dx, f2_fma(dy, dy, f2_fma(dz, dz, E2)));
            const f2x inv = pair_rsqrt<EPS0>(r2);
            const f2x mi = f2_mul(Mu, inv);  // the self pair (d = 0) adds nothing to a
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
__device__ __forceinline__ void eval_cells_n(int ipt, WarpSmem& s, int cc, int k0, int kstep, int lane,
                                             const float (&xi)[IPT_MAX], const float (&yi)[IPT_MAX],
                                             const float (&zi)[IPT_MAX], float e2) {
    switch (ipt) {
        case 1: eval_cells<1, POT, EPS0>(s, cc, k0, kstep, lane, xi, yi, zi, e2); break;
        case 2: eval_cells<(IPT_MAX < 2 ? IPT_MAX : 2), POT, EPS0>(s, cc, k0, kstep, lane, xi, yi, zi, e2); break;
        case 3: eval_cells<(IPT_MAX < 3 ? IPT_MAX : 3), POT, EPS0>(s, cc, k0, kstep, lane, xi, yi, zi, e2); break;
        default: eval_cells<IPT_MAX, POT, EPS0>(s, cc, k0, kstep, lane, xi, yi, zi, e2); break;
    }
}

template <bool POT, bool EPS0>
__device__ __forceinline__ void eval_bodies_n(int ipt, WarpSmem& s, int bc, int k0, int kstep, int lane,
                                              const float (&xi)[IPT_MAX], const float (&yi)[IPT_MAX],
                                              const float (&zi)[IPT_MAX], const int (&kself)[IPT_MAX], float e2) {
    switch (ipt) {
        case 1: eval_bodies<1, POT, EPS0>(s, bc, k0, kstep, lane, xi, yi, zi, kself, e2); break;
        case 2: eval_bodies<(IPT_MAX < 2 ? IPT_MAX : 2), POT, EPS0>(s, bc, k0, kstep, lane, xi, yi, zi, kself, e2); break;
        case 3: eval_bodies<(IPT_MAX < 3 ? IPT_MAX : 3), POT, EPS0>(s, bc, k0, kstep, lane, xi, yi, zi, kself, e2); break;
        default: eval_bodies<IPT_MAX, POT, EPS0>(s, bc, k0, kstep, lane, xi, yi, zi, kself, e2); break;
    }
}

// A far, massless entry: pads a chunk to an even count and contributes exactly zero.
constexpr float kFar = 1e18f;

// Evaluates the pending lists for the pass's i-bodies and empties them.
template <bool POT, bool EPS0>
__device__ __forceinline__ void flush(const WalkArgs& w, WarpSmem& s, int lane, int ipt, int part, int P, int nc,
                                      int nr, float ox, float oy, float oz, const float (&xi)[IPT_MAX],
                                      const float (&yi)[IPT_MAX], const float (&zi)[IPT_MAX], float e2, uint32_t plo,
                                      int np) {
    const int pad = 2 * P - 1;  // chunks padded to whole pairs per partition
    for (int c0 = 0; c0 < nc; c0 += CCH) {
        const int cc = min(CCH, nc - c0);
        const int cc2 = (cc + pad) & ~pad;
        for (int k = lane; k < cc2; k += 32) {
            if (k < cc) {
                const uint32_t nd = s.clist[c0 + k];
                float4 com, cl, q0, q1;
                if (nd & REMOTE) {
                    const uint32_t r = nd & ~REMOTE;
                    com = w.let.com[r]; q0 = w.let.q0[r]; q1 = w.let.q1[r];
                    cl = make_float4(0.f, 0.f, 0.f, 0.f);
                } else {
                    com = w.tv.nd_com[nd]; cl = w.tv.nd_comlo[nd]; q0 = w.tv.nd_q0[nd]; q1 = w.tv.nd_q1[nd];
                }
                s.cx[k] = (com.x - ox) + cl.x;
                s.cy[k] = (com.y - oy) + cl.y;
                s.cz[k] = (com.z - oz) + cl.z;
                s.cm[k] = com.w;
                s.qxx[k] = -q0.x; s.qxy[k] = -q0.y; s.qxz[k] = -q0.z; s.qyy[k] = -q0.w; s.qyz[k] = -q1.x;
                s.qzz[k] = -q1.y;
            } else {
                s.cx[k] = kFar; s.cy[k] = kFar; s.cz[k] = kFar; s.cm[k] = 0.f;
                s.qxx[k] = s.qxy[k] = s.qxz[k] = s.qyy[k] = s.qyz[k] = s.qzz[k] = 0.f;
            }
        }
        __syncwarp();
        eval_cells_n<POT, EPS0>(ipt, s, cc2, 2 * part, 2 * P, lane, xi, yi, zi, e2);
        __syncwarp();
    }
    if (nr == 0) return;
    const int total = range_prefix(s, nr, lane);
    const int Lw = 32 / P, lp = lane % Lw;
    for (int b0 = 0; b0 < total; b0 += BCH) {
        const int bc = min(BCH, total - b0);
        const int bc2 = (bc + pad) & ~pad;
        if (POT) {
            for (int i = lane; i < np; i += 32) s.kself[i] = -2;
            __syncwarp();
        }
        for (int k = lane; k < bc2; k += 32) {
            if (k < bc) {
                const uint32_t j = range_body(s, nr, b0 + k);
                if (POT && j - plo < static_cast<uint32_t>(np)) s.kself[j - plo] = k;
                float4 h, l;
                if (j & REMOTE) {
                    h = w.let.body[j & ~REMOTE];
                    l = make_float4(0.f, 0.f, 0.f, 0.f);
                } else {
                    h = w.hm[j];
                    l = w.lo[j];
                }
                s.bx[k] = (h.x - ox) + l.x;
                s.by[k] = (h.y - oy) + l.y;
                s.bz[k] = (h.z - oz) + l.z;
                s.bm[k] = h.w;
            } else {
                s.bx[k] = kFar; s.by[k] = kFar; s.bz[k] = kFar; s.bm[k] = 0.f;
            }
        }
        __syncwarp();
        int kself[IPT_MAX];
#pragma unroll
        for (int u = 0; u < IPT_MAX; ++u) {
            const int i = lp + Lw * u;
            kself[u] = POT && i < np ? s.kself[i] : -2;
        }
        eval_bodies_n<POT, EPS0>(ipt, s, bc2, 2 * part, 2 * P, lane, xi, yi, zi, kself, e2);
        __syncwarp();
    }
}

template <bool POT, bool EPS0>
__device__ void walk_pass(const WalkArgs& w, WarpSmem& s, uint32_t* stack, int lane, uint2 gr, float4 bc, float4 bh,
                          uint32_t plo, int np, unsigned long long& inter_b, unsigned long long& inter_c) {
    if (w.level) {
        bool active = false;
        for (int k = lane; k < np; k += 32) active |= w.level[plo + k] >= w.kmin;
        if (!__any_sync(0xffffffffu, active)) return;
    }
    const float ox = bc.x, oy = bc.y, oz = bc.z;
    // Entry partitions: the warp's lanes form P partitions of Lw = 32 / P lanes; every partition
    // holds all np i-bodies (ipt per lane) and evaluates every P-th pair of list entries, and the
    // partitions' sums are added at the end. P is the one of 1, 2, 4 with the least lane work
    // ipt / P (ties to the smaller P), so small groups keep every lane busy.
    int P = 1, ipt = (np + 31) >> 5;
    for (int q = 2; q <= 4; q *= 2) {
        const int iq = (np * q + 31) >> 5;
        if (iq <= IPT_MAX && iq * P < ipt * q) {
            P = q;
            ipt = iq;
        }
    }
    const int Lw = 32 / P, part = lane / Lw, lp = lane % Lw;
    float xi[IPT_MAX], yi[IPT_MAX], zi[IPT_MAX];
#pragma unroll
    for (int u = 0; u < IPT_MAX; ++u) {
        const int k = min(lp + Lw * u, np - 1);
        const float4 h = w.hm[plo + k], l = w.lo[plo + k];
        xi[u] = (h.x - ox) + l.x;
        yi[u] = (h.y - oy) + l.y;
        zi[u] = (h.z - oz) + l.z;
    }
#pragma unroll
    for (int u = 0; u < IPT_MAX; ++u)
#pragma unroll
        for (int f = 0; f < 8; ++f) s.ks[u][f][lane] = 0.f;
    const uint32_t root = w.sys ? w.sys[gr.x] : 0u;
    const float e2 = w.e2_sys ? w.e2_sys[root] : w.e2;
    uint32_t list_len = 0, cells_len = 0;
    auto fl = [&](int nc, int nr) {
        flush<POT, EPS0>(w, s, lane, ipt, part, P, nc, nr, ox, oy, oz, xi, yi, zi, e2, plo, np);
    };
    if (w.local) traverse(w.tv, s, stack, lane, gr, bc, bh, root, w.err, list_len, cells_len, fl);
    for (int t = 0; t < w.let.ntrees; ++t)
        traverse_let(w.let, s, stack, lane, bc, bh, w.let.roots[t], w.err, list_len, cells_len, fl);
    // With the local tree the own body is in the list (its leaf is inside the group, so it is
    // opened): it is not an interaction, adds nothing to a (d = 0) and is excluded from the
    // potential by index. Remote trees never hold the target.
    const uint32_t self = w.local ? 1u : 0u;
#pragma unroll
    for (int u = 0; u < IPT_MAX; ++u) {
        const float* ks = &s.ks[u][0][lane];
        float fx = ks[0] - ks[128], fy = ks[32] - ks[160], fz = ks[64] - ks[192], p = ks[96] - ks[224];
        // The partitions' sums, in a fixed order (all lanes take part in the shuffles).
        for (int o = Lw; o < 32; o <<= 1) {
            fx += __shfl_xor_sync(0xffffffffu, fx, o);
            fy += __shfl_xor_sync(0xffffffffu, fy, o);
            fz += __shfl_xor_sync(0xffffffffu, fz, o);
            if (POT) p += __shfl_xor_sync(0xffffffffu, p, o);
        }
        const int k = lp + Lw * u;
        if (part != 0 || k >= np) continue;
        const uint32_t i = plo + k;
        const float4 a = make_float4(w.G * fx, w.G * fy, w.G * fz, POT ? -w.G * p : 0.f);
        if (w.accumulate) {
            const float4 o = w.acc[i];
            w.acc[i] = make_float4(o.x + a.x, o.y + a.y, o.z + a.z, o.w + a.w);
            w.cost[i] += static_cast<float>(list_len);
        } else {
            w.acc[i] = a;
            w.cost[i] = static_cast<float>(list_len - self);
        }
    }
    inter_b += static_cast<unsigned long long>(list_len - cells_len - self) * static_cast<unsigned long long>(np);
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

namespace {
void launch_walk(Engine& e, WalkArgs& w, bool potential, bool eps0) {
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
}  // namespace

void tree_walk_remote_blocks(Engine& e, float G, float e2, bool potential, bool eps0, const LetView& let,
                             const TreeView& blocks) {
    WalkArgs w{};
    w.tv = blocks;
    BodyArrays b = e.bodies(e.cur);
    w.hm = b.hm;
    w.lo = b.lo;
    w.acc = e.acc.as<float4>();
    w.cost = b.cost;
    w.group_ctr = reinterpret_cast<unsigned*>(e.small.as<char>() + 36);
    w.inter = e.inter_counter();
    w.err = e.err_word();
    w.G = G;
    w.e2 = e2;
    w.let = let;
    w.local = 0;
    w.accumulate = 1;
    launch_walk(e, w, potential, eps0);
}

void tree_walk(Engine& e, float G, float e2, bool potential, bool eps0, const uint32_t* sys, const float* e2_sys,
               const LetView* let) {
    WalkArgs w{};
    w.sys = sys;
    w.e2_sys = e2_sys;
    if (let) w.let = *let;
    w.local = 1;
    w.accumulate = 0;
    if (e.walk_kmin >= 0) {
        w.level = e.bodies(e.cur).level;
        w.kmin = e.walk_kmin;
    }
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
    launch_walk(e, w, potential, eps0);
}

}  // namespace lg
