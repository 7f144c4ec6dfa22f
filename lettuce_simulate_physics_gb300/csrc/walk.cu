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
//    coordinates relative to the group's box centre o, (x_hi - o) + x_lo in FP32, in shared
//    memory, and every lane evaluates them for its IPT i-bodies (IPT = ceil(group size / 32)):
//    quadrupole cell terms (cuda_backend.cu:783-800 / cpu_backend.cpp:858-871 math) and
//    softened body terms. Chunk sums are added to the running sums with Kahan compensation.
// The interaction count per body is the list length minus its own entry; the reference CPU
// backend counts that self entry, so its count exceeds this one by exactly N.
#include "engine.cuh"

namespace lg {

namespace {

constexpr int WBS = 128;  // 4 warps per block
constexpr int WARPS = WBS / 32;
constexpr int SMALL_LEAF = 4;   // src/cpu_backend.cpp:29
constexpr int SCAP = 16384;     // traversal stack entries per warp (global memory)
constexpr int CL_CAP = 160, CL_FLUSH = 128;
constexpr int RL_CAP = 96, RL_FLUSH = 64;
constexpr int BR_FLUSH = 256;
constexpr int CCH = 64;   // cells converted per chunk
constexpr int BCH = 128;  // bodies converted per chunk
constexpr int PASS = 128; // i-bodies per pass (4 per lane)

struct WarpSmem {
    uint32_t clist[CL_CAP];
    uint2 rlist[RL_CAP];
    uint32_t rpre[RL_CAP + 1];
    float4 cpos[CCH];
    float4 cq0[CCH];
    float2 cq1[CCH];
    float4 bpos[BCH];
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

template <int IPT, bool POT, bool EPS0>
struct Acc {
    float sx[IPT], sy[IPT], sz[IPT], sp[IPT], cx[IPT], cy[IPT], cz[IPT], cp[IPT];
    float px[IPT], py[IPT], pz[IPT], pp[IPT];
    __device__ void zero_all() {
#pragma unroll
        for (int u = 0; u < IPT; ++u) sx[u] = sy[u] = sz[u] = sp[u] = cx[u] = cy[u] = cz[u] = cp[u] = 0.f;
    }
    __device__ void zero_partial() {
#pragma unroll
        for (int u = 0; u < IPT; ++u) px[u] = py[u] = pz[u] = pp[u] = 0.f;
    }
    __device__ void merge() {
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            kahan_add(sx[u], cx[u], px[u]);
            kahan_add(sy[u], cy[u], py[u]);
            kahan_add(sz[u], cz[u], pz[u]);
            if (POT) kahan_add(sp[u], cp[u], pp[u]);
        }
    }
};

template <int IPT, bool POT, bool EPS0>
__device__ __forceinline__ void eval_cells(const WarpSmem& s, int cc, const float (&xi)[IPT], const float (&yi)[IPT],
                                           const float (&zi)[IPT], float e2, Acc<IPT, POT, EPS0>& a) {
#pragma unroll 2
    for (int k = 0; k < cc; ++k) {
        const float4 p = s.cpos[k];
        const float4 q0 = s.cq0[k];
        const float2 q1 = s.cq1[k];
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            const float dx = p.x - xi[u], dy = p.y - yi[u], dz = p.z - zi[u];
            const float r2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmaf_rn(dz, dz, e2)));
            float inv = rsqrt_mufu(r2);
            if (EPS0) inv = r2 > 0.f ? inv : 0.f;
            const float inv2 = inv * inv, inv3 = inv * inv2, inv5 = inv3 * inv2;
            // d points from the body to the cell: a = G [M d/r^3 - Q d/r^5 + 5/2 (dQd) d/r^7].
            const float qx = __fmaf_rn(q0.x, dx, __fmaf_rn(q0.y, dy, q0.z * dz));
            const float qy = __fmaf_rn(q0.y, dx, __fmaf_rn(q0.w, dy, q1.x * dz));
            const float qz = __fmaf_rn(q0.z, dx, __fmaf_rn(q1.x, dy, q1.y * dz));
            const float dqd = __fmaf_rn(dx, qx, __fmaf_rn(dy, qy, dz * qz));
            const float t5 = dqd * inv5;
            const float f = __fmaf_rn(p.w, inv3, 2.5f * t5 * inv2);
            a.px[u] = __fmaf_rn(-qx, inv5, __fmaf_rn(f, dx, a.px[u]));
            a.py[u] = __fmaf_rn(-qy, inv5, __fmaf_rn(f, dy, a.py[u]));
            a.pz[u] = __fmaf_rn(-qz, inv5, __fmaf_rn(f, dz, a.pz[u]));
            if (POT) a.pp[u] += __fmaf_rn(p.w, inv, 0.5f * t5);
        }
    }
}

template <int IPT, bool POT, bool EPS0>
__device__ __forceinline__ void eval_bodies(const WarpSmem& s, int bc, const float (&xi)[IPT], const float (&yi)[IPT],
                                            const float (&zi)[IPT], float e2, Acc<IPT, POT, EPS0>& a) {
#pragma unroll 4
    for (int k = 0; k < bc; ++k) {
        const float4 q = s.bpos[k];
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            const float dx = q.x - xi[u], dy = q.y - yi[u], dz = q.z - zi[u];
            const float r2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmaf_rn(dz, dz, e2)));
            float inv = rsqrt_mufu(r2);
            if (EPS0) inv = r2 > 0.f ? inv : 0.f;
            const float mi = __fmul_rn(q.w, inv);  // rounded: the self term cancels exactly
            const float f = mi * (inv * inv);
            a.px[u] = __fmaf_rn(f, dx, a.px[u]);
            a.py[u] = __fmaf_rn(f, dy, a.py[u]);
            a.pz[u] = __fmaf_rn(f, dz, a.pz[u]);
            if (POT) a.pp[u] += mi;
        }
    }
}

// Evaluates the pending lists for the pass's i-bodies and empties them.
template <int IPT, bool POT, bool EPS0>
__device__ void flush(const WalkArgs& w, WarpSmem& s, int lane, int nc, int nr, float ox, float oy, float oz,
                      const float (&xi)[IPT], const float (&yi)[IPT], const float (&zi)[IPT], Acc<IPT, POT, EPS0>& a) {
    for (int c0 = 0; c0 < nc; c0 += CCH) {
        const int cc = min(CCH, nc - c0);
        for (int k = lane; k < cc; k += 32) {
            const uint32_t nd = s.clist[c0 + k];
            const float4 com = w.tv.nd_com[nd], cl = w.tv.nd_comlo[nd], q0 = w.tv.nd_q0[nd], q1 = w.tv.nd_q1[nd];
            s.cpos[k] = make_float4((com.x - ox) + cl.x, (com.y - oy) + cl.y, (com.z - oz) + cl.z, com.w);
            s.cq0[k] = q0;
            s.cq1[k] = make_float2(q1.x, q1.y);
        }
        __syncwarp();
        a.zero_partial();
        eval_cells<IPT, POT, EPS0>(s, cc, xi, yi, zi, w.e2, a);
        a.merge();
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
        for (int k = lane; k < bc; k += 32) {
            const uint32_t p = b0 + k;
            int lo = 0, hi = nr;  // last r with rpre[r] <= p
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (s.rpre[mid] <= p) lo = mid;
                else hi = mid;
            }
            const uint32_t j = s.rlist[lo].x + (p - s.rpre[lo]);
            const float4 h = w.hm[j], l = w.lo[j];
            s.bpos[k] = make_float4((h.x - ox) + l.x, (h.y - oy) + l.y, (h.z - oz) + l.z, h.w);
        }
        __syncwarp();
        a.zero_partial();
        eval_bodies<IPT, POT, EPS0>(s, bc, xi, yi, zi, w.e2, a);
        a.merge();
        __syncwarp();
    }
}

template <int IPT, bool POT, bool EPS0>
__device__ void walk_pass(const WalkArgs& w, WarpSmem& s, uint32_t* stack, int lane, uint2 gr, float4 bc, float4 bh,
                          uint32_t plo, int np, unsigned long long& inter_b, unsigned long long& inter_c) {
    const float ox = bc.x, oy = bc.y, oz = bc.z;
    float xi[IPT], yi[IPT], zi[IPT], mi[IPT];
#pragma unroll
    for (int u = 0; u < IPT; ++u) {
        const int k = min(lane + 32 * u, np - 1);
        const float4 h = w.hm[plo + k], l = w.lo[plo + k];
        xi[u] = (h.x - ox) + l.x;
        yi[u] = (h.y - oy) + l.y;
        zi[u] = (h.z - oz) + l.z;
        mi[u] = h.w;
    }
    Acc<IPT, POT, EPS0> a;
    a.zero_all();
    const unsigned lt = (1u << lane) - 1u;
    int sp = 1;
    if (lane == 0) stack[0] = 0;
    __syncwarp();
    int nc = 0, nr = 0, nbr = 0;
    uint32_t list_len = 0, cells_len = 0;
    bool overflow = false;
    // Each node is visited at most once per pass; the cap stops a malformed tree.
    const uint32_t max_iter = static_cast<uint32_t>(w.tv.T) + 64u;
    uint32_t iter = 0;
    while (sp > 0) {
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
        if (nc >= CL_FLUSH || nr >= RL_FLUSH || nbr >= BR_FLUSH) {
            flush<IPT, POT, EPS0>(w, s, lane, nc, nr, ox, oy, oz, xi, yi, zi, a);
            list_len += nc + nbr;
            cells_len += nc;
            nc = nr = nbr = 0;
        }
    }
    if (overflow) {
        if (lane == 0) atomicOr(w.err, iter > max_iter ? kErrNodeOverflow : kErrStackOverflow);
    } else {
        flush<IPT, POT, EPS0>(w, s, lane, nc, nr, ox, oy, oz, xi, yi, zi, a);
        list_len += nc + nbr;
        cells_len += nc;
    }
    const float self_inv = (POT && !EPS0) ? rsqrt_mufu(w.e2) : 0.f;
#pragma unroll
    for (int u = 0; u < IPT; ++u) {
        const int k = lane + 32 * u;
        if (k >= np) continue;
        const uint32_t i = plo + k;
        float p = a.sp[u] - a.cp[u];
        // The own body is always in the list (its leaf is inside the group, so it is opened);
        // with eps > 0 its pair has d = 0 and only adds m_i/eps to the potential.
        if (POT && !EPS0) p = __fsub_rn(p, __fmul_rn(mi[u], self_inv));
        w.acc[i] = make_float4(w.G * (a.sx[u] - a.cx[u]), w.G * (a.sy[u] - a.cy[u]), w.G * (a.sz[u] - a.cz[u]),
                               POT ? -w.G * p : 0.f);
        w.cost[i] = static_cast<float>(list_len - 1);
    }
    inter_b += static_cast<unsigned long long>(list_len - cells_len - 1) * static_cast<unsigned long long>(np);
    inter_c += static_cast<unsigned long long>(cells_len) * static_cast<unsigned long long>(np);
}

template <bool POT, bool EPS0>
__global__ void __launch_bounds__(WBS) k_walk(WalkArgs w) {
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
            switch ((np + 31) >> 5) {
                case 1: walk_pass<1, POT, EPS0>(w, s, stack, lane, gr, bc, bh, plo, np, inter_b, inter_c); break;
                case 2: walk_pass<2, POT, EPS0>(w, s, stack, lane, gr, bc, bh, plo, np, inter_b, inter_c); break;
                case 3: walk_pass<3, POT, EPS0>(w, s, stack, lane, gr, bc, bh, plo, np, inter_b, inter_c); break;
                default: walk_pass<4, POT, EPS0>(w, s, stack, lane, gr, bc, bh, plo, np, inter_b, inter_c); break;
            }
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

void tree_walk(Engine& e, float G, float e2, bool potential, bool eps0) {
    WalkArgs w;
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
