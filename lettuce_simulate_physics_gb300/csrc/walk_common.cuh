// The tree walk's list construction, shared by the force walk (walk.cu) and its vector-Jacobian
// product (walk_vjp.cu): one warp, one walk group, the reference CPU backend's opening rule
// (src/cpu_backend.cpp:816-838 build_list).
#pragma once

#include "engine.cuh"

namespace lg {
namespace walk {

constexpr int SMALL_LEAF = 4;   // src/cpu_backend.cpp:29
constexpr int SCAP = 16384;     // traversal stack entries per warp (global memory)
constexpr int CL_CAP = 160, CL_FLUSH = 128;
constexpr int RL_CAP = 96, RL_FLUSH = 64;
constexpr int BR_FLUSH = 256;

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

// Warp-cooperative depth-first traversal for the group of bodies gr with box (bc, bh), from node
// `root`. Each step pops up to 32 nodes, one per lane: a node that contains the group, or whose box
// distance d satisfies d^2 < rcrit2, is opened (src/cpu_backend.cpp:826-828); an accepted leaf of
// <= SMALL_LEAF bodies is taken as bodies, other accepted nodes as cells; opened leaves give
// bodies, opened internal nodes push their children. Cells are appended to s.clist and body
// ranges to s.rlist (ballot-compacted); flush(nc, nr) is called when a list fills and once at the
// end, and must consume them. list_len / cells_len count the entries (cells + bodies) and cells.
// Stack or node overflow sets the error word and ends the traversal.
template <class S, class F>
__device__ __forceinline__ void traverse(const TreeView& tv, S& s, uint32_t* stack, int lane, uint2 gr, float4 bc,
                                         float4 bh, uint32_t root, unsigned* err, uint32_t& list_len,
                                         uint32_t& cells_len, F&& flush) {
    const unsigned lt = (1u << lane) - 1u;
    int sp = 1;
    if (lane == 0) stack[0] = root;
    __syncwarp();
    int nc = 0, nr = 0, nbr = 0;
    bool overflow = false;
    // Each node is visited at most once per pass; the cap stops a malformed tree.
    const uint32_t max_iter = static_cast<uint32_t>(tv.T) + 64u;
    uint32_t iter = 0;
    for (;;) {
        const bool done = sp == 0;
        // One evaluation site: when the lists fill up, and once at the end.
        if (done || nc >= CL_FLUSH || nr >= RL_FLUSH || nbr >= BR_FLUSH) {
            flush(nc, nr);
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
        if (have && node >= tv.T) {
            atomicOr(err, kErrNodeOverflow);
        } else if (have) {
            const uint4 r = tv.nd_range[node];
            const float4 com = tv.nd_com[node];
            const float rc2 = tv.nd_q1[node].z;
            const float dx = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.x, bc.x)), bh.x), 0.f);
            const float dy = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.y, bc.y)), bh.y), 0.f);
            const float dz = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.z, bc.z)), bh.z), 0.f);
            const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
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
    if (overflow && lane == 0) atomicOr(err, iter > max_iter ? kErrNodeOverflow : kErrStackOverflow);
}

// List entries from a remote tree carry this bit (cell: node index; body range: first body).
constexpr uint32_t REMOTE = 0x80000000u;

// The receiver walk of a remote tree (src/backend.hpp:77-82, src/cpu_backend.cpp:787-812) for the
// group box (bc, bh), warp-cooperative like traverse(): a node with no children and no bodies, or
// whose box distance d satisfies d^2 >= rcrit2, is accepted (as bodies when it holds 1..SMALL_LEAF
// of them, else as a multipole); otherwise its bodies, or else its children, are taken. Appends
// to the same lists (entries flagged REMOTE) and flushes like traverse().
template <class S, class F>
__device__ __forceinline__ void traverse_let(const LetView& lv, S& s, uint32_t* stack, int lane, float4 bc, float4 bh,
                                             uint32_t root, unsigned* err, uint32_t& list_len, uint32_t& cells_len,
                                             F&& flush) {
    const unsigned lt = (1u << lane) - 1u;
    int sp = 1;
    if (lane == 0) stack[0] = root;
    __syncwarp();
    int nc = 0, nr = 0, nbr = 0;
    bool overflow = false;
    const uint32_t max_iter = lv.nnodes + 64u;
    uint32_t iter = 0;
    for (;;) {
        const bool done = sp == 0;
        if (done || nc >= CL_FLUSH || nr >= RL_FLUSH || nbr >= BR_FLUSH) {
            flush(nc, nr);
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
        if (have && node >= lv.nnodes) {
            atomicOr(err, kErrNodeOverflow);
        } else if (have) {
            const int4 L = lv.link[node];
            const bool terminal = L.x < 0 && L.w == 0;
            bool accept = terminal;
            if (!terminal) {
                const float4 com = lv.com[node];
                const float rc2 = lv.q1[node].z;
                const float dx = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.x, bc.x)), bh.x), 0.f);
                const float dy = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.y, bc.y)), bh.y), 0.f);
                const float dz = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.z, bc.z)), bh.z), 0.f);
                const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                accept = d2 >= rc2;
            }
            if (accept) {
                if (L.w > 0 && L.w <= SMALL_LEAF) { kind = 2; a0 = REMOTE | static_cast<uint32_t>(L.z); a1 = L.w; }
                else { kind = 1; a0 = REMOTE | node; }
            } else if (L.w > 0) {
                kind = 2; a0 = REMOTE | static_cast<uint32_t>(L.z); a1 = L.w;
            } else if (L.y > 0) {
                kind = 3; a0 = static_cast<uint32_t>(L.x); a1 = L.y;
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
    if (overflow && lane == 0) atomicOr(err, iter > max_iter ? kErrNodeOverflow : kErrStackOverflow);
}

// Prefix sums of the pending body ranges' lengths into s.rpre (nr <= RL_CAP); returns the total.
template <class S>
__device__ __forceinline__ int range_prefix(S& s, int nr, int lane) {
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
    return static_cast<int>(s.rpre[nr]);
}

// Body index of the p-th body of the pending ranges (binary search over s.rpre).
template <class S>
__device__ __forceinline__ uint32_t range_body(const S& s, int nr, uint32_t p) {
    int lo = 0, hi = nr;  // last r with rpre[r] <= p
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (s.rpre[mid] <= p) lo = mid;
        else hi = mid;
    }
    return s.rlist[lo].x + (p - s.rpre[lo]);
}

}  // namespace walk
}  // namespace lg
