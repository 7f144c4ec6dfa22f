// The tree walk's list construction, shared by the force walk (walk.cu) and its vector-Jacobian
// product (walk_vjp.cu): one warp, one walk group, the reference CPU backend's opening rule
// (src/cpu_backend.cpp:816-838 build_list).
#pragma once

#include "engine.cuh"

namespace lg {
namespace walk {

constexpr int SMALL_LEAF = 4;   // src/cpu_backend.cpp:29
constexpr int SCAP = 16384;     // global traversal stack entries per warp (LET walk; overflow of the shared stack)
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
// `root`. Each step takes up to 32 nodes, one per lane: a node that contains the group, or whose box
// distance d satisfies d^2 < rcrit2, is opened (src/cpu_backend.cpp:826-828; d^2 formed as the
// reference's compiler forms it, fma(dz, dz, fma(dx, dx, dy*dy))); an accepted leaf of
// <= SMALL_LEAF bodies is taken as bodies, other accepted nodes as cells; opened leaves give
// bodies, opened internal nodes push their children. Cells are appended to s.clist and body
// ranges to s.rlist (ballot-compacted); flush(nc, nr) is called when a list fills and once at the
// end, and must consume them. list_len / cells_len count the entries (cells + bodies) and cells.
//
// The stack lives in shared memory (s.sstk, SSTK entries) and holds child blocks, one entry per
// opened node: (first child << 3) | (children - 1), children being contiguous in the reference's
// node order. A step reads the top entries, takes the first 32 nodes they hold (a block only partly
// taken keeps its tail on the stack), and pushes one entry per node it opens, so a step does no
// global-memory round trip for the stack. When a push would overflow the shared stack, its bottom
// SPILL entries move to the warp's slice of `stack` in global memory and come back when the shared
// part empties (rare: a 1e6-body disk needs at most ~70 entries). The children of an opened node
// are prefetched into L1 when it is pushed. Stack or node overflow sets the error word and ends
// the traversal.
constexpr int SSTK = 256;   // shared-memory stack entries per warp
constexpr int SPILL = 128;  // entries moved between the shared and the global part at a time
static_assert(SSTK - SPILL >= 32 && SPILL % 32 == 0, "a spill leaves room for one step's pushes");
constexpr uint32_t kMaxNodeIndex = (1u << 29) - 1;  // first-child indices fit the packed entry

__device__ __forceinline__ void prefetch_l1(const void* p) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

template <class S, class F>
__device__ __forceinline__ void traverse(const TreeView& tv, S& s, uint32_t* stack, int lane, uint2 gr, float4 bc,
                                         float4 bh, uint32_t root, unsigned* err, uint32_t& list_len,
                                         uint32_t& cells_len, F&& flush) {
    const unsigned lt = (1u << lane) - 1u;
    int sp = 1, gsp = 0;  // entries in the shared part, entries in the global part
    if (lane == 0) s.sstk[0] = root << 3;
    __syncwarp();
    int nc = 0, nr = 0, nbr = 0;
    bool overflow = false;
    // Each node is visited at most once per pass; the cap stops a malformed tree.
    const uint32_t max_iter = static_cast<uint32_t>(tv.T) + 64u;
    uint32_t iter = 0;
    for (;;) {
        if (sp == 0 && gsp > 0) {  // refill from the global part (its top SPILL entries)
            const int k = min(SPILL, gsp);
            for (int q = lane; q < k; q += 32) s.sstk[q] = stack[gsp - k + q];
            gsp -= k;
            sp = k;
            __syncwarp();
        }
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
        // Take up to 32 nodes from the top blocks: lane l reads the l-th entry from the top.
        const int nread = min(32, sp);
        const uint32_t ent = lane < nread ? s.sstk[sp - 1 - lane] : 0u;
        const int cnt = lane < nread ? static_cast<int>(ent & 7u) + 1 : 0;
        int total;
        const int excl = warp_excl_scan(cnt, lane, total);
        const int take = min(32, total);
        // Blocks wholly taken, and the block (if any) only partly taken, which keeps its tail.
        const unsigned full = __ballot_sync(0xffffffffu, cnt > 0 && excl + cnt <= 32);
        const int nfull = __popc(full);
        const unsigned starts = __reduce_or_sync(0xffffffffu, cnt > 0 && excl < 32 ? (1u << excl) : 0u);
        if (lane == nfull && cnt > 0 && excl < 32)
            s.sstk[sp - 1 - lane] = ent + (static_cast<uint32_t>(32 - excl) << 3) - static_cast<uint32_t>(32 - excl);
        const bool have = lane < take;
        const int r = __popc(starts & (lane == 31 ? 0xffffffffu : (2u << lane) - 1u)) - 1;
        const uint32_t rent = __shfl_sync(0xffffffffu, ent, r & 31);
        const int rexcl = __shfl_sync(0xffffffffu, excl, r & 31);
        const uint32_t node = have ? (rent >> 3) + static_cast<uint32_t>(lane - rexcl) : 0u;
        sp -= nfull;
        __syncwarp();
        int kind = 0;  // 1 cell, 2 bodies, 3 children
        uint32_t a0 = 0, a1 = 0;
        if (have && node >= tv.T) {
            atomicOr(err, kErrNodeOverflow);
        } else if (have) {
            const uint4 rg = tv.nd_range[node];
            const float4 com = tv.nd_com[node];
            const float rc2 = tv.nd_q1[node].z;
            const float dx = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.x, bc.x)), bh.x), 0.f);
            const float dy = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.y, bc.y)), bh.y), 0.f);
            const float dz = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.z, bc.z)), bh.z), 0.f);
            const float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
            const bool contains = rg.x <= gr.x && gr.y <= rg.y;
            const bool leaf = rg.w == 0;
            if (!contains && d2 >= rc2) {
                if (leaf && rg.y - rg.x <= static_cast<unsigned>(SMALL_LEAF)) { kind = 2; a0 = rg.x; a1 = rg.y - rg.x; }
                else { kind = 1; a0 = node; }
            } else if (leaf) {
                kind = 2; a0 = rg.x; a1 = rg.y - rg.x;
            } else if (rg.w <= 8u && rg.z <= kMaxNodeIndex && rg.z + rg.w <= tv.T) {
                kind = 3; a0 = rg.z; a1 = rg.w;
                prefetch_l1(tv.nd_range + a0);
                prefetch_l1(tv.nd_com + a0);
                prefetch_l1(tv.nd_q1 + a0);
            } else {
                atomicOr(err, kErrNodeOverflow);
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
        const unsigned pm = __ballot_sync(0xffffffffu, kind == 3);
        const int npush = __popc(pm);
        if (sp + npush > SSTK) {  // spill the bottom SPILL entries to the global part
            if (gsp + SPILL > SCAP) {
                overflow = true;
                break;
            }
            for (int q = lane; q < SPILL; q += 32) stack[gsp + q] = s.sstk[q];
            uint32_t keep[(SSTK - SPILL) / 32];
#pragma unroll
            for (int u = 0; u < (SSTK - SPILL) / 32; ++u) {
                const int q = SPILL + lane + 32 * u;
                keep[u] = q < sp ? s.sstk[q] : 0u;
            }
            __syncwarp();
#pragma unroll
            for (int u = 0; u < (SSTK - SPILL) / 32; ++u) {
                const int q = SPILL + lane + 32 * u;
                if (q < sp) s.sstk[q - SPILL] = keep[u];
            }
            gsp += SPILL;
            sp -= SPILL;
            __syncwarp();
        }
        if (kind == 3) s.sstk[sp + __popc(pm & lt)] = (a0 << 3) | (a1 - 1u);
        sp += npush;
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
                const float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
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
