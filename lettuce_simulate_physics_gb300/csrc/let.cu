// Locally-essential trees (LETs): the reference's multi-rank support (src/backend.hpp:50-86).
//  - let_upload: remote trees to the device for the walk (walk_common.cuh traverse_let), indices
//    made global over the concatenated trees, every link checked on the host first.
//  - let_body_blocks: blocks of 128 consecutive bodies with their FP32 bounding boxes, the direct
//    method's receiver groups (src/cpu_backend.cpp:695-728).
//  - let_export: this engine's tree for a target box, built on the device level by level: a
//    node whose box distance d to the target satisfies d^2 >= rcrit2 is terminal; an opened leaf
//    exports its bodies; an opened internal node exports its children of positive mass as one
//    contiguous block. Processing each level in order and placing children blocks by a scan gives
//    exactly the reference's breadth-first order (src/cpu_backend.cpp:222-270), in which the
//    output doubles as the queue. The direct method exports one always-open root holding every
//    body (src/cpu_backend.cpp:730-747).
#include <cfloat>
#include <cstring>
#include <string>
#include <vector>

#include "engine.cuh"

namespace lg {

struct LetStore {
    // remote trees (device) and their host staging, kept until the next upload
    DevBuf com, q0, q1, link, body, roots;
    std::vector<float4> h_com, h_q0, h_q1, h_body;
    std::vector<int4> h_link;
    std::vector<uint32_t> h_roots;
    // direct-method receiver blocks
    DevBuf blk_range, blk_box, blk_count;
    // export
    DevBuf out_nodes, out_body, front_a, front_b, kind, ccount, bcount, cscan, bscan, totals;
    size_t out_n = 0, out_b = 0;
};

namespace {

void destroy_let_store(LetStore* s) { delete s; }

inline int grid_for(long long n, int bs) { return static_cast<int>((n + bs - 1) / bs); }

// One warp per block of `block` consecutive bodies: range and FP32 bounding box (centre, half).
__global__ void k_block_groups(const float4* __restrict__ hm, int n, int block, uint2* range, float4* box,
                               unsigned* count) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int nb = (n + block - 1) / block;
    if (w == 0 && lane == 0) *count = static_cast<unsigned>(nb);
    if (w >= nb) return;
    const int lo = w * block, hi = min(n, lo + block);
    const float4 h0 = hm[lo];
    float mn[3] = {h0.x, h0.y, h0.z}, mx[3] = {h0.x, h0.y, h0.z};
    for (int i = lo + lane; i < hi; i += 32) {
        const float4 h = hm[i];
        mn[0] = fminf(mn[0], h.x); mn[1] = fminf(mn[1], h.y); mn[2] = fminf(mn[2], h.z);
        mx[0] = fmaxf(mx[0], h.x); mx[1] = fmaxf(mx[1], h.y); mx[2] = fmaxf(mx[2], h.z);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
        for (int o = 16; o > 0; o >>= 1) {
            mn[c] = fminf(mn[c], __shfl_xor_sync(0xffffffffu, mn[c], o));
            mx[c] = fmaxf(mx[c], __shfl_xor_sync(0xffffffffu, mx[c], o));
        }
    if (lane == 0) {
        range[w] = make_uint2(static_cast<unsigned>(lo), static_cast<unsigned>(hi));
        box[2 * w] = make_float4(0.5f * (mn[0] + mx[0]), 0.5f * (mn[1] + mx[1]), 0.5f * (mn[2] + mx[2]), 0.f);
        box[2 * w + 1] = make_float4(0.5f * (mx[0] - mn[0]), 0.5f * (mx[1] - mn[1]), 0.5f * (mx[2] - mn[2]), 0.f);
    }
}

// Export, per level: kind (0 terminal, 1 opened leaf, 2 opened internal node) and what each
// frontier node contributes to the next level (children of positive mass) and to the bodies.
__global__ void k_let_decide(TreeView tv, const uint32_t* __restrict__ front, int nf, float4 bc, float4 bh,
                             uint32_t* kind, uint32_t* ccount, uint32_t* bcount) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nf) return;
    const uint32_t nd = front[k];
    const uint4 r = tv.nd_range[nd];
    const float4 com = tv.nd_com[nd];
    const float rc2 = tv.nd_q1[nd].z;
    const float dx = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.x, bc.x)), bh.x), 0.f);
    const float dy = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.y, bc.y)), bh.y), 0.f);
    const float dz = fmaxf(__fsub_rn(fabsf(__fsub_rn(com.z, bc.z)), bh.z), 0.f);
    const float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
    uint32_t kd = 0, c = 0, b = 0;
    if (!(d2 >= rc2)) {
        if (r.w == 0) {
            kd = 1;
            b = r.y - r.x;
        } else {
            kd = 2;
            for (uint32_t ch = r.z; ch < r.z + r.w; ++ch) c += tv.nd_com[ch].w > 0.f ? 1u : 0u;
        }
    }
    kind[k] = kd;
    ccount[k] = c;
    bcount[k] = b;
}

// Exclusive scans of the two count arrays in one block (frontiers hold at most the node count);
// totals[0], totals[1] = their sums.
__global__ void k_let_scan(const uint32_t* __restrict__ ca, const uint32_t* __restrict__ ba, int nf, uint32_t* cs,
                           uint32_t* bs, uint32_t* totals) {
    __shared__ uint32_t sc[1024], sb[1024];
    uint32_t carry_c = 0, carry_b = 0;
    for (int base = 0; base < nf; base += 1024) {
        const int k = base + static_cast<int>(threadIdx.x);
        const uint32_t vc = k < nf ? ca[k] : 0u, vb = k < nf ? ba[k] : 0u;
        sc[threadIdx.x] = vc;
        sb[threadIdx.x] = vb;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const uint32_t tc = static_cast<int>(threadIdx.x) >= o ? sc[threadIdx.x - o] : 0u;
            const uint32_t tb = static_cast<int>(threadIdx.x) >= o ? sb[threadIdx.x - o] : 0u;
            __syncthreads();
            sc[threadIdx.x] += tc;
            sb[threadIdx.x] += tb;
            __syncthreads();
        }
        if (k < nf) {
            cs[k] = carry_c + sc[threadIdx.x] - vc;
            bs[k] = carry_b + sb[threadIdx.x] - vb;
        }
        carry_c += sc[1023];
        carry_b += sb[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        totals[0] = carry_c;
        totals[1] = carry_b;
    }
}

// Writes the level's nodes (out index base + k), the next frontier and the opened leaves' bodies.
__global__ void k_let_emit(TreeView tv, const float4* __restrict__ hm, const uint32_t* __restrict__ front, int nf,
                           const uint32_t* __restrict__ kind, const uint32_t* __restrict__ ccount,
                           const uint32_t* __restrict__ bcount, const uint32_t* __restrict__ cs,
                           const uint32_t* __restrict__ bs, uint32_t base, uint32_t next_base, uint32_t body_base,
                           lg_let_node* out, uint32_t* next, float4* out_body) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nf) return;
    const uint32_t nd = front[k];
    const uint4 r = tv.nd_range[nd];
    const float4 com = tv.nd_com[nd], q0 = tv.nd_q0[nd], q1 = tv.nd_q1[nd];
    lg_let_node o;
    o.cx = com.x; o.cy = com.y; o.cz = com.z; o.mass = com.w;
    o.qxx = q0.x; o.qxy = q0.y; o.qxz = q0.z; o.qyy = q0.w; o.qyz = q1.x; o.qzz = q1.y;
    o.rcrit2 = q1.z;
    o.first_child = -1; o.child_count = 0; o.body_first = -1; o.body_count = 0;
    const uint32_t kd = kind[k];
    if (kd == 1) {
        const uint32_t b0 = body_base + bs[k], nb = bcount[k];
        o.body_first = static_cast<int32_t>(b0);
        o.body_count = static_cast<int32_t>(nb);
        for (uint32_t j = 0; j < nb; ++j) out_body[b0 + j] = hm[r.x + j];
    } else if (kd == 2) {
        // The children block, possibly empty: first_child is where it starts, as in the reference.
        o.first_child = static_cast<int32_t>(next_base + cs[k]);
        o.child_count = static_cast<int32_t>(ccount[k]);
        uint32_t j = cs[k];
        for (uint32_t ch = r.z; ch < r.z + r.w; ++ch)
            if (tv.nd_com[ch].w > 0.f) next[j++] = ch;
    }
    out[base + k] = o;
}

}  // namespace

std::unique_ptr<LetStore, void (*)(LetStore*)> make_let_store() {
    return std::unique_ptr<LetStore, void (*)(LetStore*)>(new LetStore, destroy_let_store);
}

LetView let_upload(Engine& e, const lg_let_tree* remote, size_t nremote) {
    LetStore& s = *e.lets;
    s.h_com.clear(); s.h_q0.clear(); s.h_q1.clear(); s.h_body.clear(); s.h_link.clear(); s.h_roots.clear();
    size_t nn = 0, nb = 0;
    for (size_t t = 0; t < nremote; ++t) {
        const lg_let_tree& L = remote[t];
        if (L.nnodes == 0) continue;
        if (!L.nodes) fail(kArg, "compute_forces_with: remote tree " + std::to_string(t) + " has no node array");
        if (L.nbodies > 0 && (!L.bx || !L.by || !L.bz || !L.bm))
            fail(kArg, "compute_forces_with: remote tree " + std::to_string(t) + " has no body arrays");
        nn += L.nnodes;
        nb += L.nbodies;
    }
    if (nn >= (size_t(1) << 31) || nb >= (size_t(1) << 31)) fail(kArg, "compute_forces_with: remote trees too large");
    LetView v{};
    if (nn == 0) return v;
    s.h_com.reserve(nn); s.h_q0.reserve(nn); s.h_q1.reserve(nn); s.h_link.reserve(nn); s.h_body.reserve(nb + 1);
    size_t nbase = 0, bbase = 0;
    for (size_t t = 0; t < nremote; ++t) {
        const lg_let_tree& L = remote[t];
        if (L.nnodes == 0) continue;
        for (size_t k = 0; k < L.nnodes; ++k) {
            const lg_let_node& d = L.nodes[k];
            const bool kids = d.child_count > 0, bods = d.body_count > 0;
            if (d.child_count < 0 || d.body_count < 0 ||
                (kids && (d.first_child < 0 || static_cast<size_t>(d.first_child) + d.child_count > L.nnodes)) ||
                (bods && (d.body_first < 0 || static_cast<size_t>(d.body_first) + d.body_count > L.nbodies)))
                fail(kArg, "compute_forces_with: remote tree " + std::to_string(t) + " node " + std::to_string(k) +
                               " links outside the tree");
            s.h_com.push_back(make_float4(d.cx, d.cy, d.cz, d.mass));
            s.h_q0.push_back(make_float4(d.qxx, d.qxy, d.qxz, d.qyy));
            s.h_q1.push_back(make_float4(d.qyz, d.qzz, d.rcrit2, 0.f));
            s.h_link.push_back(make_int4(d.first_child >= 0 ? static_cast<int>(d.first_child + nbase) : -1,
                                         d.child_count,
                                         bods ? static_cast<int>(d.body_first + bbase) : -1, d.body_count));
        }
        for (size_t k = 0; k < L.nbodies; ++k) s.h_body.push_back(make_float4(L.bx[k], L.by[k], L.bz[k], L.bm[k]));
        s.h_roots.push_back(static_cast<uint32_t>(nbase));
        nbase += L.nnodes;
        bbase += L.nbodies;
    }
    if (s.h_body.empty()) s.h_body.push_back(make_float4(0.f, 0.f, 0.f, 0.f));
    s.com.reserve(nn * 16); s.q0.reserve(nn * 16); s.q1.reserve(nn * 16); s.link.reserve(nn * 16);
    s.body.reserve(s.h_body.size() * 16);
    s.roots.reserve(s.h_roots.size() * 4);
    LG_CK(cudaMemcpyAsync(s.com.as<float4>(), s.h_com.data(), nn * 16, cudaMemcpyHostToDevice, e.stream));
    LG_CK(cudaMemcpyAsync(s.q0.as<float4>(), s.h_q0.data(), nn * 16, cudaMemcpyHostToDevice, e.stream));
    LG_CK(cudaMemcpyAsync(s.q1.as<float4>(), s.h_q1.data(), nn * 16, cudaMemcpyHostToDevice, e.stream));
    LG_CK(cudaMemcpyAsync(s.link.as<int4>(), s.h_link.data(), nn * 16, cudaMemcpyHostToDevice, e.stream));
    LG_CK(cudaMemcpyAsync(s.body.as<float4>(), s.h_body.data(), s.h_body.size() * 16, cudaMemcpyHostToDevice,
                          e.stream));
    LG_CK(cudaMemcpyAsync(s.roots.as<uint32_t>(), s.h_roots.data(), s.h_roots.size() * 4, cudaMemcpyHostToDevice,
                          e.stream));
    v.com = s.com.as<float4>();
    v.q0 = s.q0.as<float4>();
    v.q1 = s.q1.as<float4>();
    v.link = s.link.as<int4>();
    v.body = s.body.as<float4>();
    v.roots = s.roots.as<uint32_t>();
    v.nnodes = static_cast<uint32_t>(nn);
    v.ntrees = static_cast<int>(s.h_roots.size());
    return v;
}

TreeView let_body_blocks(Engine& e, int block) {
    LetStore& s = *e.lets;
    const int n = e.n;
    const int nb = (n + block - 1) / block;
    s.blk_range.reserve(static_cast<size_t>(nb) * 8 + 8);
    s.blk_box.reserve(static_cast<size_t>(nb) * 32 + 32);
    s.blk_count.reserve(64);
    k_block_groups<<<grid_for(static_cast<long long>(nb) * 32, 256), 256, 0, e.stream>>>(
        e.bodies(e.cur).hm, n, block, s.blk_range.as<uint2>(), s.blk_box.as<float4>(), s.blk_count.as<unsigned>());
    LG_LAUNCHED();
    ++e.launches;
    TreeView v{};
    v.grp_range = s.blk_range.as<uint2>();
    v.grp_box = s.blk_box.as<float4>();
    v.ngroups = s.blk_count.as<unsigned>();
    v.T = 0;
    return v;
}

void let_export(Engine& e, const float lo[3], const float hi[3], const lg_force_params& p, size_t* nnodes,
                size_t* nbodies) {
    LetStore& s = *e.lets;
    s.out_n = s.out_b = 0;
    const int n = e.n;
    cudaStream_t st = e.stream;
    if (n == 0) {
        *nnodes = *nbodies = 0;
        return;
    }
    const BodyArrays b = e.bodies(e.cur);
    s.out_body.reserve(static_cast<size_t>(n) * 16);
    if (p.method != LG_TREE) {
        // One always-open root holding every body; its centre of mass from FP64 sums.
        const lg_diag d = e.diagnostics();
        lg_let_node r{};
        if (d.mass > 0) {
            r.cx = static_cast<float>(d.cx);
            r.cy = static_cast<float>(d.cy);
            r.cz = static_cast<float>(d.cz);
        }
        r.mass = static_cast<float>(d.mass);
        r.rcrit2 = 3.0e38f;
        r.first_child = -1; r.child_count = 0; r.body_first = 0; r.body_count = n;
        s.out_nodes.reserve(sizeof(lg_let_node));
        LG_CK(cudaMemcpyAsync(s.out_nodes.as<lg_let_node>(), &r, sizeof r, cudaMemcpyHostToDevice, st));
        LG_CK(cudaMemcpyAsync(s.out_body.as<float4>(), b.hm, static_cast<size_t>(n) * 16, cudaMemcpyDeviceToDevice, st));
        LG_CK(cudaStreamSynchronize(st));
        s.out_n = 1;
        s.out_b = static_cast<size_t>(n);
        *nnodes = s.out_n;
        *nbodies = s.out_b;
        return;
    }
    if (!e.tree_ok) fail(kLogic, "cuda export_let: call build_tree first");
    e.ensure_tree_valid();
    size_t T = 0;
    tree_counts(e, &T, nullptr, nullptr, nullptr);
    const TreeView tv = tree_view(e);
    // Root of zero mass (or no bodies): empty LET.
    float4 root{};
    LG_CK(cudaMemcpyAsync(&root, tv.nd_com, 16, cudaMemcpyDeviceToHost, st));
    LG_CK(cudaStreamSynchronize(st));
    if (!(root.w > 0.f)) {
        *nnodes = *nbodies = 0;
        return;
    }
    s.out_nodes.reserve(T * sizeof(lg_let_node));
    for (DevBuf* d : {&s.front_a, &s.front_b, &s.kind, &s.ccount, &s.bcount, &s.cscan, &s.bscan}) d->reserve(T * 4 + 4);
    s.totals.reserve(64);
    const float4 bc = make_float4(0.5f * (lo[0] + hi[0]), 0.5f * (lo[1] + hi[1]), 0.5f * (lo[2] + hi[2]), 0.f);
    const float4 bh = make_float4(0.5f * (hi[0] - lo[0]), 0.5f * (hi[1] - lo[1]), 0.5f * (hi[2] - lo[2]), 0.f);
    uint32_t zero = 0;
    LG_CK(cudaMemcpyAsync(s.front_a.as<uint32_t>(), &zero, 4, cudaMemcpyHostToDevice, st));
    DevBuf* cur = &s.front_a;
    DevBuf* nxt = &s.front_b;
    size_t nf = 1, base = 0, bodies = 0;
    uint32_t* tot = e.pinned_small + 128;
    while (nf > 0) {
        if (base + nf > T) fail(kRuntime, "cuda export_let: more nodes than the tree holds");
        const int g = grid_for(static_cast<long long>(nf), 256);
        k_let_decide<<<g, 256, 0, st>>>(tv, cur->as<uint32_t>(), static_cast<int>(nf), bc, bh, s.kind.as<uint32_t>(),
                                        s.ccount.as<uint32_t>(), s.bcount.as<uint32_t>());
        LG_LAUNCHED();
        k_let_scan<<<1, 1024, 0, st>>>(s.ccount.as<uint32_t>(), s.bcount.as<uint32_t>(), static_cast<int>(nf),
                                       s.cscan.as<uint32_t>(), s.bscan.as<uint32_t>(), s.totals.as<uint32_t>());
        LG_LAUNCHED();
        LG_CK(cudaMemcpyAsync(tot, s.totals.as<uint32_t>(), 8, cudaMemcpyDeviceToHost, st));
        LG_CK(cudaStreamSynchronize(st));
        const size_t nc = tot[0], nbod = tot[1];
        if (base + nf + nc > T || bodies + nbod > static_cast<size_t>(n))
            fail(kRuntime, "cuda export_let: sizes exceed the tree");
        k_let_emit<<<g, 256, 0, st>>>(tv, b.hm, cur->as<uint32_t>(), static_cast<int>(nf), s.kind.as<uint32_t>(),
                                      s.ccount.as<uint32_t>(), s.bcount.as<uint32_t>(), s.cscan.as<uint32_t>(),
                                      s.bscan.as<uint32_t>(), static_cast<uint32_t>(base),
                                      static_cast<uint32_t>(base + nf), static_cast<uint32_t>(bodies),
                                      s.out_nodes.as<lg_let_node>(), nxt->as<uint32_t>(), s.out_body.as<float4>());
        LG_LAUNCHED();
        e.launches += 3;
        base += nf;
        bodies += nbod;
        nf = nc;
        std::swap(cur, nxt);
    }
    LG_CK(cudaStreamSynchronize(st));
    s.out_n = base;
    s.out_b = bodies;
    *nnodes = s.out_n;
    *nbodies = s.out_b;
}

void let_export_read(Engine& e, lg_let_node* nodes, float* bx, float* by, float* bz, float* bm) {
    LetStore& s = *e.lets;
    if (s.out_n && nodes)
        LG_CK(cudaMemcpyAsync(nodes, s.out_nodes.as<lg_let_node>(), s.out_n * sizeof(lg_let_node), cudaMemcpyDeviceToHost,
                              e.stream));
    std::vector<float4> h(s.out_b);
    if (s.out_b)
        LG_CK(cudaMemcpyAsync(h.data(), s.out_body.as<float4>(), s.out_b * 16, cudaMemcpyDeviceToHost, e.stream));
    LG_CK(cudaStreamSynchronize(e.stream));
    for (size_t k = 0; k < s.out_b; ++k) {
        if (bx) bx[k] = h[k].x;
        if (by) by[k] = h[k].y;
        if (bz) bz[k] = h[k].z;
        if (bm) bm[k] = h[k].w;
    }
}

}  // namespace lg
