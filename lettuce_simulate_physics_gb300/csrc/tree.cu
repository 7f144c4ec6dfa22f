// Tree build for the Barnes-Hut method: Morton keys, onesweep LSD radix sort, permute, key
// restarts, the octree in the reference CPU backend's exact topology and node order, walk groups,
// and the FP64 bottom-up upsweep of monopole and quadrupole moments.
//
// Parity target: the reference CPU backend (src/cpu_backend.cpp:395-664). After an upload (FP64
// positions equal to the float inputs) the keys, the sort permutation, the node array (lo, hi,
// first, nchild in the same indices), the cell geometry and the groups are bit-identical to the
// reference's; the moments use the reference's FP64 operation order, with the fused multiply-adds
// its compiler forms (GCC's default contraction on x86-64-v3 and aarch64: a product fused into the
// sum or difference that is its only use) written out as __fma_rn, everything else rounded per
// operation. rcrit2 and the walk's opening distance use the same fused float forms.
//
// Construction (no level-by-level loop, no recursion):
//  1. bbox and key frame (FP64), keys (src/cpu_backend.cpp:418-428 formula), identity values.
//  2. Onesweep radix sort (Adinets & Merrill 2022): one histogram pass for all eight 8-bit digits,
//     then one kernel per digit with decoupled look-back across tiles; digits that are constant
//     over all keys are skipped on the device. Stable, so the permutation equals the reference's.
//  3. Key restarts: runs of > 16 identical keys are re-keyed in their own bounding cube (the
//     reference's rekey, src/cpu_backend.cpp:503-530) and sorted by the new keys inside each run;
//     runs whose composite keys still tie are re-keyed again, up to FRAMES frames (depth 126).
//     Composite keys (frame 0, then the restart frames) order the bodies as the reference's nested
//     rekeys do, and a common-prefix length over them drives steps 4-6.
//  4. Leaves from key windows: body i's leaf depth is 1 + the deepest common octal prefix of any
//     window of LEAF_MAX+1 consecutive sorted keys that contains i (the first depth at which its
//     cell holds <= LEAF_MAX bodies); group depth likewise with windows of group_max+1.
//  5. Octree nodes in pre-order, enumerated per leaf: leaf l owns the ancestors at depths
//     c+1 .. depth-1, c = common prefix with the previous leaf (Karras 2012's adjacent-key rule in
//     octree form). A scan gives every node's pre-order index; body ranges, parents and children
//     follow from binary searches over the sorted keys.
//  6. Node indices of the reference (children contiguous, child blocks in parent pre-order):
//     first child of v = 1 + exclusive scan of nchild over pre-order.
//  7. Upsweep in FP64, children always combined in index order: one launch for the leaves (one
//     thread per leaf, leaves bucketed by body count), then one launch per depth from the deepest
//     (four lanes per node, each sequential sum folded by one lane). The group boxes are computed
//     on a side stream meanwhile. (A single-launch form in which the last-arriving child of each
//     node combines it was measured slower: its combines run one node per thread in sparse warps,
//     and an FP64 warp instruction costs the same however few lanes are active.)
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

#include "engine.cuh"

namespace lg {

namespace {

constexpr int LEAF_MAX = 16;   // src/cpu_backend.cpp:24
constexpr int MAX_LEVEL = 21;  // :28
constexpr int FRAMES = 6;                     // key frames: frame 0 and up to five key restarts
constexpr int MAX_DEPTH = FRAMES * MAX_LEVEL;  // 126: depths fit the 8-bit depth fields
constexpr int BS = 256;

// Key restart frames, in device memory. Frame f >= 1 re-keys, in its own bounding cube, every run
// of more than LEAF_MAX bodies whose keys in frames 0..f-1 are all equal (the reference's rekey at
// level kMaxLevel of frame f-1, src/cpu_backend.cpp:536-544); its runs are sorted by the new keys.
struct FrameTable {
    const uint64_t* key[FRAMES];  // [f >= 1] frame-f keys by sorted position (0 outside its runs)
    const int* runid[FRAMES];     // [f >= 1] the body's run in frame f, or -1
    const double* cube[FRAMES];   // [f >= 1] per run: origin xyz, side (0: coincident), 2^21 / side
    const uint8_t* nfr;           // per body: frames it has keys in (1 + its non-coincident restarts)
    int nf;                       // frames in use
};

inline int grid_for(long long n, int bs) { return static_cast<int>((n + bs - 1) / bs); }

// ---- sort control --------------------------------------------------------------------------
constexpr int RADIX = 256;
constexpr int PASSES = 8;
#ifndef LG_SORT_IPT
#define LG_SORT_IPT 8
#endif
constexpr int SORT_BS = 256;
constexpr int SORT_IPT = LG_SORT_IPT;  // keys per thread of a sort tile
constexpr int SORT_TILE = SORT_BS * SORT_IPT;
constexpr unsigned FLAG_AGG = 1u << 30, FLAG_INC = 2u << 30, VAL_MASK = (1u << 30) - 1;
#ifndef LG_LB_BATCH
#define LG_LB_BATCH 4
#endif
constexpr int LB_BATCH = LG_LB_BATCH;  // predecessors read per look-back round trip

struct SortCtl {
    unsigned sel;
    unsigned skip[PASSES];
    unsigned tile_ctr[PASSES];
    unsigned done_ctr[PASSES];
};

}  // namespace

struct TreeState {
    // sort
    DevBuf keysA, keysB, valsA, valsB, hist, lookback, ctl;
    // sorted frame-0 keys, per-body tree data
    DevBuf skey, bdepth, flag, leafid;
    // frame, key-restart runs and frames (index 0 of the per-frame buffers unused)
    DevBuf frame, runs, counts, key1tmp, nfr, ftab;
    DevBuf fkey[FRAMES], frunid[FRAMES], fcube[FRAMES];
    int nframes = 1;  // key frames of the last restarted build
    // leaves
    DevBuf leaf_first, leaf_depth, leaf_c, leaf_pre, leaf_node;
    // pre-order nodes
    DevBuf pn_lohi, pn_meta, pn_nchild, pn_cb, pn_cpu;
    // reference-order nodes
    DevBuf nd_range, nd_com, nd_comlo, nd_q0, nd_q1, nd_geo, nd_parent;
    // groups
    DevBuf gflag, gidx, grp_node, grp_range, grp_box, leaf_cnt;
    // upsweep order
    DevBuf ups, dep_nodes, leaf_order;
    // scan state
    DevBuf scan_state, scan_ctr;
    size_t K = 0, T = 0, ngroups = 0;  // sizes the last build was launched with
    int max_depth = 0;
    bool restarted = false;
    int group_max = 128;
    // Sync-free builds: sizes from the previous build with headroom; verified after the walk.
    bool have_guess = false;
    bool restart_mode = false;  // key restarts were needed last time: check for them on the host
    bool speculative = false;   // the current build used guessed sizes / assumed no restart
    double theta = 0.6;
    // Forest (ensemble) configuration: the tree covers bodies [0, n_tree) of nsys systems whose
    // ranges are sys_off[0..nsys] (device); sys[i] is body i's system (device); per-system inverse
    // opening angles. n_tree < 0 means one system over all bodies.
    int n_tree = -1;
    int nsys = 1;
    const uint32_t* sys = nullptr;
    const uint32_t* sys_off = nullptr;
    const float* inv_theta_sys = nullptr;
    uint64_t generation = 0;  // bumped by every build that may grow (reallocate) tree buffers
    DevBuf mkeys;   // forest: Morton keys before the (system, key) sort
    // merged walk groups
    bool merged = false;
    DevBuf mcount, moff, mrange, mbox;
    DevBuf sticky;  // graph mode: sticky word set when a sync-free build misses
};

namespace {

void destroy_tree(TreeState* t) { delete t; }

// ---- device helpers --------------------------------------------------------------------------
__device__ __forceinline__ uint64_t spread21(uint64_t v) {
    v &= 0x1fffffULL;
    v = (v | v << 32) & 0x1f00000000ffffULL;
    v = (v | v << 16) & 0x1f0000ff0000ffULL;
    v = (v | v << 8) & 0x100f00f00f00f00fULL;
    v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
    v = (v | v << 2) & 0x1249249249249249ULL;
    return v;
}

// Quantised coordinate of src/cpu_backend.cpp:423: uint64(clamp((v - o) * s, 0, lim)), FP64,
// round-to-nearest products, truncation. The clamp is taken after the conversion, in integers:
// the truncating conversion saturates (negative values give 0), and lim = 2^21 - 1 is an integer,
// so min(trunc(q), lim) equals trunc(clamp(q, 0, lim)) for every q, with two FP64 operations fewer.
constexpr uint64_t QLIM = (1ull << MAX_LEVEL) - 1;
__device__ __forceinline__ uint64_t quantize(double v, double o, double s) {
    const uint64_t u = __double2ull_rz(__dmul_rn(__dsub_rn(v, o), s));
    return u < QLIM ? u : QLIM;
}

__device__ __forceinline__ uint64_t morton(double x, double y, double z, double ox, double oy, double oz, double s) {
    return spread21(quantize(x, ox, s)) << 2 | spread21(quantize(y, oy, s)) << 1 | spread21(quantize(z, oz, s));
}

// Common octal prefix (0..21) of two 63-bit keys.
__device__ __forceinline__ int cpl21(uint64_t a, uint64_t b) { return (__clzll(a ^ b) - 1) / 3; }

// Forest builds (many independent systems in one pipeline) pass a per-body system index `sys`:
// bodies of different systems share no prefix (-1), so no leaf, node or group spans two systems.
// Single-system builds pass null.

// Common octal prefix over the restart frames 1..nf-1 of bodies whose frame-0 keys are equal:
// 21 per equal frame, 21 nf when every frame is equal.
__device__ __forceinline__ int cpl_frames(const FrameTable* ft, int i, int j) {
    const int nf = ft->nf;
    for (int f = 1; f < nf; ++f) {
        const uint64_t a = ft->key[f][i], b = ft->key[f][j];
        if (a != b) return MAX_LEVEL * f + cpl21(a, b);
    }
    return MAX_LEVEL * nf;
}

// Common octal prefix (0..126) of the composite keys (frame 0, then the restart frames) of bodies
// i and j; -1 across systems. ft is null when no key restart was needed.
__device__ __forceinline__ int cpl_key(const uint32_t* sys, const uint64_t* k0, const FrameTable* ft, int i, int j) {
    if (sys && sys[i] != sys[j]) return -1;
    const uint64_t a = k0[i], b = k0[j];
    if (a != b || !ft) return cpl21(a, b);
    return cpl_frames(ft, i, j);
}

__device__ __forceinline__ uint32_t sys_of(const uint32_t* sys, int i) { return sys ? sys[i] : 0u; }

// Octal digit of the composite key at depth d (1-based): digit d - 21 f of frame f = (d - 1) / 21.
__device__ __forceinline__ int digit_at(const uint64_t* k0, const FrameTable* ft, int i, int d) {
    const int f = (d - 1) / MAX_LEVEL;
    const uint64_t k = f == 0 ? k0[i] : ft->key[f][i];
    return static_cast<int>((k >> (3 * (MAX_LEVEL * (f + 1) - d))) & 7);
}

// ---- frame and keys --------------------------------------------------------------------------
// frame: [0..2] origin, [3] side, [4] scale 2^21/side.
// Bounding-box minima and maxima on the integer pipes: a double's bits mapped to a signed 64-bit
// integer that orders as the values do (-0 below +0), NaN mapped to +inf for minima and to -inf
// for maxima, so that it is ignored as fmin and fmax ignore it. FP64 issue is scarce on this part.
__device__ __forceinline__ long long ord_bits(long long b) { return b ^ ((b >> 63) & 0x7fffffffffffffffLL); }
__device__ __forceinline__ bool nan_bits(long long b) { return (b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL; }
__device__ __forceinline__ long long ord_lo(double d) {
    const long long b = __double_as_longlong(d);
    return nan_bits(b) ? 0x7ff0000000000000LL : ord_bits(b);
}
__device__ __forceinline__ long long ord_hi(double d) {
    const long long b = __double_as_longlong(d);
    return nan_bits(b) ? ord_bits(static_cast<long long>(0xfff0000000000000ULL)) : ord_bits(b);
}
__device__ __forceinline__ double ord_value(long long k) { return __longlong_as_double(ord_bits(k)); }

// v[0..2] minima, v[3..5] maxima (ordered integers) of the block's bodies, reduced over the block
// into sh (lane 0 of each warp) and returned by thread 0 in v.
__device__ __forceinline__ void box_block_reduce(long long (&v)[6], long long (*sh)[BS / 32]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        for (int o = 16; o > 0; o >>= 1) {
            const long long t = __shfl_down_sync(0xffffffffu, v[c], o);
            v[c] = c < 3 ? min(v[c], t) : max(v[c], t);
        }
        if (lane == 0) sh[c][w] = v[c];
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int c = 0; c < 6; ++c) {
            long long r = sh[c][0];
            for (int u = 1; u < BS / 32; ++u) r = c < 3 ? min(r, sh[c][u]) : max(r, sh[c][u]);
            v[c] = r;
        }
}

__device__ __forceinline__ void box_init(long long (&v)[6]) {
    for (int c = 0; c < 3; ++c) {
        v[c] = ord_bits(0x7ff0000000000000LL);                                   // +inf
        v[3 + c] = ord_bits(static_cast<long long>(0xfff0000000000000ULL));      // -inf
    }
}

__device__ __forceinline__ void box_add(long long (&v)[6], double x, double y, double z) {
    v[0] = min(v[0], ord_lo(x));
    v[1] = min(v[1], ord_lo(y));
    v[2] = min(v[2], ord_lo(z));
    v[3] = max(v[3], ord_hi(x));
    v[4] = max(v[4], ord_hi(y));
    v[5] = max(v[5], ord_hi(z));
}

// src/cpu_backend.cpp:404-406: origin = the minima; side = max extent, widened by 1e-6; 1 if all
// coincide; scale = 2^21 / side.
__device__ __forceinline__ void write_frame(const long long (&v)[6], double* f) {
    double r[6];
    for (int c = 0; c < 6; ++c) r[c] = ord_value(v[c]);
    double side = fmax(fmax(__dsub_rn(r[3], r[0]), __dsub_rn(r[4], r[1])), __dsub_rn(r[5], r[2]));
    side = side > 0 ? __dmul_rn(side, 1 + 1e-6) : 1.0;
    f[0] = r[0];
    f[1] = r[1];
    f[2] = r[2];
    f[3] = side;
    f[4] = __ddiv_rn(static_cast<double>(1u << MAX_LEVEL), side);
}

__global__ void k_frame(const BodyArrays b, int n, long long* partial, unsigned* ticket, double* frame) {
    __shared__ long long sh[6][BS / 32];
    __shared__ bool last;
    long long v[6];
    box_init(v);
    for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) box_add(v, b.x[i], b.y[i], b.z[i]);
    box_block_reduce(v, sh);
    if (threadIdx.x == 0) {
        for (int c = 0; c < 6; ++c) partial[blockIdx.x * 6 + c] = v[c];
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    box_init(v);
    for (int blk = threadIdx.x; blk < static_cast<int>(gridDim.x); blk += BS)
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const long long t = __ldcg(&partial[blk * 6 + c]);
            v[c] = c < 3 ? min(v[c], t) : max(v[c], t);
        }
    __syncthreads();
    box_block_reduce(v, sh);
    if (threadIdx.x == 0) {
        write_frame(v, frame);
        *ticket = 0;
    }
}

__global__ void k_keys(const uint32_t* __restrict__ sys, const BodyArrays b, int n, const double* __restrict__ frame,
                       uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* f = frame + 5 * sys_of(sys, i);
    keys[i] = morton(b.x[i], b.y[i], b.z[i], f[0], f[1], f[2], f[4]);
    vals[i] = static_cast<uint32_t>(i);
}

// Forest: one block per system computes its key frame over its body range [off[s], off[s + 1]).
__global__ void k_frame_sys(const BodyArrays b, const uint32_t* __restrict__ off, double* frame) {
    __shared__ long long sh[6][BS / 32];
    const uint32_t lo = off[blockIdx.x], hi = off[blockIdx.x + 1];
    long long v[6];
    box_init(v);
    for (uint32_t i = lo + threadIdx.x; i < hi; i += BS) box_add(v, b.x[i], b.y[i], b.z[i]);
    box_block_reduce(v, sh);
    if (threadIdx.x == 0) write_frame(v, frame + 5 * blockIdx.x);
}

// keys[i] = (system of body vals[i]): the second key of the forest's (system, Morton) sort.
__global__ void k_sys_keys(const uint32_t* __restrict__ sys, const uint32_t* __restrict__ vals,
                           uint64_t* __restrict__ keys, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) keys[i] = sys_of(sys, static_cast<int>(vals[i]));
}

// ---- onesweep radix sort ---------------------------------------------------------------------
__global__ void k_sort_hist(const uint64_t* __restrict__ keys, int n, unsigned* __restrict__ hist) {
    __shared__ unsigned h[PASSES][RADIX];
    for (int k = threadIdx.x; k < PASSES * RADIX; k += blockDim.x) (&h[0][0])[k] = 0;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
#pragma unroll
        for (int p = 0; p < PASSES; ++p) atomicAdd(&h[p][(k >> (8 * p)) & 255], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < PASSES * RADIX; k += blockDim.x) {
        const unsigned v = (&h[0][0])[k];
        if (v) atomicAdd(&hist[k], v);
    }
}

// Exclusive digit offsets per pass; a pass whose digit is constant over all keys is skipped.
__global__ void k_sort_offsets(unsigned* __restrict__ hist, int n, SortCtl* ctl) {
    __shared__ unsigned s[RADIX];
    const int d = threadIdx.x;
    for (int p = 0; p < PASSES; ++p) {
        const unsigned c = hist[p * RADIX + d];
        s[d] = c;
        __syncthreads();
        // Hillis-Steele inclusive scan over 256 entries.
        for (int o = 1; o < RADIX; o <<= 1) {
            unsigned t = d >= o ? s[d - o] : 0;
            __syncthreads();
            s[d] += t;
            __syncthreads();
        }
        hist[p * RADIX + d] = s[d] - c;
        const int full = __syncthreads_or(c == static_cast<unsigned>(n));
        if (d == 0) {
            ctl->skip[p] = full ? 1u : 0u;
            ctl->tile_ctr[p] = 0;
            ctl->done_ctr[p] = 0;
        }
        __syncthreads();
    }
    if (d == 0) ctl->sel = 0;
}

__global__ void __launch_bounds__(SORT_BS) k_sort_pass(uint64_t* __restrict__ kA, uint32_t* __restrict__ vA,
                                                       uint64_t* __restrict__ kB, uint32_t* __restrict__ vB, int n,
                                                       int pass, const unsigned* __restrict__ offsets,
                                                       unsigned* __restrict__ lookback, SortCtl* ctl,
                                                       unsigned* err) {
    __shared__ unsigned warp_hist[SORT_BS / 32][RADIX];
    __shared__ unsigned gbase[RADIX];       // global start of each digit for this tile
    __shared__ unsigned tstart[RADIX];      // inclusive scan of the tile's digit counts
    __shared__ uint64_t stage_k[SORT_TILE]; // the tile in digit order
    __shared__ uint32_t stage_v[SORT_TILE];
    __shared__ unsigned tile_s, sel_s;
    if (ctl->skip[pass]) return;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) {
        tile_s = atomicAdd(&ctl->tile_ctr[pass], 1u);
        sel_s = *reinterpret_cast<volatile unsigned*>(&ctl->sel);
    }
    for (int k = tid; k < (SORT_BS / 32) * RADIX; k += SORT_BS) (&warp_hist[0][0])[k] = 0;
    __syncthreads();
    const unsigned tile = tile_s;
    const unsigned ntiles = (n + SORT_TILE - 1) / SORT_TILE;
    const uint64_t* src_k = sel_s ? kB : kA;
    const uint32_t* src_v = sel_s ? vB : vA;
    uint64_t* dst_k = sel_s ? kA : kB;
    uint32_t* dst_v = sel_s ? vA : vB;
    const int shift = 8 * pass;
    const int tile0 = tile * SORT_TILE;
    const int wbase = tile0 + w * (32 * SORT_IPT);
    const int tile_n = min(SORT_TILE, n - tile0);

    uint64_t key[SORT_IPT];
    uint32_t val[SORT_IPT];
    unsigned rank[SORT_IPT];
    int dig[SORT_IPT];
    const unsigned lt = (1u << lane) - 1u;
    // Stable rank inside the tile: keys in index order (warp, round, lane).
#pragma unroll
    for (int r = 0; r < SORT_IPT; ++r) {
        const int i = wbase + r * 32 + lane;
        const bool valid = i < n;
        key[r] = valid ? src_k[i] : 0;
        val[r] = valid ? src_v[i] : 0;
        const int d = valid ? static_cast<int>((key[r] >> shift) & 255) : -1 - lane;
        dig[r] = d;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned before = __popc(peers & lt);
        unsigned basev = 0;
        if (valid) basev = warp_hist[w][d];
        __syncwarp();
        if (valid && before == 0) warp_hist[w][d] = basev + __popc(peers);
        __syncwarp();
        rank[r] = basev + before;
    }
    __syncthreads();
    {
        // Per digit (thread d): offsets of the warps inside the digit, the tile's count, then the
        // decoupled look-back across tiles for the digit's global start.
        const int d = tid;
        unsigned run = 0;
#pragma unroll
        for (int u = 0; u < SORT_BS / 32; ++u) {
            const unsigned c = warp_hist[u][d];
            warp_hist[u][d] = run;
            run += c;
        }
        const unsigned tile_count = run;
        volatile unsigned* lb = lookback + static_cast<size_t>(tile) * RADIX;
        unsigned prefix = 0;
        if (tile == 0) {
            lb[d] = FLAG_INC | tile_count;
        } else {
            lb[d] = FLAG_AGG | tile_count;
            // Look back LB_BATCH predecessors per round trip: their flags are read together and
            // taken in order (aggregates added until an inclusive prefix; an unpublished tile is
            // waited for, keeping what was added before it).
            int j = static_cast<int>(tile) - 1;
            unsigned spins = 0;
            while (j >= 0) {
                unsigned sv[LB_BATCH];
#pragma unroll
                for (int q = 0; q < LB_BATCH; ++q)
                    sv[q] = j - q >= 0 ? *reinterpret_cast<volatile const unsigned*>(
                                             &lookback[static_cast<size_t>(j - q) * RADIX + d])
                                       : FLAG_INC;
                int taken = 0;
                bool inc = false;
#pragma unroll
                for (int q = 0; q < LB_BATCH; ++q) {
                    if (inc || taken < q) break;
                    if (sv[q] & (FLAG_INC | FLAG_AGG)) {
                        prefix += sv[q] & VAL_MASK;
                        inc = (sv[q] & FLAG_INC) != 0;
                        ++taken;
                    }
                }
                if (inc) break;
                j -= taken;
                if (taken == 0 && ++spins > kSpinCap) {
                    atomicOr(err, kErrWaitTimeout);
                    break;
                }
            }
            lb[d] = FLAG_INC | ((prefix + tile_count) & VAL_MASK);
        }
        gbase[d] = offsets[pass * RADIX + d] + prefix;
        // Exclusive scan of the tile's digit counts (Hillis-Steele over 256 threads).
        tstart[d] = tile_count;
    }
    __syncthreads();
    for (int o = 1; o < RADIX; o <<= 1) {
        const unsigned t = tid >= o ? tstart[tid - o] : 0u;
        __syncthreads();
        tstart[tid] += t;
        __syncthreads();
    }
    // tstart now holds the inclusive scan: digit d starts at tstart[d - 1] (0 for d = 0).
    // Stage the tile in digit order (tile-local position = digit start + rank within the digit).
#pragma unroll
    for (int r = 0; r < SORT_IPT; ++r) {
        const int i = wbase + r * 32 + lane;
        if (i < n) {
            const int d = dig[r];
            const unsigned excl = (d > 0 ? tstart[d - 1] : 0u);
            const unsigned pos = excl + warp_hist[w][d] + rank[r];
            stage_k[pos] = key[r];
            stage_v[pos] = val[r];
        }
    }
    __syncthreads();
    // Write out: consecutive staged entries of one digit go to consecutive global addresses.
    for (int p = tid; p < tile_n; p += SORT_BS) {
        const uint64_t k = stage_k[p];
        const int d = static_cast<int>((k >> shift) & 255);
        const unsigned excl = (d > 0 ? tstart[d - 1] : 0u);
        const unsigned gpos = gbase[d] + (p - excl);
        dst_k[gpos] = k;
        dst_v[gpos] = stage_v[p];
    }
    // The last tile to finish flips the buffer selector (every tile has read it by then).
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&ctl->done_ctr[pass], 1u) == ntiles - 1) ctl->sel ^= 1u;
    }
}

// Gathers every body array into the other body set in the order of the permutation in vals;
// copies the sorted keys; optionally carries a second key array through the permutation.
__global__ void k_permute(const BodyArrays src, BodyArrays dst, const uint64_t* __restrict__ keys,
                          const uint32_t* __restrict__ vals, uint64_t* __restrict__ skey,
                          const uint64_t* __restrict__ key1_in, uint64_t* __restrict__ key1_out, int n,
                          const uint64_t* __restrict__ key_src, int n_total) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_total) return;
    // Bodies past the tree's range (the forest's direct systems) keep their place.
    const uint32_t j = i < n ? vals[i] : static_cast<uint32_t>(i);
    if (i < n && skey) skey[i] = key_src ? key_src[j] : keys[i];
    if (i >= n) {
        dst.x[i] = src.x[i]; dst.y[i] = src.y[i]; dst.z[i] = src.z[i];
        dst.hm[i] = src.hm[i]; dst.lo[i] = src.lo[i];
        dst.vx[i] = src.vx[i]; dst.vy[i] = src.vy[i]; dst.vz[i] = src.vz[i];
        dst.m[i] = src.m[i]; dst.id[i] = src.id[i]; dst.cost[i] = src.cost[i];
        dst.level[i] = src.level[i];
        return;
    }
    if (key1_in) key1_out[i] = key1_in[j];
    dst.x[i] = src.x[j];
    dst.y[i] = src.y[j];
    dst.z[i] = src.z[j];
    dst.hm[i] = src.hm[j];
    dst.lo[i] = src.lo[j];
    dst.vx[i] = src.vx[j];
    dst.vy[i] = src.vy[j];
    dst.vz[i] = src.vz[j];
    dst.m[i] = src.m[j];
    dst.id[i] = src.id[j];
    dst.cost[i] = src.cost[j];
    dst.level[i] = src.level[j];
}

// After the passes: if the sorted pairs ended in buffer B, copy them to A (so every sort returns
// its result in A), and reset the selector.
__global__ void k_sort_finish(uint64_t* __restrict__ kA, uint32_t* __restrict__ vA, const uint64_t* __restrict__ kB,
                              const uint32_t* __restrict__ vB, const SortCtl* ctl, int n) {
    if (ctl->sel == 0) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        kA[i] = kB[i];
        vA[i] = vB[i];
    }
}

// ---- exclusive scan (decoupled look-back) ----------------------------------------------------
constexpr int SCAN_BS = 256, SCAN_IPT = 8, SCAN_TILE = SCAN_BS * SCAN_IPT;
constexpr unsigned long long SFLAG_AGG = 1ull << 62, SFLAG_INC = 2ull << 62, SVAL = (1ull << 62) - 1;

__global__ void __launch_bounds__(SCAN_BS) k_scan(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int n,
                                                 unsigned long long* state, unsigned* counter, uint32_t* total,
                                                 unsigned* err) {
    __shared__ unsigned tile_s;
    __shared__ unsigned long long warp_tot[SCAN_BS / 32];
    __shared__ unsigned long long prefix_s;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) tile_s = atomicAdd(counter, 1u);
    __syncthreads();
    const unsigned tile = tile_s;
    const long long base = static_cast<long long>(tile) * SCAN_TILE + static_cast<long long>(tid) * SCAN_IPT;
    uint32_t v[SCAN_IPT];
    unsigned long long tsum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        v[k] = base + k < n ? in[base + k] : 0u;
        tsum += v[k];
    }
    // Warp inclusive scan of thread sums.
    unsigned long long incl = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (tid == 0) {
        unsigned long long run = 0;
        for (int u = 0; u < SCAN_BS / 32; ++u) {
            unsigned long long c = warp_tot[u];
            warp_tot[u] = run;
            run += c;
        }
        const unsigned long long block_total = run;
        volatile unsigned long long* st = state;
        unsigned long long prefix = 0;
        if (tile == 0) {
            st[0] = SFLAG_INC | block_total;
        } else {
            st[tile] = SFLAG_AGG | block_total;
            long long j = static_cast<long long>(tile) - 1;
            unsigned spins = 0;
            while (j >= 0) {  // LB_BATCH predecessors per round trip, taken in order (as in the sort)
                unsigned long long sv[LB_BATCH];
#pragma unroll
                for (int q = 0; q < LB_BATCH; ++q) {
                    const unsigned long long v = j - q >= 0 ? st[j - q] : 0ull;
                    sv[q] = j - q >= 0 ? v : static_cast<unsigned long long>(SFLAG_INC);
                }
                int taken = 0;
                bool inc = false;
#pragma unroll
                for (int q = 0; q < LB_BATCH; ++q) {
                    if (inc || taken < q) break;
                    if (sv[q] & (SFLAG_INC | SFLAG_AGG)) {
                        prefix += sv[q] & SVAL;
                        inc = (sv[q] & SFLAG_INC) != 0;
                        ++taken;
                    }
                }
                if (inc) break;
                j -= taken;
                if (taken == 0 && ++spins > kSpinCap) { atomicOr(err, kErrWaitTimeout); break; }
            }
            st[tile] = SFLAG_INC | ((prefix + block_total) & SVAL);
        }
        prefix_s = prefix;
        const unsigned ntiles = static_cast<unsigned>((n + SCAN_TILE - 1) / SCAN_TILE);
        if (tile == ntiles - 1 && total) *total = static_cast<uint32_t>(prefix + block_total);
    }
    __syncthreads();
    unsigned long long run = prefix_s + warp_tot[w] + (incl - tsum);
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        if (base + k < n) out[base + k] = static_cast<uint32_t>(run);
        run += v[k];
    }
}

// ---- key restarts ----------------------------------------------------------------------------
// The runs of frame f: maximal ranges of more than LEAF_MAX bodies of one system whose keys in
// frames 0..f-1 are all equal, among the bodies re-keyed in every earlier frame (nfr == f; all
// bodies for f = 1, where nfr and ft are null): appended as (start, end). ft holds frames 0..f-1.
__global__ void k_find_runs(const uint32_t* __restrict__ sys, const uint64_t* __restrict__ skey,
                            const FrameTable* ft, const uint8_t* __restrict__ nfr, int f, int n, uint2* runs,
                            unsigned* count, int cap) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i + LEAF_MAX >= n) return;
    if (nfr && nfr[i] != f) return;
    const int full = MAX_LEVEL * f;
    if (i > 0 && cpl_key(sys, skey, ft, i - 1, i) >= full) return;
    if (cpl_key(sys, skey, ft, i, i + LEAF_MAX) < full) return;
    int lo = i + LEAF_MAX, hi = n;  // first index with a different (system, composite key)
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (cpl_key(sys, skey, ft, i, mid) >= full) lo = mid + 1;
        else hi = mid;
    }
    const unsigned r = atomicAdd(count, 1u);
    if (static_cast<int>(r) < cap) runs[r] = make_uint2(static_cast<unsigned>(i), static_cast<unsigned>(lo));
}

// One block per run: FP64 bounding box (src/cpu_backend.cpp:505-512); cube = (mn, side, scale),
// side 0 marks coincident bodies (kept as one leaf).
__global__ void k_run_cube(const BodyArrays b, const uint2* runs, double* cube) {
    __shared__ double sh[6][BS / 32];
    const uint2 r = runs[blockIdx.x];
    double v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (unsigned i = r.x + threadIdx.x; i < r.y; i += BS) {
        double p[3] = {b.x[i], b.y[i], b.z[i]};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            v[c] = fmin(v[c], p[c]);
            v[3 + c] = fmax(v[3 + c], p[c]);
        }
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        for (int o = 16; o > 0; o >>= 1) {
            double t = __shfl_down_sync(0xffffffffu, v[c], o);
            v[c] = c < 3 ? fmin(v[c], t) : fmax(v[c], t);
        }
        if (lane == 0) sh[c][w] = v[c];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double q[6];
        for (int c = 0; c < 6; ++c) {
            q[c] = sh[c][0];
            for (int u = 1; u < BS / 32; ++u) q[c] = c < 3 ? fmin(q[c], sh[c][u]) : fmax(q[c], sh[c][u]);
        }
        double side = fmax(fmax(__dsub_rn(q[3], q[0]), __dsub_rn(q[4], q[1])), __dsub_rn(q[5], q[2]));
        double* o = cube + 5 * blockIdx.x;
        o[0] = q[0];
        o[1] = q[1];
        o[2] = q[2];
        if (side == 0) {
            o[3] = 0;
            o[4] = 0;
        } else {
            side = __dmul_rn(side, 1 + 1e-6);
            o[3] = side;
            o[4] = __ddiv_rn(static_cast<double>(1u << MAX_LEVEL), side);
        }
    }
}

// Frame-f keys of the bodies of non-coincident runs (0 elsewhere, from a fill); runid = the run's
// index (-1 elsewhere, from a fill); nfr = f + 1 for the re-keyed bodies.
__global__ void k_run_keys(const BodyArrays b, const uint2* runs, const double* cube, uint64_t* key1, int* runid,
                           uint8_t* nfr, int f) {
    const uint2 r = runs[blockIdx.x];
    const double* c = cube + 5 * blockIdx.x;
    const bool rekeyed = c[3] > 0;
    for (unsigned i = r.x + threadIdx.x; i < r.y; i += BS) {
        runid[i] = static_cast<int>(blockIdx.x);
        if (rekeyed) {
            key1[i] = morton(b.x[i], b.y[i], b.z[i], c[0], c[1], c[2], c[4]);
            nfr[i] = static_cast<uint8_t>(f + 1);
        }
    }
}

// Second key of the stable (run, frame key) sort: the run's first position for bodies of a run,
// the body's own position otherwise, so that every body stays inside its run.
__global__ void k_seg_keys(const uint32_t* __restrict__ vals, const int* __restrict__ runid,
                           const uint2* __restrict__ runs, uint64_t* __restrict__ keys, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t j = vals[i];
    const int r = runid[j];
    keys[i] = r >= 0 ? runs[r].x : j;
}

__global__ void k_put_table(FrameTable v, FrameTable* dst) { *dst = v; }

__global__ void k_fill_u64(uint64_t* a, uint64_t v, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}
__global__ void k_fill_i32(int* a, int v, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}
__global__ void k_iota(uint32_t* a, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = static_cast<uint32_t>(i);
}

// ---- leaves ----------------------------------------------------------------------------------
// Per body: leaf depth and group depth from window common prefixes, capped at 21 times the frames
// the body has keys in. bdepth packs (leaf depth, group depth) as bytes.
// Each block handles DEPTH_BS bodies: it first forms, in shared memory, the common prefixes
// c_w(j) = cpl(key j, key j+w) of every window start its bodies need (w = 16 and w = group_max),
// then every thread takes the maxima over its windows from shared memory.
constexpr int DEPTH_BS = 256;
constexpr int GMAX_LIMIT = 1024;

__global__ void __launch_bounds__(DEPTH_BS) k_body_depth(const uint32_t* __restrict__ sys, const uint64_t* __restrict__ k0,
                                                         const FrameTable* ft, int n, int gmax,
                                                         uint16_t* __restrict__ bdepth) {
    __shared__ int8_t c16[DEPTH_BS + LEAF_MAX];
    __shared__ int8_t cg[DEPTH_BS + GMAX_LIMIT];
    const int i0 = blockIdx.x * DEPTH_BS;
    // Window starts j in [i0 - w, i0 + DEPTH_BS): slot j - (i0 - w).
    for (int t = threadIdx.x; t < DEPTH_BS + LEAF_MAX; t += DEPTH_BS) {
        const int j = i0 - LEAF_MAX + t;
        c16[t] = static_cast<int8_t>((j >= 0 && j + LEAF_MAX < n) ? cpl_key(sys, k0, ft, j, j + LEAF_MAX) : -1);
    }
    for (int t = threadIdx.x; t < DEPTH_BS + gmax; t += DEPTH_BS) {
        const int j = i0 - gmax + t;
        cg[t] = static_cast<int8_t>((j >= 0 && j + gmax < n) ? cpl_key(sys, k0, ft, j, j + gmax) : -1);
    }
    __syncthreads();
    const int i = i0 + threadIdx.x;
    if (i >= n) return;
    // Windows containing i start at j in [i - w, i], i.e. slots [threadIdx.x, threadIdx.x + w].
    int best = -1;
    for (int t = threadIdx.x; t <= threadIdx.x + LEAF_MAX; ++t) best = max(best, static_cast<int>(c16[t]));
    // A body's keys end with the last frame it was re-keyed in: coincident bodies, and bodies of a
    // run past the last frame, stay one leaf there.
    const int cap = ft ? MAX_LEVEL * ft->nfr[i] : MAX_LEVEL;
    const int ld = min(best + 1, cap);
    int gbest = -1;
    for (int t = threadIdx.x; t <= threadIdx.x + gmax; ++t) gbest = max(gbest, static_cast<int>(cg[t]));
    const int gd = min(ld, gbest + 1);
    bdepth[i] = static_cast<uint16_t>(ld | (gd << 8));
}

__global__ void k_leaf_flags(const uint32_t* __restrict__ sys, const uint64_t* __restrict__ k0, const FrameTable* ft,
                             const uint16_t* __restrict__ bdepth, int n, uint32_t* __restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int d = bdepth[i] & 255;
    uint32_t f = 1;
    if (i > 0 && (bdepth[i - 1] & 255) == d && cpl_key(sys, k0, ft, i - 1, i) >= d) f = 0;
    flag[i] = f;
}

// leaf_first, leaf_depth, leaf_c, and the node count of each leaf (its owned ancestors + itself).
__global__ void k_leaf_info(const uint32_t* __restrict__ sys, const uint64_t* __restrict__ k0, const FrameTable* ft,
                            const uint16_t* __restrict__ bdepth, const uint32_t* __restrict__ flag,
                            const uint32_t* __restrict__ lid, int n, uint32_t* leaf_first, uint8_t* leaf_depth,
                            int8_t* leaf_c, uint32_t* leaf_nodes, int* max_depth) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !flag[i]) return;
    const uint32_t l = lid[i];
    const int d = bdepth[i] & 255;
    atomicMax(max_depth, d);
    const int c = i == 0 ? -1 : cpl_key(sys, k0, ft, i - 1, i);
    leaf_first[l] = static_cast<uint32_t>(i);
    leaf_depth[l] = static_cast<uint8_t>(d);
    leaf_c[l] = static_cast<int8_t>(c);
    leaf_nodes[l] = static_cast<uint32_t>(d - 1 - c + 1);
}

// ---- nodes -----------------------------------------------------------------------------------
struct NodeCtx {
    const uint32_t* sys;  // per-body system (forest) or null
    const uint64_t* k0;          // sorted frame-0 keys
    const FrameTable* ft;        // key restart frames, or null
    const uint32_t* leaf_first;  // K+1
    const uint8_t* leaf_depth;
    const int8_t* leaf_c;
    const uint32_t* leaf_pre;    // K+1
    const uint32_t* lid;         // per body
    const uint16_t* bdepth;
    int n;
    const unsigned* Kdev;  // leaf count (device)
    unsigned Kcap;         // capacity the leaf arrays were sized for
    unsigned nroots;       // systems in the forest (1 for one system); roots take node indices 0..nroots-1
};

__device__ __forceinline__ int leaf_count(const NodeCtx& c) { return static_cast<int>(min(*c.Kdev, c.Kcap)); }
__device__ __forceinline__ uint32_t eff(const unsigned* dev, uint32_t cap) { return min(*dev, cap); }

// Pre-order index of the node at depth d whose first body is b (b must start that node).
__device__ __forceinline__ uint32_t node_at(const NodeCtx& c, uint32_t b, int d) {
    const uint32_t l = c.lid[b];
    return c.leaf_pre[l] + static_cast<uint32_t>(d - c.leaf_c[l] - 1);
}

// End of the body range sharing `d` octal digits with body lo.
__device__ __forceinline__ uint32_t range_end(const NodeCtx& c, uint32_t lo, int d) {
    uint32_t a = lo + 1, b = static_cast<uint32_t>(c.n);
    while (a < b) {
        uint32_t mid = (a + b) >> 1;
        if (cpl_key(c.sys, c.k0, c.ft, lo, mid) >= d) a = mid + 1;
        else b = mid;
    }
    return a;
}

// Per pre-order node: (lo, hi) and meta = depth | leaf << 8 | group << 9.
__global__ void k_nodes_pre(NodeCtx c, uint32_t Tcap, const unsigned* Tdev, uint2* pn_lohi, uint16_t* pn_meta) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= eff(Tdev, Tcap)) return;
    // Leaf owning v: last l with leaf_pre[l] <= v.
    int a = 0, b = leaf_count(c);
    while (b - a > 1) {
        int mid = (a + b) >> 1;
        if (c.leaf_pre[mid] <= v) a = mid;
        else b = mid;
    }
    const int l = a;
    const int d = c.leaf_c[l] + 1 + static_cast<int>(v - c.leaf_pre[l]);
    const bool leaf = d == c.leaf_depth[l];
    const uint32_t lo = c.leaf_first[l];
    const uint32_t hi = leaf ? c.leaf_first[l + 1] : range_end(c, lo, d);
    const bool group = d == (c.bdepth[lo] >> 8);
    pn_lohi[v] = make_uint2(lo, hi);
    pn_meta[v] = static_cast<uint16_t>(d | (leaf ? 256 : 0) | (group ? 512 : 0));
}

// Children of internal pre-order node v, in order; returns the count.
template <class F>
__device__ __forceinline__ int for_children(const NodeCtx& c, const uint2* pn_lohi, uint32_t v, int d, F&& f) {
    const uint2 r = pn_lohi[v];
    uint32_t b = r.x;
    int k = 0;
    // An octree node has at most 8 children; the cap keeps a malformed range from looping.
    while (b < r.y && k < 8) {
        const uint32_t ch = node_at(c, b, d + 1);
        f(k, ch);
        const uint32_t nb = pn_lohi[ch].y;
        if (nb <= b) break;
        b = nb;
        ++k;
    }
    return k;
}

__global__ void k_nchild(NodeCtx c, uint32_t Tcap, const unsigned* Tdev, const uint2* pn_lohi, const uint16_t* pn_meta,
                         uint32_t* pn_nchild) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= Tcap) return;
    if (v >= eff(Tdev, Tcap)) {
        pn_nchild[v] = 0;  // scanned over the capacity
        return;
    }
    const uint16_t meta = pn_meta[v];
    int k = 0;
    if (!(meta & 256)) k = for_children(c, pn_lohi, v, meta & 255, [](int, uint32_t) {});
    pn_nchild[v] = static_cast<uint32_t>(k);
}

__global__ void k_cpu_index(NodeCtx c, uint32_t Tcap, const unsigned* Tdev, const uint2* pn_lohi,
                            const uint16_t* pn_meta, const uint32_t* pn_cb, uint32_t* pn_cpu) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= eff(Tdev, Tcap)) return;
    const uint16_t meta = pn_meta[v];
    if ((meta & 255) == 0) pn_cpu[v] = sys_of(c.sys, static_cast<int>(pn_lohi[v].x));  // a system's root
    if (meta & 256) return;
    const uint32_t first = c.nroots + pn_cb[v];
    for_children(c, pn_lohi, v, meta & 255, [&](int k, uint32_t ch) { pn_cpu[ch] = first + k; });
}

// Geometric centre (FP64, the reference's iterative halving, src/cpu_backend.cpp:575-582 and
// 585-592) of the node at depth d containing body b; at depth 21 f the node of a run re-keyed in
// frame f takes that run's cube (src/cpu_backend.cpp:536-544).
__device__ void node_geo(const NodeCtx& c, const double* frame, uint32_t b, int d, double& gx, double& gy, double& gz,
                         double& half) {
    frame += 5 * sys_of(c.sys, static_cast<int>(b));
    half = 0.5 * frame[3];
    gx = __dadd_rn(frame[0], half);
    gy = __dadd_rn(frame[1], half);
    gz = __dadd_rn(frame[2], half);
    for (int l = 1; l <= d; ++l) {
        const int o = digit_at(c.k0, c.ft, b, l);
        const double q = 0.5 * half;
        gx = __dadd_rn(gx, (o & 4) ? q : -q);
        gy = __dadd_rn(gy, (o & 2) ? q : -q);
        gz = __dadd_rn(gz, (o & 1) ? q : -q);
        half = q;
        if (c.ft && l % MAX_LEVEL == 0 && l / MAX_LEVEL < c.ft->nfr[b]) {
            const int f = l / MAX_LEVEL;
            const double* cb = c.ft->cube[f] + 5 * c.ft->runid[f][b];
            half = 0.5 * cb[3];
            gx = __dadd_rn(cb[0], half);
            gy = __dadd_rn(cb[1], half);
            gz = __dadd_rn(cb[2], half);
        }
    }
}

__global__ void k_nodes_out(NodeCtx c, uint32_t Tcap, const unsigned* Tdev, const uint2* pn_lohi, const uint16_t* pn_meta,
                            const uint32_t* pn_nchild, const uint32_t* pn_cb, const uint32_t* pn_cpu,
                            const double* frame, uint4* nd_range,
                            float4* nd_geo, uint32_t* nd_parent, uint32_t* leaf_node, const uint32_t* gidx,
                            uint32_t* grp_node, int* max_depth, unsigned* err) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t T = eff(Tdev, Tcap);
    if (v >= T) return;
    const uint16_t meta = pn_meta[v];
    const int d = meta & 255;
    const bool leaf = meta & 256;
    const uint2 r = pn_lohi[v];
    const uint32_t me = pn_cpu[v];
    const uint32_t nch = pn_nchild[v];
    const uint32_t first = leaf ? r.x : c.nroots + pn_cb[v];
    if (me >= T || (!leaf && first + nch > T) || r.x >= r.y || r.y > static_cast<uint32_t>(c.n)) {
        atomicOr(err, kErrNodeOverflow);
        return;
    }
    nd_range[me] = make_uint4(r.x, r.y, first, leaf ? 0u : nch);
    double gx, gy, gz, half;
    node_geo(c, frame, r.x, d, gx, gy, gz, half);
    nd_geo[me] = make_float4(static_cast<float>(gx), static_cast<float>(gy), static_cast<float>(gz),
                             static_cast<float>(half));
    if (v == 0) nd_parent[0] = 0xffffffffu;
    if (!leaf)
        for (uint32_t k = 0; k < nch; ++k) nd_parent[first + k] = me;
    if (leaf) {
        const uint32_t l = c.lid[r.x];
        if (l < static_cast<uint32_t>(leaf_count(c))) leaf_node[l] = me;
        else atomicOr(err, kErrNodeOverflow);
    }
    if (meta & 512) {
        const uint32_t gi = gidx[v];
        if (gi < T) grp_node[gi] = v;
        else atomicOr(err, kErrNodeOverflow);
    }
    atomicMax(max_depth, d);
}

// Group boxes from the bodies' float positions (src/cpu_backend.cpp:604-616).
__global__ void k_groups(const uint32_t* grp_node, const uint2* pn_lohi, uint32_t Tcap, const unsigned* Tdev,
                         const BodyArrays b, const unsigned* ngroups, uint2* grp_range, float4* grp_box) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t T = eff(Tdev, Tcap);
    if (g >= *ngroups || g >= Tcap) return;
    const uint32_t v = grp_node[g];
    if (v >= T) return;
    const uint2 r = pn_lohi[v];
    if (r.x >= r.y) return;
    float4 p = b.hm[r.x];
    float mnx = p.x, mny = p.y, mnz = p.z, mxx = mnx, mxy = mny, mxz = mnz;
    for (uint32_t i = r.x + 1; i < r.y; ++i) {
        p = b.hm[i];
        mnx = fminf(mnx, p.x); mny = fminf(mny, p.y); mnz = fminf(mnz, p.z);
        mxx = fmaxf(mxx, p.x); mxy = fmaxf(mxy, p.y); mxz = fmaxf(mxz, p.z);
    }
    grp_range[g] = r;
    grp_box[2 * g] = make_float4(__fmul_rn(0.5f, __fadd_rn(mnx, mxx)), __fmul_rn(0.5f, __fadd_rn(mny, mxy)),
                                 __fmul_rn(0.5f, __fadd_rn(mnz, mxz)), 0.f);
    grp_box[2 * g + 1] = make_float4(__fmul_rn(0.5f, __fsub_rn(mxx, mnx)), __fmul_rn(0.5f, __fsub_rn(mxy, mny)),
                                     __fmul_rn(0.5f, __fsub_rn(mxz, mnz)), 0.f);
}

// ---- merged walk groups (GB300 grouping; off by default) ------------------------------------
// The reference's groups are the largest subtrees of <= group_max bodies, which the octree's
// eight-way split leaves small (a few dozen bodies). Runs of consecutive sibling groups (same
// parent, contiguous bodies) are packed greedily, in order, into groups of <= group_max bodies:
// fewer, fuller walk groups. Every packed group is still contained in its parent, whose walk
// rule opens it, so the lists stay exact-rule lists for the larger box.
__device__ __forceinline__ uint32_t group_parent(const uint32_t* grp_node, const uint32_t* pn_cpu,
                                                 const uint32_t* nd_parent, uint32_t T, uint32_t g) {
    const uint32_t v = grp_node[g];
    if (v >= T) return 0xffffffffu;
    const uint32_t c = pn_cpu[v];
    return c < T ? nd_parent[c] : 0xffffffffu;
}

template <bool WRITE>
__global__ void k_merge_groups(const uint32_t* grp_node, const uint32_t* pn_cpu, const uint32_t* nd_parent,
                               const uint2* grp_range, const unsigned* ngroups, uint32_t Tcap, const unsigned* Tdev,
                               int gmax, uint32_t* mcount, const uint32_t* moff, uint2* mrange) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= Tcap) return;
    const uint32_t T = eff(Tdev, Tcap), G = min(*ngroups, Tcap);
    if (g >= G) {
        if (!WRITE) mcount[g] = 0;
        return;
    }
    const uint32_t P = group_parent(grp_node, pn_cpu, nd_parent, T, g);
    const bool start = g == 0 || group_parent(grp_node, pn_cpu, nd_parent, T, g - 1) != P ||
                       grp_range[g - 1].y != grp_range[g].x;
    if (!start) {
        if (!WRITE) mcount[g] = 0;
        return;
    }
    uint32_t bins = 0, cur = 0, lo = grp_range[g].x, hi = lo;
    for (uint32_t h = g; h < G; ++h) {
        const uint2 r = grp_range[h];
        if (h > g && (group_parent(grp_node, pn_cpu, nd_parent, T, h) != P || r.x != hi)) break;
        const uint32_t sz = r.y - r.x;
        if (cur > 0 && cur + sz > static_cast<uint32_t>(gmax)) {
            if (WRITE) mrange[moff[g] + bins] = make_uint2(lo, hi);
            ++bins;
            cur = 0;
            lo = r.x;
        }
        cur += sz;
        hi = r.y;
    }
    if (WRITE) mrange[moff[g] + bins] = make_uint2(lo, hi);
    ++bins;
    if (!WRITE) mcount[g] = bins;
}

__global__ void k_merged_boxes(const uint2* mrange, const unsigned* mcount_total, uint32_t cap, const BodyArrays b,
                               float4* box) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= *mcount_total || g >= cap) return;
    const uint2 r = mrange[g];
    if (r.x >= r.y) return;
    float4 p = b.hm[r.x];
    float mnx = p.x, mny = p.y, mnz = p.z, mxx = mnx, mxy = mny, mxz = mnz;
    for (uint32_t i = r.x + 1; i < r.y; ++i) {
        p = b.hm[i];
        mnx = fminf(mnx, p.x); mny = fminf(mny, p.y); mnz = fminf(mnz, p.z);
        mxx = fmaxf(mxx, p.x); mxy = fmaxf(mxy, p.y); mxz = fmaxf(mxz, p.z);
    }
    box[2 * g] = make_float4(__fmul_rn(0.5f, __fadd_rn(mnx, mxx)), __fmul_rn(0.5f, __fadd_rn(mny, mxy)),
                             __fmul_rn(0.5f, __fadd_rn(mnz, mxz)), 0.f);
    box[2 * g + 1] = make_float4(__fmul_rn(0.5f, __fsub_rn(mxx, mnx)), __fmul_rn(0.5f, __fsub_rn(mxy, mny)),
                                 __fmul_rn(0.5f, __fsub_rn(mxz, mnz)), 0.f);
}

// ---- upsweep ---------------------------------------------------------------------------------
struct Moments {
    float4* com;    // (cx, cy, cz, m), the reference's stored floats
    float4* comlo;  // FP64 com minus its float, as floats
    float4* q0;     // (qxx, qxy, qxz, qyy)
    float4* q1;     // (qyz, qzz, rcrit2, 0)
};

// rcrit2 = (2 half / theta + |com - centre|)^2 capped at FLT_MAX (src/cpu_backend.cpp:595-600), with
// |com - centre|^2 as the reference's compiler forms it: fma(dz, dz, fma(dx, dx, dy*dy)).
__device__ __forceinline__ float rcrit2_of(float cx, float cy, float cz, float4 g, float inv_theta) {
    const float dx = __fsub_rn(cx, g.x), dy = __fsub_rn(cy, g.y), dz = __fsub_rn(cz, g.z);
    const float s = __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
    const double r = __dadd_rn(__dmul_rn(static_cast<double>(__fmul_rn(2.f, g.w)), static_cast<double>(inv_theta)),
                               __dsqrt_rn(static_cast<double>(s)));
    const double r2 = __dmul_rn(r, r);
    return static_cast<float>(r2 < static_cast<double>(FLT_MAX) ? r2 : static_cast<double>(FLT_MAX));
}

__device__ void store_moments(Moments mo, uint32_t node, double M, double cx, double cy, double cz, double qxx,
                              double qxy, double qxz, double qyy, double qyz, double qzz, float4 g, float inv_theta) {
    const float fx = static_cast<float>(cx), fy = static_cast<float>(cy), fz = static_cast<float>(cz);
    mo.com[node] = make_float4(fx, fy, fz, static_cast<float>(M));
    mo.comlo[node] = make_float4(static_cast<float>(__dsub_rn(cx, fx)), static_cast<float>(__dsub_rn(cy, fy)),
                                 static_cast<float>(__dsub_rn(cz, fz)), 0.f);
    mo.q0[node] = make_float4(static_cast<float>(qxx), static_cast<float>(qxy), static_cast<float>(qxz),
                              static_cast<float>(qyy));
    mo.q1[node] = make_float4(static_cast<float>(qyz), static_cast<float>(qzz), rcrit2_of(fx, fy, fz, g, inv_theta), 0.f);
}

#define DADD __dadd_rn
#define DMUL __dmul_rn
#define DSUB __dsub_rn
#define DFMA __fma_rn

// Upsweep bookkeeping: internal nodes bucketed by depth, leaves bucketed by body count.
constexpr int NDEP = MAX_DEPTH + 2;  // depth buckets (depth <= MAX_DEPTH + 1 with headroom)
constexpr int NLSZ = 18;   // leaf-size buckets: 1..16, then larger
struct UpsweepIndex {
    unsigned dep_count[NDEP], dep_off[NDEP + 1], dep_cur[NDEP];
    unsigned lsz_count[NLSZ], lsz_off[NLSZ + 1], lsz_cur[NLSZ];
};

__device__ __forceinline__ int lsz_bucket(uint32_t cnt) { return cnt > 16 ? 17 : static_cast<int>(cnt); }

// Pass 1: bucket counts (block-aggregated). Pass 2 (phase 1): scatter into bucket order.
__global__ void k_upsweep_bucket(const uint2* pn_lohi, const uint16_t* pn_meta, const uint32_t* pn_cpu, uint32_t Tcap,
                                 const unsigned* Tdev, UpsweepIndex* ix, int phase, uint32_t* dep_nodes,
                                 uint32_t* leaf_order) {
    const uint32_t T = eff(Tdev, Tcap);
    __shared__ unsigned sc[NDEP + NLSZ], sbase[NDEP + NLSZ];
    for (int k = threadIdx.x; k < NDEP + NLSZ; k += blockDim.x) sc[k] = 0;
    __syncthreads();
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    int bucket = -1;
    unsigned rank = 0;
    uint32_t me = 0;
    if (v < T) {
        const uint16_t meta = pn_meta[v];
        me = pn_cpu[v];
        if (meta & 256) {
            const uint2 r = pn_lohi[v];
            bucket = NDEP + lsz_bucket(r.y - r.x);
        } else {
            bucket = meta & 255;
        }
        rank = atomicAdd(&sc[bucket], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < NDEP + NLSZ; k += blockDim.x) {
        if (!sc[k]) continue;
        if (phase == 0) {
            atomicAdd(k < NDEP ? &ix->dep_count[k] : &ix->lsz_count[k - NDEP], sc[k]);
        } else {
            sbase[k] = k < NDEP ? ix->dep_off[k] + atomicAdd(&ix->dep_cur[k], sc[k])
                                : ix->lsz_off[k - NDEP] + atomicAdd(&ix->lsz_cur[k - NDEP], sc[k]);
        }
    }
    if (phase == 0) return;
    __syncthreads();
    if (bucket < 0) return;
    const unsigned pos = sbase[bucket] + rank;
    if (bucket < NDEP) dep_nodes[pos] = me;
    else leaf_order[pos] = me;
}

__global__ void k_upsweep_offsets(UpsweepIndex* ix) {
    if (threadIdx.x != 0) return;
    unsigned run = 0;
    for (int k = 0; k < NDEP; ++k) { ix->dep_off[k] = run; run += ix->dep_count[k]; }
    ix->dep_off[NDEP] = run;
    run = 0;
    for (int k = 0; k < NLSZ; ++k) { ix->lsz_off[k] = run; run += ix->lsz_count[k]; }
    ix->lsz_off[NLSZ] = run;
}

// Leaf moments about each leaf's centre of mass in FP64 (src/cpu_backend.cpp:619-640), one
// thread per leaf, leaves taken in body-count order so a warp's loops have equal trip counts.
__global__ void k_leaf_moments(const uint32_t* __restrict__ leaf_order, uint32_t Kcap, const unsigned* Kdev,
                               uint32_t Tcap, const unsigned* Tdev, const uint4* __restrict__ nd_range,
                               const float4* __restrict__ nd_geo, const BodyArrays b, Moments mo, float inv_theta,
                               const float* __restrict__ inv_theta_sys, const uint32_t* __restrict__ sys, unsigned* err) {
    const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t T = eff(Tdev, Tcap);
    if (l >= eff(Kdev, Kcap)) return;
    const uint32_t node = leaf_order[l];
    if (node >= T) {
        atomicOr(err, kErrNodeOverflow);
        return;
    }
    const uint4 r = nd_range[node];
    const float4 g = nd_geo[node];
    if (inv_theta_sys) inv_theta = inv_theta_sys[sys_of(sys, static_cast<int>(r.x))];
    double M = 0, sx = 0, sy = 0, sz = 0;
    for (uint32_t i = r.x; i < r.y; ++i) {
        const double m = b.m[i];
        M = DADD(M, m);
        sx = DADD(sx, DMUL(m, b.x[i]));
        sy = DADD(sy, DMUL(m, b.y[i]));
        sz = DADD(sz, DMUL(m, b.z[i]));
    }
    const double cx = M > 0 ? __ddiv_rn(sx, M) : g.x, cy = M > 0 ? __ddiv_rn(sy, M) : g.y,
                 cz = M > 0 ? __ddiv_rn(sz, M) : g.z;
    double qxx = 0, qxy = 0, qxz = 0, qyy = 0, qyz = 0, qzz = 0;
    for (uint32_t i = r.x; i < r.y; ++i) {
        const double m = b.m[i], dx = DSUB(b.x[i], cx), dy = DSUB(b.y[i], cy), dz = DSUB(b.z[i], cz);
        const double r2 = DFMA(dz, dz, DFMA(dx, dx, DMUL(dy, dy)));
        const double m3 = DMUL(m, 3.0);
        qxx = DFMA(m, DFMA(DMUL(3.0, dx), dx, -r2), qxx);
        qyy = DFMA(m, DFMA(DMUL(3.0, dy), dy, -r2), qyy);
        qzz = DFMA(m, DFMA(DMUL(3.0, dz), dz, -r2), qzz);
        qxy = DFMA(DMUL(m3, dx), dy, qxy);
        qxz = DFMA(DMUL(m3, dx), dz, qxz);
        qyz = DFMA(DMUL(m3, dy), dz, qyz);
    }
    store_moments(mo, node, M, cx, cy, cz, qxx, qxy, qxz, qyy, qyz, qzz, g, inv_theta);
}

// Internal nodes of one depth: combine the children (already final) in index order, FP64, the
// parallel-axis theorem for the traceless quadrupole (src/cpu_backend.cpp:642-663).
// Four lanes per node, eight nodes per warp. Lane j forms the terms of children j and j + 4 (the
// per-child FP64 work runs in parallel); each of the reference's sequential child-order sums is
// then folded by one lane only, from terms shuffled in child order: M, sx, sy, sz by lanes 0..3;
// qxx and qyy by lane 0, qzz and qxy by lane 1, qxz by lane 2, qyz by lane 3. Lanes 1..3 divide
// their first sum by M together. Every FP64 operation of the reference, as its compiler forms it
// (fused multiply-adds included), is done once, in its order, so the moments are the reference's
// bit for bit. (On this part an FP64 warp instruction holds a
// scheduler's FP64 unit for about 64 cycles: the form keeps the number of FP64 warp instructions
// per node low and spreads the nodes of a level over all schedulers.)
__device__ __forceinline__ double shfl_d(double v, int src_lane) { return __shfl_sync(0xffffffffu, v, src_lane); }

constexpr int COMBINE_BS = 128;
constexpr int COMBINE_NODES = COMBINE_BS / 4;  // nodes per block and round

__global__ void __launch_bounds__(COMBINE_BS) k_combine_level(const uint32_t* __restrict__ dep_nodes,
                                                              const UpsweepIndex* ix, int depth, uint32_t Tcap,
                                                              const unsigned* Tdev, const uint4* __restrict__ nd_range,
                                                              const float4* __restrict__ nd_geo, Moments mo,
                                                              float inv_theta, const float* __restrict__ inv_theta_sys,
                                                              const uint32_t* __restrict__ sys, unsigned* err) {
    const uint32_t T = eff(Tdev, Tcap);
    const unsigned lo = ix->dep_off[depth], hi = ix->dep_off[depth + 1];
    const int lane = threadIdx.x & 31, j = lane & 3, base = lane & ~3;
    const unsigned warps = (gridDim.x * blockDim.x) >> 5;
    const unsigned wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    for (unsigned k0 = lo + 8 * wid; k0 < hi; k0 += 8 * warps) {  // warp-uniform
        const unsigned k = k0 + static_cast<unsigned>(lane >> 2);
        bool valid = k < hi;
        uint32_t p = valid ? dep_nodes[k] : 0u;
        uint4 r = make_uint4(0, 0, 0, 0);
        if (valid) {
            if (p >= T) {
                if (j == 0) atomicOr(err, kErrNodeOverflow);
                valid = false;
            } else {
                r = nd_range[p];
                if (r.w == 0 || r.w > 8 || r.z + r.w > T) {
                    if (j == 0) atomicOr(err, kErrNodeOverflow);
                    valid = false;
                }
            }
        }
        const int nch = valid ? static_cast<int>(r.w) : 0;
        // Terms of the lane's children c = j + 4 sl (zeros past the last child: never added).
        double m[2], ccx[2], ccy[2], ccz[2], mx[2], my[2], mz[2];
        float4 qa[2], qb[2];
#pragma unroll
        for (int sl = 0; sl < 2; ++sl) {
            const int c = j + 4 * sl;
            float4 cm = make_float4(0.f, 0.f, 0.f, 0.f);
            qa[sl] = cm;
            qb[sl] = cm;
            if (c < nch) {
                cm = mo.com[r.z + c];
                qa[sl] = mo.q0[r.z + c];
                qb[sl] = mo.q1[r.z + c];
            }
            m[sl] = cm.w;
            ccx[sl] = cm.x;
            ccy[sl] = cm.y;
            ccz[sl] = cm.z;
            mx[sl] = DMUL(m[sl], ccx[sl]);
            my[sl] = DMUL(m[sl], ccy[sl]);
            mz[sl] = DMUL(m[sl], ccz[sl]);
        }
        // Monopole sums in child order: lane j folds M (0), sx (1), sy (2), sz (3).
        double f1 = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int src = base + (q & 3), sl = q >> 2;
            const double vm = shfl_d(m[sl], src), vx = shfl_d(mx[sl], src), vy = shfl_d(my[sl], src),
                         vz = shfl_d(mz[sl], src);
            const double v = j == 0 ? vm : j == 1 ? vx : j == 2 ? vy : vz;
            if (q < nch) f1 = DADD(f1, v);
        }
        const double M = shfl_d(f1, base);
        const float4 g = valid ? nd_geo[p] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float gj = j == 1 ? g.x : j == 2 ? g.y : g.z;
        const double cj = M > 0 ? __ddiv_rn(f1, M) : static_cast<double>(gj);  // lane 0's is unused
        const double cx = shfl_d(cj, base + 1), cy = shfl_d(cj, base + 2), cz = shfl_d(cj, base + 3);
        // Quadrupole terms of the lane's children about the new centre.
        double txx[2], tyy[2], tzz[2], txy[2], txz[2], tyz[2];
#pragma unroll
        for (int sl = 0; sl < 2; ++sl) {
            const double dx = DSUB(ccx[sl], cx), dy = DSUB(ccy[sl], cy), dz = DSUB(ccz[sl], cz);
            const double r2 = DFMA(dz, dz, DFMA(dx, dx, DMUL(dy, dy)));
            const double m3 = DMUL(m[sl], 3.0);
            txx[sl] = DFMA(m[sl], DFMA(DMUL(3.0, dx), dx, -r2), static_cast<double>(qa[sl].x));
            tyy[sl] = DFMA(m[sl], DFMA(DMUL(3.0, dy), dy, -r2), static_cast<double>(qa[sl].w));
            tzz[sl] = DFMA(m[sl], DFMA(DMUL(3.0, dz), dz, -r2), static_cast<double>(qb[sl].y));
            txy[sl] = DFMA(DMUL(m3, dx), dy, static_cast<double>(qa[sl].y));
            txz[sl] = DFMA(DMUL(m3, dx), dz, static_cast<double>(qa[sl].z));
            tyz[sl] = DFMA(DMUL(m3, dy), dz, static_cast<double>(qb[sl].x));
        }
        // Quadrupole sums in child order: lane 0 folds qxx and qyy, lane 1 qzz and qxy, lane 2 qxz,
        // lane 3 qyz.
        double fa = 0, fb = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int src = base + (q & 3), sl = q >> 2;
            const double vxx = shfl_d(txx[sl], src), vyy = shfl_d(tyy[sl], src), vzz = shfl_d(tzz[sl], src),
                         vxy = shfl_d(txy[sl], src), vxz = shfl_d(txz[sl], src), vyz = shfl_d(tyz[sl], src);
            const double va = j == 0 ? vxx : j == 1 ? vzz : j == 2 ? vxz : vyz;
            const double vb = j == 0 ? vyy : vxy;
            if (q < nch) {
                fa = DADD(fa, va);
                if (j < 2) fb = DADD(fb, vb);
            }
        }
        const double qzz = shfl_d(fa, base + 1), qxy = shfl_d(fb, base + 1), qxz = shfl_d(fa, base + 2),
                     qyz = shfl_d(fa, base + 3);
        if (valid && j == 0)
            store_moments(mo, p, M, cx, cy, cz, fa, qxy, qxz, fb, qyz, qzz, g,
                          inv_theta_sys ? inv_theta_sys[sys_of(sys, static_cast<int>(r.x))] : inv_theta);
    }
}

#undef DADD
#undef DMUL
#undef DSUB


__global__ void k_lid(uint32_t* lid, const uint32_t* flag, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) lid[i] = lid[i] + flag[i] - 1;
}

__global__ void k_leaf_tail(uint32_t* leaf_first, const unsigned* K, int n) { leaf_first[*K] = static_cast<uint32_t>(n); }

__global__ void k_gflag(const uint16_t* pn_meta, uint32_t Tcap, const unsigned* Tdev, uint32_t* gflag) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < Tcap) gflag[v] = v < eff(Tdev, Tcap) ? (pn_meta[v] >> 9) & 1u : 0u;
}

__global__ void k_probe() {}

// ---- host helpers ----------------------------------------------------------------------------
void scan_u32(Engine& e, TreeState& t, const uint32_t* in, uint32_t* out, int n, uint32_t* total) {
    if (n <= 0) return;
    const int tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    t.scan_state.reserve(static_cast<size_t>(tiles) * 8);
    t.scan_ctr.reserve(256);
    LG_CK(cudaMemsetAsync(t.scan_state.as<char>(), 0, static_cast<size_t>(tiles) * 8, e.stream));
    LG_CK(cudaMemsetAsync(t.scan_ctr.as<char>(), 0, 4, e.stream));
    k_scan<<<tiles, SCAN_BS, 0, e.stream>>>(in, out, n, t.scan_state.as<unsigned long long>(), t.scan_ctr.as<unsigned>(),
                                           total, e.err_word());
    LG_LAUNCHED();
    ++e.launches;
}

// Sorts (keys, vals) held in (keysA, valsA); result in the buffer ctl->sel selects.
void sort_pairs(Engine& e, TreeState& t, int n) {
    cudaStream_t s = e.stream;
    const int tiles = (n + SORT_TILE - 1) / SORT_TILE;
    t.hist.reserve(PASSES * RADIX * 4);
    t.lookback.reserve(static_cast<size_t>(PASSES) * tiles * RADIX * 4);
    t.ctl.reserve(sizeof(SortCtl));
    LG_CK(cudaMemsetAsync(t.hist.as<char>(), 0, PASSES * RADIX * 4, s));
    LG_CK(cudaMemsetAsync(t.lookback.as<char>(), 0, static_cast<size_t>(PASSES) * tiles * RADIX * 4, s));
    const int hb = std::min(e.sms * 4, std::max(1, grid_for(n, 1024)));
    k_sort_hist<<<hb, 256, 0, s>>>(t.keysA.as<uint64_t>(), n, t.hist.as<unsigned>());
    LG_LAUNCHED();
    k_sort_offsets<<<1, RADIX, 0, s>>>(t.hist.as<unsigned>(), n, t.ctl.as<SortCtl>());
    LG_LAUNCHED();
    for (int p = 0; p < PASSES; ++p) {
        k_sort_pass<<<tiles, SORT_BS, 0, s>>>(t.keysA.as<uint64_t>(), t.valsA.as<uint32_t>(), t.keysB.as<uint64_t>(),
                                              t.valsB.as<uint32_t>(), n, p, t.hist.as<unsigned>(),
                                              t.lookback.as<unsigned>() + static_cast<size_t>(p) * tiles * RADIX,
                                              t.ctl.as<SortCtl>(), e.err_word());
        LG_LAUNCHED();
    }
    k_sort_finish<<<std::max(1, std::min(4 * e.sms, grid_for(n, BS))), BS, 0, s>>>(
        t.keysA.as<uint64_t>(), t.valsA.as<uint32_t>(), t.keysB.as<uint64_t>(), t.valsB.as<uint32_t>(),
        t.ctl.as<SortCtl>(), n);
    LG_LAUNCHED();
    e.launches += 3 + PASSES;
}

void reserve_sort(TreeState& t, int n) {
    const size_t cnt = static_cast<size_t>(n) + 1;
    t.keysA.reserve(cnt * 8); t.keysB.reserve(cnt * 8);
    t.valsA.reserve(cnt * 4); t.valsB.reserve(cnt * 4);
    t.skey.reserve(cnt * 8);
}

}  // namespace

std::unique_ptr<TreeState, void (*)(TreeState*)> make_tree_state() {
    return std::unique_ptr<TreeState, void (*)(TreeState*)>(new TreeState, destroy_tree);
}

const void* probe_kernel() { return reinterpret_cast<const void*>(k_probe); }

void tree_sort(Engine& e) {
    TreeState& t = *e.tree;
    const int n = t.n_tree >= 0 ? t.n_tree : e.n;
    const int n_total = e.n;
    const uint32_t* sys = t.sys;
    cudaStream_t s = e.stream;
    if (n >= (1 << 30)) fail(kRuntime, "cuda tree: n >= 2^30 exceeds the sort's look-back counters");
    reserve_sort(t, n);
    t.frame.reserve(static_cast<size_t>(std::max(t.nsys, 1)) * 5 * 8 + 64);
    t.counts.reserve(64);
    t.restarted = false;
    t.nframes = 1;
    if (sys) {
        k_frame_sys<<<t.nsys, BS, 0, s>>>(e.bodies(e.cur), t.sys_off, t.frame.as<double>());
    } else {
        const int fb = std::min(2 * e.sms, grid_for(n, BS));
        e.diag_partial.reserve(static_cast<size_t>(fb) * 12 * 8);
        k_frame<<<fb, BS, 0, s>>>(e.bodies(e.cur), n, e.diag_partial.as<long long>(), e.ticket(), t.frame.as<double>());
    }
    LG_LAUNCHED();
    if (sys) t.mkeys.reserve(static_cast<size_t>(n) * 8 + 8);
    k_keys<<<grid_for(n, BS), BS, 0, s>>>(sys, e.bodies(e.cur), n, t.frame.as<double>(),
                                          sys ? t.mkeys.as<uint64_t>() : t.keysA.as<uint64_t>(), t.valsA.as<uint32_t>());
    LG_LAUNCHED();
    e.launches += 2;
    if (sys) LG_CK(cudaMemcpyAsync(t.keysA.as<uint64_t>(), t.mkeys.as<uint64_t>(), static_cast<size_t>(n) * 8,
                                   cudaMemcpyDeviceToDevice, s));
    sort_pairs(e, t, n);
    if (sys) {
        // Forest: stable sort by system on top of the key order -> (system, key) order.
        k_sys_keys<<<grid_for(n, BS), BS, 0, s>>>(sys, t.valsA.as<uint32_t>(), t.keysA.as<uint64_t>(), n);
        LG_LAUNCHED();
        ++e.launches;
        sort_pairs(e, t, n);
    }
    int other = e.cur ^ 1;
    k_permute<<<grid_for(n_total, BS), BS, 0, s>>>(e.bodies(e.cur), e.bodies(other), t.keysA.as<uint64_t>(),
                                                   t.valsA.as<uint32_t>(), t.skey.as<uint64_t>(), nullptr, nullptr, n,
                                                   sys ? t.mkeys.as<uint64_t>() : nullptr, n_total);
    LG_LAUNCHED();
    ++e.launches;
    e.cur = other;

    // Key restarts (src/cpu_backend.cpp:536-544): runs of identical keys longer than a leaf.
    unsigned* counts = t.counts.as<unsigned>();
    LG_CK(cudaMemsetAsync(counts, 0, 64, s));
    const int run_cap = std::max(1, n / (LEAF_MAX + 1) + 1);  // runs hold more than LEAF_MAX bodies each
    t.runs.reserve(static_cast<size_t>(run_cap) * 8);
    k_find_runs<<<grid_for(n, BS), BS, 0, s>>>(sys, t.skey.as<uint64_t>(), nullptr, nullptr, 1, n, t.runs.as<uint2>(),
                                               counts, run_cap);
    LG_LAUNCHED();
    ++e.launches;
    // Key restarts are rare: unless the last build needed them, assume none and let the check after
    // the walk (tree_verify) catch a miss; otherwise read the run count now.
    t.speculative = t.have_guess && !t.restart_mode;
    if (t.speculative) return;
    LG_CK(cudaMemcpyAsync(e.pinned_small, counts, 4, cudaMemcpyDeviceToHost, s));
    LG_CK(cudaStreamSynchronize(s));
    // Runs are disjoint and longer than LEAF_MAX, so there are fewer than run_cap.
    unsigned R = std::min(e.pinned_small[0], static_cast<unsigned>(run_cap));
    t.restart_mode = R > 0;
    if (R == 0) return;
    t.restarted = true;
    ++t.generation;
    t.key1tmp.reserve(static_cast<size_t>(n) * 8 + 8);
    t.nfr.reserve(static_cast<size_t>(n) + 8);
    t.ftab.reserve(sizeof(FrameTable));
    uint64_t* key1 = t.key1tmp.as<uint64_t>();
    uint8_t* nfr = t.nfr.as<uint8_t>();
    LG_CK(cudaMemsetAsync(nfr, 1, static_cast<size_t>(n), s));
    FrameTable ft{};
    ft.key[0] = t.skey.as<uint64_t>();
    ft.nfr = nfr;
    // Frame by frame: re-key the runs in their own cubes, then a stable sort by (run, new key), which
    // keeps every body inside its run. Inside a run the earlier frames' keys, run indices and nfr
    // are all equal, so only the bodies and the new keys move.
    for (int f = 1; f < FRAMES && R > 0; ++f) {
        BodyArrays b = e.bodies(e.cur);
        t.fkey[f].reserve(static_cast<size_t>(n) * 8 + 8);
        t.frunid[f].reserve(static_cast<size_t>(n) * 4 + 4);
        t.fcube[f].reserve(static_cast<size_t>(R) * 5 * 8);
        int* runid = t.frunid[f].as<int>();
        k_fill_i32<<<grid_for(n, BS), BS, 0, s>>>(runid, -1, n);
        LG_LAUNCHED();
        k_fill_u64<<<grid_for(n, BS), BS, 0, s>>>(key1, 0ull, n);
        LG_LAUNCHED();
        k_run_cube<<<R, BS, 0, s>>>(b, t.runs.as<uint2>(), t.fcube[f].as<double>());
        LG_LAUNCHED();
        k_run_keys<<<R, BS, 0, s>>>(b, t.runs.as<uint2>(), t.fcube[f].as<double>(), key1, runid, nfr, f);
        LG_LAUNCHED();
        LG_CK(cudaMemcpyAsync(t.keysA.as<uint64_t>(), key1, static_cast<size_t>(n) * 8, cudaMemcpyDeviceToDevice, s));
        k_iota<<<grid_for(n, BS), BS, 0, s>>>(t.valsA.as<uint32_t>(), n);
        LG_LAUNCHED();
        sort_pairs(e, t, n);
        k_seg_keys<<<grid_for(n, BS), BS, 0, s>>>(t.valsA.as<uint32_t>(), runid, t.runs.as<uint2>(),
                                                  t.keysA.as<uint64_t>(), n);
        LG_LAUNCHED();
        sort_pairs(e, t, n);
        const int other = e.cur ^ 1;
        k_permute<<<grid_for(n_total, BS), BS, 0, s>>>(e.bodies(e.cur), e.bodies(other), t.keysA.as<uint64_t>(),
                                                       t.valsA.as<uint32_t>(), nullptr, key1, t.fkey[f].as<uint64_t>(), n,
                                                       nullptr, n_total);
        LG_LAUNCHED();
        e.cur = other;
        ft.key[f] = t.fkey[f].as<uint64_t>();
        ft.runid[f] = runid;
        ft.cube[f] = t.fcube[f].as<double>();
        ft.nf = f + 1;
        t.nframes = f + 1;
        k_put_table<<<1, 1, 0, s>>>(ft, t.ftab.as<FrameTable>());
        LG_LAUNCHED();
        e.launches += 8;
        if (f + 1 == FRAMES) break;  // runs left now stay leaves at depth MAX_DEPTH
        // The next frame's runs: bodies re-keyed in this frame whose composite keys still tie.
        LG_CK(cudaMemsetAsync(counts + 6, 0, 4, s));
        k_find_runs<<<grid_for(n, BS), BS, 0, s>>>(sys, t.skey.as<uint64_t>(), t.ftab.as<FrameTable>(), nfr, f + 1, n,
                                                   t.runs.as<uint2>(), counts + 6, run_cap);
        LG_LAUNCHED();
        ++e.launches;
        LG_CK(cudaMemcpyAsync(e.pinned_small, counts + 6, 4, cudaMemcpyDeviceToHost, s));
        LG_CK(cudaStreamSynchronize(s));
        R = std::min(e.pinned_small[0], static_cast<unsigned>(run_cap));
    }
}

void tree_build(Engine& e, double theta) {
    TreeState& t = *e.tree;
    const int n = t.n_tree >= 0 ? t.n_tree : e.n;
    const uint32_t* sys = t.sys;
    cudaStream_t s = e.stream;
    t.group_max = e.group_max;
    t.theta = theta;
    const uint64_t* k0 = t.skey.as<uint64_t>();
    const FrameTable* ft = t.restarted ? t.ftab.as<FrameTable>() : nullptr;
    unsigned* counts = t.counts.as<unsigned>();
    const unsigned* Kdev = counts + 1;
    const unsigned* Tdev = counts + 2;
    const size_t n1 = static_cast<size_t>(n) + 1;
    t.bdepth.reserve(n1 * 2);
    t.flag.reserve(n1 * 4);
    t.leafid.reserve(n1 * 4);
    t.leaf_first.reserve(n1 * 4);
    t.leaf_depth.reserve(n1);
    t.leaf_c.reserve(n1);
    t.leaf_cnt.reserve(n1 * 4);
    t.leaf_pre.reserve(n1 * 4);
    t.leaf_node.reserve(n1 * 4);
    const int gb = grid_for(n, BS);
    if (t.group_max > GMAX_LIMIT) fail(kRuntime, "cuda tree build: group size above 1024");
    k_body_depth<<<grid_for(n, DEPTH_BS), DEPTH_BS, 0, s>>>(sys, k0, ft, n, t.group_max,
                                                            t.bdepth.as<uint16_t>());
    LG_LAUNCHED();
    k_leaf_flags<<<gb, BS, 0, s>>>(sys, k0, ft, t.bdepth.as<uint16_t>(), n, t.flag.as<uint32_t>());
    LG_LAUNCHED();
    e.launches += 2;
    scan_u32(e, t, t.flag.as<uint32_t>(), t.leafid.as<uint32_t>(), n, counts + 1);
    LG_CK(cudaMemsetAsync(t.leaf_cnt.as<char>(), 0, n1 * 4, s));
    k_leaf_info<<<gb, BS, 0, s>>>(sys, k0, ft, t.bdepth.as<uint16_t>(), t.flag.as<uint32_t>(), t.leafid.as<uint32_t>(), n,
                                  t.leaf_first.as<uint32_t>(), t.leaf_depth.as<uint8_t>(), t.leaf_c.as<int8_t>(),
                                  t.leaf_cnt.as<uint32_t>(), reinterpret_cast<int*>(counts + 4));
    LG_LAUNCHED();
    k_lid<<<gb, BS, 0, s>>>(t.leafid.as<uint32_t>(), t.flag.as<uint32_t>(), n);
    LG_LAUNCHED();
    k_leaf_tail<<<1, 1, 0, s>>>(t.leaf_first.as<uint32_t>(), counts + 1, n);
    LG_LAUNCHED();
    e.launches += 3;
    scan_u32(e, t, t.leaf_cnt.as<uint32_t>(), t.leaf_pre.as<uint32_t>(), n + 1, counts + 2);
    // Sizes: exact (one host read) for the first build and after a miss; otherwise the previous
    // build's with headroom, checked by tree_verify once the force call synchronises.
    size_t K, T;
    int depth;
    const bool spec = t.have_guess && (t.speculative || t.restarted);
    if (spec) {
        K = t.K;
        T = t.T;
        depth = t.max_depth;
        t.speculative = true;
    } else {
        LG_CK(cudaMemcpyAsync(e.pinned_small, counts, 32, cudaMemcpyDeviceToHost, s));
        LG_CK(cudaStreamSynchronize(s));
        const size_t Kx = e.pinned_small[1], Tx = e.pinned_small[2];
        const int dx = static_cast<int>(e.pinned_small[4]);
        if (Kx < 1 || Kx > static_cast<size_t>(n) || Tx < Kx)
            fail(kRuntime, "cuda tree build: bad leaf/node count " + std::to_string(Kx) + "/" + std::to_string(Tx));
        // Headroom for the sync-free builds that follow (LETTUCE_GB300_TREE_HEADROOM percent, default
        // 25, plus a fixed slack unless it is 0): more memory against fewer exact rebuilds.
        size_t pct = 25;
        if (const char* h = std::getenv("LETTUCE_GB300_TREE_HEADROOM")) pct = static_cast<size_t>(std::atoi(h));
        const size_t slack = pct ? 1024 : 0;
        K = std::min(static_cast<size_t>(n), Kx + Kx * pct / 100 + slack);
        T = Tx + Tx * pct / 100 + slack;
        depth = std::min(dx + (pct ? 2 : 0), MAX_DEPTH + 1);
        t.K = K;
        t.T = T;
        t.max_depth = depth;
        t.have_guess = true;
        ++t.generation;
        t.speculative = false;
    }
    t.pn_lohi.reserve(T * 8);
    t.pn_meta.reserve(T * 2);
    t.pn_nchild.reserve(T * 4);
    t.pn_cb.reserve(T * 4);
    t.pn_cpu.reserve(T * 4);
    t.gflag.reserve(T * 4);
    t.gidx.reserve(T * 4);
    t.grp_node.reserve(T * 4);
    t.grp_range.reserve(T * 8);
    t.grp_box.reserve(T * 32);
    for (DevBuf* d : {&t.nd_range, &t.nd_com, &t.nd_comlo, &t.nd_q0, &t.nd_q1, &t.nd_geo}) d->reserve(T * 16);
    t.nd_parent.reserve(T * 4);
    const uint32_t Tc = static_cast<uint32_t>(T), Kc = static_cast<uint32_t>(K);
    NodeCtx c{sys, k0, ft, t.leaf_first.as<uint32_t>(), t.leaf_depth.as<uint8_t>(), t.leaf_c.as<int8_t>(),
              t.leaf_pre.as<uint32_t>(), t.leafid.as<uint32_t>(), t.bdepth.as<uint16_t>(), n, Kdev, Kc,
              static_cast<unsigned>(sys ? t.nsys : 1)};
    const int tb = grid_for(static_cast<long long>(T), BS);
    // Index arrays start out of range (0xff..): a slot the construction fails to fill is caught by
    // the range checks below instead of being followed.
    LG_CK(cudaMemsetAsync(t.pn_cpu.as<char>(), 0xff, T * 4, s));
    LG_CK(cudaMemsetAsync(t.grp_node.as<char>(), 0xff, T * 4, s));
    LG_CK(cudaMemsetAsync(t.leaf_node.as<char>(), 0xff, K * 4, s));
    LG_CK(cudaMemsetAsync(t.nd_parent.as<char>(), 0xff, T * 4, s));
    LG_CK(cudaMemsetAsync(t.nd_range.as<char>(), 0, T * 16, s));
    LG_CK(cudaMemsetAsync(t.grp_range.as<char>(), 0, T * 8, s));
    k_nodes_pre<<<tb, BS, 0, s>>>(c, Tc, Tdev, t.pn_lohi.as<uint2>(), t.pn_meta.as<uint16_t>());
    LG_LAUNCHED();
    k_nchild<<<tb, BS, 0, s>>>(c, Tc, Tdev, t.pn_lohi.as<uint2>(), t.pn_meta.as<uint16_t>(), t.pn_nchild.as<uint32_t>());
    LG_LAUNCHED();
    e.launches += 2;
    scan_u32(e, t, t.pn_nchild.as<uint32_t>(), t.pn_cb.as<uint32_t>(), static_cast<int>(T), nullptr);
    k_gflag<<<tb, BS, 0, s>>>(t.pn_meta.as<uint16_t>(), Tc, Tdev, t.gflag.as<uint32_t>());
    LG_LAUNCHED();
    ++e.launches;
    scan_u32(e, t, t.gflag.as<uint32_t>(), t.gidx.as<uint32_t>(), static_cast<int>(T), counts + 3);
    k_cpu_index<<<tb, BS, 0, s>>>(c, Tc, Tdev, t.pn_lohi.as<uint2>(), t.pn_meta.as<uint16_t>(), t.pn_cb.as<uint32_t>(),
                                  t.pn_cpu.as<uint32_t>());
    LG_LAUNCHED();
    k_nodes_out<<<tb, BS, 0, s>>>(c, Tc, Tdev, t.pn_lohi.as<uint2>(), t.pn_meta.as<uint16_t>(),
                                  t.pn_nchild.as<uint32_t>(), t.pn_cb.as<uint32_t>(), t.pn_cpu.as<uint32_t>(),
                                  t.frame.as<double>(), t.nd_range.as<uint4>(), t.nd_geo.as<float4>(),
                                  t.nd_parent.as<uint32_t>(), t.leaf_node.as<uint32_t>(), t.gidx.as<uint32_t>(),
                                  t.grp_node.as<uint32_t>(), reinterpret_cast<int*>(counts + 4), e.err_word());
    LG_LAUNCHED();
    t.merged = e.walk_merge && !sys;
    // The group boxes do not depend on the moments: with the reference groups they are computed on
    // the side stream while the FP64 upsweep runs, and joined back before the build returns.
    cudaStream_t gs = s;
    if (!t.merged) {
        LG_CK(cudaEventRecord(e.fork_ev, s));
        LG_CK(cudaStreamWaitEvent(e.side, e.fork_ev, 0));
        gs = e.side;
    }
    k_groups<<<tb, BS, 0, gs>>>(t.grp_node.as<uint32_t>(), t.pn_lohi.as<uint2>(), Tc, Tdev, e.bodies(e.cur), counts + 3,
                                t.grp_range.as<uint2>(), t.grp_box.as<float4>());
    LG_LAUNCHED();
    if (!t.merged) LG_CK(cudaEventRecord(e.join_ev, e.side));
    e.launches += 3;
    if (t.merged) {
        t.mcount.reserve(T * 4 + 4);
        t.moff.reserve(T * 4 + 4);
        t.mrange.reserve(T * 8 + 8);
        t.mbox.reserve(T * 32 + 32);
        k_merge_groups<false><<<tb, BS, 0, s>>>(t.grp_node.as<uint32_t>(), t.pn_cpu.as<uint32_t>(),
                                                t.nd_parent.as<uint32_t>(), t.grp_range.as<uint2>(), counts + 3, Tc,
                                                Tdev, std::min(e.merge_cap, t.group_max), t.mcount.as<uint32_t>(),
                                                nullptr, nullptr);
        LG_LAUNCHED();
        scan_u32(e, t, t.mcount.as<uint32_t>(), t.moff.as<uint32_t>(), static_cast<int>(T), counts + 5);
        k_merge_groups<true><<<tb, BS, 0, s>>>(t.grp_node.as<uint32_t>(), t.pn_cpu.as<uint32_t>(),
                                               t.nd_parent.as<uint32_t>(), t.grp_range.as<uint2>(), counts + 3, Tc,
                                               Tdev, std::min(e.merge_cap, t.group_max), nullptr,
                                               t.moff.as<uint32_t>(), t.mrange.as<uint2>());
        LG_LAUNCHED();
        k_merged_boxes<<<tb, BS, 0, s>>>(t.mrange.as<uint2>(), counts + 5, Tc, e.bodies(e.cur), t.mbox.as<float4>());
        LG_LAUNCHED();
        e.launches += 3;
    }
    // Upsweep: leaves (by size), then internal nodes level by level from the deepest.
    t.ups.reserve(sizeof(UpsweepIndex));
    t.dep_nodes.reserve(T * 4);
    t.leaf_order.reserve(K * 4);
    UpsweepIndex* ix = t.ups.as<UpsweepIndex>();
    LG_CK(cudaMemsetAsync(ix, 0, sizeof(UpsweepIndex), s));
    k_upsweep_bucket<<<tb, BS, 0, s>>>(t.pn_lohi.as<uint2>(), t.pn_meta.as<uint16_t>(), t.pn_cpu.as<uint32_t>(), Tc, Tdev,
                                       ix, 0, nullptr, nullptr);
    LG_LAUNCHED();
    k_upsweep_offsets<<<1, 32, 0, s>>>(ix);
    LG_LAUNCHED();
    k_upsweep_bucket<<<tb, BS, 0, s>>>(t.pn_lohi.as<uint2>(), t.pn_meta.as<uint16_t>(), t.pn_cpu.as<uint32_t>(), Tc, Tdev,
                                       ix, 1, t.dep_nodes.as<uint32_t>(), t.leaf_order.as<uint32_t>());
    LG_LAUNCHED();
    const float inv_theta = theta > 0 ? static_cast<float>(1.0 / theta) : FLT_MAX;
    Moments mo{t.nd_com.as<float4>(), t.nd_comlo.as<float4>(), t.nd_q0.as<float4>(), t.nd_q1.as<float4>()};
    k_leaf_moments<<<grid_for(static_cast<long long>(K), 128), 128, 0, s>>>(
        t.leaf_order.as<uint32_t>(), Kc, Kdev, Tc, Tdev, t.nd_range.as<uint4>(), t.nd_geo.as<float4>(), e.bodies(e.cur),
        mo, inv_theta, t.inv_theta_sys, sys, e.err_word());
    LG_LAUNCHED();
    e.launches += 4;
    const int cb = std::max(1, std::min(2 * e.sms, grid_for(static_cast<long long>(T), COMBINE_NODES)));
    for (int d = depth - 1; d >= 0; --d) {
        k_combine_level<<<cb, COMBINE_BS, 0, s>>>(t.dep_nodes.as<uint32_t>(), ix, d, Tc, Tdev, t.nd_range.as<uint4>(),
                                           t.nd_geo.as<float4>(), mo, inv_theta, t.inv_theta_sys, sys, e.err_word());
        LG_LAUNCHED();
        ++e.launches;
    }
    if (!t.merged) LG_CK(cudaStreamWaitEvent(s, e.join_ev, 0));
}

// After a synchronising point: true if the tree built with guessed sizes is valid (no key restart
// was missed, leaves, nodes and depth within what was launched). Otherwise records the exact need
// so that the caller's rebuild takes the exact path.
bool tree_verify(Engine& e, const unsigned* counts_host) {
    TreeState& t = *e.tree;
    if (!t.speculative) return true;
    const unsigned R = counts_host[0], K = counts_host[1], T = counts_host[2];
    const int depth = static_cast<int>(counts_host[4]);
    const bool ok = (t.restarted || R == 0) && K <= t.K && T <= t.T && depth <= t.max_depth;
    if (!ok) {
        if (!t.restarted && R > 0) t.restart_mode = true;
        t.have_guess = false;  // next build reads exact sizes
    }
    return ok;
}

const unsigned* tree_counts_device(Engine& e) { return e.tree->counts.as<unsigned>(); }

namespace {
// Sets *sticky when the build just launched exceeded what it was launched for, or a key restart
// was needed: the same test as tree_verify, on the device, for step loops without host reads.
__global__ void k_tree_check(const unsigned* __restrict__ counts, unsigned K, unsigned T, int depth, int restarted,
                             unsigned* sticky) {
    const bool ok = (restarted || counts[0] == 0) && counts[1] <= K && counts[2] <= T &&
                    static_cast<int>(counts[4]) <= depth;
    if (!ok) atomicOr(sticky, 1u);
}
}  // namespace

void tree_set_forest(Engine& e, int n_tree, int nsys, const uint32_t* sys, const uint32_t* sys_off,
                     const float* inv_theta_sys) {
    TreeState& t = *e.tree;
    t.n_tree = n_tree;
    t.nsys = nsys;
    t.sys = sys;
    t.sys_off = sys_off;
    t.inv_theta_sys = inv_theta_sys;
    t.have_guess = false;
    t.restart_mode = false;
}

bool tree_sync_free_ready(const Engine& e) { return e.tree->have_guess && !e.tree->restart_mode; }
uint64_t tree_generation(const Engine& e) { return e.tree->generation; }

void tree_check_async(Engine& e, unsigned* sticky) {
    TreeState& t = *e.tree;
    if (!t.speculative) return;
    k_tree_check<<<1, 1, 0, e.stream>>>(t.counts.as<unsigned>(), static_cast<unsigned>(t.K),
                                        static_cast<unsigned>(t.T), t.max_depth, t.restarted ? 1 : 0, sticky);
    LG_LAUNCHED();
    ++e.launches;
}
void tree_reset_guess(Engine& e) {
    e.tree->have_guess = false;
    e.tree->restart_mode = false;
}
double tree_theta(const Engine& e) { return e.tree->theta; }

TreeView tree_view(Engine& e) {
    TreeState& t = *e.tree;
    TreeView v;
    v.nd_range = t.nd_range.as<uint4>();
    v.nd_com = t.nd_com.as<float4>();
    v.nd_comlo = t.nd_comlo.as<float4>();
    v.nd_q0 = t.nd_q0.as<float4>();
    v.nd_q1 = t.nd_q1.as<float4>();
    v.grp_range = t.merged ? t.mrange.as<uint2>() : t.grp_range.as<uint2>();
    v.grp_box = t.merged ? t.mbox.as<float4>() : t.grp_box.as<float4>();
    v.ngroups = t.counts.as<unsigned>() + (t.merged ? 5 : 3);
    v.T = t.T;  // capacity the build was launched with (>= the node count)
    v.nd_parent = t.nd_parent.as<uint32_t>();
    v.body_leaf = t.leafid.as<uint32_t>();
    v.leaf_node = t.leaf_node.as<uint32_t>();
    v.nleaves = t.counts.as<unsigned>() + 1;
    v.K = t.K;
    return v;
}

void tree_counts(Engine& e, size_t* nodes, size_t* leaves, size_t* groups, int* max_depth) {
    TreeState& t = *e.tree;
    if (!e.tree_ok) fail(kLogic, "tree introspection: call build_tree (tree method) first");
    e.ensure_tree_valid();
    LG_CK(cudaMemcpyAsync(e.pinned_small, t.counts.as<unsigned>(), 32, cudaMemcpyDeviceToHost, e.stream));
    LG_CK(cudaStreamSynchronize(e.stream));
    if (nodes) *nodes = e.pinned_small[2];
    if (leaves) *leaves = e.pinned_small[1];
    if (groups) *groups = e.pinned_small[t.merged ? 5 : 3];
    if (max_depth) *max_depth = static_cast<int>(e.pinned_small[4]);
}

// The reference's key array after a build (src/cpu_backend.cpp:884-906 key_): each body's key in
// the last frame it was re-keyed in (rekey overwrites key_ inside a run; a coincident run keeps
// the keys it had).
void tree_keys(Engine& e, uint64_t* keys, size_t n) {
    TreeState& t = *e.tree;
    if (!e.tree_ok) fail(kLogic, "tree introspection: call build_tree (tree method) first");
    e.ensure_tree_valid();
    if (n < static_cast<size_t>(e.n)) fail(kArg, "tree_keys: output holds fewer than n keys");
    const size_t N = static_cast<size_t>(e.n);
    LG_CK(cudaMemcpyAsync(keys, t.skey.as<uint64_t>(), N * 8, cudaMemcpyDeviceToHost, e.stream));
    if (t.restarted) {
        std::vector<uint8_t> nfr(N);
        std::vector<std::vector<uint64_t>> fk(t.nframes);
        LG_CK(cudaMemcpyAsync(nfr.data(), t.nfr.as<uint8_t>(), N, cudaMemcpyDeviceToHost, e.stream));
        for (int f = 1; f < t.nframes; ++f) {
            fk[f].resize(N);
            LG_CK(cudaMemcpyAsync(fk[f].data(), t.fkey[f].as<uint64_t>(), N * 8, cudaMemcpyDeviceToHost, e.stream));
        }
        LG_CK(cudaStreamSynchronize(e.stream));
        for (size_t i = 0; i < N; ++i)
            if (nfr[i] > 1) keys[i] = fk[nfr[i] - 1][i];
    }
    LG_CK(cudaStreamSynchronize(e.stream));
}

void tree_nodes(Engine& e, uint32_t* range4, float* moments11, float* geo4, size_t nodes) {
    TreeState& t = *e.tree;
    if (!e.tree_ok) fail(kLogic, "tree introspection: call build_tree (tree method) first");
    size_t T = 0;
    tree_counts(e, &T, nullptr, nullptr, nullptr);
    if (nodes < T) fail(kArg, "tree_nodes: output holds fewer than the node count");
    if (range4) LG_CK(cudaMemcpyAsync(range4, t.nd_range.as<uint4>(), T * 16, cudaMemcpyDeviceToHost, e.stream));
    if (geo4) LG_CK(cudaMemcpyAsync(geo4, t.nd_geo.as<float4>(), T * 16, cudaMemcpyDeviceToHost, e.stream));
    if (moments11) {
        std::vector<float4> com(T), q0(T), q1(T);
        LG_CK(cudaMemcpyAsync(com.data(), t.nd_com.as<float4>(), T * 16, cudaMemcpyDeviceToHost, e.stream));
        LG_CK(cudaMemcpyAsync(q0.data(), t.nd_q0.as<float4>(), T * 16, cudaMemcpyDeviceToHost, e.stream));
        LG_CK(cudaMemcpyAsync(q1.data(), t.nd_q1.as<float4>(), T * 16, cudaMemcpyDeviceToHost, e.stream));
        LG_CK(cudaStreamSynchronize(e.stream));
        for (size_t k = 0; k < T; ++k) {
            float* o = moments11 + 11 * k;
            o[0] = com[k].x; o[1] = com[k].y; o[2] = com[k].z; o[3] = com[k].w;
            o[4] = q0[k].x; o[5] = q0[k].y; o[6] = q0[k].z; o[7] = q0[k].w;
            o[8] = q1[k].x; o[9] = q1[k].y; o[10] = q1[k].z;
        }
    }
    LG_CK(cudaStreamSynchronize(e.stream));
}

void tree_groups(Engine& e, float* box6, uint32_t* lohi, size_t groups) {
    TreeState& t = *e.tree;
    if (!e.tree_ok) fail(kLogic, "tree introspection: call build_tree (tree method) first");
    size_t G = 0;
    tree_counts(e, nullptr, nullptr, &G, nullptr);
    if (groups < G) fail(kArg, "tree_groups: output holds fewer than the group count");
    // The walk's groups (merged ones when the engine packs them).
    const uint2* range = t.merged ? t.mrange.as<uint2>() : t.grp_range.as<uint2>();
    const float4* gbox = t.merged ? t.mbox.as<float4>() : t.grp_box.as<float4>();
    if (lohi) LG_CK(cudaMemcpyAsync(lohi, range, G * 8, cudaMemcpyDeviceToHost, e.stream));
    if (box6) {
        std::vector<float4> box(2 * G);
        LG_CK(cudaMemcpyAsync(box.data(), gbox, G * 32, cudaMemcpyDeviceToHost, e.stream));
        LG_CK(cudaStreamSynchronize(e.stream));
        for (size_t g = 0; g < G; ++g) {
            box6[6 * g] = box[2 * g].x; box6[6 * g + 1] = box[2 * g].y; box6[6 * g + 2] = box[2 * g].z;
            box6[6 * g + 3] = box[2 * g + 1].x; box6[6 * g + 4] = box[2 * g + 1].y; box6[6 * g + 5] = box[2 * g + 1].z;
        }
    }
    LG_CK(cudaStreamSynchronize(e.stream));
}

lg_memory_estimate memory_need(uint64_t n, int method) {
    lg_memory_estimate r{};
    // Two body sets (80 B), accelerations (16 B), staging (12 B), plus fixed buffers.
    r.device = 192 * n + (uint64_t(64) << 20);
    if (method == LG_TREE) r.device += 112 * n;  // keys, sort buffers, per-body tree data, ~0.2 n nodes
    r.host = 0;
    return r;
}

size_t tree_held_bytes(const Engine& e) {
    const TreeState& t = *e.tree;
    size_t h = 0;
    for (const DevBuf* d : {&t.keysA, &t.keysB, &t.valsA, &t.valsB, &t.hist, &t.lookback, &t.ctl, &t.skey, &t.key1tmp,
                            &t.nfr, &t.ftab, &t.bdepth, &t.flag, &t.leafid, &t.frame, &t.runs, &t.counts,
                            &t.leaf_first, &t.leaf_depth, &t.leaf_c, &t.leaf_pre, &t.leaf_node, &t.pn_lohi,
                            &t.pn_meta, &t.pn_nchild, &t.pn_cb, &t.pn_cpu, &t.nd_range, &t.nd_com, &t.nd_comlo,
                            &t.nd_q0, &t.nd_q1, &t.nd_geo, &t.nd_parent, &t.gflag, &t.gidx, &t.grp_node, &t.leaf_cnt, &t.ups, &t.dep_nodes, &t.leaf_order,
                            &t.grp_range, &t.grp_box, &t.scan_state, &t.scan_ctr})
        h += d->capacity();
    for (int f = 1; f < FRAMES; ++f) h += t.fkey[f].capacity() + t.frunid[f].capacity() + t.fcube[f].capacity();
    return h;
}

}  // namespace lg
