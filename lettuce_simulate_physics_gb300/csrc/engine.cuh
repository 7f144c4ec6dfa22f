// The engine object behind the C ABI, and the tree stages it calls.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <memory>
#include <string>

#include "../../include/lettuce_gb300.h"
#include "lg_engine.cuh"

namespace lg {

// NVTX range around the host-side enqueue of one phase (sort, build, walk, direct, kick, drift),
// for timeline profilers; a no-op unless a profiler injects itself (nvtx3 is header-only).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

struct TreeState;     // tree.cu
struct AdjointState;  // adjoint.cu
struct LetStore;      // let.cu

// Read-only view of the built tree for the walk.
struct TreeView {
    const uint4* nd_range;    // (lo, hi, first, nchild), reference node order
    const float4* nd_com;     // (cx, cy, cz, m)
    const float4* nd_comlo;   // low parts of the FP64 centre of mass
    const float4* nd_q0;      // (qxx, qxy, qxz, qyy)
    const float4* nd_q1;      // (qyz, qzz, rcrit2, 0)
    const uint2* grp_range;   // walk groups (lo, hi), reference order
    const float4* grp_box;    // 2 per group: (bx, by, bz, 0), (hx, hy, hz, 0)
    const unsigned* ngroups;  // device-side group count
    size_t T;
    // For the walk's vector-Jacobian product: parent of every node (root: 0xffffffff), leaf of
    // every body, node of every leaf.
    const uint32_t* nd_parent;
    const uint32_t* body_leaf;
    const uint32_t* leaf_node;
    const unsigned* nleaves;  // device-side leaf count
    size_t K;
};

// Remote (locally-essential) trees on the device, back to back: per node the centre of mass and
// mass, the quadrupole (xx, xy, xz, yy) and (yz, zz, rcrit2, 0), and (first_child, child_count,
// body_first, body_count) as indices into these arrays; bodies as (x, y, z, m); the roots of the
// ntrees non-empty trees.
struct LetView {
    const float4* com = nullptr;
    const float4* q0 = nullptr;
    const float4* q1 = nullptr;
    const int4* link = nullptr;
    const float4* body = nullptr;
    const uint32_t* roots = nullptr;
    uint32_t nnodes = 0;
    int ntrees = 0;
};

struct BodySet {
    DevBuf x, y, z, hm, lo, vx, vy, vz, m, cost, id, level;
};

struct Engine {
    explicit Engine(int device);
    ~Engine();

    // Backend semantics (src/backend.hpp:89-141).
    void upload(size_t count, const float* x, const float* y, const float* z, const float* vx, const float* vy,
                const float* vz, const float* m, const uint32_t* id);
    void upload64(size_t count, const double* x, const double* y, const double* z, const float* vx, const float* vy,
                  const float* vz, const float* m, const uint32_t* id);
    void download(float* x, float* y, float* z, float* vx, float* vy, float* vz, float* m, uint32_t* id);
    void build_tree(const lg_force_params& p);
    void compute_forces_with(const lg_force_params& p, bool potential, const lg_let_tree* remote, size_t nremote);
    void kick(double dt);
    void drift(double dt);
    lg_diag diagnostics();
    double exact_potential_energy(double G, double eps);
    lg_phase_times get_times();
    void local_bounds(float lo[3], float hi[3]);
    bool body_costs(float* cost, size_t count);
    void read_accel(float* ax, float* ay, float* az, float* pot);
    void read_pos64(double* x, double* y, double* z);
    void flush_l2();
    // Block (hierarchical) time steps, block.cu.
    void block_step(const lg_force_params& p, double dt, int max_level, double eta, int steps);
    size_t held_bytes() const;

    BodyArrays bodies(int which) const;
    void reserve_bodies(size_t count);
    unsigned* err_word() const;
    unsigned* ticket() const;
    unsigned long long* inter_counter() const;
    double* dscratch() const;
    float elapsed(int a, int b) const;
    void check_device_errors(const char* where);
    void ensure_tree_valid();  // rebuilds exactly if a sync-free build guessed wrong

    // Device, stream, events.
    int dev = 0;
    int sms = 0;
    int l2_bytes = 0;
    std::string name;
    cudaStream_t stream = nullptr;
    // Side stream for build work that overlaps the moment upsweep (group boxes), forked from and
    // joined back into `stream` with the two events.
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    enum { EV_BUILD0, EV_SORTED, EV_BUILT, EV_WALK0, EV_WALK1, EV_KICK0, EV_KICK1, EV_DRIFT0, EV_DRIFT1, EV_COUNT };
    cudaEvent_t events[EV_COUNT] = {};
    static constexpr int kUserEvents = 16;
    cudaEvent_t user_events[kUserEvents] = {};

    // Walk settings (LETTUCE_CUDA_WALK / LETTUCE_CUDA_GROUP).
    bool walk_body = false;
    int group_max = 128;
    // Walk groups: the reference's groups (default: interaction lists and counts equal to the
    // reference CPU backend's), or with LETTUCE_GB300_WALK_GROUPS=merged consecutive sibling groups
    // packed into groups of up to LETTUCE_GB300_WALK_MERGE_CAP bodies (fewer, fuller groups; faster
    // on some distributions, slower on others).
    bool walk_merge = false;
    int merge_cap = 128;
    DirectShape direct_shape_override{0, 0, 0};
    // Block time steps: the walk skips passes whose bodies all have levels below walk_kmin (< 0: off).
    int walk_kmin = -1;
    bool block_ready = false;

    // State.
    int n = 0;
    int cur = 0;  // which BodySet holds the current bodies
    BodySet set[2];
    DevBuf acc;          // float4 per body
    DevBuf staging;      // 3 floats per body for upload/download
    DevBuf partial;      // split-j partial sums (scratch)
    DevBuf diag_partial; // per-block FP64 partials
    DevBuf flush_buf;
    DevBuf walk_stack;   // per-warp traversal stacks of the tree walk
    DevBuf vjp_scratch;  // per-node adjoints of the tree walk's vector-Jacobian product
    DevBuf small;        // error word, tickets, counters, FP64 results
    unsigned* pinned_small = nullptr;
    bool has_pe = false, acc_ok = true, tree_ok = false, costs_ok = false;
    bool kick_rec = false, drift_rec = false, pend_tree_times = false;
    lg_phase_times times{};
    uint64_t launches = 0;
    uint64_t last_body_pairs = 0, last_cell_terms = 0;
    std::unique_ptr<TreeState, void (*)(TreeState*)> tree{nullptr, nullptr};
    std::unique_ptr<AdjointState, void (*)(AdjointState*)> adjoint{nullptr, nullptr};
    std::unique_ptr<LetStore, void (*)(LetStore*)> lets{nullptr, nullptr};
};

extern thread_local std::string g_last_error;

// tree.cu
std::unique_ptr<TreeState, void (*)(TreeState*)> make_tree_state();
void tree_sort(Engine& e);                    // keys, radix sort, permute (+ key restarts)
void tree_build(Engine& e, double theta);     // octree, groups, moments
size_t tree_held_bytes(const Engine& e);
TreeView tree_view(Engine& e);
bool tree_verify(Engine& e, const unsigned* counts_host);
const unsigned* tree_counts_device(Engine& e);
void tree_reset_guess(Engine& e);
double tree_theta(const Engine& e);
// Forest mode (ensembles): the tree covers bodies [0, n_tree) of nsys systems; sys (per body),
// sys_off (nsys + 1 body offsets) and inv_theta_sys (per system) are device arrays the caller
// keeps alive. n_tree < 0 restores the single-system tree.
void tree_set_forest(Engine& e, int n_tree, int nsys, const uint32_t* sys, const uint32_t* sys_off,
                     const float* inv_theta_sys);
// True when the next build takes no host read (sizes guessed from the previous build).
bool tree_sync_free_ready(const Engine& e);
// Changes whenever a build may have reallocated tree buffers (captured graphs must be redone).
uint64_t tree_generation(const Engine& e);
// Device-side form of tree_verify for a sync-free build: ORs 1 into *sticky on a miss.
void tree_check_async(Engine& e, unsigned* sticky);
void tree_counts(Engine& e, size_t* nodes, size_t* leaves, size_t* groups, int* max_depth);
void tree_keys(Engine& e, uint64_t* keys, size_t n);
void tree_nodes(Engine& e, uint32_t* lohi_first_nchild, float* moments11, float* geo4, size_t nodes);
void tree_groups(Engine& e, float* box6, uint32_t* lohi, size_t groups);
lg_memory_estimate memory_need(uint64_t n, int method);
const void* probe_kernel();
// walk.cu
// sys/e2_sys: forest walk (per-body system, per-system squared softening); nullptr for one tree.
// let: remote trees walked after the local one (nullptr: none).
void tree_walk(Engine& e, float G, float e2, bool potential, bool eps0, const uint32_t* sys = nullptr,
               const float* e2_sys = nullptr, const LetView* let = nullptr);
// Remote trees only, for groups given by `blocks` (grp_range, grp_box, ngroups); adds to acc and
// cost (the direct method's remote part).
void tree_walk_remote_blocks(Engine& e, float G, float e2, bool potential, bool eps0, const LetView& let,
                             const TreeView& blocks);
// let.cu: remote trees to the device; blocks of consecutive bodies with their boxes; export.
std::unique_ptr<LetStore, void (*)(LetStore*)> make_let_store();
LetView let_upload(Engine& e, const lg_let_tree* remote, size_t nremote);
TreeView let_body_blocks(Engine& e, int block);
void let_export(Engine& e, const float lo[3], const float hi[3], const lg_force_params& p, size_t* nnodes,
                size_t* nbodies);
void let_export_read(Engine& e, lg_let_node* nodes, float* bx, float* by, float* bz, float* bm);
// walk_vjp.cu: vector-Jacobian product of the tree forces over the current tree's interaction
// lists (the lists are those of the force walk on the same tree), with the cell moments
// differentiated through the bodies: g (4 arrays of n doubles: x, y, z, m; current body order)
// accumulates d(sum_i w_i . a_i / G)/d(x, m). w: float4 weights per body (current order).
void tree_walk_vjp(Engine& e, const float4* w, float e2, bool eps0, double* g);
// walk_vjp.cu: vector-Jacobian product of the tree forces over the current tree's interaction
// lists (the lists are those of the force walk on the same tree), with the cell moments
// differentiated through the bodies: g (4 arrays of n doubles: x, y, z, m; current body order)
// accumulates d(sum_i w_i . a_i / G)/d(x, m). w: float4 weights per body (current order).
void tree_walk_vjp(Engine& e, const float4* w, float e2, bool eps0, double* g);
// adjoint.cu
std::unique_ptr<AdjointState, void (*)(AdjointState*)> make_adjoint_state();
void adjoint_forward(Engine& e, AdjointState& a, const lg_force_params& p, double dt, int steps, int every);
// tx, ty, tz: the target x* (loss sum m |x_T - x*|^2), or with seeded the caller's dL/dx_T (by id).
double adjoint_backward(Engine& e, AdjointState& a, const double* tx, const double* ty, const double* tz, double* gx,
                        double* gy, double* gz, double* gvx, double* gvy, double* gvz, double* gm, bool seeded);
// render.cu
void render(Engine& e, const lg_render_options& o, unsigned char* rgb, double* extent_used);
// integrate.cu
double probe_fp32_peak(cudaStream_t s, int sms, unsigned* sink);
void probe_waits(cudaStream_t s, unsigned polls, const unsigned* never_set, unsigned* err);

}  // namespace lg
