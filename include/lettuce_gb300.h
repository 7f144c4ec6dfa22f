/* lettuce_gb300.h -- C ABI of the GB300 force-and-integrate engine for lettuce.
 *
 * The engine is a drop-in for the reference's CUDA backend (NotMaxwell/lettuce_simulate_physics,
 * src/cuda_backend.cu) behind the reference's C++ interface `class Backend` (src/backend.hpp:89-141).
 * Every entry point below names the Backend member or factory it replaces. The C++ adapter that
 * implements `Backend` over this ABI is lettuce_simulate_physics_gb300/integration/gb300_backend.cpp.
 *
 * Conventions
 *  - Every call returns an lg_status; on failure lg_last_error() holds a message for this thread.
 *    LG_ERR_RUNTIME is the reference's std::runtime_error, LG_ERR_LOGIC its std::logic_error
 *    (a call made in the wrong state, e.g. kick after build_tree without a force call).
 *  - Pointers are host pointers to plain arrays; sizes are element counts.
 *  - One engine = one device, one non-blocking stream (plus an internal second stream, forked from
 *    and joined back into it, for work that overlaps inside one call: the group boxes of a tree
 *    build, the adjoint's VJP sweep). kick and drift are asynchronous; times, diagnostics,
 *    download, body_costs and the force calls synchronise, as in the reference.
 *  - Bodies cross the boundary as float32 (the reference's Bodies, src/bodies.hpp:7-10); inside,
 *    positions are FP64 and the drift is FP64. download() rounds positions to float.
 */
#ifndef LETTUCE_GB300_H
#define LETTUCE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    LG_OK = 0,
    LG_ERR_RUNTIME = 1,     /* std::runtime_error in the reference */
    LG_ERR_LOGIC = 2,       /* std::logic_error in the reference */
    LG_ERR_ARG = 3,         /* invalid argument (null pointer, size mismatch) */
    LG_ERR_UNAVAILABLE = 4  /* no usable device or no kernel image (make_cuda_backend -> nullptr) */
} lg_status;

enum { LG_DIRECT = 0, LG_TREE = 1 }; /* ForceMethod, src/backend.hpp:12 */

typedef struct lg_engine lg_engine;

/* ForceParams, src/backend.hpp:14-19. */
typedef struct {
    double G;
    double eps;   /* Plummer softening: a = G m d / (|d|^2 + eps^2)^(3/2) */
    double theta; /* tree opening angle */
    int32_t method;
    int32_t reserved;
} lg_force_params;

/* Diag, src/backend.hpp:31-39. */
typedef struct {
    double mass, ke, pe;
    int32_t has_pe, reserved;
    double px, py, pz;
    double lx, ly, lz;
    double cx, cy, cz;
} lg_diag;

/* PhaseTimes, src/backend.hpp:41-50 (milliseconds, measured with CUDA events). */
typedef struct {
    double force_ms, sort_ms, build_ms, walk_ms, step_ms;
    uint64_t interactions;
    double comm_ms, balance_ms;
} lg_phase_times;

/* MemoryNeed, src/backend.hpp:24-27. */
typedef struct {
    uint64_t device, host;
} lg_memory_estimate;

/* Message of the last failed call on this thread ("" if none). */
const char* lg_last_error(void);

/* cuda_compiled(), src/backend.hpp:146: 1 (this library is the CUDA build). */
int lg_compiled(void);
/* cuda_device_count(), src/backend.hpp:148: visible devices, 0 without a driver. */
int lg_device_count(void);

/* make_cuda_backend(device, why), src/backend.hpp:145 and src/cuda_backend.cu:2026-2048.
 * LG_ERR_UNAVAILABLE (message = why) when the device is missing or has no sm_103a image. Reads
 * LETTUCE_CUDA_WALK=group|body and LETTUCE_CUDA_GROUP=<max bodies per walk group> (default 128, the
 * reference CPU backend's group rule, src/cpu_backend.cpp:27), as the reference reads its walk
 * settings at construction (src/cuda_backend.cu:1239-1254). */
lg_status lg_create(int device, lg_engine** out);
/* ~Backend(). */
void lg_destroy(lg_engine* e);

/* Backend::name(), src/backend.hpp:93: "cuda: <device> (sm_XY, N SMs, M GB), <walk>". */
lg_status lg_name(const lg_engine* e, char* buf, size_t cap);

/* Backend::upload(const Bodies&), src/backend.hpp:95. Accelerations are zeroed. */
lg_status lg_upload(lg_engine* e, size_t n, const float* x, const float* y, const float* z, const float* vx,
                    const float* vy, const float* vz, const float* m, const uint32_t* id);
/* Number of resident bodies (Bodies::size() of the next download). */
lg_status lg_size(const lg_engine* e, size_t* n);
/* Backend::download(Bodies&), src/backend.hpp:97: current (possibly sorted) order, ids identify. */
lg_status lg_download(lg_engine* e, float* x, float* y, float* z, float* vx, float* vy, float* vz, float* m,
                      uint32_t* id);

/* Backend::compute_forces(p, potential), src/backend.hpp:102. */
lg_status lg_compute_forces(lg_engine* e, const lg_force_params* p, int potential);
/* Backend::kick(dt), src/backend.hpp:103: v += a dt. LG_ERR_LOGIC if the accelerations are stale. */
lg_status lg_kick(lg_engine* e, double dt);
/* Backend::drift(dt), src/backend.hpp:104: x += v dt, in FP64. */
lg_status lg_drift(lg_engine* e, double dt);
/* Backend::diagnostics(), src/backend.hpp:106: FP64 reductions over the FP64 state. */
lg_status lg_diagnostics(lg_engine* e, lg_diag* out);
/* Backend::exact_potential_energy(G, eps), src/backend.hpp:108: O(N^2) FP64 pair sum. */
lg_status lg_exact_potential_energy(lg_engine* e, double G, double eps, double* out);
/* Backend::times(), src/backend.hpp:110. */
lg_status lg_times(lg_engine* e, lg_phase_times* out);

/* Backend::local_bounds(), src/backend.hpp:115: lo[3], hi[3] of the current positions. */
lg_status lg_local_bounds(lg_engine* e, float lo[3], float hi[3]);
/* Backend::build_tree(p), src/backend.hpp:118: sort and build for the current positions;
 * invalidates accelerations, potential and costs; no-op for the direct method. */
lg_status lg_build_tree(lg_engine* e, const lg_force_params* p);
/* LetNode, src/backend.hpp:62-75: the same 60-byte layout, so a LetTree's node array can be passed
 * as is. Receiver rule (src/backend.hpp:77-82): a node with no children and no bodies, or with
 * |box distance|^2 >= rcrit2, is a multipole; otherwise its bodies, or else its children. */
typedef struct {
    float cx, cy, cz;
    float mass;
    float qxx, qxy, qxz, qyy, qyz, qzz;
    float rcrit2;
    int32_t first_child, child_count;
    int32_t body_first, body_count;
} lg_let_node;

/* LetTree, src/backend.hpp:83-86: nodes (root first) and its bodies. */
typedef struct {
    const lg_let_node* nodes;
    size_t nnodes;
    const float *bx, *by, *bz, *bm;
    size_t nbodies;
} lg_let_tree;

/* Backend::compute_forces_with(p, potential, remote), src/backend.hpp:128-129: forces from the
 * resident bodies' own tree (or direct sum) plus the `nremote` locally-essential trees of other
 * ranks, walked on the device with the receiver rule (tree method: per walk group; direct method:
 * per block of 128 consecutive bodies, as src/cpu_backend.cpp:695-717). LG_ERR_LOGIC for the tree
 * method without a current tree. */
lg_status lg_compute_forces_with(lg_engine* e, const lg_force_params* p, int potential, const lg_let_tree* remote,
                                 size_t nremote);
/* Backend::export_let(target, p), src/backend.hpp:120-124: the part of this engine's tree that any
 * target inside the box lo..hi could open, built on the device in the reference's breadth-first
 * order (src/cpu_backend.cpp:222-270); the direct method exports one always-open root holding every
 * body. lg_export_let builds it and returns its sizes; lg_export_let_read copies it out (arrays of
 * the sizes returned). LG_ERR_LOGIC for the tree method without a current tree. */
lg_status lg_export_let(lg_engine* e, const float lo[3], const float hi[3], const lg_force_params* p, size_t* nnodes,
                        size_t* nbodies);
lg_status lg_export_let_read(lg_engine* e, lg_let_node* nodes, float* bx, float* by, float* bz, float* bm);
/* Backend::memory_need(n, method), src/backend.hpp:131. */
lg_status lg_memory_need(uint64_t n, int method, lg_memory_estimate* out);
/* Backend::device_memory(free, total), src/backend.hpp:134-137; free includes what the engine holds. */
lg_status lg_device_memory(lg_engine* e, uint64_t* free_bytes, uint64_t* total_bytes);
/* Backend::body_costs(cost), src/backend.hpp:141: interactions per body of the last force call, in
 * download order (sum == interactions). *valid = 0 when there is none (the reference returns false). */
lg_status lg_body_costs(lg_engine* e, float* cost, size_t n, int* valid);

/* ---- Extensions: no counterpart in the reference interface ------------------------------------ */

/* RenderOptions, src/render.hpp:15-21: view "xy" | "xz" | "yz" | "<yaw_deg>,<pitch_deg>";
 * extent = half-width in world units (0: 1.2 x the 99th-percentile radius about the centre of
 * mass); color 0 = density, 1 = speed. */
typedef struct {
    int32_t width, height;
    const char* view;
    double extent;
    int32_t color;
    int32_t reserved;
} lg_render_options;

/* render_image(bodies, options), src/render.hpp:28-33 (src/render.cpp:83-224), on the device from
 * the resident bodies: mass splatted bilinearly into a float image (integer sums: independent of
 * atomic order), log tone map, the reference's colour ramps. rgb: width * height * 3 bytes, row 0
 * at the top; *extent_used = the half-width used. No graphics API is involved: the image is a
 * plain device buffer copied to rgb. */
lg_status lg_render(lg_engine* e, const lg_render_options* o, unsigned char* rgb, double* extent_used);

/* Block (hierarchical) time steps (no reference counterpart; the reference lists them as not done
 * yet, docs/design.md:70-71). `steps` steps of size dt, each made of 2^max_level substeps: a body
 * on level k advances with dt / 2^k in kick-drift-kick form (opening half kick where its step
 * starts, every body drifts each substep in FP64, forces and the closing half kick where its step
 * ends; tree walks skip the groups with no body ending a step). Levels: dt_i = eta sqrt(eps / |a_i|),
 * k_i = the smallest k with dt / 2^k <= dt_i, clamped to [0, max_level] and, when changed, to the
 * levels whose step starts at that time. The first call after an upload evaluates every force and
 * level. lg_block_levels reads the levels in download order. */
lg_status lg_block_step(lg_engine* e, const lg_force_params* p, double dt, int max_level, double eta, int steps);
lg_status lg_block_levels(lg_engine* e, uint8_t* levels, size_t n);

/* FP64-preserving restart (no reference counterpart). lg_upload64 is lg_upload with FP64 positions.
 * A float snapshot (the reference's .snap, src/snapshot.hpp:1-27) loses the FP64 state; the sidecar
 * written next to it by lg_write_fp64_sidecar holds, in download order, the ids and the low parts
 * x - (double)(float)x (exact in FP64). lg_read_fp64_sidecar checks n and the ids against the
 * snapshot's bodies and rebuilds the FP64 positions bit for bit (host only, no engine). */
lg_status lg_upload64(lg_engine* e, size_t n, const double* x, const double* y, const double* z, const float* vx,
                      const float* vy, const float* vz, const float* m, const uint32_t* id);
lg_status lg_write_fp64_sidecar(lg_engine* e, const char* path, uint64_t step);
lg_status lg_read_fp64_sidecar(const char* path, size_t n, const uint32_t* id, const float* x, const float* y,
                               const float* z, double* x64, double* y64, double* z64, uint64_t* step);

/* Accelerations and potential in the current body order (the reference tests read them through
 * kick(1) on zero velocities; this reads them directly). pot may be NULL. */
lg_status lg_read_accel(lg_engine* e, float* ax, float* ay, float* az, float* pot);
/* FP64 positions in the current body order. */
lg_status lg_read_pos64(lg_engine* e, double* x, double* y, double* z);

/* Tree introspection after build_tree: the sorted Morton keys (frame-0 keys), and the octree in
 * the reference CPU backend's node order and layout (src/cpu_backend.cpp:35-43): per node
 * lo, hi, first, nchild; moments cx, cy, cz, m, qxx, qxy, qxz, qyy, qyz, qzz, rcrit2 as floats;
 * geometric centre and half side. Any output pointer may be NULL. */
lg_status lg_tree_counts(lg_engine* e, size_t* nodes, size_t* leaves, size_t* groups, int* max_depth);
lg_status lg_tree_keys(lg_engine* e, uint64_t* keys, size_t n);
lg_status lg_tree_nodes(lg_engine* e, uint32_t* lohi_first_nchild, float* moments11, float* geo4, size_t nodes);
/* Walk groups in the reference's order: box centre and half (float 6) and body range (u32 2). */
lg_status lg_tree_groups(lg_engine* e, float* box6, uint32_t* lohi, size_t groups);

/* Timing helpers on the engine's stream (CUDA events; slot 0..15). */
lg_status lg_event_record(lg_engine* e, int slot);
lg_status lg_event_elapsed(lg_engine* e, int slot_a, int slot_b, float* ms);
lg_status lg_synchronize(lg_engine* e);
/* Writes a device buffer larger than L2 on the engine's stream (cache flush between timed steps). */
lg_status lg_flush_l2(lg_engine* e);
/* Number of engine kernel launches issued so far (a counter kept by the host side). */
lg_status lg_launch_count(const lg_engine* e, uint64_t* count);
/* Split of the last force call's interactions: body-body pairs and body-cell (quadrupole) terms;
 * body_pairs + cell_terms == interactions. For the direct method cell_terms = 0. */
lg_status lg_interaction_split(lg_engine* e, uint64_t* body_pairs, uint64_t* cell_terms);
/* Measured FP32 FMA throughput of this device (a dependent-free FFMA loop over every SM, timed
 * with CUDA events on the engine's stream), in TFLOP/s: the roofline denominator of the force
 * kernels. */
lg_status lg_probe_fp32_peak(lg_engine* e, double* tflops);
/* Self-test of failure detection (no reference counterpart): one block waits on an mbarrier no one
 * arrives on and on a flag no one sets, `polls` polls each (1 .. 2^20), with the bounded-wait
 * primitives the kernels use. Both waits give up; the call returns LG_ERR_RUNTIME with "device wait
 * timed out" in lg_last_error(), the error word is cleared and the engine stays usable. */
lg_status lg_probe_wait_timeout(lg_engine* e, unsigned polls);
/* Page-locked host memory for transfers that overlap (cudaMallocHost / cudaFreeHost). */
lg_status lg_host_alloc(size_t bytes, void** out);
lg_status lg_host_free(void* p);

/* ---- Adjoint of the leapfrog (no counterpart in the reference) -------------------------------
 * Reverse-mode derivative of the loss L = sum_i m_i |x_i(T) - x*_i|^2 after `steps` KDK steps of
 * size dt from the resident state, with direct-summation or tree forces (p->method).
 * lg_adjoint_forward runs the steps (the final state stays resident, as after ordinary steps) and
 * keeps FP64-position / FP32-velocity checkpoints every `checkpoint_every` steps.
 * lg_adjoint_backward takes x* (FP64, indexed by body id; ids must be 0..n-1) and returns L and
 * dL/dx0, dL/dv0, dL/dm (FP64, indexed by id); it recomputes each segment from its checkpoint and
 * applies one vector-Jacobian product per step: pairwise for direct forces; for tree forces over
 * the step's interaction lists, held fixed ("frozen": the segment replay rebuilds the same tree
 * from bit-identical positions), with the cell moments differentiated through the bodies.
 * Afterwards the resident state is no longer the final state (upload again to continue). */
lg_status lg_adjoint_forward(lg_engine* e, const lg_force_params* p, double dt, int steps, int checkpoint_every);
lg_status lg_adjoint_backward(lg_engine* e, const double* target_x, const double* target_y, const double* target_z,
                              double* loss, double* gx, double* gy, double* gz, double* gvx, double* gvy, double* gvz,
                              double* gm);
/* Backward pass for any loss of the final positions: the caller passes dL/dx(T) (FP64, by body id;
 * computed from the final state the forward pass left resident) and receives dL/dx0, dL/dv0 and
 * the part of dL/dm that flows through the dynamics (an explicit dependence of L on the masses is
 * the caller's to add). Losses that depend on the final velocities are not covered. */
lg_status lg_adjoint_backward_seeded(lg_engine* e, const double* dldx, const double* dldy, const double* dldz,
                                     double* gx, double* gy, double* gz, double* gvx, double* gvy, double* gvz,
                                     double* gm);

/* ---- Batched ensembles (no reference counterpart) ----------------------------------------------
 * Many independent systems of uneven N advanced together: every force phase is one launch pipeline
 * over all systems (a batched direct-sum launch per i-bodies-per-thread class, one forest tree for
 * the tree systems: one sort, one build, one walk), and a run of steps can be captured as one CUDA
 * graph. Each system has its own softening, opening angle and method; G and dt are shared. */
typedef struct lg_ensemble lg_ensemble;

typedef struct {
    double run_ms;          /* device time of the last lg_ensemble_run (CUDA events) */
    int steps;              /* steps of the last run */
    int used_graph;         /* 1 if the last run replayed a captured graph */
    int captures;           /* graphs captured so far */
    int recoveries;         /* runs redone with exact tree sizes after a sync-free build missed */
    int nsys, nsys_tree, nsys_direct;
    size_t n, n_tree, n_direct;
    unsigned long long launches_per_step; /* kernels launched per step (both streams) */
    unsigned long long last_interactions; /* body pairs + cell terms of the last force phase */
} lg_ensemble_stats;

/* Tuning: i-bodies per thread (1, 2, 4 or 8) and j-bodies per shared-memory stage (256, or 128
 * with 1, 2 or 4 i-bodies per thread) of the batched direct kernel for systems with N < 2048,
 * N < 4096 and larger (classes 0-2), and the walk group size of the forest tree. */
typedef struct {
    int direct_ipt[3];
    int walk_group;
    int tuned;              /* 1 after lg_ensemble_tune measured or loaded them */
    int direct_tile[3];
} lg_ensemble_tuning;

lg_status lg_ensemble_create(int device, lg_ensemble** out);
lg_status lg_ensemble_destroy(lg_ensemble* en);
/* Systems back to back in the input arrays: system s has counts[s] bodies, softening eps[s] > 0,
 * opening angle theta[s] (tree systems) and method[s] (LG_DIRECT or LG_TREE). */
lg_status lg_ensemble_upload(lg_ensemble* en, size_t nsys, const uint32_t* counts, const double* eps,
                             const double* theta, const int* method, double G, const float* x, const float* y,
                             const float* z, const float* vx, const float* vy, const float* vz, const float* m,
                             const uint32_t* id);
/* `steps` kick-drift-kick steps of size dt; use_graph != 0 captures them as one CUDA graph (reused
 * by later runs with the same steps and dt). Synchronises. */
lg_status lg_ensemble_run(lg_ensemble* en, double dt, int steps, int use_graph);
/* Per-system total energy (kinetic + potential, FP64; input system order) at the current state;
 * evaluates forces with potentials. ke / pe may be NULL. */
lg_status lg_ensemble_energy(lg_ensemble* en, double* energy, double* ke, double* pe);
/* Bodies in input system order; within a system, in the engine's current order (ids identify). */
lg_status lg_ensemble_download(lg_ensemble* en, float* x, float* y, float* z, float* vx, float* vy, float* vz,
                               float* m, uint32_t* id);
/* Accelerations and potentials of the last force phase, in lg_ensemble_download's order. */
lg_status lg_ensemble_read_accel(lg_ensemble* en, float* ax, float* ay, float* az, float* pot);
/* Times the candidates on the resident ensemble and keeps the fastest; with a cache file named by
 * LETTUCE_GB300_TUNE_CACHE, an entry for this device is loaded instead (and new results saved). */
lg_status lg_ensemble_tune(lg_ensemble* en);
lg_status lg_ensemble_get_tuning(lg_ensemble* en, lg_ensemble_tuning* out);
lg_status lg_ensemble_set_tuning(lg_ensemble* en, const lg_ensemble_tuning* t);
lg_status lg_ensemble_get_stats(lg_ensemble* en, lg_ensemble_stats* out);

/* Direct-summation forces with no device allocation. No counterpart in the reference: it is for
 * callers that cannot allocate device memory when they need forces, such as a code that owns all
 * device memory through its own fixed arena, or a stepping loop that must avoid cudaMalloc's
 * implicit device synchronisation. The caller passes device arrays of the current device, each
 * 16-byte aligned: posm[n] float4 (x, y, z, m) and poslo[n] float4 (low parts of FP64 positions,
 * x - (double)(float)x, or zeros), and receives acc[n] float4 (ax, ay, az, phi; phi only with
 * potential != 0) on its stream (a cudaStream_t, NULL for the legacy stream). Pointers that are
 * misaligned or not device memory of the current device are rejected with LG_ERR_ARG before any
 * work is enqueued. The call synchronises that stream before it returns.
 * Scratch is a static device array inside this library (16 MiB of split-j partial sums plus a
 * status word), held by every GPU that loads the library until the process exits; n above
 * 1,048,576 is rejected with LG_ERR_ARG. Each call looks up the array's device address in the
 * current context (cudaGetSymbolAddress), so a context that was reset and recreated gets the new
 * address; the first call on a device also loads the module, so make that first call before any
 * stream capture. All calls share the array and it keeps the last call's contents, so calls that
 * overlap on the GPU (other streams, other host threads) race and must not be issued. */
lg_status lg_direct_forces_noalloc(const void* posm, const void* poslo, int n, double G, double eps, int potential,
                                   void* acc, void* stream);

#ifdef __cplusplus
}
#endif
#endif
