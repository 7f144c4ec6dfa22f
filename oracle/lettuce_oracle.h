/* lettuce_oracle.h -- CPU oracle for the lettuce force-and-integrate path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE. Only tests/, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py load this library, and only as the checker or the timed CPU baseline. The GPU
 * engine never calls it and never falls back to it.
 *
 * It restates, in C, the algorithm of the reference's OpenMP backend (src/cpu_backend.cpp):
 * blocked direct summation, Morton keys, the stable 11-bit LSD radix sort, the top-down octree with
 * key restarts, double-precision moments, group interaction lists and the quadrupole evaluation,
 * plus kick, drift, diagnostics and the exact potential energy. It adds an FP64 brute-force direct
 * sum (the oracle every force field is reported against) and an FP64 adjoint of the direct-sum
 * leapfrog. Parity of the restatement is pinned against the reference itself (oracle/_ref, built
 * from the reference sources by oracle/Makefile) and the golden vectors under tests/golden/.
 */
#ifndef LETTUCE_ORACLE_H
#define LETTUCE_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_backend or_backend;

/* Node of the octree, field for field the reference's Node (src/cpu_backend.cpp:35-43). */
typedef struct {
    float cx, cy, cz, m;
    float qxx, qxy, qxz, qyy, qyz, qzz;
    float rcrit2;
    uint32_t first, nchild, lo, hi;
} or_node;

/* Geometric cell: centre and half side (src/cpu_backend.cpp:46). */
typedef struct { float gx, gy, gz, half; } or_geo;

/* Walk group: bounding box of a subtree of consecutive sorted bodies (src/cpu_backend.cpp:50). */
typedef struct { float bx, by, bz, hx, hy, hz; uint32_t lo, hi; } or_group;

enum { OR_DIRECT = 0, OR_TREE = 1 };

or_backend* or_create(int threads);
void or_destroy(or_backend* b);
int or_threads(const or_backend* b);

void or_upload(or_backend* b, size_t n, const float* x, const float* y, const float* z, const float* vx,
               const float* vy, const float* vz, const float* m, const uint32_t* id);
size_t or_size(const or_backend* b);
void or_download(const or_backend* b, float* x, float* y, float* z, float* vx, float* vy, float* vz, float* m,
                 uint32_t* id);
/* Accelerations and potential in the current body order. */
void or_accel(const or_backend* b, float* ax, float* ay, float* az, float* pot);

void or_build_tree(or_backend* b, int method, double theta);
void or_compute_forces_with(or_backend* b, int method, double G, double eps, double theta, int potential);
void or_compute_forces(or_backend* b, int method, double G, double eps, double theta, int potential);
void or_kick(or_backend* b, double dt);
void or_drift(or_backend* b, double dt);
/* out: mass, ke, pe, px, py, pz, lx, ly, lz, cx, cy, cz; returns has_pe. */
int or_diagnostics(const or_backend* b, double out[12]);
double or_exact_potential_energy(const or_backend* b, double G, double eps);
/* out: force, sort, build, walk, step ms; returns interactions. */
uint64_t or_times(const or_backend* b, double out[5]);
/* Per-body interaction counts of the last force call in body order; 0 if none. */
int or_body_costs(const or_backend* b, float* cost);

/* Tree introspection after or_build_tree (tree method). */
size_t or_num_nodes(const or_backend* b);
size_t or_num_groups(const or_backend* b);
size_t or_num_leaves(const or_backend* b);
int or_max_depth(const or_backend* b);
void or_get_nodes(const or_backend* b, or_node* out);
void or_get_geo(const or_backend* b, or_geo* out);
void or_get_groups(const or_backend* b, or_group* out);
void or_get_leaves(const or_backend* b, uint32_t* out);
/* Sorted Morton keys (after any key restarts) and the sort frame (ox, oy, oz, side). */
void or_get_keys(const or_backend* b, uint64_t* out);
void or_get_frame(const or_backend* b, double out[4]);

/* FP64 brute-force direct sum over float inputs, self excluded by index; the force oracle. */
void or_direct_fp64(size_t n, const float* x, const float* y, const float* z, const float* m, double G, double eps,
                    double* ax, double* ay, double* az, double* pot, int threads);

/* FP64 reference for the adjoint of a direct-sum KDK leapfrog (see lettuce_oracle.c). */
double or_adjoint_direct_fp64(size_t n, const double* x0, const double* v0, const double* m, double G, double eps,
                              double dt, int steps, const double* xstar, double* gx, double* gv, double* gm,
                              int threads);
/* The loss alone (forward only) for finite differences. */
double or_loss_direct_fp64(size_t n, const double* x0, const double* v0, const double* m, double G, double eps,
                           double dt, int steps, const double* xstar, int threads);

/* FP64 tree forces over frozen interaction lists (test oracle of the engine's tree adjoint): one
 * entry per force call of a trajectory of `steps` steps; per call s: nn[s] nodes (range4: lo, hi,
 * first, nchild; comrc: FP32 cx, cy, cz, rcrit2), ng[s] groups (glohi; gbox: bx, by, bz, hx, hy,
 * hz), perm: sorted position -> id (n per call). Arrays of all calls back to back. */
typedef struct or_frozen or_frozen;
or_frozen* or_frozen_create(size_t n, int steps, const uint32_t* nn, const uint32_t* ng, const uint32_t* perm_all,
                            const uint32_t* range4_all, const float* comrc_all, const uint32_t* glohi_all,
                            const float* gbox_all);
void or_frozen_destroy(or_frozen* f);
/* L = sum m |x_T - x*|^2 after the KDK steps (x0, v0, xstar: 3 per id; m per id). */
double or_frozen_loss(const or_frozen* f, const double* x0, const double* v0, const double* m, double G, double eps,
                      double dt, const double* xstar, int threads);
void or_frozen_accel(const or_frozen* f, int s, const double* x, const double* m, double G, double eps, double* a,
                     int threads);

/* FP64 block (hierarchical) time steps with direct forces (test oracle of the engine's block steps):
 * x, v (3 per body, FP64) advanced in place; level (per body) = the final levels. */
void or_block_direct_fp64(size_t n, double* x, double* v, const double* m, double G, double eps, double dt, int K,
                          double eta, int steps, uint8_t* level, int threads);

#ifdef __cplusplus
}
#endif
#endif
