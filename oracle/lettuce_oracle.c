/* lettuce_oracle.c -- CPU oracle (test infrastructure; see lettuce_oracle.h).
 *
 * A C restatement of the reference OpenMP backend, src/cpu_backend.cpp. Each function names the
 * lines it follows. It is the checker for the GPU engine and the timed "port" CPU baseline; nothing
 * in the product path links or calls it.
 *
 * Portability: host C only (GCC vector extensions, OpenMP), no ISA intrinsics, so it builds and
 * gives the same results on x86-64 and aarch64. The pair kernel uses 1/sqrtf, the reference's
 * non-AVX path (src/cpu_backend.cpp:76-78); the reference built with AVX uses rsqrt plus one
 * Newton step instead (relative difference ~1e-7).
 */
#include "lettuce_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

enum {
    LEAF_MAX = 16,    /* src/cpu_backend.cpp:24 kLeafMax */
    GROUP_MAX = 128,  /* :27 kGroupMax */
    MAX_LEVEL = 21,   /* :28 kMaxLevel */
    SMALL_LEAF = 4,   /* :29 kSmallLeaf */
    RADIX_BITS = 11,  /* :30 kRadixBits */
    RADIX_BUCKETS = 1 << RADIX_BITS,
    PAR_MIN = 1 << 16 /* :32 kParMin */
};

static double now_ms(void) { return 1e3 * omp_get_wtime(); }

/* Morton bit spread of a 21-bit integer: bit b moves to bit 3b (src/cpu_backend.cpp:52-60). */
static uint64_t spread21(uint64_t v) {
    v &= 0x1fffffULL;
    v = (v | v << 32) & 0x1f00000000ffffULL;
    v = (v | v << 16) & 0x1f0000ff0000ffULL;
    v = (v | v << 8) & 0x100f00f00f00f00fULL;
    v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
    v = (v | v << 2) & 0x1249249249249249ULL;
    return v;
}

typedef float v8f __attribute__((vector_size(32)));
typedef int32_t v8i __attribute__((vector_size(32)));

static inline v8f ld8f(const float* p) { v8f v; memcpy(&v, p, sizeof v); return v; }
static inline v8i ld8i(const int32_t* p) { v8i v; memcpy(&v, p, sizeof v); return v; }
/* Pairwise lane sum in the reference's order (src/cpu_backend.cpp:70). */
static inline float hsum8(v8f v) { return ((v[0] + v[4]) + (v[1] + v[5])) + ((v[2] + v[6]) + (v[3] + v[7])); }

/* 1/sqrt(r2) where mask is set, 0 elsewhere (src/cpu_backend.cpp:72-83, portable branch). */
static inline v8f rsqrt_masked(v8f r2, v8i mask) {
    v8f y;
    for (int l = 0; l < 8; ++l) y[l] = 1.f / sqrtf(r2[l]);
    return (v8f)((v8i)y & mask);
}

/* Body-body over n (multiple of 8) sources, skipping the source whose index equals self
 * (src/cpu_backend.cpp:85-105). */
static inline void p2p8(const float* bx, const float* by, const float* bz, const float* bm, const int32_t* idx,
                        int32_t base, long n, float xi, float yi, float zi, int32_t self, float e2, int pot,
                        float* oax, float* oay, float* oaz, float* op) {
    v8f ax = {0}, ay = {0}, az = {0}, p = {0};
    const v8i lane = {0, 1, 2, 3, 4, 5, 6, 7};
    for (long k = 0; k < n; k += 8) {
        v8f dx = ld8f(bx + k) - xi, dy = ld8f(by + k) - yi, dz = ld8f(bz + k) - zi;
        v8f r2 = dx * dx + dy * dy + dz * dz + e2;
        v8i j = idx ? ld8i(idx + k) : lane + (int32_t)(base + k);
        v8f inv = rsqrt_masked(r2, (v8i)(r2 > 0.f) & (j != self));
        v8f mi = ld8f(bm + k) * inv;
        v8f f = mi * inv * inv;
        ax += f * dx; ay += f * dy; az += f * dz;
        if (pot) p += mi;
    }
    *oax += hsum8(ax); *oay += hsum8(ay); *oaz += hsum8(az);
    if (pot) *op += hsum8(p);
}

/* Per-thread interaction-list scratch (src/cpu_backend.cpp:112-131). */
typedef struct {
    float *bx, *by, *bz, *bm;
    int32_t* bi;
    float *nx, *ny, *nz, *nm, *qxx, *qxy, *qxz, *qyy, *qyz, *qzz;
    size_t capb, capn;
    uint32_t* stack;
    size_t capstack;
    size_t nb, nn;
} scratch_t;

static void* grow_buf(void* p, size_t bytes) {
    void* q = realloc(p, bytes ? bytes : 1);
    if (!q) abort();
    return q;
}

static void need_bodies(scratch_t* s, size_t n) {
    if (s->capb >= n) return;
    size_t c = n > 2 * s->capb ? n : 2 * s->capb;
    s->bx = grow_buf(s->bx, c * 4); s->by = grow_buf(s->by, c * 4); s->bz = grow_buf(s->bz, c * 4);
    s->bm = grow_buf(s->bm, c * 4); s->bi = grow_buf(s->bi, c * 4);
    s->capb = c;
}

static void need_nodes(scratch_t* s, size_t n) {
    if (s->capn >= n) return;
    size_t c = n > 2 * s->capn ? n : 2 * s->capn;
    float** v[10] = {&s->nx, &s->ny, &s->nz, &s->nm, &s->qxx, &s->qxy, &s->qxz, &s->qyy, &s->qyz, &s->qzz};
    for (int k = 0; k < 10; ++k) *v[k] = grow_buf(*v[k], c * 4);
    s->capn = c;
}

struct or_backend {
    int nt;
    size_t n, cap;
    float *x, *y, *z, *vx, *vy, *vz, *m, *ax, *ay, *az, *pot, *cost;
    uint32_t* id;
    int cost_valid; /* cost_.size() == n_ */
    int has_pot, tree_ok;
    double pend_sort_ms, pend_build_ms;
    double t_force, t_sort, t_build, t_walk, t_step, kick_ms, drift_ms;
    uint64_t interactions;
    /* tree */
    double ox, oy, oz, side;
    uint64_t *key, *key2;
    uint32_t *idx, *idx2, *tmpu;
    float* tmpf;
    size_t* hist;
    int hist_threads;
    or_node* nodes;
    size_t nnodes, capnodes;
    or_geo* geo;
    size_t capgeo;
    or_group* groups;
    size_t ngroups, capgroups;
    uint32_t* leaves;
    size_t nleaves, capleaves;
    int max_depth;
    scratch_t* scratch;
};

or_backend* or_create(int threads) {
    or_backend* b = calloc(1, sizeof *b);
    if (!b) abort();
    b->nt = threads > 0 ? threads : omp_get_max_threads();
    b->scratch = calloc((size_t)b->nt, sizeof(scratch_t));
    b->side = 1;
    return b;
}

void or_destroy(or_backend* b) {
    if (!b) return;
    float* fs[] = {b->x, b->y, b->z, b->vx, b->vy, b->vz, b->m, b->ax, b->ay, b->az, b->pot, b->cost, b->tmpf};
    for (size_t k = 0; k < sizeof fs / sizeof fs[0]; ++k) free(fs[k]);
    free(b->id); free(b->key); free(b->key2); free(b->idx); free(b->idx2); free(b->tmpu); free(b->hist);
    free(b->nodes); free(b->geo); free(b->groups); free(b->leaves);
    for (int t = 0; t < b->nt; ++t) {
        scratch_t* s = &b->scratch[t];
        void* ps[] = {s->bx, s->by, s->bz, s->bm, s->bi, s->nx, s->ny, s->nz, s->nm,
                      s->qxx, s->qxy, s->qxz, s->qyy, s->qyz, s->qzz, s->stack};
        for (size_t k = 0; k < sizeof ps / sizeof ps[0]; ++k) free(ps[k]);
    }
    free(b->scratch);
    free(b);
}

int or_threads(const or_backend* b) { return b->nt; }

static void reserve(or_backend* b, size_t n) {
    if (b->cap >= n && b->cap) return;
    size_t c = n ? n : 1;
    float** fs[] = {&b->x, &b->y, &b->z, &b->vx, &b->vy, &b->vz, &b->m, &b->ax, &b->ay, &b->az, &b->pot, &b->cost,
                    &b->tmpf};
    for (size_t k = 0; k < sizeof fs / sizeof fs[0]; ++k) *fs[k] = grow_buf(*fs[k], c * 4);
    b->id = grow_buf(b->id, c * 4); b->tmpu = grow_buf(b->tmpu, c * 4);
    b->idx = grow_buf(b->idx, c * 4); b->idx2 = grow_buf(b->idx2, c * 4);
    b->key = grow_buf(b->key, c * 8); b->key2 = grow_buf(b->key2, c * 8);
    b->cap = c;
}

/* upload (src/cpu_backend.cpp:146-156): copies the state, zeroes a and phi, drops tree and costs. */
void or_upload(or_backend* b, size_t n, const float* x, const float* y, const float* z, const float* vx,
               const float* vy, const float* vz, const float* m, const uint32_t* id) {
    reserve(b, n);
    b->n = n;
    memcpy(b->x, x, n * 4); memcpy(b->y, y, n * 4); memcpy(b->z, z, n * 4);
    memcpy(b->vx, vx, n * 4); memcpy(b->vy, vy, n * 4); memcpy(b->vz, vz, n * 4);
    memcpy(b->m, m, n * 4); memcpy(b->id, id, n * 4);
    memset(b->ax, 0, n * 4); memset(b->ay, 0, n * 4); memset(b->az, 0, n * 4); memset(b->pot, 0, n * 4);
    b->has_pot = 0;
    b->tree_ok = 0;
    b->cost_valid = 0;
}

size_t or_size(const or_backend* b) { return b->n; }

void or_download(const or_backend* b, float* x, float* y, float* z, float* vx, float* vy, float* vz, float* m,
                 uint32_t* id) {
    size_t n = b->n;
    memcpy(x, b->x, n * 4); memcpy(y, b->y, n * 4); memcpy(z, b->z, n * 4);
    memcpy(vx, b->vx, n * 4); memcpy(vy, b->vy, n * 4); memcpy(vz, b->vz, n * 4);
    memcpy(m, b->m, n * 4); memcpy(id, b->id, n * 4);
}

void or_accel(const or_backend* b, float* ax, float* ay, float* az, float* pot) {
    size_t n = b->n;
    memcpy(ax, b->ax, n * 4); memcpy(ay, b->ay, n * 4); memcpy(az, b->az, n * 4);
    if (pot) memcpy(pot, b->pot, n * 4);
}

/* ---- direct (src/cpu_backend.cpp:353-392) ------------------------------------------------- */
static void direct(or_backend* b, float G, float e2, int pot) {
    enum { IB = 128, JT = 4096 };
    const size_t n = b->n;
    const float *X = b->x, *Y = b->y, *Z = b->z, *M = b->m;
    const long nblk = (long)((n + IB - 1) / IB);
#pragma omp parallel for num_threads(b->nt) schedule(dynamic, 1)
    for (long blk = 0; blk < nblk; ++blk) {
        const size_t i0 = (size_t)blk * IB, i1 = n < i0 + IB ? n : i0 + IB;
        float sax[IB] = {0}, say[IB] = {0}, saz[IB] = {0}, sp[IB] = {0};
        for (size_t j0 = 0; j0 < n; j0 += JT) {
            const size_t j1 = n < j0 + JT ? n : j0 + JT;
            for (size_t i = i0; i < i1; ++i) {
                const float xi = X[i], yi = Y[i], zi = Z[i];
                const int32_t ii = (int32_t)i;
                float ax = 0, ay = 0, az = 0, p = 0;
                const size_t jv = j0 + ((j1 - j0) & ~(size_t)7);
                p2p8(X + j0, Y + j0, Z + j0, M + j0, NULL, (int32_t)j0, (long)(jv - j0), xi, yi, zi, ii, e2, pot,
                     &ax, &ay, &az, &p);
                for (size_t j = jv; j < j1; ++j) {
                    float dx = X[j] - xi, dy = Y[j] - yi, dz = Z[j] - zi;
                    float r2 = dx * dx + dy * dy + dz * dz + e2;
                    float inv = (r2 > 0.f && (int32_t)j != ii) ? 1.f / sqrtf(r2) : 0.f;
                    float mi = M[j] * inv;
                    float f = mi * inv * inv;
                    ax += f * dx; ay += f * dy; az += f * dz;
                    if (pot) p += mi;
                }
                sax[i - i0] += ax; say[i - i0] += ay; saz[i - i0] += az;
                if (pot) sp[i - i0] += p;
            }
        }
        for (size_t i = i0; i < i1; ++i) {
            b->ax[i] = G * sax[i - i0]; b->ay[i] = G * say[i - i0]; b->az[i] = G * saz[i - i0];
            if (pot) b->pot[i] = -G * sp[i - i0];
        }
    }
}

/* ---- sort (src/cpu_backend.cpp:395-499) ---------------------------------------------------- */
static void bbox_range(const or_backend* b, size_t lo, size_t hi, int par, float mn[3], float mx[3]) {
    float mnx = b->x[lo], mny = b->y[lo], mnz = b->z[lo], mxx = mnx, mxy = mny, mxz = mnz;
    const long l0 = (long)lo, l1 = (long)hi;
#pragma omp parallel for num_threads(b->nt) if (par) reduction(min : mnx, mny, mnz) reduction(max : mxx, mxy, mxz)
    for (long i = l0; i < l1; ++i) {
        mnx = fminf(mnx, b->x[i]); mny = fminf(mny, b->y[i]); mnz = fminf(mnz, b->z[i]);
        mxx = fmaxf(mxx, b->x[i]); mxy = fmaxf(mxy, b->y[i]); mxz = fmaxf(mxz, b->z[i]);
    }
    mn[0] = mnx; mn[1] = mny; mn[2] = mnz;
    mx[0] = mxx; mx[1] = mxy; mx[2] = mxz;
}

static double max3(double a, double b, double c) { double t = a > b ? a : b; return t > c ? t : c; }

static inline uint64_t quantize(float v, double o, double s, double lim) {
    double q = ((double)v - o) * s;
    if (q < 0.0) q = 0.0;
    if (q > lim) q = lim;
    return (uint64_t)q;
}

/* make_keys (src/cpu_backend.cpp:418-428): key = x<<2 | y<<1 | z of the 21-bit quantised coordinates. */
static void make_keys(or_backend* b, size_t lo, size_t hi, double ox, double oy, double oz, double side, int par) {
    const double s = (double)(1u << MAX_LEVEL) / side;
    const double lim = (double)((1u << MAX_LEVEL) - 1);
    const long l0 = (long)lo, l1 = (long)hi;
#pragma omp parallel for num_threads(b->nt) schedule(static) if (par)
    for (long i = l0; i < l1; ++i) {
        b->key[i] = spread21(quantize(b->x[i], ox, s, lim)) << 2 | spread21(quantize(b->y[i], oy, s, lim)) << 1 |
                    spread21(quantize(b->z[i], oz, s, lim));
        b->idx[i] = (uint32_t)i;
    }
}

/* permute (src/cpu_backend.cpp:431-450): gathers every body array of [lo, hi) in idx order. */
static void permute(or_backend* b, size_t lo, size_t hi, int par) {
    const long l0 = (long)lo, l1 = (long)hi;
    const size_t n = hi - lo;
    float* arrs[] = {b->x, b->y, b->z, b->vx, b->vy, b->vz, b->m};
    for (int a = 0; a < 7; ++a) {
        float* src = arrs[a];
        float* dst = b->tmpf;
#pragma omp parallel for num_threads(b->nt) schedule(static) if (par)
        for (long i = l0; i < l1; ++i) dst[i] = src[b->idx[i]];
        memcpy(src + lo, dst + lo, n * 4);
    }
#pragma omp parallel for num_threads(b->nt) schedule(static) if (par)
    for (long i = l0; i < l1; ++i) b->tmpu[i] = b->id[b->idx[i]];
    memcpy(b->id + lo, b->tmpu + lo, n * 4);
    if (b->cost_valid) {
#pragma omp parallel for num_threads(b->nt) schedule(static) if (par)
        for (long i = l0; i < l1; ++i) b->tmpf[i] = b->cost[b->idx[i]];
        memcpy(b->cost + lo, b->tmpf + lo, n * 4);
    }
}

/* Stable LSD radix sort of (key, idx) over [lo, hi) with T threads, 11-bit digits, constant
 * digits skipped (src/cpu_backend.cpp:453-499). */
static void radix_sort(or_backend* b, size_t lo, size_t hi, int T) {
    const size_t n = hi - lo;
    if (b->hist_threads < T) {
        b->hist = grow_buf(b->hist, (size_t)T * RADIX_BUCKETS * sizeof(size_t));
        b->hist_threads = T;
    }
    size_t* hist = b->hist;
    uint64_t *ks = b->key + lo, *kd = b->key2 + lo;
    uint32_t *is = b->idx + lo, *id = b->idx2 + lo;
    for (int shift = 0; shift < 63; shift += RADIX_BITS) {
        int skip = 0;
#pragma omp parallel num_threads(T)
        {
            const int t = omp_get_thread_num(), nth = omp_get_num_threads();
            const size_t b0 = n * (size_t)t / (size_t)nth, b1 = n * (size_t)(t + 1) / (size_t)nth;
            size_t* h = &hist[(size_t)t * RADIX_BUCKETS];
            memset(h, 0, RADIX_BUCKETS * sizeof(size_t));
            for (size_t i = b0; i < b1; ++i) ++h[(ks[i] >> shift) & (RADIX_BUCKETS - 1)];
#pragma omp barrier
#pragma omp single
            {
                size_t off = 0;
                for (int d = 0; d < RADIX_BUCKETS; ++d) {
                    size_t tot = 0;
                    for (int u = 0; u < nth; ++u) {
                        size_t c = hist[(size_t)u * RADIX_BUCKETS + d];
                        hist[(size_t)u * RADIX_BUCKETS + d] = off;
                        off += c;
                        tot += c;
                    }
                    if (tot == n) skip = 1;
                }
            }
            if (!skip) {
                for (size_t i = b0; i < b1; ++i) {
                    size_t dst = h[(ks[i] >> shift) & (RADIX_BUCKETS - 1)]++;
                    kd[dst] = ks[i];
                    id[dst] = is[i];
                }
            }
        }
        if (!skip) {
            uint64_t* tk = ks; ks = kd; kd = tk;
            uint32_t* ti = is; is = id; id = ti;
        }
    }
    if (ks == b->key + lo) return;
    if (lo == 0 && hi == b->n) {
        uint64_t* tk = b->key; b->key = b->key2; b->key2 = tk;
        uint32_t* ti = b->idx; b->idx = b->idx2; b->idx2 = ti;
    } else {
        memcpy(b->key + lo, ks, n * 8);
        memcpy(b->idx + lo, is, n * 4);
    }
}

/* sort_bodies (src/cpu_backend.cpp:395-415). */
static void sort_bodies(or_backend* b) {
    const size_t n = b->n;
    float mn[3], mx[3];
    bbox_range(b, 0, n, 1, mn, mx);
    double side = max3((double)mx[0] - mn[0], (double)mx[1] - mn[1], (double)mx[2] - mn[2]);
    side = side > 0 ? side * (1 + 1e-6) : 1.0;
    b->ox = mn[0]; b->oy = mn[1]; b->oz = mn[2]; b->side = side;
    make_keys(b, 0, n, b->ox, b->oy, b->oz, side, 1);
    radix_sort(b, 0, n, b->nt);
    permute(b, 0, n, 1);
}

static int cmp_kv(const void* pa, const void* pb) {
    const uint64_t* a = pa;
    const uint64_t* c = pb;
    if (a[0] != c[0]) return a[0] < c[0] ? -1 : 1;
    return a[1] < c[1] ? -1 : (a[1] > c[1]);
}

/* rekey (src/cpu_backend.cpp:503-530): keys [lo, hi) in their own bounding cube, re-sorts and
 * permutes them; returns 0 when they all coincide. */
static int rekey(or_backend* b, uint32_t lo, uint32_t hi, double* gx, double* gy, double* gz, double* half) {
    const int par = hi - lo >= PAR_MIN;
    float mn[3], mx[3];
    bbox_range(b, lo, hi, par, mn, mx);
    double side = max3((double)mx[0] - mn[0], (double)mx[1] - mn[1], (double)mx[2] - mn[2]);
    if (side == 0) return 0;
    side *= 1 + 1e-6;
    make_keys(b, lo, hi, mn[0], mn[1], mn[2], side, par);
    if (!par) {
        /* (key, index) order: the order a stable sort gives. */
        size_t cnt = hi - lo;
        uint64_t* kv = malloc(cnt * 16);
        if (!kv) abort();
        for (uint32_t i = lo; i < hi; ++i) { kv[2 * (i - lo)] = b->key[i]; kv[2 * (i - lo) + 1] = i; }
        qsort(kv, cnt, 16, cmp_kv);
        for (uint32_t i = lo; i < hi; ++i) { b->key[i] = kv[2 * (i - lo)]; b->idx[i] = (uint32_t)kv[2 * (i - lo) + 1]; }
        free(kv);
    } else {
        radix_sort(b, lo, hi, b->nt);
    }
    permute(b, lo, hi, par);
    *half = 0.5 * side;
    *gx = mn[0] + *half; *gy = mn[1] + *half; *gz = mn[2] + *half;
    return 1;
}

/* ---- build (src/cpu_backend.cpp:534-664) --------------------------------------------------- */
static uint32_t push_node(or_backend* b, uint32_t lo, uint32_t hi) {
    if (b->nnodes == b->capnodes) {
        b->capnodes = b->capnodes ? 2 * b->capnodes : 1024;
        b->nodes = grow_buf(b->nodes, b->capnodes * sizeof(or_node));
    }
    or_node* c = &b->nodes[b->nnodes];
    memset(c, 0, sizeof *c);
    c->lo = lo; c->hi = hi;
    return (uint32_t)b->nnodes++;
}

static void sync_geo(or_backend* b) {
    if (b->capgeo < b->capnodes) {
        b->capgeo = b->capnodes;
        b->geo = grow_buf(b->geo, b->capgeo * sizeof(or_geo));
    }
}

static void push_group(or_backend* b, uint32_t lo, uint32_t hi) {
    if (b->ngroups == b->capgroups) {
        b->capgroups = b->capgroups ? 2 * b->capgroups : 1024;
        b->groups = grow_buf(b->groups, b->capgroups * sizeof(or_group));
    }
    or_group g = {0, 0, 0, 0, 0, 0, lo, hi};
    b->groups[b->ngroups++] = g;
}

static void push_leaf(or_backend* b, uint32_t ni) {
    if (b->nleaves == b->capleaves) {
        b->capleaves = b->capleaves ? 2 * b->capleaves : 1024;
        b->leaves = grow_buf(b->leaves, b->capleaves * 4);
    }
    b->leaves[b->nleaves++] = ni;
}

/* First index in [from, hi) whose octant digit at shift is >= o (keys sorted). */
static uint32_t octant_bound(const uint64_t* k, uint32_t from, uint32_t hi, int shift, int o) {
    uint32_t a = from, c = hi;
    while (a < c) {
        uint32_t mid = a + (c - a) / 2;
        if ((int)((k[mid] >> shift) & 7) < o) a = mid + 1;
        else c = mid;
    }
    return a;
}

static void build_node(or_backend* b, uint32_t ni, int level, int depth, double gx, double gy, double gz,
                       double half, int in_group) {
    const uint32_t lo = b->nodes[ni].lo, hi = b->nodes[ni].hi;
    if (depth > b->max_depth) b->max_depth = depth;
    int leaf = hi - lo <= (uint32_t)LEAF_MAX;
    if (!leaf && level == MAX_LEVEL) {
        if (rekey(b, lo, hi, &gx, &gy, &gz, &half)) level = 0;
        else leaf = 1;
    }
    or_geo ge = {(float)gx, (float)gy, (float)gz, (float)half};
    b->geo[ni] = ge;
    if (!in_group && (hi - lo <= (uint32_t)GROUP_MAX || leaf)) {
        push_group(b, lo, hi);
        in_group = 1;
    }
    if (leaf) {
        b->nodes[ni].first = lo;
        b->nodes[ni].nchild = 0;
        push_leaf(b, ni);
        return;
    }
    const int shift = 3 * (MAX_LEVEL - 1 - level);
    uint32_t bound[9];
    bound[0] = lo;
    for (int o = 1; o < 8; ++o) bound[o] = octant_bound(b->key, bound[o - 1], hi, shift, o);
    bound[8] = hi;
    const uint32_t first = (uint32_t)b->nnodes;
    uint32_t nc = 0;
    for (int o = 0; o < 8; ++o)
        if (bound[o + 1] > bound[o]) { push_node(b, bound[o], bound[o + 1]); ++nc; }
    sync_geo(b);
    b->nodes[ni].first = first;
    b->nodes[ni].nchild = nc;
    const double q = 0.5 * half;
    uint32_t c = first;
    for (int o = 0; o < 8; ++o) {
        if (bound[o + 1] == bound[o]) continue;
        build_node(b, c++, level + 1, depth + 1, gx + ((o & 4) ? q : -q), gy + ((o & 2) ? q : -q),
                   gz + ((o & 1) ? q : -q), q, in_group);
    }
}

/* The reference as its compiler builds it (GCC's default -ffp-contract=fast; FMA on x86-64-v3 and
 * aarch64) fuses a product into the sum or difference that is its only use: x*x + y*y + z*z becomes
 * fma(z, z, fma(x, x, y*y)), in float and in double; m*(3*d*d - r2) accumulated into q becomes
 * fma(m, fma(3*d, d, -r2), q); m*3*d*e into q becomes fma(m*3*d, e, q). This file is built without
 * contraction, so those fused forms are spelled out where the reference's results depend on them
 * (opening tests, rcrit2, quadrupoles); products of two floats are exact in double and are left
 * as they are. */
static inline float sq3f(float x, float y, float z) { return fmaf(z, z, fmaf(x, x, y * y)); }
static inline double sq3(double x, double y, double z) { return fma(z, z, fma(x, x, y * y)); }

/* rcrit2 = (2 half / theta + |com - centre|)^2, capped at FLT_MAX (src/cpu_backend.cpp:595-600). */
static void finish_node(or_node* nd, const or_geo* g, float inv_theta) {
    float dx = nd->cx - g->gx, dy = nd->cy - g->gy, dz = nd->cz - g->gz;
    double r = (double)(2 * g->half) * inv_theta + sqrt((double)sq3f(dx, dy, dz));
    double r2 = r * r;
    nd->rcrit2 = (float)(r2 < (double)FLT_MAX ? r2 : (double)FLT_MAX);
}

static void build_octree(or_backend* b, double theta) {
    b->nnodes = 0; b->ngroups = 0; b->nleaves = 0; b->max_depth = 0;
    push_node(b, 0, (uint32_t)b->n);
    sync_geo(b);
    const double h = 0.5 * b->side;
    build_node(b, 0, 0, 0, b->ox + h, b->oy + h, b->oz + h, h, 0);

    const float inv_theta = theta > 0 ? (float)(1.0 / theta) : FLT_MAX;
    const long ng = (long)b->ngroups;
#pragma omp parallel for num_threads(b->nt) schedule(dynamic, 16)
    for (long g = 0; g < ng; ++g) {
        or_group* gr = &b->groups[g];
        float mnx = b->x[gr->lo], mny = b->y[gr->lo], mnz = b->z[gr->lo], mxx = mnx, mxy = mny, mxz = mnz;
        for (uint32_t i = gr->lo; i < gr->hi; ++i) {
            mnx = fminf(mnx, b->x[i]); mny = fminf(mny, b->y[i]); mnz = fminf(mnz, b->z[i]);
            mxx = fmaxf(mxx, b->x[i]); mxy = fmaxf(mxy, b->y[i]); mxz = fmaxf(mxz, b->z[i]);
        }
        gr->bx = 0.5f * (mnx + mxx); gr->by = 0.5f * (mny + mxy); gr->bz = 0.5f * (mnz + mxz);
        gr->hx = 0.5f * (mxx - mnx); gr->hy = 0.5f * (mxy - mny); gr->hz = 0.5f * (mxz - mnz);
    }

    /* Leaf moments about each leaf's centre of mass in double (src/cpu_backend.cpp:619-640). */
    const long nl = (long)b->nleaves;
#pragma omp parallel for num_threads(b->nt) schedule(dynamic, 64)
    for (long l = 0; l < nl; ++l) {
        or_node* nd = &b->nodes[b->leaves[l]];
        const or_geo* ge = &b->geo[b->leaves[l]];
        double M = 0, sx = 0, sy = 0, sz = 0;
        for (uint32_t i = nd->lo; i < nd->hi; ++i) {
            double mi = b->m[i];
            M += mi; sx += mi * b->x[i]; sy += mi * b->y[i]; sz += mi * b->z[i];
        }
        double cx = M > 0 ? sx / M : ge->gx, cy = M > 0 ? sy / M : ge->gy, cz = M > 0 ? sz / M : ge->gz;
        double qxx = 0, qxy = 0, qxz = 0, qyy = 0, qyz = 0, qzz = 0;
        for (uint32_t i = nd->lo; i < nd->hi; ++i) {
            double mi = b->m[i], dx = b->x[i] - cx, dy = b->y[i] - cy, dz = b->z[i] - cz;
            double r2 = sq3(dx, dy, dz);
            qxx = fma(mi, fma(3 * dx, dx, -r2), qxx); qyy = fma(mi, fma(3 * dy, dy, -r2), qyy);
            qzz = fma(mi, fma(3 * dz, dz, -r2), qzz);
            qxy = fma(mi * 3 * dx, dy, qxy); qxz = fma(mi * 3 * dx, dz, qxz); qyz = fma(mi * 3 * dy, dz, qyz);
        }
        nd->cx = (float)cx; nd->cy = (float)cy; nd->cz = (float)cz; nd->m = (float)M;
        nd->qxx = (float)qxx; nd->qxy = (float)qxy; nd->qxz = (float)qxz;
        nd->qyy = (float)qyy; nd->qyz = (float)qyz; nd->qzz = (float)qzz;
        finish_node(nd, ge, inv_theta);
    }

    /* Internal nodes: serial reverse sweep, parallel-axis theorem in double (:642-663). */
    for (long ni = (long)b->nnodes - 1; ni >= 0; --ni) {
        or_node* nd = &b->nodes[ni];
        if (nd->nchild == 0) continue;
        double M = 0, sx = 0, sy = 0, sz = 0;
        for (uint32_t c = nd->first; c < nd->first + nd->nchild; ++c) {
            const or_node* ch = &b->nodes[c];
            M += ch->m; sx += (double)ch->m * ch->cx; sy += (double)ch->m * ch->cy; sz += (double)ch->m * ch->cz;
        }
        const or_geo* ge = &b->geo[ni];
        double cx = M > 0 ? sx / M : ge->gx, cy = M > 0 ? sy / M : ge->gy, cz = M > 0 ? sz / M : ge->gz;
        double qxx = 0, qxy = 0, qxz = 0, qyy = 0, qyz = 0, qzz = 0;
        for (uint32_t c = nd->first; c < nd->first + nd->nchild; ++c) {
            const or_node* ch = &b->nodes[c];
            double mc = ch->m, dx = ch->cx - cx, dy = ch->cy - cy, dz = ch->cz - cz;
            double r2 = sq3(dx, dy, dz);
            qxx += fma(mc, fma(3 * dx, dx, -r2), (double)ch->qxx); qyy += fma(mc, fma(3 * dy, dy, -r2), (double)ch->qyy);
            qzz += fma(mc, fma(3 * dz, dz, -r2), (double)ch->qzz);
            qxy += fma(mc * 3 * dx, dy, (double)ch->qxy); qxz += fma(mc * 3 * dx, dz, (double)ch->qxz);
            qyz += fma(mc * 3 * dy, dz, (double)ch->qyz);
        }
        nd->cx = (float)cx; nd->cy = (float)cy; nd->cz = (float)cz; nd->m = (float)M;
        nd->qxx = (float)qxx; nd->qxy = (float)qxy; nd->qxz = (float)qxz;
        nd->qyy = (float)qyy; nd->qyz = (float)qyz; nd->qzz = (float)qzz;
        finish_node(nd, ge, inv_theta);
    }
}

/* build_tree (src/cpu_backend.cpp:168-178). */
void or_build_tree(or_backend* b, int method, double theta) {
    b->pend_sort_ms = b->pend_build_ms = 0;
    if (method != OR_TREE || b->n == 0) return;
    double ts = now_ms();
    sort_bodies(b);
    b->pend_sort_ms = now_ms() - ts;
    double tb = now_ms();
    build_octree(b, theta);
    b->pend_build_ms = now_ms() - tb;
    b->tree_ok = 1;
}

/* ---- walk (src/cpu_backend.cpp:667-689, 770-882) ------------------------------------------- */
static void pad_lists(scratch_t* s) {
    const size_t nb8 = (s->nb + 7) & ~(size_t)7, nn8 = (s->nn + 7) & ~(size_t)7;
    need_bodies(s, nb8);
    need_nodes(s, nn8);
    for (size_t k = s->nb; k < nb8; ++k) { s->bx[k] = s->by[k] = s->bz[k] = s->bm[k] = 0; s->bi[k] = -1; }
    for (size_t k = s->nn; k < nn8; ++k) {
        s->nx[k] = s->ny[k] = s->nz[k] = s->nm[k] = 0;
        s->qxx[k] = s->qxy[k] = s->qxz[k] = s->qyy[k] = s->qyz[k] = s->qzz[k] = 0;
    }
}

static void push_bodies(const or_backend* b, scratch_t* s, uint32_t lo, uint32_t hi) {
    need_bodies(s, s->nb + (hi - lo));
    for (uint32_t j = lo; j < hi; ++j, ++s->nb) {
        s->bx[s->nb] = b->x[j]; s->by[s->nb] = b->y[j]; s->bz[s->nb] = b->z[j]; s->bm[s->nb] = b->m[j];
        s->bi[s->nb] = (int32_t)j;
    }
}

static void push_cell(scratch_t* s, const or_node* nd) {
    need_nodes(s, s->nn + 1);
    const size_t k = s->nn++;
    s->nx[k] = nd->cx; s->ny[k] = nd->cy; s->nz[k] = nd->cz; s->nm[k] = nd->m;
    s->qxx[k] = nd->qxx; s->qxy[k] = nd->qxy; s->qxz[k] = nd->qxz;
    s->qyy[k] = nd->qyy; s->qyz[k] = nd->qyz; s->qzz[k] = nd->qzz;
}

/* build_list (src/cpu_backend.cpp:816-838): depth-first, children pushed last-first. */
static void build_list(const or_backend* b, const or_group* gr, scratch_t* s) {
    s->nb = s->nn = 0;
    uint32_t sp = 0;
    s->stack[sp++] = 0;
    while (sp) {
        const or_node* nd = &b->nodes[s->stack[--sp]];
        float dx = fmaxf(fabsf(nd->cx - gr->bx) - gr->hx, 0.f);
        float dy = fmaxf(fabsf(nd->cy - gr->by) - gr->hy, 0.f);
        float dz = fmaxf(fabsf(nd->cz - gr->bz) - gr->hz, 0.f);
        int contains = nd->lo <= gr->lo && gr->hi <= nd->hi;
        if (!contains && sq3f(dx, dy, dz) >= nd->rcrit2) {
            if (nd->nchild == 0 && nd->hi - nd->lo <= (uint32_t)SMALL_LEAF) push_bodies(b, s, nd->lo, nd->hi);
            else push_cell(s, nd);
        } else if (nd->nchild == 0) {
            push_bodies(b, s, nd->lo, nd->hi);
        } else {
            for (uint32_t c = nd->first + nd->nchild; c-- > nd->first;) s->stack[sp++] = c;
        }
    }
}

/* eval_group (src/cpu_backend.cpp:841-882), overwrite form. */
static void eval_group(or_backend* b, const or_group* gr, const scratch_t* s, float G, float e2, int pot) {
    const long nb = (long)((s->nb + 7) & ~(size_t)7), nn = (long)((s->nn + 7) & ~(size_t)7);
    for (uint32_t i = gr->lo; i < gr->hi; ++i) {
        const float xi = b->x[i], yi = b->y[i], zi = b->z[i];
        float ax = 0, ay = 0, az = 0, p = 0;
        p2p8(s->bx, s->by, s->bz, s->bm, s->bi, 0, nb, xi, yi, zi, (int32_t)i, e2, pot, &ax, &ay, &az, &p);
        v8f vax = {0}, vay = {0}, vaz = {0}, vp = {0};
        for (long k = 0; k < nn; k += 8) {
            v8f dx = ld8f(s->nx + k) - xi, dy = ld8f(s->ny + k) - yi, dz = ld8f(s->nz + k) - zi;
            v8f r2 = dx * dx + dy * dy + dz * dz + e2;
            v8f inv = rsqrt_masked(r2, (v8i)(r2 > 0.f));
            v8f inv2 = inv * inv, inv3 = inv * inv2, inv5 = inv3 * inv2;
            v8f xx = ld8f(s->qxx + k), xy = ld8f(s->qxy + k), xz = ld8f(s->qxz + k);
            v8f yy = ld8f(s->qyy + k), yz = ld8f(s->qyz + k), zz = ld8f(s->qzz + k);
            v8f qx = xx * dx + xy * dy + xz * dz;
            v8f qy = xy * dx + yy * dy + yz * dz;
            v8f qz = xz * dx + yz * dy + zz * dz;
            v8f dqd = dx * qx + dy * qy + dz * qz;
            v8f mk = ld8f(s->nm + k);
            v8f f = mk * inv3 + 2.5f * dqd * inv5 * inv2;
            vax += f * dx - qx * inv5; vay += f * dy - qy * inv5; vaz += f * dz - qz * inv5;
            if (pot) vp += mk * inv + 0.5f * dqd * inv5;
        }
        ax += hsum8(vax); ay += hsum8(vay); az += hsum8(vaz);
        if (pot) p += hsum8(vp);
        b->ax[i] = G * ax; b->ay[i] = G * ay; b->az[i] = G * az;
        if (pot) b->pot[i] = -G * p;
    }
}

static uint64_t walk(or_backend* b, float G, float e2, int pot) {
    const long ng = (long)b->ngroups;
    uint64_t inter = 0;
#pragma omp parallel num_threads(b->nt) reduction(+ : inter)
    {
        scratch_t* s = &b->scratch[omp_get_thread_num()];
        const size_t stack_need = 8 * (size_t)(b->max_depth + 2);
        if (s->capstack < stack_need) {
            s->stack = grow_buf(s->stack, stack_need * 4);
            s->capstack = stack_need;
        }
#pragma omp for schedule(dynamic, 4)
        for (long g = 0; g < ng; ++g) {
            const or_group* gr = &b->groups[g];
            build_list(b, gr, s);
            pad_lists(s);
            eval_group(b, gr, s, G, e2, pot);
            const size_t len = s->nb + s->nn;
            for (uint32_t i = gr->lo; i < gr->hi; ++i) b->cost[i] = (float)len;
            inter += (uint64_t)len * (gr->hi - gr->lo);
        }
    }
    return inter;
}

/* compute_forces_with without remote trees (src/cpu_backend.cpp:180-204). */
void or_compute_forces_with(or_backend* b, int method, double G, double eps, double theta, int potential) {
    double t0 = now_ms();
    double step = b->t_step;
    if (method == OR_TREE && b->n > 0 && !b->tree_ok) or_build_tree(b, method, theta);
    b->t_sort = b->pend_sort_ms;
    b->t_build = b->pend_build_ms;
    b->pend_sort_ms = b->pend_build_ms = 0;
    b->t_force = b->t_walk = 0;
    b->interactions = 0;
    b->t_step = step;
    b->has_pot = potential;
    b->cost_valid = 1;
    if (b->n == 0) return;
    const float Gf = (float)G, e2 = (float)(eps * eps);
    double tw = now_ms();
    if (method == OR_DIRECT) {
        direct(b, Gf, e2, potential);
        b->interactions = (uint64_t)b->n * b->n;
        for (size_t i = 0; i < b->n; ++i) b->cost[i] = (float)b->n;
    } else {
        b->interactions = walk(b, Gf, e2, potential);
    }
    b->t_walk = now_ms() - tw;
    b->t_force = b->t_sort + b->t_build + (now_ms() - t0);
}

void or_compute_forces(or_backend* b, int method, double G, double eps, double theta, int potential) {
    or_build_tree(b, method, theta);
    or_compute_forces_with(b, method, G, eps, theta, potential);
}

/* kick/drift (src/cpu_backend.cpp:279-305), FP32. */
void or_kick(or_backend* b, double dt) {
    double t0 = now_ms();
    const float h = (float)dt;
    const long n = (long)b->n;
#pragma omp parallel for simd num_threads(b->nt) schedule(static)
    for (long i = 0; i < n; ++i) {
        /* v += a h as the reference's compiler forms it: one fused multiply-add */
        b->vx[i] = fmaf(b->ax[i], h, b->vx[i]); b->vy[i] = fmaf(b->ay[i], h, b->vy[i]);
        b->vz[i] = fmaf(b->az[i], h, b->vz[i]);
    }
    b->kick_ms = now_ms() - t0;
    b->t_step = b->kick_ms + b->drift_ms;
}

void or_drift(or_backend* b, double dt) {
    double t0 = now_ms();
    const float h = (float)dt;
    const long n = (long)b->n;
#pragma omp parallel for simd num_threads(b->nt) schedule(static)
    for (long i = 0; i < n; ++i) {
        /* x += v h, fused as in the reference's build */
        b->x[i] = fmaf(b->vx[i], h, b->x[i]); b->y[i] = fmaf(b->vy[i], h, b->y[i]);
        b->z[i] = fmaf(b->vz[i], h, b->z[i]);
    }
    b->has_pot = 0;
    b->tree_ok = 0;
    b->drift_ms = now_ms() - t0;
    b->t_step = b->kick_ms + b->drift_ms;
}

/* diagnostics (src/cpu_backend.cpp:307-329). */
int or_diagnostics(const or_backend* b, double out[12]) {
    double mass = 0, ke = 0, pe = 0, px = 0, py = 0, pz = 0, lx = 0, ly = 0, lz = 0, cx = 0, cy = 0, cz = 0;
    const long n = (long)b->n;
#pragma omp parallel for num_threads(b->nt) schedule(static) \
    reduction(+ : mass, ke, pe, px, py, pz, lx, ly, lz, cx, cy, cz)
    for (long i = 0; i < n; ++i) {
        double m = b->m[i], x = b->x[i], y = b->y[i], z = b->z[i], vx = b->vx[i], vy = b->vy[i], vz = b->vz[i];
        mass += m;
        ke += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        pe += 0.5 * m * (double)b->pot[i];
        px += m * vx; py += m * vy; pz += m * vz;
        lx += m * (y * vz - z * vy); ly += m * (z * vx - x * vz); lz += m * (x * vy - y * vx);
        cx += m * x; cy += m * y; cz += m * z;
    }
    out[0] = mass; out[1] = ke; out[2] = b->has_pot ? pe : 0;
    out[3] = px; out[4] = py; out[5] = pz;
    out[6] = lx; out[7] = ly; out[8] = lz;
    out[9] = mass > 0 ? cx / mass : 0; out[10] = mass > 0 ? cy / mass : 0; out[11] = mass > 0 ? cz / mass : 0;
    return b->has_pot;
}

/* exact_potential_energy (src/cpu_backend.cpp:331-347). */
double or_exact_potential_energy(const or_backend* b, double G, double eps) {
    const double e2 = eps * eps;
    const long n = (long)b->n;
    double pe = 0;
#pragma omp parallel for num_threads(b->nt) schedule(dynamic, 64) reduction(+ : pe)
    for (long i = 0; i < n; ++i) {
        const double xi = b->x[i], yi = b->y[i], zi = b->z[i];
        double s = 0;
        for (long j = i + 1; j < n; ++j) {
            double dx = b->x[j] - xi, dy = b->y[j] - yi, dz = b->z[j] - zi;
            double r2 = dx * dx + dy * dy + dz * dz + e2;
            if (r2 > 0) s += (double)b->m[j] / sqrt(r2);
        }
        pe -= (double)b->m[i] * s;
    }
    return G * pe;
}

uint64_t or_times(const or_backend* b, double out[5]) {
    out[0] = b->t_force; out[1] = b->t_sort; out[2] = b->t_build; out[3] = b->t_walk; out[4] = b->t_step;
    return b->interactions;
}

int or_body_costs(const or_backend* b, float* cost) {
    if (!b->cost_valid || b->n == 0) return 0;
    memcpy(cost, b->cost, b->n * 4);
    return 1;
}

size_t or_num_nodes(const or_backend* b) { return b->nnodes; }
size_t or_num_groups(const or_backend* b) { return b->ngroups; }
size_t or_num_leaves(const or_backend* b) { return b->nleaves; }
int or_max_depth(const or_backend* b) { return b->max_depth; }
void or_get_nodes(const or_backend* b, or_node* out) { memcpy(out, b->nodes, b->nnodes * sizeof(or_node)); }
void or_get_geo(const or_backend* b, or_geo* out) { memcpy(out, b->geo, b->nnodes * sizeof(or_geo)); }
void or_get_groups(const or_backend* b, or_group* out) { memcpy(out, b->groups, b->ngroups * sizeof(or_group)); }
void or_get_leaves(const or_backend* b, uint32_t* out) { memcpy(out, b->leaves, b->nleaves * 4); }
void or_get_keys(const or_backend* b, uint64_t* out) { memcpy(out, b->key, b->n * 8); }
void or_get_frame(const or_backend* b, double out[4]) { out[0] = b->ox; out[1] = b->oy; out[2] = b->oz; out[3] = b->side; }

/* ---- FP64 brute force (pattern of tests/test_cuda_backend.cpp:63-85) ------------------------ */
void or_direct_fp64(size_t n, const float* x, const float* y, const float* z, const float* m, double G, double eps,
                    double* ax, double* ay, double* az, double* pot, int threads) {
    const double e2 = eps * eps;
    const long ln = (long)n;
    int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for num_threads(nt) schedule(dynamic, 16)
    for (long i = 0; i < ln; ++i) {
        double sx = 0, sy = 0, sz = 0, sp = 0;
        const double xi = x[i], yi = y[i], zi = z[i];
        for (long j = 0; j < ln; ++j) {
            if (j == i) continue;
            double dx = (double)x[j] - xi, dy = (double)y[j] - yi, dz = (double)z[j] - zi;
            double s2 = dx * dx + dy * dy + dz * dz + e2;
            if (!(s2 > 0)) continue;
            double inv = 1 / sqrt(s2);
            double f = m[j] * inv * inv * inv;
            sx += f * dx; sy += f * dy; sz += f * dz;
            sp += m[j] * inv;
        }
        ax[i] = G * sx; ay[i] = G * sy; az[i] = G * sz;
        if (pot) pot[i] = -G * sp;
    }
}

/* ---- FP64 adjoint of the direct-sum KDK leapfrog ---------------------------------------------
 * The reference has no adjoint; this is the project's own FP64 restatement of the discrete
 * adjoint, used only to check the GPU adjoint. The forward map is the reference's step order
 * (src/simulation.cpp:416-419): forces at x0, then per step kick(dt/2), drift(dt),
 * forces, kick(dt/2). Loss L = sum_i m_i |x_i(T) - xstar_i|^2.
 *
 * Accelerations a_i = G sum_{j!=i} m_j K(x_j - x_i), K(d) = d / s^3, s^2 = |d|^2 + eps^2.
 * Vector-Jacobian products for an adjoint w on a:
 *   dL/dx_k += G sum_{j!=k} M(x_j - x_k) (m_k w_j - m_j w_k),  M(d) u = u/s^3 - 3 d (d.u)/s^5
 *   dL/dm_k += -G sum_{j!=k} w_j . (x_j - x_k)/s^3  ... written below as G sum_j w_j . K(x_k - x_j)
 */
static void accel_fp64(long n, const double* x, const double* m, double G, double e2, double* a, int nt) {
#pragma omp parallel for num_threads(nt) schedule(static)
    for (long i = 0; i < n; ++i) {
        double s0 = 0, s1 = 0, s2 = 0;
        for (long j = 0; j < n; ++j) {
            if (j == i) continue;
            double dx = x[3 * j] - x[3 * i], dy = x[3 * j + 1] - x[3 * i + 1], dz = x[3 * j + 2] - x[3 * i + 2];
            double r2 = dx * dx + dy * dy + dz * dz + e2;
            if (!(r2 > 0)) continue;
            double inv = 1 / sqrt(r2), f = m[j] * inv * inv * inv;
            s0 += f * dx; s1 += f * dy; s2 += f * dz;
        }
        a[3 * i] = G * s0; a[3 * i + 1] = G * s1; a[3 * i + 2] = G * s2;
    }
}

/* gx += J^T w (positions), gm += (da/dm)^T w. */
static void vjp_fp64(long n, const double* x, const double* m, double G, double e2, const double* w, double* gx,
                     double* gm, int nt) {
#pragma omp parallel for num_threads(nt) schedule(static)
    for (long k = 0; k < n; ++k) {
        double g0 = 0, g1 = 0, g2 = 0, h = 0;
        for (long j = 0; j < n; ++j) {
            if (j == k) continue;
            double dx = x[3 * j] - x[3 * k], dy = x[3 * j + 1] - x[3 * k + 1], dz = x[3 * j + 2] - x[3 * k + 2];
            double r2 = dx * dx + dy * dy + dz * dz + e2;
            if (!(r2 > 0)) continue;
            double inv = 1 / sqrt(r2), inv3 = inv * inv * inv, inv5 = inv3 * inv * inv;
            double ux = m[k] * w[3 * j] - m[j] * w[3 * k];
            double uy = m[k] * w[3 * j + 1] - m[j] * w[3 * k + 1];
            double uz = m[k] * w[3 * j + 2] - m[j] * w[3 * k + 2];
            double du = dx * ux + dy * uy + dz * uz;
            g0 += ux * inv3 - 3 * dx * du * inv5;
            g1 += uy * inv3 - 3 * dy * du * inv5;
            g2 += uz * inv3 - 3 * dz * du * inv5;
            /* a_j depends on m_k through G m_k K(x_k - x_j) = -G m_k K(d). */
            h -= (w[3 * j] * dx + w[3 * j + 1] * dy + w[3 * j + 2] * dz) * inv3;
        }
        gx[3 * k] += G * g0; gx[3 * k + 1] += G * g1; gx[3 * k + 2] += G * g2;
        gm[k] += G * h;
    }
}

static double forward_fp64(long n, double* x, double* v, const double* m, double G, double e2, double dt, int steps,
                           double* traj, int nt) {
    double* a = malloc((size_t)n * 3 * sizeof(double));
    if (!a) abort();
    accel_fp64(n, x, m, G, e2, a, nt);
    if (traj) memcpy(traj, x, (size_t)n * 3 * sizeof(double));
    for (int s = 0; s < steps; ++s) {
        for (long k = 0; k < 3 * n; ++k) v[k] += 0.5 * dt * a[k];
        for (long k = 0; k < 3 * n; ++k) x[k] += dt * v[k];
        accel_fp64(n, x, m, G, e2, a, nt);
        for (long k = 0; k < 3 * n; ++k) v[k] += 0.5 * dt * a[k];
        if (traj) memcpy(traj + (size_t)(s + 1) * n * 3, x, (size_t)n * 3 * sizeof(double));
    }
    free(a);
    return 0;
}

static double loss_of(long n, const double* x, const double* m, const double* xstar) {
    double L = 0;
    for (long i = 0; i < n; ++i) {
        double dx = x[3 * i] - xstar[3 * i], dy = x[3 * i + 1] - xstar[3 * i + 1], dz = x[3 * i + 2] - xstar[3 * i + 2];
        L += m[i] * (dx * dx + dy * dy + dz * dz);
    }
    return L;
}

double or_loss_direct_fp64(size_t n, const double* x0, const double* v0, const double* m, double G, double eps,
                           double dt, int steps, const double* xstar, int threads) {
    int nt = threads > 0 ? threads : omp_get_max_threads();
    long ln = (long)n;
    double* x = malloc(n * 3 * sizeof(double));
    double* v = malloc(n * 3 * sizeof(double));
    if (!x || !v) abort();
    memcpy(x, x0, n * 3 * sizeof(double));
    memcpy(v, v0, n * 3 * sizeof(double));
    forward_fp64(ln, x, v, m, G, eps * eps, dt, steps, NULL, nt);
    double L = loss_of(ln, x, m, xstar);
    free(x); free(v);
    return L;
}

double or_adjoint_direct_fp64(size_t n, const double* x0, const double* v0, const double* m, double G, double eps,
                              double dt, int steps, const double* xstar, double* gx, double* gv, double* gm,
                              int threads) {
    int nt = threads > 0 ? threads : omp_get_max_threads();
    long ln = (long)n;
    const double e2 = eps * eps;
    size_t n3 = n * 3;
    double* traj = malloc((size_t)(steps + 1) * n3 * sizeof(double));
    double* x = malloc(n3 * sizeof(double));
    double* v = malloc(n3 * sizeof(double));
    double* w = malloc(n3 * sizeof(double));
    if (!traj || !x || !v || !w) abort();
    memcpy(x, x0, n3 * sizeof(double));
    memcpy(v, v0, n3 * sizeof(double));
    forward_fp64(ln, x, v, m, G, e2, dt, steps, traj, nt);
    double L = loss_of(ln, x, m, xstar);
    /* Terminal adjoints. */
    double* lx = gx;
    double* lv = gv;
    for (long i = 0; i < ln; ++i) {
        for (int c = 0; c < 3; ++c) {
            lx[3 * i + c] = 2 * m[i] * (x[3 * i + c] - xstar[3 * i + c]);
            lv[3 * i + c] = 0;
        }
        double dx = x[3 * i] - xstar[3 * i], dy = x[3 * i + 1] - xstar[3 * i + 1], dz = x[3 * i + 2] - xstar[3 * i + 2];
        gm[i] = dx * dx + dy * dy + dz * dz;
    }
    /* Reverse sweep. Step s maps (x_s, v_s) -> (x_{s+1}, v_{s+1}):
     *   vh = v + h a(x_s); x' = x + dt vh; v' = vh + h a(x'), h = dt/2.
     * Reverse: lvh = lv'; lx' += J(x')^T (h lv'); lx = lx'; lvh += dt lx'; lv = lvh;
     *          lx += J(x_s)^T (h lvh). */
    for (int s = steps - 1; s >= 0; --s) {
        const double* xs1 = traj + (size_t)(s + 1) * n3;
        const double* xs = traj + (size_t)s * n3;
        for (size_t k = 0; k < n3; ++k) w[k] = 0.5 * dt * lv[k];
        vjp_fp64(ln, xs1, m, G, e2, w, lx, gm, nt);
        for (size_t k = 0; k < n3; ++k) lv[k] += dt * lx[k];
        for (size_t k = 0; k < n3; ++k) w[k] = 0.5 * dt * lv[k];
        vjp_fp64(ln, xs, m, G, e2, w, lx, gm, nt);
    }
    free(traj); free(x); free(v); free(w);
    return L;
}

/* ---- FP64 tree forces over frozen interaction lists --------------------------------------------
 * Test oracle of the engine's tree adjoint (no reference counterpart). For every force call of a
 * trajectory the caller passes the tree the engine built: its sorted body order (position -> id),
 * node ranges and children (the reference node layout), the FP32 centres of mass and rcrit2 its
 * opening test used, and the walk groups with their boxes. The interaction lists are rebuilt with
 * the walk's opening rule (src/cpu_backend.cpp:816-838) in the same FP32 arithmetic, so they are
 * the engine's lists; the forces then use them in FP64 with every cell's moments recomputed from
 * the current positions (M = sum m, com = sum m x / M, Q = sum m (3 e e^T - |e|^2 I)):
 *   a_i = G [sum_cells M d/r^3 - Q d/r^5 + 5/2 (d.Q.d) d/r^7 + sum_bodies m_j d/r^3],
 *   d = X - x_i, r^2 = |d|^2 + eps^2.
 * or_frozen_loss runs the KDK steps with the step-s lists at force call s and returns
 * L = sum m |x_T - x*|^2; central differences of it check the engine's adjoint. */
typedef struct {
    uint32_t nn, ng;
    uint32_t* range4;    /* 4 per node */
    uint32_t* perm;      /* n */
    uint32_t* glohi;     /* 2 per group */
    uint32_t* coff;      /* ng + 1: cells of group g at cells[coff[g] .. coff[g+1]) */
    uint32_t* cells;
    uint32_t* boff;      /* ng + 1: body ranges of group g at branges[2 boff[g] ..) */
    uint32_t* branges;
} fz_step;

struct or_frozen {
    size_t n;
    int steps;
    fz_step* st;
};

typedef struct {
    uint32_t* p;
    size_t n, cap;
} u32vec;

static void u32_push(u32vec* v, uint32_t x) {
    if (v->n == v->cap) {
        v->cap = v->cap ? 2 * v->cap : 256;
        v->p = realloc(v->p, v->cap * 4);
        if (!v->p) abort();
    }
    v->p[v->n++] = x;
}

or_frozen* or_frozen_create(size_t n, int steps, const uint32_t* nn, const uint32_t* ng, const uint32_t* perm_all,
                            const uint32_t* range4_all, const float* comrc_all, const uint32_t* glohi_all,
                            const float* gbox_all) {
    or_frozen* f = calloc(1, sizeof(or_frozen));
    if (!f) abort();
    f->n = n;
    f->steps = steps;
    f->st = calloc((size_t)steps, sizeof(fz_step));
    if (!f->st) abort();
    size_t no = 0, go = 0;
    for (int s = 0; s < steps; ++s) {
        fz_step* t = &f->st[s];
        t->nn = nn[s];
        t->ng = ng[s];
        t->range4 = malloc((size_t)t->nn * 16);
        t->perm = malloc(n * 4);
        t->glohi = malloc((size_t)t->ng * 8);
        t->coff = malloc(((size_t)t->ng + 1) * 4);
        t->boff = malloc(((size_t)t->ng + 1) * 4);
        if (!t->range4 || !t->perm || !t->glohi || !t->coff || !t->boff) abort();
        memcpy(t->range4, range4_all + 4 * no, (size_t)t->nn * 16);
        memcpy(t->perm, perm_all + (size_t)s * n, n * 4);
        memcpy(t->glohi, glohi_all + 2 * go, (size_t)t->ng * 8);
        const float* crc = comrc_all + 4 * no;
        const float* gbox = gbox_all + 6 * go;
        u32vec cells = {0}, br = {0}, stack = {0};
        for (uint32_t g = 0; g < t->ng; ++g) {
            t->coff[g] = (uint32_t)cells.n;
            t->boff[g] = (uint32_t)(br.n / 2);
            const uint32_t glo = t->glohi[2 * g], ghi = t->glohi[2 * g + 1];
            const float bx = gbox[6 * g], by = gbox[6 * g + 1], bz = gbox[6 * g + 2];
            const float hx = gbox[6 * g + 3], hy = gbox[6 * g + 4], hz = gbox[6 * g + 5];
            stack.n = 0;
            u32_push(&stack, 0);
            while (stack.n) {
                const uint32_t nd = stack.p[--stack.n];
                const uint32_t* r = t->range4 + 4 * nd;
                const float* c = crc + 4 * nd;
                const float dx = fmaxf(fabsf(c[0] - bx) - hx, 0.f);
                const float dy = fmaxf(fabsf(c[1] - by) - hy, 0.f);
                const float dz = fmaxf(fabsf(c[2] - bz) - hz, 0.f);
                const float d2 = sq3f(dx, dy, dz);
                const int contains = r[0] <= glo && ghi <= r[1];
                const int leaf = r[3] == 0;
                if (!contains && d2 >= c[3]) {
                    if (leaf && r[1] - r[0] <= 4) { u32_push(&br, r[0]); u32_push(&br, r[1]); }
                    else u32_push(&cells, nd);
                } else if (leaf) {
                    u32_push(&br, r[0]); u32_push(&br, r[1]);
                } else {
                    for (uint32_t k = 0; k < r[3]; ++k) u32_push(&stack, r[2] + k);
                }
            }
        }
        t->coff[t->ng] = (uint32_t)cells.n;
        t->boff[t->ng] = (uint32_t)(br.n / 2);
        t->cells = cells.p;
        t->branges = br.p;
        free(stack.p);
        no += t->nn;
        go += t->ng;
    }
    return f;
}

void or_frozen_destroy(or_frozen* f) {
    if (!f) return;
    for (int s = 0; s < f->steps; ++s) {
        fz_step* t = &f->st[s];
        free(t->range4); free(t->perm); free(t->glohi); free(t->coff); free(t->cells); free(t->boff);
        free(t->branges);
    }
    free(f->st);
    free(f);
}

/* Forces of force call s at positions x (3 per id), masses m (per id). */
static void frozen_accel(const or_frozen* f, int s, const double* x, const double* m, double G, double e2, double* a,
                         double* mom /* 10 per node */, int nt) {
    const fz_step* t = &f->st[s];
    const long nn = (long)t->nn;
#pragma omp parallel for num_threads(nt) schedule(dynamic, 64)
    for (long c = 0; c < nn; ++c) {
        const uint32_t lo = t->range4[4 * c], hi = t->range4[4 * c + 1];
        double M = 0, sx = 0, sy = 0, sz = 0;
        for (uint32_t p = lo; p < hi; ++p) {
            const uint32_t j = t->perm[p];
            M += m[j]; sx += m[j] * x[3 * j]; sy += m[j] * x[3 * j + 1]; sz += m[j] * x[3 * j + 2];
        }
        const double cx = M > 0 ? sx / M : 0, cy = M > 0 ? sy / M : 0, cz = M > 0 ? sz / M : 0;
        double q[6] = {0, 0, 0, 0, 0, 0};
        for (uint32_t p = lo; p < hi; ++p) {
            const uint32_t j = t->perm[p];
            const double ex = x[3 * j] - cx, ey = x[3 * j + 1] - cy, ez = x[3 * j + 2] - cz;
            const double r2 = ex * ex + ey * ey + ez * ez;
            q[0] += m[j] * (3 * ex * ex - r2); q[1] += m[j] * 3 * ex * ey; q[2] += m[j] * 3 * ex * ez;
            q[3] += m[j] * (3 * ey * ey - r2); q[4] += m[j] * 3 * ey * ez; q[5] += m[j] * (3 * ez * ez - r2);
        }
        double* o = mom + 10 * c;
        o[0] = M; o[1] = cx; o[2] = cy; o[3] = cz;
        for (int k = 0; k < 6; ++k) o[4 + k] = q[k];
    }
    const long ng = (long)t->ng;
#pragma omp parallel for num_threads(nt) schedule(dynamic, 4)
    for (long g = 0; g < ng; ++g) {
        for (uint32_t p = t->glohi[2 * g]; p < t->glohi[2 * g + 1]; ++p) {
            const uint32_t i = t->perm[p];
            const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
            double ax = 0, ay = 0, az = 0;
            for (uint32_t k = t->coff[g]; k < t->coff[g + 1]; ++k) {
                const double* o = mom + 10 * t->cells[k];
                const double dx = o[1] - xi, dy = o[2] - yi, dz = o[3] - zi;
                const double r2 = dx * dx + dy * dy + dz * dz + e2;
                const double inv = 1 / sqrt(r2), inv2 = inv * inv, inv3 = inv * inv2, inv5 = inv3 * inv2;
                const double inv7 = inv5 * inv2;
                const double qx = o[4] * dx + o[5] * dy + o[6] * dz;
                const double qy = o[5] * dx + o[7] * dy + o[8] * dz;
                const double qz = o[6] * dx + o[8] * dy + o[9] * dz;
                const double dqd = dx * qx + dy * qy + dz * qz;
                const double fr = o[0] * inv3 + 2.5 * dqd * inv7;
                ax += fr * dx - qx * inv5;
                ay += fr * dy - qy * inv5;
                az += fr * dz - qz * inv5;
            }
            for (uint32_t k = t->boff[g]; k < t->boff[g + 1]; ++k) {
                for (uint32_t q = t->branges[2 * k]; q < t->branges[2 * k + 1]; ++q) {
                    const uint32_t j = t->perm[q];
                    if (j == i) continue;
                    const double dx = x[3 * j] - xi, dy = x[3 * j + 1] - yi, dz = x[3 * j + 2] - zi;
                    const double r2 = dx * dx + dy * dy + dz * dz + e2;
                    if (!(r2 > 0)) continue;
                    const double inv = 1 / sqrt(r2), fr = m[j] * inv * inv * inv;
                    ax += fr * dx; ay += fr * dy; az += fr * dz;
                }
            }
            a[3 * i] = G * ax; a[3 * i + 1] = G * ay; a[3 * i + 2] = G * az;
        }
    }
}

double or_frozen_loss(const or_frozen* f, const double* x0, const double* v0, const double* m, double G, double eps,
                      double dt, const double* xstar, int threads) {
    const int nt = threads > 0 ? threads : omp_get_max_threads();
    const size_t n = f->n, n3 = 3 * n;
    uint32_t maxnn = 1;
    for (int s = 0; s < f->steps; ++s) maxnn = f->st[s].nn > maxnn ? f->st[s].nn : maxnn;
    double* x = malloc(n3 * 8);
    double* v = malloc(n3 * 8);
    double* a = malloc(n3 * 8);
    double* mom = malloc((size_t)maxnn * 80);
    if (!x || !v || !a || !mom) abort();
    memcpy(x, x0, n3 * 8);
    memcpy(v, v0, n3 * 8);
    const double e2 = eps * eps, h = 0.5 * dt;
    frozen_accel(f, 0, x, m, G, e2, a, mom, nt);
    for (int s = 0; s < f->steps; ++s) {
        for (size_t k = 0; k < n3; ++k) v[k] += h * a[k];
        for (size_t k = 0; k < n3; ++k) x[k] += dt * v[k];
        if (s + 1 < f->steps) {
            frozen_accel(f, s + 1, x, m, G, e2, a, mom, nt);
            for (size_t k = 0; k < n3; ++k) v[k] += h * a[k];
        }
    }
    const double L = loss_of((long)n, x, m, xstar);
    free(x); free(v); free(a); free(mom);
    return L;
}

/* Accelerations of force call s at positions x (3 per id) over its frozen lists (3 per id out). */
void or_frozen_accel(const or_frozen* f, int s, const double* x, const double* m, double G, double eps, double* a,
                     int threads) {
    const int nt = threads > 0 ? threads : omp_get_max_threads();
    uint32_t nn = f->st[s].nn ? f->st[s].nn : 1;
    double* mom = malloc((size_t)nn * 80);
    if (!mom) abort();
    frozen_accel(f, s, x, m, G, eps * eps, a, mom, nt);
    free(mom);
}

/* ---- FP64 block (hierarchical) time steps, direct forces ----------------------------------------
 * Test oracle of the engine's block steps (no reference counterpart): `steps` steps of dt, each of
 * 2^K substeps. At substep boundary s, bodies whose level k has s a multiple of 2^(K-k) get the
 * opening half kick dt/2^k/2; every body drifts by dt/2^K; at boundary s+1 the bodies ending a
 * step get fresh forces, the closing half kick and a new level: the smallest k with
 * dt/2^k <= eta sqrt(eps/|a|), i.e. k = ceil(log2((dt/eta) sqrt(|a|/eps))) by frexp, clamped to
 * [kmin, K] with kmin = K - trailing zeros of s+1 (0 at the end of the step). Positions, velocities
 * and accelerations in FP64; x, v (3 per body) are updated in place, levels written to level. */
static int or_level_for(const double* a, double dt, double eta, double eps, int kmin, int kmax) {
    const double am = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (!(am > 0)) return kmin;
    const double r = dt / eta * sqrt(am / eps);
    if (!(r > 1)) return kmin;
    int e = 0;
    const double f = frexp(r, &e);
    int k = f == 0.5 ? e - 1 : e;
    return k < kmin ? kmin : (k > kmax ? kmax : k);
}

static int or_tz(unsigned v) {
    int t = 0;
    while (v && !(v & 1u)) { v >>= 1; ++t; }
    return t;
}

void or_block_direct_fp64(size_t n, double* x, double* v, const double* m, double G, double eps, double dt, int K,
                          double eta, int steps, uint8_t* level, int threads) {
    const int nt = threads > 0 ? threads : omp_get_max_threads();
    const long ln = (long)n;
    const double e2 = eps * eps, epsl = eps > 0 ? eps : 1e-30;
    double* a = malloc(n * 3 * sizeof(double));
    if (!a) abort();
    accel_fp64(ln, x, m, G, e2, a, nt);
    for (long i = 0; i < ln; ++i) level[i] = (uint8_t)or_level_for(a + 3 * i, dt, eta, epsl, 0, K);
    const unsigned sub = 1u << K;
    const double ds = ldexp(dt, -K);
    for (int st = 0; st < steps; ++st) {
        for (unsigned s = 0; s < sub; ++s) {
            const int kopen = s == 0 ? 0 : K - or_tz(s);
            for (long i = 0; i < ln; ++i)
                if (level[i] >= kopen) {
                    const double h = 0.5 * ldexp(dt, -level[i]);
                    for (int c = 0; c < 3; ++c) v[3 * i + c] += h * a[3 * i + c];
                }
            for (long k = 0; k < 3 * ln; ++k) x[k] += ds * v[k];
            const unsigned s1 = s + 1;
            const int kclose = s1 == sub ? 0 : K - or_tz(s1);
            double* an = malloc(n * 3 * sizeof(double));
            if (!an) abort();
            accel_fp64(ln, x, m, G, e2, an, nt);
            for (long i = 0; i < ln; ++i)
                if (level[i] >= kclose) {
                    for (int c = 0; c < 3; ++c) a[3 * i + c] = an[3 * i + c];
                    const double h = 0.5 * ldexp(dt, -level[i]);
                    for (int c = 0; c < 3; ++c) v[3 * i + c] += h * a[3 * i + c];
                    level[i] = (uint8_t)or_level_for(a + 3 * i, dt, eta, epsl, kclose, K);
                }
            free(an);
        }
    }
    free(a);
}
