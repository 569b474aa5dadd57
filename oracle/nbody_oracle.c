/*
 * nbody_oracle.c -- CPU restatement of the drons/nbody force path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Nothing in the product links or
 * calls this file; it is loaded by tests/, __graft_entry__.smoke() and the
 * CPU legs of bench.py.  Compiled with -ffp-contract=off so that every
 * operation rounds as written, like a non-contracting build of the reference.
 *
 * Parity pin: the solver restatements below reproduce the reference's golden
 * vectors test/data/{euler,rk4,rkdp,rkdp-corr,rkck,rkf}.txt from
 * test/data/initial_state.txt at the reference tolerance (1e-12 abs,
 * test/solver/test_nbody_solver.cpp:74-85).
 */
#include "nbody_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MIN_DISTANCE 1e-8 /* nbody/nbtype.h:79 (compared with r^2) */
#define ORC_BLOCK 64          /* nbody/nbtype.h:77 NBODY_DATA_BLOCK_SIZE */

/* ------------------------------------------------------------------------ */
/* heap index algebra -- nbody/nbody_space_heap_func_priv.h:4-73            */
/* ------------------------------------------------------------------------ */
uint64_t orc_left_idx(uint64_t idx) { return idx << 1; }
uint64_t orc_rght_idx(uint64_t idx) { return (idx << 1) + 1; }
uint64_t orc_parent_idx(uint64_t idx) { return idx >> 1; }

/* Shift out the trailing run of 1 bits (walk up while 'right'), then step to
 * the right sibling.  For an all-ones index this lands on the root (1). */
uint64_t orc_next_down(uint64_t idx)
{
    uint64_t inv = ~idx;
    int tz = 0;
    while (tz < 64 && ((inv >> tz) & 1u) == 0) ++tz;
    idx = (tz >= 64) ? 0 : (idx >> tz);
    return idx + 1;
}
uint64_t orc_skip_idx(uint64_t idx) { return orc_next_down(idx); }
uint64_t orc_next_up(uint64_t idx, uint64_t tree_size)
{
    uint64_t left = orc_left_idx(idx);
    if (left < tree_size) return left;
    return orc_next_down(idx);
}

/* ------------------------------------------------------------------------ */
/* pair force -- nbody/nbody_data.cpp:35-44 (G = 1)                          */
/* ------------------------------------------------------------------------ */
void orc_force(const double v1[3], const double v2[3], double m1, double m2,
               double out[3])
{
    double dx = v1[0] - v2[0], dy = v1[1] - v2[1], dz = v1[2] - v2[2];
    double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < ORC_MIN_DISTANCE) r2 = ORC_MIN_DISTANCE;
    double k = ((-1.0 * m1) * m2) / (r2 * sqrt(r2));
    out[0] = dx * k;
    out[1] = dy * k;
    out[2] = dz * k;
}

/* ------------------------------------------------------------------------ */
/* direct engines                                                            */
/* ------------------------------------------------------------------------ */
static void simple_row(size_t n, const double* y, const double* mass,
                       double* f, size_t b1)
{
    const double* rx = y;
    const double* ry = y + n;
    const double* rz = y + 2 * n;
    double v1[3] = {rx[b1], ry[b1], rz[b1]};
    double tf[3] = {0.0, 0.0, 0.0};
    for (size_t b2 = 0; b2 != n; ++b2) {
        if (b1 == b2) continue;
        double v2[3] = {rx[b2], ry[b2], rz[b2]};
        double fo[3];
        orc_force(v1, v2, mass[b1], mass[b2], fo);
        tf[0] += fo[0];
        tf[1] += fo[1];
        tf[2] += fo[2];
    }
    f[b1] = y[3 * n + b1];
    f[n + b1] = y[4 * n + b1];
    f[2 * n + b1] = y[5 * n + b1];
    f[3 * n + b1] = tf[0] / mass[b1];
    f[4 * n + b1] = tf[1] / mass[b1];
    f[5 * n + b1] = tf[2] / mass[b1];
}

/* nbody/nbody_engine_simple.cpp:116-173, nbody/nbody_engine_openmp.cpp:19-77 */
void orc_fcompute_simple(size_t n, const double* y, const double* mass,
                         double* f, int nthreads)
{
    if (nthreads <= 1) {
        for (size_t b1 = 0; b1 < n; ++b1) simple_row(n, y, mass, f, b1);
        return;
    }
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (long long b1 = 0; b1 < (long long)n; ++b1)
        simple_row(n, y, mass, f, (size_t)b1);
}

/* nbody/nbody_engine_block.cpp:51-125 with tail blocks */
void orc_fcompute_block(size_t n, const double* y, const double* mass,
                        double* f, int nthreads)
{
    orc_fcompute_block_range(n, y, mass, f, 0, n, nthreads);
}

void orc_fcompute_block_range(size_t n, const double* y, const double* mass,
                              double* f, size_t row0, size_t row1, int nthreads)
{
    const double* rx = y;
    const double* ry = y + n;
    const double* rz = y + 2 * n;
    long long b0 = (long long)(row0 / ORC_BLOCK);
    long long nblocks = (long long)((row1 + ORC_BLOCK - 1) / ORC_BLOCK);
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) schedule(dynamic, 1)
    for (long long ib = b0; ib < nblocks; ++ib) {
        size_t n1 = (size_t)ib * ORC_BLOCK;
        size_t c1 = (n - n1 < ORC_BLOCK) ? n - n1 : ORC_BLOCK;
        double x1[ORC_BLOCK], y1[ORC_BLOCK], z1[ORC_BLOCK];
        double fx[ORC_BLOCK], fy[ORC_BLOCK], fz[ORC_BLOCK];
        for (size_t b1 = 0; b1 != c1; ++b1) {
            x1[b1] = rx[n1 + b1];
            y1[b1] = ry[n1 + b1];
            z1[b1] = rz[n1 + b1];
            fx[b1] = fy[b1] = fz[b1] = 0.0;
        }
        for (size_t n2 = 0; n2 < n; n2 += ORC_BLOCK) {
            size_t c2 = (n - n2 < ORC_BLOCK) ? n - n2 : ORC_BLOCK;
            double x2[ORC_BLOCK], y2[ORC_BLOCK], z2[ORC_BLOCK], m2[ORC_BLOCK];
            for (size_t b2 = 0; b2 != c2; ++b2) {
                x2[b2] = rx[n2 + b2];
                y2[b2] = ry[n2 + b2];
                z2[b2] = rz[n2 + b2];
                m2[b2] = mass[n2 + b2];
            }
            for (size_t b1 = 0; b1 != c1; ++b1) {
                for (size_t b2 = 0; b2 != c2; ++b2) {
                    double dx = x1[b1] - x2[b2];
                    double dy = y1[b1] - y2[b2];
                    double dz = z1[b1] - z2[b2];
                    double r2 = dx * dx + dy * dy + dz * dz;
                    if (r2 < ORC_MIN_DISTANCE) r2 = ORC_MIN_DISTANCE;
                    double r = sqrt(r2);
                    double coeff = m2[b2] / (r * r2);
                    fx[b1] -= dx * coeff;
                    fy[b1] -= dy * coeff;
                    fz[b1] -= dz * coeff;
                }
            }
        }
        for (size_t b1 = 0; b1 != c1; ++b1) {
            size_t i = n1 + b1;
            f[i] = y[3 * n + i];
            f[n + i] = y[4 * n + i];
            f[2 * n + i] = y[5 * n + i];
            f[3 * n + i] = fx[b1];
            f[4 * n + i] = fy[b1];
            f[5 * n + i] = fz[b1];
        }
    }
}

/* Softened FP64 direct sum for selected rows (error judge, no reference
 * counterpart: the softened form of the block kernel's pair term). */
void orc_accel_rows(size_t n, const double* y, const double* mass, double eps,
                    const int64_t* rows, size_t nrows, double* acc,
                    int nthreads)
{
    const double* rx = y;
    const double* ry = y + n;
    const double* rz = y + 2 * n;
    const double eps2 = eps * eps;
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) schedule(dynamic, 4)
    for (long long r = 0; r < (long long)nrows; ++r) {
        size_t i = rows ? (size_t)rows[r] : (size_t)r;
        double xi = rx[i], yi = ry[i], zi = rz[i];
        double ax = 0.0, ay = 0.0, az = 0.0;
        for (size_t j = 0; j < n; ++j) {
            if (j == i) continue;
            double dx = rx[j] - xi, dy = ry[j] - yi, dz = rz[j] - zi;
            double r2 = dx * dx + dy * dy + dz * dz + eps2;
            if (r2 < ORC_MIN_DISTANCE) r2 = ORC_MIN_DISTANCE;
            double inv = 1.0 / sqrt(r2);
            double s = mass[j] * inv * inv * inv;
            ax += dx * s;
            ay += dy * s;
            az += dz * s;
        }
        acc[3 * r + 0] = ax;
        acc[3 * r + 1] = ay;
        acc[3 * r + 2] = az;
    }
}

/* ------------------------------------------------------------------------ */
/* buffer algebra                                                            */
/* ------------------------------------------------------------------------ */
/* nbody/nbody_engine_simple.cpp:245-264 */
void orc_fill(double* a, double v, size_t n)
{
    for (size_t i = 0; i < n; ++i) a[i] = v;
}
/* nbody/nbody_engine_simple.cpp:266-291 */
void orc_fmadd_inplace(double* a, const double* b, double c, size_t n)
{
    for (size_t i = 0; i < n; ++i) a[i] += b[i] * c;
}
/* nbody/nbody_engine_simple.cpp:293-339 */
void orc_fmadd(double* a, const double* b, const double* c, double d, size_t n)
{
    for (size_t i = 0; i < n; ++i) a[i] = b[i] + c[i] * d;
}
/* nbody/nbody_engine.cpp:47-66: zero coefficients are skipped */
void orc_fmaddn_inplace(double* a, const double* const* b, const double* c,
                        size_t csize, size_t n)
{
    if (c == NULL) return;
    for (size_t k = 0; k != csize; ++k) {
        if (c[k] == 0.0) continue;
        orc_fmadd_inplace(a, b[k], c[k], n);
    }
}
/* nbody/nbody_engine.cpp:75-115: b == NULL means a = sum */
void orc_fmaddn(double* a, const double* b, const double* const* c,
                const double* d, size_t dsize, size_t n)
{
    if (d == NULL) return;
    int init = 0;
    if (b == NULL) {
        orc_fill(a, 0.0, n);
        init = 1;
    }
    for (size_t k = 0; k != dsize; ++k) {
        if (d[k] == 0.0) continue;
        if (init)
            orc_fmadd(a, a, c[k], d[k], n);
        else
            orc_fmadd(a, b, c[k], d[k], n);
        init = 1;
    }
}
/* nbody/nbody_engine_simple.cpp:341-394 with summation_k (summation.h:8-14) */
void orc_fmaddn_corr(double* a, double* corr, const double* const* b,
                     const double* c, size_t csize, size_t n)
{
    if (c == NULL) return;
    for (size_t i = 0; i < n; ++i) {
        for (size_t k = 0; k < csize; ++k) {
            if (c[k] == 0.0) continue;
            volatile double term = b[k][i] * c[k];
            volatile double corrected = term - corr[i];
            volatile double new_sum = a[i] + corrected;
            corr[i] = (new_sum - a[i]) - corrected;
            a[i] = new_sum;
        }
    }
}
/* nbody/nbody_engine_simple.cpp:396-419 (0 for an empty buffer, as the CUDA
 * engine nbody/nbody_engine_cuda.cpp:509-514) */
double orc_fmaxabs(const double* a, size_t n)
{
    if (n == 0) return 0.0;
    double r = fabs(a[0]);
    for (size_t i = 0; i < n; ++i) {
        double v = fabs(a[i]);
        if (v > r) r = v;
    }
    return r;
}
/* nbody/nbody_engine_simple.cpp:175-199: first 3*count entries only */
void orc_clamp(double* y, size_t count, double b)
{
    double diam = 2.0 * b;
    for (size_t i = 0; i < 3 * count; ++i) {
        if (y[i] > +b) y[i] -= diam;
        if (y[i] < -b) y[i] += diam;
    }
}

/* ------------------------------------------------------------------------ */
/* kd heap                                                                   */
/* ------------------------------------------------------------------------ */
int orc_heap_alloc(orc_heap* h, size_t count)
{
    memset(h, 0, sizeof(*h));
    h->count = count;
    h->size = 2 * count;
    h->com = (double*)calloc(3 * h->size, sizeof(double));
    h->mass = (double*)calloc(h->size, sizeof(double));
    h->r2 = (double*)calloc(h->size, sizeof(double));
    h->bmin = (double*)calloc(3 * h->size, sizeof(double));
    h->bmax = (double*)calloc(3 * h->size, sizeof(double));
    h->body_n = (int64_t*)malloc(h->size * sizeof(int64_t));
    if (!h->com || !h->mass || !h->r2 || !h->bmin || !h->bmax || !h->body_n) {
        orc_heap_free(h);
        return -1;
    }
    for (size_t i = 0; i < h->size; ++i) h->body_n[i] = -1;
    return 0;
}

void orc_heap_free(orc_heap* h)
{
    free(h->com);
    free(h->mass);
    free(h->r2);
    free(h->bmin);
    free(h->bmax);
    free(h->body_n);
    memset(h, 0, sizeof(*h));
}

static double vlen(double x, double y, double z) { return sqrt(x * x + y * y + z * z); }

/* nbody/nbody_space_heap.cpp:119-134 */
static void heap_update(orc_heap* h, size_t idx, size_t l, size_t r)
{
    double* c = h->com;
    h->mass[idx] = h->mass[l] + h->mass[r];
    for (int d = 0; d < 3; ++d)
        c[3 * idx + d] = (c[3 * l + d] * h->mass[l] + c[3 * r + d] * h->mass[r]) / h->mass[idx];
    for (int d = 0; d < 3; ++d) {
        double a = h->bmin[3 * l + d], b = h->bmin[3 * r + d];
        h->bmin[3 * idx + d] = (b < a) ? b : a;
        a = h->bmax[3 * l + d];
        b = h->bmax[3 * r + d];
        h->bmax[3 * idx + d] = (a < b) ? b : a;
    }
    const double* mn = h->bmin + 3 * idx;
    const double* mx = h->bmax + 3 * idx;
    double rr = vlen(mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]) * 0.5 +
                vlen((mx[0] + mn[0]) / 2 - c[3 * idx + 0],
                     (mx[1] + mn[1]) / 2 - c[3 * idx + 1],
                     (mx[2] + mn[2]) / 2 - c[3 * idx + 2]);
    h->r2[idx] = (rr * rr) * h->lambda2;
}

static const double* g_sort_key; /* qsort has no context argument */
static int cmp_by_key(const void* pa, const void* pb)
{
    int64_t a = *(const int64_t*)pa, b = *(const int64_t*)pb;
    double ka = g_sort_key[a], kb = g_sort_key[b];
    if (ka < kb) return -1;
    if (kb < ka) return 1;
    return (a < b) ? -1 : (a > b);
}

/* nbody/nbody_space_heap.cpp:136-190: the left child takes the count/2
 * smallest bodies along the current axis (nth_element; here a full sort with
 * index tie-break, which yields the same subsets for distinct keys). */
static void heap_build_p(orc_heap* h, size_t count, int64_t* ind,
                         const double* r[3], const double* mass, size_t idx,
                         int dim)
{
    if (count == 1) {
        int64_t b = ind[0];
        for (int d = 0; d < 3; ++d) {
            h->com[3 * idx + d] = r[d][b];
            h->bmin[3 * idx + d] = r[d][b];
            h->bmax[3 * idx + d] = r[d][b];
        }
        h->mass[idx] = mass[b];
        h->body_n[idx] = b;
        return;
    }
    size_t left = count / 2;
    g_sort_key = r[dim];
    qsort(ind, count, sizeof(int64_t), cmp_by_key);
    int nd = (dim + 1) % 3;
    heap_build_p(h, left, ind, r, mass, 2 * idx, nd);
    heap_build_p(h, count - left, ind + left, r, mass, 2 * idx + 1, nd);
    heap_update(h, idx, 2 * idx, 2 * idx + 1);
}

int orc_heap_build(orc_heap* h, size_t count, const double* rx,
                   const double* ry, const double* rz, const double* mass,
                   double lambda)
{
    if (count == 0 || (count & (count - 1)) != 0) return -1; /* 2^k only */
    if (h->count != count) {
        orc_heap_free(h);
        if (orc_heap_alloc(h, count) != 0) return -2;
    }
    int64_t* ind = (int64_t*)malloc(count * sizeof(int64_t));
    if (!ind) return -2;
    for (size_t i = 0; i < count; ++i) ind[i] = (int64_t)i;
    h->lambda2 = lambda * lambda;
    const double* r[3] = {rx, ry, rz};
    heap_build_p(h, count, ind, r, mass, 1, 0);
    free(ind);
    return 0;
}

/* nbody/nbody_space_heap.cpp:39-62 */
void orc_heap_rebuild(orc_heap* h, size_t count, const double* rx,
                      const double* ry, const double* rz, double lambda)
{
    h->lambda2 = lambda * lambda;
    for (size_t idx = count; idx < 2 * count; ++idx) {
        int64_t b = h->body_n[idx];
        double p[3] = {rx[b], ry[b], rz[b]};
        for (int d = 0; d < 3; ++d) {
            h->com[3 * idx + d] = p[d];
            h->bmin[3 * idx + d] = p[d];
            h->bmax[3 * idx + d] = p[d];
        }
    }
    for (size_t lc = count; lc > 0; lc /= 2)
        for (size_t idx = lc / 2; idx < lc; ++idx)
            heap_update(h, idx, 2 * idx, 2 * idx + 1);
}

static double dist2(const double a[3], const double* b)
{
    double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return dx * dx + dy * dy + dz * dz;
}

/* nbody/nbody_space_heap.cpp:64-97 */
void orc_heap_traverse(const orc_heap* h, const double v1[3], double m1,
                       double out[3])
{
    size_t stack[64];
    size_t sp = 0;
    out[0] = out[1] = out[2] = 0.0;
    stack[sp++] = 1;
    while (sp != 0) {
        size_t curr = stack[--sp];
        double d2 = dist2(v1, h->com + 3 * curr);
        if (d2 > h->r2[curr]) {
            double fo[3];
            orc_force(v1, h->com + 3 * curr, m1, h->mass[curr], fo);
            out[0] += fo[0];
            out[1] += fo[1];
            out[2] += fo[2];
        } else {
            size_t l = 2 * curr, r = 2 * curr + 1;
            if (r < h->size && sp < 64) stack[sp++] = r;
            if (l < h->size && sp < 64) stack[sp++] = l;
        }
    }
}

/* nbody/nbody_space_heap_stackless.cpp:3-28 */
void orc_heap_traverse_stackless(const orc_heap* h, const double v1[3],
                                 double m1, double out[3])
{
    uint64_t curr = 1;
    out[0] = out[1] = out[2] = 0.0;
    do {
        double d2 = dist2(v1, h->com + 3 * curr);
        if (d2 > h->r2[curr]) {
            double fo[3];
            orc_force(v1, h->com + 3 * curr, m1, h->mass[curr], fo);
            out[0] += fo[0];
            out[1] += fo[1];
            out[2] += fo[2];
            curr = orc_skip_idx(curr);
        } else {
            curr = orc_next_up(curr, h->size);
        }
    } while (curr != 1);
}

uint64_t orc_heap_visits(const orc_heap* h, const double v1[3])
{
    uint64_t curr = 1, visits = 0;
    do {
        ++visits;
        double d2 = dist2(v1, h->com + 3 * curr);
        curr = (d2 > h->r2[curr]) ? orc_skip_idx(curr) : orc_next_up(curr, h->size);
    } while (curr != 1);
    return visits;
}

/* nbody/nbody_engine_simple_bh.cpp:16-93 */
int orc_fcompute_bh(orc_heap* h, int layout, int traverse, size_t step,
                    size_t build_rate, double lambda, size_t n,
                    const double* y, const double* mass, double* f,
                    int nthreads)
{
    const double* rx = y;
    const double* ry = y + n;
    const double* rz = y + 2 * n;
    if (build_rate == 0 || h->count == 0 || (step % build_rate) == 0) {
        int rc = orc_heap_build(h, n, rx, ry, rz, mass, lambda);
        if (rc != 0) return rc;
    } else {
        orc_heap_rebuild(h, n, rx, ry, rz, lambda);
    }
    long long total = (long long)n;
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) schedule(dynamic, 4)
    for (long long t = 0; t < total; ++t) {
        size_t b1;
        double v1[3];
        if (traverse == 0) { /* cycle: body order, position from y */
            b1 = (size_t)t;
            v1[0] = rx[b1];
            v1[1] = ry[b1];
            v1[2] = rz[b1];
        } else { /* nested_tree: leaf order, position from the leaf */
            size_t idx = n + (size_t)t;
            b1 = (size_t)h->body_n[idx];
            v1[0] = h->com[3 * idx + 0];
            v1[1] = h->com[3 * idx + 1];
            v1[2] = h->com[3 * idx + 2];
        }
        double tf[3];
        double m1 = mass[b1];
        if (layout == 2)
            orc_heap_traverse_stackless(h, v1, m1, tf);
        else
            orc_heap_traverse(h, v1, m1, tf);
        f[b1] = y[3 * n + b1];
        f[n + b1] = y[4 * n + b1];
        f[2 * n + b1] = y[5 * n + b1];
        f[3 * n + b1] = tf[0] / m1;
        f[4 * n + b1] = tf[1] / m1;
        f[5 * n + b1] = tf[2] / m1;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* conservation checks -- nbody/nbody_data.cpp:57-145                        */
/* ------------------------------------------------------------------------ */
typedef struct { double s, c; } kahan;
/* nbody/summation.h:8-14 */
static void kadd(kahan* k, double v)
{
    double corrected = v - k->c;
    double ns = k->s + corrected;
    k->c = (ns - k->s) - corrected;
    k->s = ns;
}

/* nbody/nbody_data.cpp:46-55 */
static double potential_pair(const double* y, const double* mass, size_t n,
                             size_t b1, size_t b2)
{
    double dx = y[b1] - y[b2], dy = y[n + b1] - y[n + b2], dz = y[2 * n + b1] - y[2 * n + b2];
    double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < ORC_MIN_DISTANCE) return 0.0;
    return -((1.0 * mass[b1]) * mass[b2]) / sqrt(r2);
}

void orc_statistics(size_t n, const double* y, const double* mass,
                    double out[12], int nthreads)
{
    (void)nthreads;
    const double *rx = y, *ry = y + n, *rz = y + 2 * n;
    const double *vx = y + 3 * n, *vy = y + 4 * n, *vz = y + 5 * n;
    kahan P[3] = {{0, 0}, {0, 0}, {0, 0}}, L[3] = {{0, 0}, {0, 0}, {0, 0}};
    kahan C[3] = {{0, 0}, {0, 0}, {0, 0}}, KE = {0, 0}, PE = {0, 0}, M = {0, 0};
    /* summation() starts from element 0 and Kahan-adds the rest
     * (nbody/summation.h:20-47); starting from 0 + element 0 is identical. */
    for (size_t i = 0; i < n; ++i) {
        double m = mass[i];
        double px = vx[i] * m, py = vy[i] * m, pz = vz[i] * m;
        kadd(&P[0], px);
        kadd(&P[1], py);
        kadd(&P[2], pz);
        /* r ^ (v m) : nbody/vertex.h cross product */
        kadd(&L[0], ry[i] * pz - rz[i] * py);
        kadd(&L[1], rz[i] * px - rx[i] * pz);
        kadd(&L[2], rx[i] * py - ry[i] * px);
        kadd(&KE, (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]) * m);
        kadd(&C[0], rx[i] * m);
        kadd(&C[1], ry[i] * m);
        kadd(&C[2], rz[i] * m);
        kadd(&M, m);
    }
    for (size_t k = 0; k < n * n; ++k) {
        size_t b1 = k / n, b2 = k % n;
        kadd(&PE, (b1 == b2) ? 0.0 : potential_pair(y, mass, n, b1, b2));
    }
    for (int d = 0; d < 3; ++d) {
        out[d] = P[d].s;
        out[3 + d] = L[d].s;
        out[8 + d] = C[d].s / M.s;
    }
    out[6] = KE.s / 2;
    out[7] = PE.s / 2;
    out[11] = M.s;
}

/* ------------------------------------------------------------------------ */
/* solvers over the oracle 'simple' engine (callers of the engine API)       */
/* ------------------------------------------------------------------------ */
typedef struct {
    int steps;
    const double* a; /* [steps][steps] row-major, lower triangle used */
    const double* b1;
    const double* b2;
    const double* c;
} orc_table;

/* Dormand-Prince 5(4): nbody/nbody_solver_rkdp.cpp:30-62 */
static const double DP_A[7 * 7] = {
    0, 0, 0, 0, 0, 0, 0,
    1.0 / 5, 0, 0, 0, 0, 0, 0,
    3.0 / 40, 9.0 / 40, 0, 0, 0, 0, 0,
    44.0 / 45, -56.0 / 15, 32.0 / 9, 0, 0, 0, 0,
    19372.0 / 6561, -25360.0 / 2187, 64448.0 / 6561, -212.0 / 729, 0, 0, 0,
    9017.0 / 3168, -355.0 / 33, 46732.0 / 5247, 49.0 / 176, -5103.0 / 18656, 0, 0,
    35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84, 0};
static const double DP_B1[7] = {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84, 0};
static const double DP_B2[7] = {5179.0 / 57600, 0, 7571.0 / 16695, 393.0 / 640, -92097.0 / 339200, 187.0 / 2100, 1.0 / 40};
static const double DP_C[7] = {0, 1.0 / 5, 3.0 / 10, 4.0 / 5, 8.0 / 9, 1, 1};

/* Cash-Karp: nbody/nbody_solver_rkck.cpp:30-62 */
static const double CK_A[6 * 6] = {
    0, 0, 0, 0, 0, 0,
    1.0 / 5, 0, 0, 0, 0, 0,
    3.0 / 40, 9.0 / 40, 0, 0, 0, 0,
    3.0 / 10, -9.0 / 10, 6.0 / 5, 0, 0, 0,
    -11.0 / 54, 5.0 / 2, -70.0 / 27, 35.0 / 27, 0, 0,
    1631.0 / 55296, 175.0 / 512, 575.0 / 13824, 44275.0 / 110592, 253.0 / 4096, 0};
static const double CK_B1[6] = {37.0 / 378, 0, 250.0 / 621, 125.0 / 594, 0, 512.0 / 1771};
static const double CK_B2[6] = {2825.0 / 27648, 0, 18575.0 / 48384, 13525.0 / 55296, 277.0 / 14336, 1.0 / 4};
static const double CK_C[6] = {0, 1.0 / 5, 3.0 / 10, 3.0 / 5, 1, 7.0 / 8};

/* Fehlberg 7(8): nbody/nbody_solver_rkf.cpp:30-71 */
static const double F_A[13 * 13] = {
    0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
    2.0 / 27, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
    1.0 / 36, 1.0 / 12, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
    1.0 / 24, 0, 1.0 / 8, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
    5.0 / 12, 0, -25.0 / 16, 25.0 / 16, 0, 0, 0, 0, 0, 0, 0, 0, 0,
    1.0 / 20, 0, 0, 1.0 / 4, 1.0 / 5, 0, 0, 0, 0, 0, 0, 0, 0,
    -25.0 / 108, 0, 0, 125.0 / 108, -65.0 / 27, 125.0 / 54, 0, 0, 0, 0, 0, 0, 0,
    31.0 / 300, 0, 0, 0, 61.0 / 225, -2.0 / 9, 13.0 / 900, 0, 0, 0, 0, 0, 0,
    2.0, 0, 0, -53.0 / 6, 704.0 / 45, -107.0 / 9, 67.0 / 90, 3.0, 0, 0, 0, 0, 0,
    -91.0 / 108, 0, 0, 23.0 / 108, -976.0 / 135, 311.0 / 54, -19.0 / 60, 17.0 / 6, -1.0 / 12, 0, 0, 0, 0,
    2383.0 / 4100, 0, 0, -341.0 / 164, 4496.0 / 1025, -301.0 / 82, 2133.0 / 4100, 45.0 / 82, 45.0 / 164, 18.0 / 41, 0, 0, 0,
    3.0 / 205, 0, 0, 0, 0, -6.0 / 41, -3.0 / 205, -3.0 / 41, 3.0 / 41, 6.0 / 41, 0, 0, 0,
    -1777.0 / 4100, 0, 0, -341.0 / 164, 4496.0 / 1025, -289.0 / 82, 2193.0 / 4100, 51.0 / 82, 33.0 / 164, 12.0 / 41, 0, 1.0, 0};
static const double F_B1[13] = {41.0 / 840, 0, 0, 0, 0, 34.0 / 105, 9.0 / 35, 9.0 / 35, 9.0 / 280, 9.0 / 280, 41.0 / 840, 0, 0};
static const double F_B2[13] = {0, 0, 0, 0, 0, 34.0 / 105, 9.0 / 35, 9.0 / 35, 9.0 / 280, 9.0 / 280, 0, 41.0 / 840, 41.0 / 840};
static const double F_C[13] = {0, 2.0 / 27, 1.0 / 9, 1.0 / 6, 5.0 / 12, 1.0 / 2, 5.0 / 6, 1.0 / 6, 2.0 / 3, 1.0 / 3, 1, 0, 1};

typedef struct {
    size_t n, ps;
    const double* mass;
    uint64_t fcount;
    /* butcher state: nbody/nbody_solver_rk_butcher.h */
    const orc_table* bt;
    double** k;
    double* t;
    double** ystack;
    double* ycorr;
    double* tcorr;
    size_t max_recursion, subdiv;
    double err_thr, min_step;
    int correction;
} orc_solver;

static void s_fcompute(orc_solver* s, const double* y, double* f)
{
    orc_fcompute_simple(s->n, y, s->mass, f, 1);
    s->fcount++;
}

/* nbody/nbody_solver_rk_butcher.cpp:130-162 */
static void sub_step_explicit(orc_solver* s, const double* y, double* coeff, double dt)
{
    const orc_table* bt = s->bt;
    for (int i = 0; i < bt->steps; ++i) {
        if (i == 0) {
            s_fcompute(s, y, s->k[0]);
        } else {
            for (int n = 0; n != i; ++n) coeff[n] = dt * bt->a[i * bt->steps + n];
            if (s->correction) {
                memcpy(s->tcorr, s->ycorr, s->ps * sizeof(double));
                memcpy(s->t, y, s->ps * sizeof(double));
                orc_fmaddn_corr(s->t, s->tcorr, (const double* const*)s->k, coeff, (size_t)i, s->ps);
            } else {
                orc_fmaddn(s->t, y, (const double* const*)s->k, coeff, (size_t)i, s->ps);
            }
            s_fcompute(s, s->t, s->k[i]);
        }
    }
}

/* nbody/nbody_solver_rk_butcher.cpp:164-248 */
static void sub_step(orc_solver* s, size_t substeps, double t, double dt, double* y,
                     size_t level)
{
    const orc_table* bt = s->bt;
    double coeff[16];
    for (size_t sub = 0; sub != substeps; ++sub, t += dt) {
        sub_step_explicit(s, y, coeff, dt);
        double max_error = 0.0;
        for (int n = 0; n != bt->steps; ++n) coeff[n] = bt->b2[n] - bt->b1[n];
        orc_fmaddn(s->t, NULL, (const double* const*)s->k, coeff, (size_t)bt->steps, s->ps);
        max_error = orc_fmaxabs(s->t, s->ps);
        int can = (level < s->max_recursion) && dt > s->min_step;
        int need = max_error > s->err_thr;
        if (can && need) {
            double ndt = dt / (double)s->subdiv;
            double* cy = s->ystack[level];
            memcpy(cy, y, s->ps * sizeof(double));
            sub_step(s, s->subdiv, t, ndt, cy, level + 1);
            memcpy(y, cy, s->ps * sizeof(double));
        } else {
            for (int n = 0; n != bt->steps; ++n) coeff[n] = bt->b2[n] * dt;
            if (s->correction)
                orc_fmaddn_corr(y, s->ycorr, (const double* const*)s->k, coeff, (size_t)bt->steps, s->ps);
            else
                orc_fmaddn_inplace(y, (const double* const*)s->k, coeff, (size_t)bt->steps, s->ps);
        }
    }
}

static double* dalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

int orc_solver_run(const char* name, size_t n, double* y, const double* mass,
                   double* t_io, double max_time, double min_step,
                   double max_step, size_t max_recursion,
                   size_t substep_subdivisions, double error_threshold,
                   int correction, uint64_t* fcompute_count)
{
    static const orc_table DP = {7, DP_A, DP_B1, DP_B2, DP_C};
    static const orc_table CK = {6, CK_A, CK_B1, CK_B2, CK_C};
    static const orc_table FE = {13, F_A, F_B1, F_B2, F_C};
    orc_solver s;
    memset(&s, 0, sizeof(s));
    s.n = n;
    s.ps = 6 * n;
    s.mass = mass;
    s.max_recursion = max_recursion;
    s.subdiv = substep_subdivisions;
    s.err_thr = error_threshold;
    s.min_step = min_step;
    s.correction = correction;
    int kind;
    if (strcmp(name, "euler") == 0) kind = 0;
    else if (strcmp(name, "rk4") == 0) kind = 1;
    else if (strcmp(name, "rkdp") == 0) { kind = 2; s.bt = &DP; }
    else if (strcmp(name, "rkck") == 0) { kind = 2; s.bt = &CK; }
    else if (strcmp(name, "rkf") == 0) { kind = 2; s.bt = &FE; }
    else return -1;

    double t = *t_io;
    double dt = max_step; /* nbody/nbody_solver.cpp:58 */
    double* tmp = dalloc(s.ps);
    double* kk[13] = {0};
    int nk = (kind == 1) ? 4 : (kind == 2 ? s.bt->steps : 1);
    for (int i = 0; i < nk; ++i) kk[i] = dalloc(s.ps);
    s.k = kk;
    s.t = tmp;
    double** ys = NULL;
    if (kind == 2) {
        ys = (double**)calloc(max_recursion ? max_recursion : 1, sizeof(double*));
        for (size_t i = 0; i < max_recursion; ++i) ys[i] = dalloc(s.ps);
        s.ystack = ys;
        if (correction) {
            s.ycorr = dalloc(s.ps);
            s.tcorr = dalloc(s.ps);
        }
    }
    while (t < max_time) {
        if (kind == 0) { /* nbody/nbody_solver_euler.cpp:19-31 */
            s_fcompute(&s, y, kk[0]);
            orc_fmadd_inplace(y, kk[0], dt, s.ps);
        } else if (kind == 1) { /* nbody/nbody_solver_rk4.cpp:19-48 */
            s_fcompute(&s, y, kk[0]);
            orc_fmadd(tmp, y, kk[0], dt / 2.0, s.ps);
            s_fcompute(&s, tmp, kk[1]);
            orc_fmadd(tmp, y, kk[1], dt / 2.0, s.ps);
            s_fcompute(&s, tmp, kk[2]);
            orc_fmadd(tmp, y, kk[2], dt, s.ps);
            s_fcompute(&s, tmp, kk[3]);
            const double co[4] = {dt / 6.0, dt / 3.0, dt / 3.0, dt / 6.0};
            orc_fmaddn_inplace(y, (const double* const*)kk, co, 4, s.ps);
        } else { /* nbody/nbody_solver_rk_butcher.cpp:60-67 */
            sub_step(&s, 1, t, dt, y, 0);
        }
        t += dt; /* nbody/nbody_data.cpp advise_time */
    }
    *t_io = t;
    if (fcompute_count) *fcompute_count = s.fcount;
    free(tmp);
    for (int i = 0; i < nk; ++i) free(kk[i]);
    if (ys) {
        for (size_t i = 0; i < max_recursion; ++i) free(ys[i]);
        free(ys);
    }
    free(s.ycorr);
    free(s.tcorr);
    return 0;
}
