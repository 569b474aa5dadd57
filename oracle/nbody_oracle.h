/*
 * nbody_oracle.h -- CPU restatement of the drons/nbody force path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GB300
 * engine: only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * reference legs of bench.py load it.  The product (libnbody_gb300.so)
 * never links, calls or falls back to it.
 *
 * Every function restates one piece of the reference in plain C and names
 * the reference file:line it follows.  Pinned against the reference's own
 * golden vectors (test/data/<solver>.txt, 16 bodies, t = 0.3, 1e-12 abs)
 * and the heap-index known answers of test/engine/test_nbody_engine.cpp.
 */
#ifndef NBODY_ORACLE_H
#define NBODY_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- heap index algebra: nbody/nbody_space_heap_func_priv.h:4-73 ---- */
uint64_t orc_left_idx(uint64_t idx);
uint64_t orc_rght_idx(uint64_t idx);
uint64_t orc_parent_idx(uint64_t idx);
uint64_t orc_next_down(uint64_t idx);
uint64_t orc_skip_idx(uint64_t idx);
uint64_t orc_next_up(uint64_t idx, uint64_t tree_size);

/* ---- pair force: nbody/nbody_data.cpp:35-44 ---- */
void orc_force(const double v1[3], const double v2[3], double m1, double m2,
               double out[3]);

/* ---- direct engines (state y = [rx|ry|rz|vx|vy|vz], f = [v|a]) ---- */
/* nbody/nbody_engine_simple.cpp:116-173 (nthreads=1) and
 * nbody/nbody_engine_openmp.cpp:19-77 (nthreads>1): same arithmetic. */
void orc_fcompute_simple(size_t n, const double* y, const double* mass,
                         double* f, int nthreads);
/* nbody/nbody_engine_block.cpp:14-126: 64x64 tiles, a = -sum m_j dr/r^3.
 * The reference needs n % 64 == 0; this restatement also handles tails. */
void orc_fcompute_block(size_t n, const double* y, const double* mass,
                        double* f, int nthreads);
/* The block engine restricted to the 64-row blocks covering [row0, row1):
 * a bounded sample of the same work for CPU timing. */
void orc_fcompute_block_range(size_t n, const double* y, const double* mass,
                              double* f, size_t row0, size_t row1,
                              int nthreads);
/* FP64 direct-sum accelerations for selected rows with Plummer softening
 * eps (r^2 + eps^2) and the reference clamp r^2 >= 1e-8 (nbtype.h:79).
 * Used as the error judge of the mixed-precision and Barnes-Hut paths.
 * rows == NULL means rows 0..nrows-1.  acc is [nrows][3]. */
void orc_accel_rows(size_t n, const double* y, const double* mass, double eps,
                    const int64_t* rows, size_t nrows, double* acc,
                    int nthreads);

/* ---- buffer algebra: nbody/nbody_engine.cpp:47-115 and
 *      nbody/nbody_engine_simple.cpp:245-419 ---- */
void orc_fill(double* a, double v, size_t n);
void orc_fmadd_inplace(double* a, const double* b, double c, size_t n);
void orc_fmadd(double* a, const double* b, const double* c, double d, size_t n);
void orc_fmaddn_inplace(double* a, const double* const* b, const double* c,
                        size_t csize, size_t n);
void orc_fmaddn(double* a, const double* b, const double* const* c,
                const double* d, size_t dsize, size_t n);
void orc_fmaddn_corr(double* a, double* corr, const double* const* b,
                     const double* c, size_t csize, size_t n);
double orc_fmaxabs(const double* a, size_t n);
void orc_clamp(double* y, size_t count, double b);

/* ---- kd heap: nbody/nbody_space_heap.cpp, nbody_space_heap_stackless.cpp ---- */
typedef struct orc_heap {
    size_t   count;       /* bodies (power of two) */
    size_t   size;        /* heap size = 2 * count */
    double*  com;         /* [size][3] */
    double*  mass;        /* [size] */
    double*  r2;          /* [size] critical radius squared (0 for leaves) */
    double*  bmin;        /* [size][3] */
    double*  bmax;        /* [size][3] */
    int64_t* body_n;      /* [size] body of a leaf, -1 for internal nodes */
    double   lambda2;     /* distance_to_node_radius_ratio ^ 2 */
} orc_heap;

int  orc_heap_alloc(orc_heap* h, size_t count);
void orc_heap_free(orc_heap* h);
/* build: nbody/nbody_space_heap.cpp:13-37,136-190 (median kd split x,y,z) */
int  orc_heap_build(orc_heap* h, size_t count, const double* rx,
                    const double* ry, const double* rz, const double* mass,
                    double lambda);
/* rebuild (refit): nbody/nbody_space_heap.cpp:39-62 */
void orc_heap_rebuild(orc_heap* h, size_t count, const double* rx,
                      const double* ry, const double* rz, double lambda);
/* stack walk nbody/nbody_space_heap.cpp:64-97 */
void orc_heap_traverse(const orc_heap* h, const double v1[3], double m1,
                       double out[3]);
/* stackless walk nbody/nbody_space_heap_stackless.cpp:3-28 */
void orc_heap_traverse_stackless(const orc_heap* h, const double v1[3],
                                 double m1, double out[3]);
/* simple_bh fcompute nbody/nbody_engine_simple_bh.cpp:16-93.
 * layout 1 = heap, 2 = heap_stackless; traverse 0 = cycle, 1 = nested_tree.
 * Builds when build_rate == 0 or h empty or step % build_rate == 0, else refits. */
int  orc_fcompute_bh(orc_heap* h, int layout, int traverse, size_t step,
                     size_t build_rate, double lambda, size_t n,
                     const double* y, const double* mass, double* f,
                     int nthreads);
/* Node visit count of the stackless walk for one body (for traffic models). */
uint64_t orc_heap_visits(const orc_heap* h, const double v1[3]);

/* ---- conservation checks: nbody/nbody_data.cpp:57-145,
 *      nbody/summation_proxy.h, nbody/summation.h:8-47 (Kahan) ----
 * out: P[3], L[3], kinetic, potential, mass_center[3], total_mass
 * (kinetic and potential already halved as in print_statistics). */
void orc_statistics(size_t n, const double* y, const double* mass,
                    double out[12], int nthreads);

/* ---- solvers (callers of the engine API) restated to pin the oracle
 *      against test/data goldens ----
 * name: euler | rk4 | rkdp | rkck | rkf.  Integrates y (6n, SoA) with the
 * reference 'simple' engine from t0 to max_time with the reference run loop
 * nbody/nbody_solver.cpp:55-105 (dt = max_step every advise).
 * Butcher params as nbody/nbody_solver_rk_butcher.cpp:130-248.
 * Returns 0 on success, -1 on unknown solver. t_io: in t0, out final time. */
int orc_solver_run(const char* name, size_t n, double* y, const double* mass,
                   double* t_io, double max_time, double min_step,
                   double max_step, size_t max_recursion,
                   size_t substep_subdivisions, double error_threshold,
                   int correction, uint64_t* fcompute_count);

#ifdef __cplusplus
}
#endif

#endif /* NBODY_ORACLE_H */
