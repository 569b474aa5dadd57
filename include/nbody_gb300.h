/*
 * nbody_gb300.h -- C ABI of the GB300 force engine for drons/nbody.
 *
 * The engine is a drop-in for the reference's `nbody_engine` interface
 * (nbody/nbody_engine.h:16-96): a reference-side adapter class subclasses
 * nbody_engine, registers under a new alias in nbody_create_engine
 * (nbody/nbody_engines.cpp:4-193) and forwards every virtual to the entry
 * point named beside it below.  Plain pointers and sizes only; every call
 * returns an nbg_status (the reference's CUDACHECK exit(3) becomes a status
 * plus a message from nbg_last_error).  One engine = one GPU, one stream.
 *
 * Buffers are engine-owned device allocations (the reference's `memory`
 * subclass, nbody/nbody_engine_cuda_memory.cpp:4-22).  Vector operations act
 * on size()/8 doubles of their first operand, as the reference CUDA engine
 * does (nbody/nbody_engine_cuda.cpp:368-530).  A handle that this engine did
 * not create is rejected with NBG_ERR_FOREIGN_BUFFER and no side effect --
 * the reference logs "x is not smemory" and returns
 * (test/engine/test_nbody_engine.cpp:761-1010).
 */
#ifndef NBODY_GB300_H
#define NBODY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NBG_ABI_VERSION 1

typedef enum nbg_status {
    NBG_OK = 0,
    NBG_ERR_INVALID_ARG = 1,     /* NULL or out-of-range argument */
    NBG_ERR_FOREIGN_BUFFER = 2,  /* handle not created by this engine */
    NBG_ERR_SIZE_MISMATCH = 3,   /* buffer smaller than the operation needs */
    NBG_ERR_OUT_OF_MEMORY = 4,   /* device or pinned allocation failed */
    NBG_ERR_CUDA = 5,            /* CUDA runtime error (message in last_error) */
    NBG_ERR_UNSUPPORTED = 6,     /* e.g. Barnes-Hut with N not a power of two */
    NBG_ERR_NOT_INITIALIZED = 7, /* nbg_init has not been called */
    NBG_ERR_DEVICE_TIMEOUT = 8,  /* a bounded device-side wait gave up */
    NBG_ERR_DEVICE_ERROR = 9,    /* a kernel reported an error flag */
    NBG_ERR_TOO_LARGE = 10       /* request exceeds a fixed, preallocated capacity */
} nbg_status;

typedef struct nbg_engine nbg_engine; /* opaque engine */
typedef struct nbg_buffer nbg_buffer; /* opaque device buffer */

enum nbg_algo { NBG_ALGO_DIRECT = 0, NBG_ALGO_BH = 1 };
enum nbg_precision {
    NBG_PREC_FP64 = 0,  /* FP64 pair math, reference operation order */
    NBG_PREC_MIXED = 1  /* FP32 pair math, compensated FP32 sums, FP64 state */
};
enum nbg_tree_layout { NBG_LAYOUT_HEAP = 1, NBG_LAYOUT_HEAP_STACKLESS = 2 };
enum nbg_traverse { NBG_TRAVERSE_CYCLE = 0, NBG_TRAVERSE_NESTED_TREE = 1 };

/* Engine parameters: the keys nbody_create_engine reads from its QVariantMap
 * (nbody/nbody_engines.cpp:21-76) plus the new engine's own keys. */
typedef struct nbg_params {
    uint32_t struct_size;       /* sizeof(nbg_params), set by nbg_params_default */
    int32_t device;             /* CUDA device ordinal ("device", default 0) */
    int32_t algo;               /* nbg_algo */
    int32_t precision;          /* nbg_precision */
    double softening;           /* Plummer epsilon; 0 = reference clamp r^2>=1e-8 only */
    double distance_to_node_radius_ratio; /* lambda = 1/theta (default 10) */
    uint64_t tree_build_rate;   /* 0 = rebuild every fcompute, else refit between builds */
    int32_t tree_layout;        /* nbg_tree_layout (default heap_stackless) */
    int32_t traverse_type;      /* nbg_traverse (default nested_tree) */
    int32_t learned;            /* 1 = apply the learned monopole correction (BH, mixed) */
    int32_t block_size;         /* accepted for key compatibility; must be 0 or >0 */
    double learned_tight_ratio; /* tight opening ratio lambda_t of the learned band (default 2) */
} nbg_params;

void nbg_params_default(nbg_params* p);
const char* nbg_status_string(nbg_status s);
int nbg_abi_version(void);

/* nbody_create_engine(param) for the new alias (nbody/nbody_engines.cpp:4) */
nbg_status nbg_engine_create(const nbg_params* p, nbg_engine** out);
/* ~nbody_engine */
void nbg_engine_destroy(nbg_engine* e);
/* nbody_engine::type_name (nbody/nbody_engine.h:40) */
const char* nbg_type_name(const nbg_engine* e);
/* Message of the last failing call on this engine ("" if none). */
const char* nbg_last_error(const nbg_engine* e);

/* nbody_engine::init (nbody/nbody_engine.h:43; nbody_engine_cuda.cpp:91-139).
 * vertices/velocities are AoS [count][3] like nbody_data. */
nbg_status nbg_init(nbg_engine* e, size_t count, const double* vertices,
                    const double* velocities, const double* mass);
/* nbody_engine::get_data (nbody/nbody_engine.h:45): engine y -> AoS arrays */
nbg_status nbg_get_data(nbg_engine* e, double* vertices, double* velocities);
/* nbody_engine::problem_size (= 6 N) and get_y */
size_t nbg_problem_size(const nbg_engine* e);
nbg_buffer* nbg_get_y(nbg_engine* e);

/* nbody_engine::fcompute (nbody/nbody_engine.h:61): f = [v ; a(y)].
 * `step` is the caller's nbody_data step, read by the tree_build_rate rule
 * (nbody/nbody_engine_simple_bh.cpp:53-60). */
nbg_status nbg_fcompute(nbg_engine* e, double t, uint64_t step,
                        const nbg_buffer* y, nbg_buffer* f);
/* nbody_engine::clamp (nbody/nbody_engine.h:63; nbody_engine_cuda_impl.cu:724-747) */
nbg_status nbg_clamp(nbg_engine* e, nbg_buffer* y, double b);

/* nbody_engine::create_buffer / free_buffer (nbody/nbody_engine.h:65-66) */
nbg_status nbg_create_buffer(nbg_engine* e, size_t bytes, nbg_buffer** out);
nbg_status nbg_free_buffer(nbg_engine* e, nbg_buffer* b);
/* nbody_engine::memory::size (nbody/nbody_engine.h:27) */
size_t nbg_buffer_size(const nbg_buffer* b);
/* Raw device address of a buffer (for callers that launch their own work). */
void* nbg_buffer_device_ptr(nbg_buffer* b);
/* read_buffer / write_buffer (nbody/nbody_engine.h:69-70): copy size() bytes.
 * read_buffer returns after the copy has landed in dst. */
nbg_status nbg_read_buffer(nbg_engine* e, void* dst, const nbg_buffer* src);
nbg_status nbg_write_buffer(nbg_engine* e, nbg_buffer* dst, const void* src);
/* copy_buffer a = b, equal sizes (nbody/nbody_engine_cuda.cpp:318-345) */
nbg_status nbg_copy_buffer(nbg_engine* e, nbg_buffer* a, const nbg_buffer* b);
/* fill_buffer a[i] = value over size()/8 doubles */
nbg_status nbg_fill_buffer(nbg_engine* e, nbg_buffer* a, double value);
/* fmadd_inplace a[i] += b[i]*c (nbody/nbody_engine.h:76) */
nbg_status nbg_fmadd_inplace(nbg_engine* e, nbg_buffer* a, const nbg_buffer* b,
                             double c);
/* fmadd a[i] = b[i] + c[i]*d (nbody/nbody_engine.h:78) */
nbg_status nbg_fmadd(nbg_engine* e, nbg_buffer* a, const nbg_buffer* b,
                     const nbg_buffer* c, double d);
/* fmaddn_inplace a[i] += sum_k b[k][i]*c[k], one fused pass
 * (nbody/nbody_engine.cpp:47-66: c == NULL is a no-op, zero c[k] skipped,
 * csize > bcount is an error). */
nbg_status nbg_fmaddn_inplace(nbg_engine* e, nbg_buffer* a,
                              const nbg_buffer* const* b, size_t bcount,
                              const double* c, size_t csize);
/* fmaddn_corr: Kahan-compensated fmaddn_inplace with per-element carry
 * (nbody/nbody_engine_simple.cpp:341-394) */
nbg_status nbg_fmaddn_corr(nbg_engine* e, nbg_buffer* a, nbg_buffer* corr,
                           const nbg_buffer* const* b, size_t bcount,
                           const double* c, size_t csize);
/* fmaddn a[i] = b[i] + sum_k c[k][i]*d[k]; b == NULL means a = sum
 * (nbody/nbody_engine.cpp:75-115), one fused pass */
nbg_status nbg_fmaddn(nbg_engine* e, nbg_buffer* a, const nbg_buffer* b,
                      const nbg_buffer* const* c, size_t ccount,
                      const double* d, size_t dsize);
/* fmaxabs result = max |a[i]| (0 for an empty buffer) */
nbg_status nbg_fmaxabs(nbg_engine* e, const nbg_buffer* a, double* result);

/* Wait for all work queued on the engine stream; reports device error flags. */
nbg_status nbg_synchronize(nbg_engine* e);
/* The engine's CUDA stream (cudaStream_t) for callers that order their own work. */
void* nbg_stream(nbg_engine* e);

/* Page-locked host memory for fast write_buffer / read_buffer. */
nbg_status nbg_host_alloc(size_t bytes, void** out);
void nbg_host_free(void* p);

/* ---- measurement (no reference counterpart) ---- */
/* Kernel ids for nbg_profile_query. */
enum nbg_kernel_id {
    NBG_K_DIRECT = 0,     /* direct-sum force kernel (either precision) */
    NBG_K_TREE_BUILD = 1, /* whole tree build/refit sequence */
    NBG_K_BH_WALK = 2,    /* Barnes-Hut traversal kernel */
    NBG_K_VECOPS = 3,     /* buffer algebra kernels */
    NBG_K_ENS_STEP = 4,   /* one whole ensemble RK step (graph launch) */
    NBG_K_JUDGE = 5,      /* the learned path's per-step judge */
    NBG_K_COUNT = 8
};
/* Enable CUDA-event timing of each kernel class on the engine stream. */
nbg_status nbg_profile_enable(nbg_engine* e, int enable);
/* Accumulated device time (ms) and launches of one kernel class; resets it. */
nbg_status nbg_profile_query(nbg_engine* e, int kernel_id, double* total_ms,
                             uint64_t* launches);
/* Conservation sums of print_statistics (nbody/nbody_data.cpp:57-145) on the
 * GPU in FP64: out = P[3], L[3], KE, PE (both halved as the reference does),
 * mass centre[3], total mass.  With softening eps > 0 the pair potential is
 * -m_i m_j / sqrt(r^2 + eps^2), the potential of the integrated force. */
nbg_status nbg_statistics(nbg_engine* e, const nbg_buffer* y, double out[12]);

/* Barnes-Hut walk counters since the last call (mixed walk): node visits
 * (per warp: every visit is one broadcast node load) and accepted
 * body-node interactions; resets them. */
nbg_status nbg_bh_counters(nbg_engine* e, uint64_t* visits, uint64_t* interactions);
/* Deepest per-warp node stack of the group walk since the last
 * nbg_bh_counters call (which resets it), and the stack capacity of the
 * current tree (48 entries per level + 32); a walk that would exceed the
 * capacity stops and reports NBG_ERR_DEVICE_ERROR. */
nbg_status nbg_bh_stack_peak(nbg_engine* e, uint64_t* peak, uint64_t* capacity);
/* Groups the group walk handed to the per-body fallback walk since the last
 * nbg_bh_counters call: a group walk gives up after "bh.test_cap" node tests
 * (default max(N / 4, 2^16)), which only groups spread over much of the
 * system reach, and its bodies are walked one by one. */
nbg_status nbg_bh_fallback_groups(nbg_engine* e, uint64_t* groups);
/* ---- learned monopole correction (no reference counterpart) ----
 * A 16 -> 64 -> 64 -> 3 GELU MLP (BF16 weights, FP32 accumulate) predicts,
 * for a body-cell interaction accepted at the engine's ratio lambda_l but
 * inside the band lambda_l < lambda <= learned_tight_ratio, the residual
 * between the cell's exact subtree acceleration and its monopole, in units
 * of m / s^2 (s = cell radius).  Its three outputs c weight the vectors
 * u/|u|, Q u/|u| and the mass-centre offset o of the features (g = c0 u/|u|
 * + c1 Q u/|u| + c2 o); nbg_learn_predict returns c.  Used when
 * nbg_params.learned = 1 (Barnes-Hut, mixed precision); tuning keys:
 * "learned.walk" 1 (default): the default group walk (64-body groups)
 * records each group's band cells and the network evaluates the band
 * (body, cell) rows in 128-row tiles on the tcgen05 tensor cores, the
 * per-body sums taken in a fixed order (with other walk settings --
 * "bh.walk" 0, "bh.group" 32 or 128, "bh.order" 2, "bh.acc_smem" 0,
 * "bh.freeze_within_step" 1 -- the learned path takes the per-body walk);
 * 0: the warp-coherent per-body walk with one mma.sync batch per band
 * cell; "learned.group" one sample per
 * (body, cell) (0, default) or per (warp, cell) at the warp centroid (1, on
 * the per-body walk); "learned.weighted" (0 default, 1: training loss
 * weighted by the cell's force scale (m / s^2)^2).
 * Judge and fallback: at the first fcompute of every engine step a direct
 * sum on a seeded sample of bodies ("learned.judge_samples", default 4096,
 * rounded down to a power of two; "learned.judge_seed", default 1) measures
 * the relative force error of the learned walk and of the plain walk at the
 * tight ratio learned_tight_ratio (theta = 0.5 by default) on the same
 * bodies; when the learned p99 is the larger, the plain walk (the engine's
 * Barnes-Hut path without the correction, tree rebuilt at the tight ratio)
 * computes that fcompute and every other fcompute of the step.
 * "learned.judge" = 0 turns the judge and the fallback off. */
size_t nbg_learn_param_count(void);
nbg_status nbg_learn_set_weights(nbg_engine* e, const float* w, size_t count);
nbg_status nbg_learn_get_weights(nbg_engine* e, float* w, size_t count);
/* Glorot-uniform initialisation from a seed (biases zero). */
nbg_status nbg_learn_init_weights(nbg_engine* e, uint64_t seed);
/* Build the tree of the engine's current state and append up to max_samples
 * (features, target) samples: exact subtree sums for in-band interactions of
 * randomly chosen bodies; cells with more than 2^max_subtree_log2 bodies
 * are skipped.  The samples follow the seeded order of the chosen bodies, so
 * equal states and seeds give equal samples. */
nbg_status nbg_learn_generate(nbg_engine* e, size_t max_samples, uint64_t seed,
                              int max_subtree_log2, size_t* produced);
size_t nbg_learn_sample_count(const nbg_engine* e);
/* Copy samples [offset, offset + count): x [count][16], t [count][4],
 * meta [count][2] = (body, cell); any output may be NULL. */
nbg_status nbg_learn_read_samples(nbg_engine* e, size_t offset, size_t count, float* x,
                                  float* t, int* meta);
nbg_status nbg_learn_clear_samples(nbg_engine* e);
/* Adam on the stored samples (MSE), cosine-decayed learning rate; a seeded
 * val_fraction of the samples is held out and scored at the end.  Gradients
 * are summed in a fixed order: equal samples and seeds give equal weights. */
nbg_status nbg_learn_train(nbg_engine* e, int epochs, size_t batch, double lr, uint64_t seed,
                           double val_fraction, double* train_mse, double* val_mse);
/* Sum of squared errors and the gradient of the mean loss over host samples
 * (x [count][16], t [count][4]) with the current weights: the training
 * kernels' forward and backward pass, for gradient checks. */
nbg_status nbg_learn_loss_grad(nbg_engine* e, const float* x, const float* t, size_t count,
                               double* loss_sum, float* grad);
/* Network outputs g (x [count][16] -> out [count][3]) with the inference
 * routine of the walk. */
nbg_status nbg_learn_predict(nbg_engine* e, const float* x, size_t count, float* out);
/* The same outputs from the tensor-core (tcgen05) inference of
 * "learned.walk" = 1: 128-row tiles, BF16 operands in shared memory, FP32
 * accumulators in tensor memory.  count <= 2^30. */
nbg_status nbg_learn_predict_tc(nbg_engine* e, const float* x, size_t count, float* out);
/* For checks of the tcgen05 layouts: each row's tensor-memory accumulators
 * of that forward pass, acc [count][144]: the first layer's D1 = X W1 + b1
 * (0..63), the second layer's D2 = GELU(D1) W2 + b2 (64..127) and the
 * third layer's D3 = GELU(D2) W3 + b3 (128..143; 131..143 zero); each
 * bias is added by the tensor core, as three BF16 terms against a block of
 * ones. */
nbg_status nbg_learn_tc_accumulators(nbg_engine* e, const float* x, size_t count, float* acc);
/* The judge's figures: out[0] engine step judged last, [1] p50 and [2] p99
 * relative error of the learned forces, [3] p50 and [4] p99 of the plain
 * walk at the tight ratio, [5] RMS learned, [6] RMS plain, [7] 1 when that
 * step ran the plain walk, [8] sampled bodies, [9] steps judged and [10]
 * steps that fell back since the engine was created.  All zero before the
 * first judged step.  count >= NBG_JUDGE_STATS. */
#define NBG_JUDGE_STATS 11
nbg_status nbg_learn_judge_stats(nbg_engine* e, double* out, size_t count);
/* Network rows the learned walk evaluated for band interactions (one per
 * body-cell pair, or per warp-cell pair with "learned.group" = 1) since the
 * last nbg_bh_counters call, which resets it. */
nbg_status nbg_learn_band_rows(nbg_engine* e, uint64_t* rows);
/* Body index of each leaf of the last tree (leaf order), [N]. */
nbg_status nbg_tree_leaves(nbg_engine* e, int* body_of_leaf);

/* Number of kernels this engine has launched since creation. */
uint64_t nbg_launch_count(const nbg_engine* e);

/* Tuning knobs (set by the autotuner or by hand; no reference counterpart).
 * Keys: "direct.symmetric" (1: each unordered pair evaluated once and
 *       applied to both bodies, the default; 0: one-sided kernel),
 *       "direct.sym_g" (4 or 3: packed A-body pairs per lane of the
 *       symmetric kernel; 3 runs 5 CTAs per SM),
 *       "direct.sym_blocks" (4 or 5: CTAs per SM the symmetric kernel's
 *       register budget is set for), "direct.sym_unroll" (1, 2, 4 or 8:
 *       unroll of its 32-step rotation loop, default 4),
 *       "direct.pairs_per_lane" (2 or 4 packed i-pairs per lane, one-sided),
 *       "direct.unroll" (2, 4 or 8: j-loop unroll),
 *       "direct.blocks_per_sm" (CTAs per SM of the persistent direct grid),
 *       "direct.uniform_mass" (1, the default: when every body has the same
 *       mass the symmetric kernel weights pairs by r^-3 alone and scales the
 *       sums by the mass once, in FP64; 0: the general kernel),
 *       "bh.walk" (1: group walk with interaction lists, 0: warp-coherent
 *       stackless walk) for the mixed-precision Barnes-Hut path,
 *       "bh.group" (64 (default), 32 or 128 bodies per warp in the group
 *       walk; 128 with monopole cells only),
 *       "bh.walk_npl" (node tests per lane and traversal step of the
 *       group walk: 2, the default with monopole cells, or 1, the default
 *       with quadrupole cells),
 *       "bh.build" (0: the reference's kd-median tree, always for FP64;
 *       mixed precision: 1 leaves in Morton order, 2 in Hilbert order (the
 *       default), every node the two halves of its range -- one sort
 *       instead of three, a different tree with compact cells),
 *       "bh.fp64_nodes" (mixed precision: 1 forms the FP64 node arrays as
 *       the FP64 path does; default 0, only the FP32 records the mixed walks
 *       read, from FP32 bounding boxes),
 *       "bh.test_cap" (node tests after which a group walk hands its bodies
 *       to the per-body walk; 0, the default, is "bh.test_cap_ratio"
 *       (default 2) times the median tests of 32 sampled groups of the
 *       current tree; curve trees only, the kd tree is not capped),
 *       "bh.order" (1: monopole cells as the reference; 2: accepted cells
 *       add their quadrupole term, from FP32 second moments per node),
 *       "bh.walk_blocks" (4, 5, 6 or 8: CTAs per SM the group walk's register
 *       budget is set for; the quadrupole walk of 64-body groups takes 3,
 *       its default, or 4), "bh.acc_smem" (1: the 64-body walk keeps its
 *       accumulators in shared memory, the default; 0: in registers),
 *       "bh.persistent" (1, the default: the group walk runs as many CTAs
 *       as fit at once, its warps taking groups from a counter; 0: one CTA
 *       per four groups),
 *       "bh.eval_unroll" (1, 2 or 4: unroll of the interaction-list loop of
 *       the 64-body walk, at 5 CTAs per SM with shared-memory accumulators
 *       or at 4 with register accumulators),
 *       "bh.refit_within_step" (0, the default: the reference's rule, a full
 *       build when tree_build_rate is 0 or step % rate == 0; 1: a full
 *       build at the first fcompute of each engine step and refits of that
 *       topology for the step's other stages),
 *       "bh.freeze_within_step" (1: as "bh.refit_within_step", and every
 *       acceptance test of the step uses the records of the step's build,
 *       so each body meets the same cells at every stage and its force is a
 *       smooth function of the positions; the default group walk only)). */
nbg_status nbg_tune_set(nbg_engine* e, const char* key, int64_t value);
nbg_status nbg_tune_get(nbg_engine* e, const char* key, int64_t* value);

/* Autotuner: times every candidate configuration of the engine's force path
 * (direct: symmetric / one-sided kernel, i-pairs per lane, unroll, CTAs per
 * SM; Barnes-Hut: walk form) on the current state, `reps` calls each after
 * one untimed call, with CUDA events; keeps the fastest in the tuning table
 * and writes a JSON report of all timings into report[report_len] (may be
 * NULL).  The engine must be initialized; results in y are not touched. */
nbg_status nbg_autotune(nbg_engine* e, int reps, char* report, size_t report_len);

/* ---- allocation-free direct sum (no counterpart in the reference) ----
 * For callers that must not allocate GPU memory -- e.g. a host application
 * that hands out all device memory from its own arena, or a time-critical
 * loop where an allocation and its implicit device synchronisation are not
 * allowed.  Computes f = [v ; a(y)] for n bodies with the mixed-precision
 * direct sum (FP32 pairs, compensated sums, FP64 in and out; softening >= 0,
 * 0 = the reference clamp r^2 >= 1e-8), exactly like nbg_fcompute of a
 * mixed-precision direct engine.  y (6n doubles), mass (n) and f (6n) are
 * device pointers on the current device; stream is a cudaStream_t (NULL =
 * the default stream).  It calls no allocator: the kernel's packed-body
 * scratch is a fixed array compiled into the library, present on every GPU
 * that loads it until the process exits, which caps n at
 * NBG_NOALLOC_MAX_BODIES (larger n returns NBG_ERR_TOO_LARGE and touches
 * nothing).  The first call on a device looks up that array's device address
 * (one-time set-up, with that device current).  Under CUDA's lazy module
 * loading (the default) the array and the kernel's code are placed on a GPU
 * when the library's direct-sum code is first used there, so when this call
 * is that first use, the CUDA driver loads the module inside it (its own
 * allocation, done once); a caller that must see no allocation at all in its
 * loop makes one call during set-up, or sets CUDA_MODULE_LOADING=EAGER.
 * Returns after f holds the result (the error word is read on `stream`).
 * All calls share the one array: calls that overlap on the GPU (from
 * several host threads or streams) race and must be serialised. */
#define NBG_NOALLOC_MAX_BODIES 131072
nbg_status nbg_direct_mixed_noalloc(const double* y, const double* mass, double* f,
                                    size_t n, double softening, void* stream);

/* ---- batched ensemble (no reference counterpart as a whole) ----
 * Many independent systems of uneven size, each integrated with its own
 * adaptive Dormand-Prince step (the rkdp table of
 * nbody/nbody_solver_rkdp.cpp:30-62) around the mixed-precision direct sum.
 * Per step and per system the device computes the embedded error
 * dt * max |sum (b2 - b1) k|, accepts (y += dt sum b2 k) or rejects, and sets
 * the next dt; one step is captured once as a CUDA graph and replayed.  The
 * same object stepping a single system is the engine-owned fused RK step. */
typedef struct nbg_ensemble nbg_ensemble;
typedef struct nbg_ensemble_params {
    uint32_t struct_size; /* sizeof(nbg_ensemble_params) */
    int32_t device;
    double softening;     /* Plummer epsilon (0 = reference clamp) */
    double tolerance;     /* per-system embedded error bound */
    double dt_initial;
    double dt_min;
    double dt_max;
    int32_t use_graph;    /* 1 = replay a captured CUDA graph per step */
} nbg_ensemble_params;
void nbg_ensemble_params_default(nbg_ensemble_params* p);
nbg_status nbg_ensemble_create(const nbg_ensemble_params* p, nbg_ensemble** out);
void nbg_ensemble_destroy(nbg_ensemble* s);
const char* nbg_ensemble_last_error(const nbg_ensemble* s);
/* counts[nsys]; vertices / velocities AoS [sum counts][3], systems concatenated. */
nbg_status nbg_ensemble_init(nbg_ensemble* s, size_t nsys, const uint32_t* counts,
                             const double* vertices, const double* velocities,
                             const double* mass);
/* Queue `steps` RK attempts for every system (asynchronous). */
nbg_status nbg_ensemble_step(nbg_ensemble* s, int steps);
nbg_status nbg_ensemble_synchronize(nbg_ensemble* s);
/* Per system (any pointer may be NULL): time, next dt, accepted, rejected. */
nbg_status nbg_ensemble_status(nbg_ensemble* s, double* t, double* dt, uint32_t* accepted,
                               uint32_t* rejected);
nbg_status nbg_ensemble_get_state(nbg_ensemble* s, double* vertices, double* velocities);
/* f = [v ; a] of the current state, SoA [6][sum counts] (parity checks). */
nbg_status nbg_ensemble_fcompute(nbg_ensemble* s, double* f);
/* 12 FP64 conservation sums per system (layout of nbg_statistics, softened
 * potential of the ensemble's softening). */
nbg_status nbg_ensemble_statistics(nbg_ensemble* s, double* out);
/* Tuning keys "ensemble.symmetric" (1, the default: every unordered pair of
 * a system evaluated once for both bodies, the reaction sums kept as
 * per-range partials and added in a fixed order, so results stay
 * bit-reproducible; the partials take sum_s ceil(N_s / (256 G)) N_s floats
 * per component, and above 8 GiB the one-sided kernel runs instead; 0: the
 * one-sided kernel), "ensemble.pairs_per_lane" (1
 * or 2: i-tile of 256 or 512 bodies per work unit), "ensemble.blocks_per_sm"
 * (0 = as many as fit),
 * "ensemble.unroll" (2, 4 or 8: j-loop unroll of the force kernel),
 * "ensemble.uniform_mass" (1, the default: when every system has equal
 * masses, pairs are weighted by r^-3 alone and each system's mass scales its
 * sums once, in FP64; 0: the mass-weighted kernel) and
 * "ensemble.hold_after_reject" (1, the default: a system's step may not grow
 * right after a rejected step; 0: it may, up to 5x) and
 * "ensemble.pi_control" (1: PI step control on accepted steps, fewer
 * rejections and smaller steps; 0, the default: the error of the current
 * step only); a change takes effect from the next step (the step graph is
 * captured again). */
nbg_status nbg_ensemble_tune_set(nbg_ensemble* s, const char* key, int64_t value);
/* Autotuner of the ensemble force kernel (tile shape and grid), timed on the
 * current state; keeps the fastest; JSON report as nbg_autotune. */
nbg_status nbg_ensemble_autotune(nbg_ensemble* s, int reps, char* report, size_t report_len);
uint64_t nbg_ensemble_launch_count(const nbg_ensemble* s);
/* Accumulated device time of the force kernel (then reset); enable/disable timing. */
nbg_status nbg_ensemble_profile(nbg_ensemble* s, int enable, double* force_ms,
                                uint64_t* force_launches);

/* ---- frame stream writer (nbody/nbody_data_stream.cpp) ----
 * Writes the reference's stream format: <base>.idx (header lines
 * "#coord_size 8", "#body_count N", "#box_size B", then one
 * "step<TAB>time<TAB>part<TAB>offset" line per frame), <base><part>.dat
 * (per frame N vertices then N velocities, 3 doubles per body; a new part
 * once the current one has reached max_part_size), <base>.col (4 floats per
 * body) and <base>.mass (N doubles).  Frames of engine state are queued on
 * the engine stream (transpose to the frame layout + copy into one of two
 * pinned buffers) and written by a host thread, so file writes overlap the
 * simulation. */
typedef struct nbg_stream_writer nbg_stream_writer;
/* nbody_data_stream::open (nbody/nbody_data_stream.cpp:168-196): makes the
 * directory, opens part 0 and the index.  e may be NULL (host frames only);
 * otherwise the writer uses e's stream and must be closed before e is
 * destroyed.
 * append != 0 continues the stream at <base>: the last part number is read
 * from its index and no header is written (the reference's append_to). */
nbg_status nbg_stream_open(nbg_engine* e, const char* base_name, int64_t max_part_size, int append,
                           nbg_stream_writer** out);
/* What the reference takes from nbody_data for the header
 * (nbody/nbody_data_stream.cpp:62-98): body count, box size, colours (4
 * floats per body; NULL writes zeros) and masses.  Required before writing. */
nbg_status nbg_stream_set_header(nbg_stream_writer* w, size_t count, uint64_t box_size,
                                 const float* colors, const double* mass);
/* nbody_data_stream::write (nbody/nbody_data_stream.cpp:107-160) for the
 * engine state y (an engine buffer): returns once the frame's copy is queued;
 * blocks only while both pinned buffers hold frames not yet written.  A
 * failed asynchronous write is reported by the next write, flush or close. */
nbg_status nbg_stream_write(nbg_stream_writer* w, const nbg_buffer* y, uint64_t step, double time);
/* The same for a frame in host memory (vertices and velocities, 3 doubles per
 * body), written before the call returns. */
nbg_status nbg_stream_write_host(nbg_stream_writer* w, const double* vertices,
                                 const double* velocities, uint64_t step, double time);
/* Waits until every queued frame is on disk. */
nbg_status nbg_stream_flush(nbg_stream_writer* w);
/* Flush, close the files and free the writer (nbody_data_stream::close). */
nbg_status nbg_stream_close(nbg_stream_writer* w);
const char* nbg_stream_last_error(const nbg_stream_writer* w);

/* FP32 FFMA throughput probe: runs a dependent-chain FMA kernel on the
 * engine's device and returns the measured FP32 FLOP/s (2 per FMA). */
nbg_status nbg_measure_fp32_peak(nbg_engine* e, double* flops);

#ifdef __cplusplus
}
#endif

#endif /* NBODY_GB300_H */
