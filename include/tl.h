/*
 * tl.h - C ABI of the GB300 tau-leaping engine (libtl.so).
 *
 * Plain C: no C++ or CUDA types cross this boundary.  Every array argument is
 * a HOST pointer; the library copies what it needs to the device and back.
 * No call ever exits the process: every failure is reported as a tl_status.
 *
 * Reference interface replaced (CSSL-UWM/tau_leaping, paths inside that
 * project):
 *   class Model                      tau_leaping/model.h:20-98
 *   Model::ReadXML                   tau_leaping/model.cpp:17-60
 *   Model::Clone / InitSeeds         tau_leaping/model.cu:766-775, :420-425
 *   Model::PerformCalc               tau_leaping/model.cu:640-737
 *   Model::Step and the leap helpers tau_leaping/model.cu:180-598
 *   CSRMatrixPacked::CompTau         tau_leaping/CSRMatrixPacked.cu:423-462
 *   CSRMatrixPacked::FireReactions   tau_leaping/CSRMatrixPacked.cu:494-503
 *   statistics (mean / stddev grid)  tau_leaping/statistics.cpp:15-111
 *
 * Threading: one model handle per host thread.  Calls on one handle are
 * serialised by the caller; the library keeps no global mutable state other
 * than the per-device scratch described at tl_simulate.
 */
#ifndef TL_H_
#define TL_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TL_ABI_VERSION 2

typedef enum tl_status {
    TL_OK = 0,
    TL_ERR_INVALID_ARGUMENT = 1, /* bad pointer / size / option             */
    TL_ERR_INVALID_MODEL = 2,    /* inconsistent model description          */
    TL_ERR_UNSUPPORTED = 3,      /* reaction order > 2, |v| outside [-2,5]  */
    TL_ERR_OVERFLOW = 4,         /* population left the int32/int64 range  */
    TL_ERR_STEP_CAP = 5,         /* max_steps reached (results truncated)   */
    TL_ERR_CUDA = 6,             /* CUDA runtime error                      */
    TL_ERR_WAIT_TIMEOUT = 7,     /* a bounded device wait gave up           */
    TL_ERR_NO_DEVICE = 8,        /* no usable CUDA device                   */
    TL_ERR_OUT_OF_MEMORY = 9,
    TL_ERR_IO = 10,              /* file could not be opened / written      */
    TL_ERR_PARSE = 11,           /* StochKit XML could not be parsed        */
    TL_ERR_NUMERIC = 12          /* negative or non-finite rate, or a leap
                                    still negative after max_halvings
                                    halvings of tau                        */
} tl_status;

typedef struct tl_model tl_model;

/* ------------------------------------------------------------------------ */
/* Model                                                                    */
/* ------------------------------------------------------------------------ */

/*
 * Host description of a reaction network, channel (column) major, exactly the
 * layout the reference builds in ReadXMLToMatrixStruct
 * (tau_leaping/CSCHostMatrixData.cpp:19-107): for channel j the entries
 * col_ptr[j] .. col_ptr[j+1]-1 list species rows in ascending order with a
 * signed stoichiometry, reactants negative and products positive.  A species
 * that is both reactant and product of one channel may appear twice.
 * The library derives reaction orders, first/second reactant indices
 * (tau_leaping/CSCMatrix.cu:185-251), the packed species-row CSR
 * (tau_leaping/CSRMatrixPacked.cu:22-31, packing functions.h:126-130) and a
 * net-stoichiometry CSR/CSC.  Inputs stay owned by the caller.
 */
typedef struct tl_model_desc {
    int32_t n_species;       /* N                                            */
    int32_t n_channels;      /* M                                            */
    int32_t nnz;             /* entries in the CSC arrays                    */
    const int64_t *x0;       /* [N] initial populations (>= 0)               */
    const double *rate;      /* [M] rate constants c_j (>= 0)                */
    const int32_t *col_ptr;  /* [M+1]                                        */
    const int32_t *row_ind;  /* [nnz] species index of each entry            */
    const int8_t *stoich;    /* [nnz] signed stoichiometry                   */
    int32_t pop_bits;        /* 32 or 64; 0 = 32 unless x0 needs 64          */
} tl_model_desc;

/* Build a device-resident model (replaces Model::ReadXML's device part). */
tl_status tl_model_create(const tl_model_desc *desc, tl_model **out);

/* Parse a StochKit-2 XML file (replaces Model::ReadXML, model.cpp:17). */
tl_status tl_model_from_stochkit(const char *path, int32_t pop_bits,
                                 tl_model **out);

void tl_model_destroy(tl_model *m);

typedef struct tl_model_info {
    int32_t n_species, n_channels, nnz_raw, nnz_net, pop_bits;
    int32_t max_order;
} tl_model_info;

tl_status tl_model_get_info(const tl_model *m, tl_model_info *info);

/* Species name for index i (models read from XML; "S<i+1>" otherwise).
 * The returned pointer lives as long as the model. */
const char *tl_model_species_name(const tl_model *m, int32_t i);

/* Index of a species name, or -1. */
int32_t tl_model_species_index(const tl_model *m, const char *name);

/* Copy the model description back (any pointer may be NULL); sizes from
 * tl_model_get_info (nnz_raw entries). */
tl_status tl_model_get_desc(const tl_model *m, int64_t *x0, double *rate,
                            int32_t *col_ptr, int32_t *row_ind,
                            int8_t *stoich);

/* Write the model as StochKit-2 XML (readable by the reference's -f). */
tl_status tl_model_write_stochkit(const tl_model *m, const char *path);

/* Seeded model generator (replaces toy_system_gen/main.cpp, whose RNG is
 * seeded from time()).  Families of the reference's examples / generator. */
enum tl_gen_family {
    TL_GEN_DIMER = 1,   /* dimerisation decay, x0 = (x0_max, 0, 0)          */
    TL_GEN_TOY = 2,     /* random network, 1-2 reactants, 1-2 products      */
    TL_GEN_CHAIN = 3,   /* cyclic chain S_i -> S_(i+1 mod N) at rate_min    */
    TL_GEN_COLLOID = 4  /* colloidal aggregation, N^2/2 channels            */
};

typedef struct tl_gen_params {
    int32_t family;
    int32_t n_species;
    int32_t n_channels;   /* toy only                                       */
    int32_t pop_bits;     /* 0 = auto                                       */
    int64_t x0_min, x0_max;
    double rate_min, rate_max;      /* toy: log-uniform range; chain: rate  */
    double rate_assoc, rate_dissoc; /* colloid                              */
    uint64_t seed;
} tl_gen_params;

/* Defaults of the benchmark configuration of each family. */
void tl_gen_params_init(tl_gen_params *g, int32_t family);
tl_status tl_model_generate(const tl_gen_params *g, tl_model **out);

/* Copy the derived tables back to the host (any pointer may be NULL).
 * order/s0/s1: [M]; csr_row_ptr: [N+1]; csr_valcol: [nnz_raw], reference
 * packing (col<<3)|((v+2)&7) on the reference's raw entries. */
tl_status tl_model_get_tables(const tl_model *m, int8_t *order, int32_t *s0,
                              int32_t *s1, int32_t *csr_row_ptr,
                              int32_t *csr_valcol);

/* ------------------------------------------------------------------------ */
/* Simulation                                                               */
/* ------------------------------------------------------------------------ */

enum tl_variant {
    TL_VARIANT_AUTO = 0,   /* autotuner picks                                */
    TL_VARIANT_THREAD = 1, /* fused persistent, one realization per thread   */
    TL_VARIANT_WARP = 2,   /* fused persistent, one realization per warp     */
    TL_VARIANT_CTA = 3,    /* fused persistent, one realization per CTA      */
    TL_VARIANT_PLAIN = 4,  /* FP32, one realization per thread, one launch
                              per step: the unfused baseline form           */
    TL_VARIANT_LANES2 = 5,  /* fused persistent, one realization per 2, 4,  */
    TL_VARIANT_LANES4 = 6,  /* 8 or 16 lanes of a warp; AUTO takes 8 or 16  */
    TL_VARIANT_LANES8 = 7,  /* for models up to 128 or 256 channels on      */
    TL_VARIANT_LANES16 = 8  /* ensembles that fill the GPU many times over   */
};

/* Behaviour flags. */
#define TL_FLAG_SENSITIVITY (1u << 0)   /* accumulate likelihood-ratio scores */
#define TL_FLAG_KEEP_SAMPLES (1u << 1)  /* return per-realization samples    */
#define TL_FLAG_AUTOTUNE_MEASURE (1u << 2) /* AUTO: time candidate plans on a
                                             prefix of the ensemble, cache
                                             the fastest in the model       */
#define TL_FLAG_NO_STAGE (1u << 3)       /* read model tables through L1/L2
                                            instead of staging them in
                                            shared memory (tuning knob)     */
#define TL_FLAG_GLOBAL_SLOTS (1u << 5)  /* CTA groups: keep each realization's
                                            state in global memory (L2) even
                                            when it fits in shared memory
                                            (tuning and checking knob; larger
                                            states always do)              */
#define TL_FLAG_GRAPH (1u << 4)          /* PLAIN: replay the per-step launches
                                            as a captured CUDA graph of 16
                                            steps between completion polls  */
/* Reference-compatibility switches (each reproduces one behaviour of the
 * shipped reference; default off = Cao-Gillespie-Petzold 2006 semantics). */
#define TL_FLAG_COMPAT_G (1u << 8)       /* g read from channel order at the
                                           species index (CSRMatrixPacked.cu:353) */
#define TL_FLAG_COMPAT_CRIT (1u << 9)    /* 2S->: critical iff 2*x < n_c
                                           (functions.h:115)                     */
#define TL_FLAG_COMPAT_STOICH (1u << 10) /* mu/sigma^2 over the raw duplicate
                                           entries and over every species row
                                           (CSRMatrixPacked.cu:330-355)          */
#define TL_FLAG_COMPAT_TAU2 (1u << 11)   /* critical / SSA waiting time uses the
                                           chosen channel's propensity
                                           (model.cu:596)                        */
#define TL_FLAG_COMPAT_SSA (1u << 12)    /* direct-method steps advance time
                                           without firing (model.cu:442-446)    */
#define TL_FLAG_COMPAT_POISSON (1u << 13) /* Knuth product below mean 80 (cap
                                           300), |Normal(mean,mean)| above
                                           (model.cu:477-520)                   */
#define TL_FLAG_COMPAT_REFERENCE                                               \
    (TL_FLAG_COMPAT_G | TL_FLAG_COMPAT_CRIT | TL_FLAG_COMPAT_STOICH |          \
     TL_FLAG_COMPAT_TAU2 | TL_FLAG_COMPAT_SSA | TL_FLAG_COMPAT_POISSON)

typedef struct tl_run_cfg {
    double t_final;          /* simulation end time (the reference's -t)     */
    double eps;              /* CGP epsilon (-e, default 0.03)               */
    int64_t n_realizations;  /* per rate set (-n)                            */
    uint64_t seed;           /* Philox key                                   */
    int32_t n_intervals;     /* grid t_k = k*t_final/n_intervals, k=0..n (-i)*/
    int32_t n_tracked;       /* species recorded on the grid (-r)            */
    const int32_t *tracked;  /* [n_tracked] species indices                  */
    int32_t n_rate_sets;     /* 0: the model's rates; else rate_sets rows    */
    const double *rate_sets; /* [n_rate_sets][M]                             */
    const double *t_final_sets; /* [n_rate_sets] per-set end time or NULL    */
    int32_t variant;         /* enum tl_variant                              */
    int32_t block_threads;   /* threads per CTA, 0 = auto                    */
    uint32_t flags;          /* TL_FLAG_*                                    */
    int32_t n_critical;      /* n_c, 0 = 5 (model.cu:225)                    */
    int32_t ssa_factor;      /* SSA fallback when tau1 < ssa_factor/a0,
                                0 = 10 (model.h:34)                          */
    int32_t ssa_block;       /* direct steps per fallback, 0 = 100
                                (model.cu:343)                               */
    int64_t max_steps;       /* per-realization step cap (-a), 0 = none      */
    void *stream;            /* cudaStream_t to run on; NULL = default stream */
    int64_t realization_offset; /* first realization id of this call: a
                                   shard [off, off+n) of a larger ensemble
                                   draws the same streams as in one call   */
    int32_t max_halvings;    /* a leap whose update leaves a population
                                negative is rejected and retried with tau
                                halved (Cao, Gillespie, Petzold 2006); a
                                realization whose leap is still rejected
                                after this many halvings stops and the call
                                returns TL_ERR_NUMERIC.  0 = 64            */
    int32_t stage_wait_polls; /* polls of the bounded wait for the model
                                tables' copy into shared memory: 0 = 2^22;
                                < 0 = none, so that the wait gives up at
                                once and the call returns
                                TL_ERR_WAIT_TIMEOUT (checks the timeout
                                path; the copy is still drained before a
                                CTA exits)                                 */
} tl_run_cfg;

/* Fill cfg with the reference's defaults (eps 0.03, 1 interval, ...). */
void tl_run_cfg_init(tl_run_cfg *cfg);

typedef struct tl_result {
    /* Caller-owned output buffers; any may be NULL.  S = max(1,n_rate_sets),
     * P = n_intervals+1, K = n_tracked, R = n_realizations.               */
    double *times;     /* [S][P]   grid times                               */
    double *mean;      /* [S][P][K] ensemble mean                           */
    double *stddev;    /* [S][P][K] sample stddev (n-1), like
                          StepStat2StdDev (statistics.cpp:67-87)            */
    int64_t *samples;  /* [S][R][P][K] per-realization samples, needs
                          TL_FLAG_KEEP_SAMPLES                               */
    /* Scalar outputs. */
    int64_t leaps;      /* accepted tau-leaps, all realizations              */
    int64_t ssa_steps;  /* direct-method steps                               */
    int64_t rejections; /* leaps rejected for a negative population          */
    int64_t truncated;  /* realizations stopped by max_steps                 */
    double kernel_ms;   /* device time of the simulation launch(es)          */
    double total_ms;    /* host wall time of the call                        */
    int32_t variant_used, block_threads_used, grid_used, launches;
} tl_result;

/*
 * Run n_realizations (per rate set) from x0 to t_final and reduce the tracked
 * species on the grid.  Replaces the realization loop of the reference's main
 * (tau_leaping.cpp:144-150) + Model::PerformCalc + statistics.
 * Realization r of rate set s draws every random number from Philox4x32-10
 * keyed by seed with counter (channel|0xFFFFFFFF, step, r, s<<8|block), so
 * results do not depend on the variant's scheduling or on other sets.
 */
tl_status tl_simulate(tl_model *m, const tl_run_cfg *cfg, tl_result *res);

/*
 * Several (model, configuration) pairs in ONE persistent launch.  Each item
 * is simulated exactly as tl_simulate would (same streams, same outputs in
 * its result; grad non-NULL adds tl_sensitivity's gradients).  Small models
 * (<= 16 species and channels) run 32 realizations per warp, one per lane;
 * larger ones one realization per warp; every warp takes work from one
 * counter, so rate sets with uneven step counts or t_final balance out.
 * Models must share the device and the population width; variant and
 * stream fields of the items' cfg are ignored (stream is the argument).
 */
typedef struct tl_batch_item {
    tl_model *model;
    const tl_run_cfg *cfg;
    tl_result *result;     /* may be NULL                                   */
    struct tl_grad_result *grad; /* non-NULL: sensitivities for this item   */
} tl_batch_item;

tl_status tl_simulate_batch(tl_batch_item *items, int32_t n_items,
                            void *stream);

/*
 * tl_simulate without any device allocation.  No counterpart in the
 * reference (it allocates per realization with Thrust vectors).
 *
 * For callers that cannot call cudaMalloc: a host whose GPU memory is owned
 * by a pool allocator that has already reserved the device, and
 * latency-bound loops that cannot take cudaMalloc / cudaFree's implicit
 * device-wide synchronisation.  The caller passes inputs and outputs as for
 * tl_simulate; every piece of device scratch of the run (rate and t_final
 * tables, per-realization grid samples, counters, reduced statistics, and
 * the per-CTA state of models past shared memory) lives in one file-scope
 * device array of TL_STATIC_SCRATCH_BYTES that every GPU loading libtl.so
 * holds until the process exits.
 *  - The model's tables must already be on the device: any earlier
 *    tl_simulate / tl_eval_leap / tl_replay call on the model uploads them;
 *    otherwise TL_ERR_INVALID_ARGUMENT.
 *  - A run whose scratch exceeds TL_STATIC_SCRATCH_BYTES (about
 *    S*R*(n_intervals+1)*n_tracked*4 bytes for 32-bit populations, plus
 *    small tables) is rejected with TL_ERR_INVALID_ARGUMENT and a message
 *    giving both sizes.  The plain form, sensitivities and the measured
 *    autotuner are not available here (TL_ERR_UNSUPPORTED / ignored).
 *  - The first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress) with that device current and keeps it for the
 *    life of the process; make that first call before any stream capture,
 *    and do not use the library across a cudaDeviceReset.
 *  - All calls share the one array, which keeps the last call's contents
 *    (counters are cleared at the start of each call).  Calls that overlap
 *    on the GPU - from two host threads, or on two streams - race on it.
 *  - The call waits for its stream before it returns.  res->kernel_ms is
 *    host-timed from launch to completion (no CUDA event is created).
 */
#define TL_STATIC_SCRATCH_BYTES (16u << 20)
tl_status tl_simulate_static(tl_model *m, const tl_run_cfg *cfg,
                             tl_result *res);

/* ------------------------------------------------------------------------ */
/* Sensitivity ("backward")                                                 */
/* ------------------------------------------------------------------------ */

typedef struct tl_grad_result {
    /* [S][K][M]: d E[X_k(t_final)] / d c_j and its standard error. */
    double *grad;
    double *grad_stderr;
    double *mean_final; /* [S][K] E[X_k(t_final)]                         */
} tl_grad_result;

/*
 * Likelihood-ratio sensitivities of the tracked species' means at t_final
 * with respect to every rate constant.  Runs the same forward pass as
 * tl_simulate with score accumulation (sum over steps of
 * (k_j - a_j*dt)/c_j) and reduces Cov(X_k(T), score_j) per set.
 * res may be NULL.
 */
tl_status tl_sensitivity(tl_model *m, const tl_run_cfg *cfg, tl_result *res,
                         tl_grad_result *grad);

/* ------------------------------------------------------------------------ */
/* Parity entry points (same device functions the fused kernel uses)        */
/* ------------------------------------------------------------------------ */

/*
 * Leap quantities for n_states population vectors x[n][N]:
 * a[n][M] propensities, crit[n][M] criticality, mu/sigma2[n][N] CGP
 * moments, tau1[n] the CGP bound, a0[n] total propensity.  Any output may be
 * NULL.  Replaces CalcPropensities (model.cu:213-247) + CompTau
 * (CSRMatrixPacked.cu:423-462).
 */
tl_status tl_eval_leap(tl_model *m, const int64_t *x, int32_t n_states,
                       double eps, uint32_t flags, int32_t n_critical,
                       float *a, uint8_t *crit, float *mu, float *sigma2,
                       float *tau1, double *a0);

/*
 * Integer replay: x_{l+1} = x_l + V k_l for l < n_leaps, starting at x0[N],
 * with firing counts k[n_leaps][M].  Writes every state x_out[n_leaps][N].
 * Uses the raw (reference) entries when raw != 0, else the net CSR; both
 * give the same integers.  Replaces FireReactions
 * (CSRMatrixPacked.cu:464-503) with its loop bound fixed to the species
 * count.  Returns TL_ERR_OVERFLOW if a state leaves the population type.
 */
tl_status tl_replay(tl_model *m, const int64_t *x0, const int32_t *k,
                    int32_t n_leaps, int32_t raw, int64_t *x_out);

/* Philox4x32-10 on the device: out[i] = philox(ctr[i], key[i]). */
tl_status tl_philox(const uint32_t *ctr, const uint32_t *key, int32_t n,
                    uint32_t *out);

/*
 * Poisson sampler on the device: out[i] ~ Poisson(mean[i]), drawn exactly as
 * the simulation draws channel i of realization 0 in step `step` (the first
 * word from the block shared by channels 4(i/4)..4(i/4)+3, then the private
 * stream (i, step, 0, b)) under seed; compat != 0 selects the reference's
 * sampler.  For distribution tests.
 */
tl_status tl_poisson(const float *mean, int32_t n, uint64_t seed,
                     uint32_t step, int32_t compat, int32_t *out);

/* ------------------------------------------------------------------------ */
/* Sharding across processes / GPUs                                         */
/* ------------------------------------------------------------------------ */

/*
 * Merge per-shard statistics of disjoint realization ranges (each shard run
 * with its own realization_offset) into the statistics of the union, with
 * Chan, Golub and LeVeque's pairwise update of (count, mean, M2).
 * means/stddevs: [n_parts][L]; counts: [n_parts]; stddev is the sample
 * (n-1) deviation as tl_simulate returns it.  Host only, no device call.
 * Replaces nothing in the reference (it never splits an ensemble).
 */
tl_status tl_merge_moments(int32_t n_parts, int32_t L, const int64_t *counts,
                           const double *means, const double *stddevs,
                           int64_t *count_out, double *mean_out,
                           double *stddev_out);

/* ------------------------------------------------------------------------ */
/* Misc                                                                     */
/* ------------------------------------------------------------------------ */

const char *tl_status_str(tl_status s);
/* Last error detail for this host thread (CUDA error string, parse error). */
const char *tl_last_error(void);
int32_t tl_abi_version(void);
/* Select the CUDA device used by subsequent tl_model_* calls on this thread
 * (the reference's -d, honoured unlike tau_leaping.cpp:48). */
tl_status tl_set_device(int32_t device);

#ifdef __cplusplus
}
#endif

#endif /* TL_H_ */
