/*
 * libmgbf -- GB300-native multigrid beta filter (MGBF) filtering pipeline.
 *
 * C-ABI drop-in for the filtering path of the reference's Fortran modules.
 * Every entry point below names the reference interface it replaces
 * (paths inside the reference project):
 *
 *   mg_entrymod.f90:36   mg_initialize            -> mgbf_create / mgbf_create_from_namelist
 *   mg_parameter.f90:179 init_mg_parameter        -> mgbf_config_read_namelist
 *   mg_filtering.f90:67  filtering_procedure      -> mgbf_filtering_procedure
 *   mg_entrymod.f90:222  mg_finalize              -> mgbf_destroy
 *
 * The field is operated on in place, in the reference's layout
 * VALL(km_all, 1-hx:im+hx, 1-hy:jm+hy) (mg_intstate.f90:157; level index
 * fastest), over the whole filter grid im = nxPE*im_filt, jm = nyPE*jm_filt
 * held by one GPU, or in a compact (km_all, im, jm) layout without halos.
 * The caller owns the field; the handle owns setup tables and scratch.
 *
 * Errors are returned as negative codes (the reference calls `stop`).
 * No entry point exits the process.  Calls on distinct handles are
 * thread-safe; one handle is used by one host thread at a time.
 */
#ifndef MGBF_H
#define MGBF_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MGBF_ABI_VERSION 1
#define MGBF_MAX_GEN 16

/* ---- status codes ---------------------------------------------------- */
#define MGBF_OK 0
#define MGBF_ERR_ARG (-1)          /* null pointer, bad enum, bad size          */
#define MGBF_ERR_CONFIG (-2)       /* inconsistent configuration                */
#define MGBF_ERR_REACH (-3)        /* filter reach exceeds halo (getlinesum stop) */
#define MGBF_ERR_DIVISIBILITY (-4) /* grid not divisible by 2^(gm-1), too small  */
#define MGBF_ERR_UNSUPPORTED (-5)  /* mgbf_proc outside the supported set        */
#define MGBF_ERR_CUDA (-6)         /* CUDA runtime error                         */
#define MGBF_ERR_NAMELIST (-7)     /* namelist syntax / unknown field            */
#define MGBF_ERR_IO (-8)           /* file cannot be read                        */
#define MGBF_ERR_TIMEOUT (-9)      /* bounded device wait ran out                */
#define MGBF_ERR_NOMEM (-10)       /* allocation failed                          */

/* ---- storage types and memory spaces ---------------------------------- */
#define MGBF_F64 0   /* double storage, double arithmetic                    */
#define MGBF_F32 1   /* float storage, float arithmetic                      */
#define MGBF_BF16 2  /* bfloat16 storage, float arithmetic                   */

#define MGBF_MEM_DEVICE 0
#define MGBF_MEM_HOST 1

#define MGBF_LAYOUT_HALO 0     /* VALL(km_all, 1-hx:im+hx, 1-hy:jm+hy)       */
#define MGBF_LAYOUT_COMPACT 1  /* (km_all, im, jm)                            */

/*
 * Configuration: the fields of namelist &PARAMETERS_MGBETA
 * (mg_parameter.f90:190-208) with the same names and meaning, plus a few
 * extensions at the end.  mgbf_config_init() sets the defaults below.
 */
typedef struct mgbf_config {
    double mg_ampl01, mg_ampl02, mg_ampl03;
    double mg_weig1, mg_weig2, mg_weig3, mg_weig4, mg_weig5;
    int hx, hy, hz, p;
    int mgbf_line, mgbf_proc, n_ens;
    int lm_a, lm, km2, km3;
    int l_loc, l_loc_vertical, l_filt_g1, l_lin_vertical, l_lin_horizontal;
    int l_quad_horizontal, l_new_map, l_vertical_filter;
    int ldelta, lquart, lhelm;
    int gm_max;
    int nm0, mm0, nxPE, nyPE, im_filt, jm_filt;
    /* ---- extensions (0 keeps reference behaviour) ---- */
    int gm_uncapped;                 /* 1: gm = gm_max, not min(gm_max, def_maxgen(nxPE,nyPE)) */
    int n_weig_ext;                  /* >0: use weig_ext[0..n-1] as a_1..a_n (gens beyond n reuse the last) */
    double weig_ext[MGBF_MAX_GEN];
    double helm_b[MGBF_MAX_GEN];     /* Helmholtz b per generation (reference: 0) */
    int layout;                      /* MGBF_LAYOUT_HALO (reference) or MGBF_LAYOUT_COMPACT */
} mgbf_config;

/* Derived sizes of a created handle. */
typedef struct mgbf_dims {
    int im, jm;            /* generation-1 filter grid                       */
    int km_all;            /* leading dimension of the field                 */
    int km, km3_all;
    int gm;                /* generations actually used                      */
    int hx, hy, hz;
    int reach_h, reach_z;  /* filter reach (<= halo)                          */
    int layout;
    size_t field_elems;    /* elements of one field in the handle's layout   */
    int hbeta_kernel;      /* 1: moment kernel, 0: direct-sum kernel          */
    int reach_line;        /* fast filters' line reach (-1: procs 3/8 unusable) */
    int nm0, mm0;          /* analysis grid of the transfers                  */
    int km_a_all;          /* leading dimension of WORKA: (km2+lm_a*km3)*n_ens */
    size_t anal_elems;     /* elements of WORKA(km_a_all, nm0, mm0)           */
} mgbf_dims;

typedef struct mgbf_handle mgbf_handle;

/* Defaults of the reference's namelist fields (the shipped RUN/mgbf.nml
 * values for the booleans; sizes zero so they must be given). */
int mgbf_config_init(mgbf_config* cfg);

/* Parse &PARAMETERS_MGBETA from a namelist file (replaces the read in
 * init_mg_parameter, mg_parameter.f90:210-212).  Unknown fields are an error.
 * Extension fields may appear in the same group.  The optional errbuf gets a
 * one-line message. */
int mgbf_config_read_namelist(const char* path, mgbf_config* cfg, char* errbuf, size_t errlen);

/* Validate a configuration and build a handle: FP64 setup of the filter
 * tables (def_mg_weights, mg_intstate.f90:296-433; def_offset_coef,
 * mg_interpolate.f90:61-86) and device scratch for the coarse generations.
 * Replaces mg_initialize (mg_entrymod.f90:36) for the filtering path.
 * Uses the current CUDA device. */
int mgbf_create(const mgbf_config* cfg, mgbf_handle** out);

/* mgbf_config_read_namelist + mgbf_create. */
int mgbf_create_from_namelist(const char* path, mgbf_handle** out);

/* Sizes derived at creation. */
int mgbf_get_dims(const mgbf_handle* h, mgbf_dims* dims);

/* The three line filters of procedures 2 and 7 as set up at creation
 * (init_mg_line, mg_intstate.f90:436-480): per color q = 0..2 the
 * generator (gen[2q], gen[2q+1]), integer half-span h[q], formal half-span
 * hs[q] and weights fil[9q + i], i = 0..h[q] (zero beyond).  Returns the
 * setup's error (MGBF_ERR_REACH, ...) when those procedures cannot run. */
int mgbf_get_line_filters(const mgbf_handle* h, int gen[6], int hspan[3], double hs[3], double fil[27]);

/*
 * filtering_procedure(mg_filt) (mg_filtering.f90:67-120) on the field in
 * place.  Supported: 1 = filtering_rad2_bckg (mg_filtering.f90:560-680),
 * 6 = filtering_rad2_ens (mg_filtering.f90:1000-1147), and the fast 1D+1D
 * variants 3 = filtering_fast_bckg (mg_filtering.f90:825-997) and
 * 8 = filtering_fast_ens (mg_filtering.f90:1316-1506), whose horizontal
 * filter is vrbeta1 along x and y with el = mg_ampl02 (no cholaspect), and
 * 4 = filtering_rad3 (mg_filtering.f90:123-257: the 3D ball vrbeta3 with
 * aspect mg_ampl03 on the 3D variables, the 2D radial filter on the 2D
 * ones, no separate vertical filter; like the reference, its adjoint side
 * keeps only the interior of the 3D scatter and folds the caller's VALL
 * halo, so the operator is not symmetric), and
 * 2 = filtering_lin2_bckg (mg_filtering.f90:683-822: per generation the
 * three "dibeta" line filters of the triad decomposition, jp_pbfil3.f90,
 * of the Cholesky factor of the inverse aspect that init_mg_line sees;
 * MGBF_ERR_REACH when a line filter's spread is beyond the moment table or
 * its reach beyond the halo; with mgbf_line off the reference never sets
 * the line filters up and every one is a copy, here too), and
 * 7 = filtering_lin2_ens
 * (mg_filtering.f90:1150-1313: the same line filters over the stacked
 * members, l_filt_g1 and lquart as for 6, ending like the reference with the
 * ADJOINT vertical filter sup_vrbeta1T_ens, so the operator is not
 * symmetric), and
 * 5 = filtering_lin3 (mg_filtering.f90:260-557: the 2D variables through the
 * line filters of 2, the 3D variables through the seven colors of the hexad
 * decomposition, jp_pbfil3.f90:798-904, of the Cholesky factor of the
 * inverse 3D aspect mg_ampl03, each color a dibeta line along its 3D
 * generator between the reference's 3D halo routines, whose generation-1
 * forms mirror the east edge about the last column and fold the east column
 * and north row onto themselves, so the operator is not symmetric; no
 * separate vertical filter).  Any other value is a no-op returning MGBF_OK,
 * as the reference's select has no default case.
 *   vall:   field pointer (device or host, per mem), laid out per the
 *           handle's layout, element type per dtype.
 *   stream: cudaStream_t (NULL = legacy default stream).  Device calls are
 *           asynchronous on the stream; host calls return after the result
 *           is back in vall.
 */
int mgbf_filtering_procedure(mgbf_handle* h, int mg_filt, void* vall, int dtype, int mem,
                             void* stream);

/*
 * Transfers between the analysis grid WORKA(km_a_all, nm0, mm0) (level
 * index fastest) and the filter field VALL, the new map of the reference's
 * driver (RBETA_TEST.f90:46-98 with l_new_map):
 *   mgbf_anal_to_filt  = anal_to_filt_all2 (mg_transfer.f90:154-181, 339-403):
 *     l_vertical_adjoint_spec2 when lm_a = 2*lm-1, VALL = 0, the adjoint
 *     offset interpolation (lsqr, or quad / lin per l_quad_horizontal /
 *     l_lin_horizontal) and bocoT_2d over the interpolation halo (3/2/1).
 *   mgbf_filt_to_anal  = filt_to_anal_all2 (mg_transfer.f90:184-203, 406-464):
 *     boco_2d fills VALL's interpolation halo (in place, halo layout), the
 *     direct interpolation, l_vertical_direct_spec2 when lm_a = 2*lm-1.
 * The analysis grid is nm0 x mm0 over nxPE x nyPE ranks, each rank's nm0/nxPE
 * points over the same length as its im_filt filter points.  lm_a must be
 * lm, or 2*lm-1 with km2 = 0; l_new_map = false (the old map) returns
 * MGBF_ERR_UNSUPPORTED.  dtype/mem/stream as in mgbf_filtering_procedure.
 */
int mgbf_anal_to_filt(mgbf_handle* h, const void* worka, void* vall, int dtype, int mem, void* stream);
int mgbf_filt_to_anal(mgbf_handle* h, void* vall, void* worka, int dtype, int mem, void* stream);

/* Adjoint of filtering_procedure(mg_filt), run through the explicit
 * transposed chain (no reference counterpart: the reference's adjoint test
 * is an empty stub, RBETA_TEST.f90:64-69).  Procedures 1, 2, 3, 6 and 8 are
 * self-adjoint, so the result equals the forward up to rounding; 4, 5 and
 * 7 are not and return MGBF_ERR_UNSUPPORTED. */
int mgbf_filtering_procedure_adjoint(mgbf_handle* h, int mg_filt, void* vall, int dtype, int mem,
                                     void* stream);

/*
 * Gradients for y = L(a) x (no reference counterpart):
 *   gx = L^T gy, and ga[g] = sum over points of u_g * v_g with
 *   u_g = B_g R_g Bz^T x, v_g = B_g R_g Bz^T gy, for g = 1..gm.
 * x, gy, gx: fields in the handle's layout (gx may alias gy).  ga: host
 * array of gm doubles.  Coarse generations are recomputed from x.
 * Returns after ga is on the host.  Procedures 4, 5 and 7 (not
 * self-adjoint) return MGBF_ERR_UNSUPPORTED.
 */
int mgbf_apply_with_weight_grads(mgbf_handle* h, int mg_filt, const void* x, const void* gy,
                                 void* gx, double* ga, int dtype, int mem, void* stream);

/* Device-side status: MGBF_ERR_TIMEOUT if a bounded wait inside a kernel
 * (a TMA-fed pipeline stage) ran out since the last check, else MGBF_OK.
 * Synchronises with the device and clears the status. */
int mgbf_status(mgbf_handle* h);

/* Polls of a row's mbarrier before a TMA-fed radial kernel gives up
 * (default 2^20, restored by polls < 0; no reference counterpart: the
 * reference has no device waits).  A block that gives up records
 * MGBF_ERR_TIMEOUT for mgbf_status, waits for its own copies still in
 * flight and returns; its output rows are then incomplete.  polls = 0 makes
 * every such wait give up at once, which lets a test exercise that path on
 * a healthy GPU. */
int mgbf_set_wait_limit(mgbf_handle* h, int polls);

/* Vertical filter passes of the radial procedures (1, 6): 2 (the default)
 * runs them as the reference does, Bz^T first (sup_vrbeta1T_bck / _ens,
 * mg_filtering.f90:583, 1026) and Bz last (sup_vrbeta1_bck / _ens, :674,
 * 1140); 1 applies M = Bz Bz^T once, in the last prolongation.  Both give the same operator: the vertical filter acts on
 * every column alike and the rest of the chain on every level alike, so
 * Bz H Bz^T = H Bz Bz^T; results differ by rounding.  With 1 the
 * restriction writes no generation-1 copy of the field and generation 1's
 * first radial pass reads the caller's field itself, one write of the field
 * less per call.  Used where it applies (FP32/BF16, the radial moment
 * kernel at reach <= 16, vertical reach <= 4, generation 1 filtered, no
 * persistent sides); elsewhere the two passes run.  No reference
 * counterpart. */
int mgbf_set_vertical_passes(mgbf_handle* h, int passes);

/* Autotuner of tile shapes: times the radial-filter kernel variants (TMA
 * pipelines of one or two rows per barrier, cp.async staging) and output
 * rows per block for every generation and pass of the handle, on the
 * handle's own scratch buffers, and keeps the fastest for later calls.
 * Synchronous; needs no field.  The choice changes results only by
 * rounding (summation order). */
int mgbf_autotune(mgbf_handle* h, int dtype, void* stream);

/* Pins the radial-filter kernel variant (0: TMA, two rows per barrier;
 * 1: TMA, one row per barrier; 2: cp.async staging; 3: TMA, two rows per
 * barrier filtered one after the other) and output rows per block
 * (<= 0: the default) for every generation and pass; variant < 0 returns
 * to the defaults.  FP64 always uses its one kernel.  For tests and manual
 * tuning; mgbf_autotune chooses by measurement. */
int mgbf_set_tuning(mgbf_handle* h, int dtype, int variant, int rows);

/* Replace the per-generation weights a_1..a_n (n <= gm) without rebuilding. */
int mgbf_set_weights(mgbf_handle* h, const double* a, int n);

/* Release the handle (replaces mg_finalize / deallocate_mg_intstate). */
int mgbf_destroy(mgbf_handle* h);

/* ------------------------------------------------------------------------
 * Stage timers: the counterpart of the reference's mg_timers (btim/etim
 * around every stage, mg_timers.f90:70-104; per-rank report,
 * mg_timers.f90:106-199).  When enabled, every kernel launch of the
 * library is bracketed by CUDA events on its stream and accumulated per
 * stage under the reference's timer names: vfiltT, upsend, hfiltT (first
 * radial pass, with the weighting), hfilt (second radial pass), dnsend,
 * vfilt, dnsend+vfilt (the last prolongation fused with the vertical
 * forward filter), plus copy, halo and wgrad.  Process-wide; not for concurrent use
 * from several host threads.
 */
typedef struct mgbf_timer_stat {
    char name[16];
    long long count;       /* launches                                      */
    double total_ms;       /* summed CUDA-event durations                    */
    double points;         /* grid points processed (sum over launches)      */
} mgbf_timer_stat;

/* on != 0 enables and resets the timers; 0 disables them. */
int mgbf_timers_enable(int on);
/* Synchronises outstanding timer events and copies up to max stats. */
int mgbf_timers_read(mgbf_timer_stat* out, int max, int* n);

/* Static description of a status code. */
const char* mgbf_strerror(int code);

/* Message of the most recent failure on the calling thread. */
const char* mgbf_last_error(void);

/* ------------------------------------------------------------------------
 * Batched ensemble extension (no single reference counterpart: the
 * reference needs one run per variable group because one lm and one
 * mg_ampl02 serve every variable, mg_parameter.f90:293-294,
 * mg_intstate.f90:383-390).  A batch is a list of variable groups on one
 * horizontal grid; each group is a compact (nk, im, jm) field of nk =
 * members * levels columns with its own horizontal reach, vertical filter
 * and levels.  All groups are filtered by one call.
 */
typedef struct mgbf_group_desc {
    int nk;               /* leading dimension of this group's field           */
    int lm;               /* levels per vertical column (1: 2D, no z filter)   */
    int nzcol;            /* z columns at offsets (c-1)*lm; 0 = no z filter     */
    int hx, hy, hz, p;
    double mg_ampl01, mg_ampl02;
} mgbf_group_desc;

typedef struct mgbf_batch mgbf_batch;

/* im, jm: generation-1 grid; gm generations; weights a_1..a_gm; lquart as in
 * the namelist; l_filt_g1 as in filtering_rad2_ens. */
int mgbf_batch_create(int im, int jm, int gm, const double* weights, int lquart, int l_filt_g1,
                      const mgbf_group_desc* groups, int ngroups, mgbf_batch** out);
/* fields[g]: device pointer to group g's compact field; filtered in place.
 * adjoint != 0 runs the transposed chain. */
int mgbf_batch_apply(mgbf_batch* b, void* const* fields, int dtype, int adjoint, void* stream);
int mgbf_batch_destroy(mgbf_batch* b);
/* enable != 0: replay each distinct call (same field pointers, dtype and
 * direction) as one CUDA graph, captured on its first call after the
 * batch's device memory exists (the first call of a dtype runs directly);
 * graphs are bypassed while stage timers are on.  0 releases the graphs. */
int mgbf_batch_use_graphs(mgbf_batch* b, int enable);
/* Procedure a batch runs: 6 (filtering_rad2_ens, the default) or 8
 * (filtering_fast_ens, mg_filtering.f90:1316-1506: the 1D+1D line filters
 * with el = mg_ampl02).  8 fails with MGBF_ERR_DIVISIBILITY when a group's
 * line reach exceeds its hx/hy or the coarsest generation.  Releases graphs
 * captured before. */
int mgbf_batch_set_procedure(mgbf_batch* b, int mg_filt);

/* As mgbf_status, for a batch. */
int mgbf_batch_status(mgbf_batch* b);
/* As mgbf_set_weights, for a batch (releases graphs captured before). */
int mgbf_batch_set_weights(mgbf_batch* b, const double* a, int n);
/* As mgbf_set_wait_limit, for a batch (releases graphs captured before). */
int mgbf_batch_set_wait_limit(mgbf_batch* b, int polls);
/* As mgbf_set_vertical_passes, for a batch (releases graphs captured before). */
int mgbf_batch_set_vertical_passes(mgbf_batch* b, int passes);
/* As mgbf_autotune, for a batch (releases graphs captured before). */
int mgbf_batch_autotune(mgbf_batch* b, int dtype, void* stream);
/* With blocks_per_sm > 0, runs each radial side (the pass after the
 * restriction, and the pass before the prolongation) of every variable
 * group as one persistent launch over all its generations: blocks_per_sm
 * resident blocks per SM (at most as many as fit) take tiles from a device
 * counter, instead of one launch per generation (FP32/BF16 storage with the
 * moment kernel; otherwise per generation).  0 (the default) launches per
 * generation.  Releases graphs captured before.  The reference has no
 * counterpart: its generations are filtered one after another on each
 * rank. */
int mgbf_batch_use_persistent(mgbf_batch* b, int blocks_per_sm);
/* Scheduling priority of the kernels in a batch's CUDA graphs (with
 * mgbf_batch_use_graphs): 0 (the default) leaves every kernel at the launch
 * stream's priority; 1 gives the memory-bound kernels (vertical filter,
 * restriction, prolongation) the device's highest priority and the radial
 * kernels its lowest; 2 the reverse.  The variable groups run as concurrent
 * graph branches, so the priority decides whose blocks the SMs take first
 * when one group's radial pass and another's restriction or prolongation
 * are both waiting.  Releases graphs captured before.  The reference has no
 * counterpart. */
int mgbf_batch_set_priorities(mgbf_batch* b, int mode);
/* The radial-filter kernel a batch runs for variable group `group`,
 * generation `gen` (0-based) and pass (0: the pass after the restriction,
 * 1: the pass before the prolongation) in storage type dtype: *variant as
 * in mgbf_set_tuning (-1: no moment kernel for this group, or not tuned:
 * the default) and *rows, the output rows per block (0: the default).
 * Extension for reporting what the autotuner chose; the reference has no
 * counterpart. */
int mgbf_batch_get_tuning(const mgbf_batch* b, int dtype, int group, int gen, int pass, int* variant, int* rows);
/* Pins the radial-filter kernel of one group, generation and pass (as
 * mgbf_batch_get_tuning reports it): variant as in mgbf_set_tuning (-1
 * returns to the default), rows the output rows per block (0: the
 * default).  Releases graphs captured before.  No reference counterpart. */
int mgbf_batch_set_tuning(mgbf_batch* b, int dtype, int group, int gen, int pass, int variant, int rows);

/* ------------------------------------------------------------------------
 * Allocation-free radial filtering (no counterpart in the reference).
 *
 * For callers that cannot allocate device memory -- work being captured
 * into a CUDA graph, applications whose device memory is all handed out by
 * their own pool, fixed memory budgets -- this computes
 *     y = weight * B(B(x))
 * on one compact FP32 field x (nk, im, jm) (level index fastest), where B is
 * the radial beta filter with half-sample mirror boundaries: the
 * generation-1 filtering of filtering_procedure with one generation and no
 * vertical filter.  x and y are device pointers supplied by the caller (y may
 * equal x).  Its two intermediate fields live in a static device array of
 * 2 * MGBF_NOALLOC_MAX_ELEMS floats (64 MiB) that every GPU loading the
 * library holds until exit; nk*(im+2*(reach+8))*jm must not exceed
 * MGBF_NOALLOC_MAX_ELEMS, larger fields return MGBF_ERR_ARG.  The radial
 * support must be the disk of radius reach+1/2 with p = 2 and a compiled
 * reach (4,5,6,8,10,12,16,24), else MGBF_ERR_UNSUPPORTED.  The first call on
 * a device looks up the array's device address and should come before any
 * stream capture (a lookup that fails returns MGBF_ERR_CUDA and is retried
 * by the next call).  Calls share the array, so calls that overlap on the GPU
 * race and must be ordered by the caller.  Asynchronous on `stream`.
 */
#define MGBF_NOALLOC_MAX_ELEMS ((size_t)8 << 20)
int mgbf_radial_filter_noalloc(const float* x, float* y, int nk, int im, int jm, int p, double mg_ampl02,
                               int hx, int hy, double weight, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MGBF_H */
