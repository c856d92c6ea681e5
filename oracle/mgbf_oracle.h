/*
 * FP64 CPU oracle for the MGBF filtering pipeline (test infrastructure only).
 *
 * This is a plain-C restatement of the reference's CPU algorithm for
 * filtering_procedure(1) (filtering_rad2_bckg), filtering_procedure(6)
 * (filtering_rad2_ens) and the fast 1D+1D variants filtering_procedure(3)
 * (filtering_fast_bckg) and (8) (filtering_fast_ens), evaluated on the
 * whole filter grid as one domain.
 * It exists to check the CUDA library; only tests, the smoke check and the
 * CPU-baseline leg of the benchmark call it.  Nothing in the shipped library
 * links or executes it.
 *
 * Parity status: unpinned.  The reference is Fortran 90 + MPI and no Fortran
 * compiler or MPI exists on the machines this project is built and tested on,
 * and the reference ships no tests, golden vectors or known-answer data for
 * this path.  The restatement is pinned only by its own invariants (adjoint
 * pairs, unit row sums, self-adjointness, symmetry) and by agreement with an
 * independent literal emulation of the reference's MPI tiling
 * (oracle/virtual_ranks.py).
 *
 * Storage follows the reference's VALL(km_all, 1-hx:im+hx, 1-hy:jm+hy)
 * (src.mgbf/mg_intstate.f90:157): level index fastest, then i, then j, FP64.
 */
#ifndef MGBF_ORACLE_H
#define MGBF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_GEN 16
/* proc 2 line filters: moment-table size nh and filter buffer nfil
 * (mg_parameter.f90:562-563) */
#define ORC_DIB_NH 6
#define ORC_DIB_NFIL (ORC_DIB_NH + 2)

typedef struct orc_cfg {
    int I, J;            /* generation-1 filter grid (im00 x jm00)            */
    int nk;              /* leading dimension of VALL (km_all)                */
    int hx, hy, hz;      /* halo widths (filter reach limits)                 */
    int p;               /* beta-function exponent (integer, as in reference) */
    double ampl01;       /* mg_ampl01: vertical aspect                        */
    double ampl02;       /* mg_ampl02: horizontal aspect                      */
    int gm;              /* number of generations                             */
    double a[ORC_MAX_GEN];  /* per-generation weights a_g (a[0] = gen 1)      */
    double b[ORC_MAX_GEN];  /* Helmholtz Laplacian coefficients (reference: 0) */
    int lhelm;           /* use weighting_helm form                           */
    int proc;            /* 1 rad2_bckg, 6 rad2_ens, 3 fast_bckg, 8 fast_ens, 4 rad3, 2 lin2_bckg,
                            7 lin2_ens, 5 lin3 */
    int l_vertical_filter;
    int l_filt_g1;       /* procs 6 and 8 only                                */
    int lquart;          /* quadratic (3-point) interpolation                 */
    int lm;              /* levels per vertical column                        */
    int nzcol;           /* number of z columns at offsets (k-1)*lm           */
    int nthreads;        /* OpenMP threads (<=0: runtime default)             */
    double ampl03;       /* mg_ampl03: aspect of the 3D filter (proc 4)       */
    int mgbf_line;       /* init_mg_line ran (procs 2, 5, 7: else identities) */
} orc_cfg;

/* Error codes (negative), mirroring the library's. */
#define ORC_OK 0
#define ORC_ERR_ARG (-1)
#define ORC_ERR_REACH (-3)
#define ORC_ERR_DIV (-4)

/* Apply the whole filtering procedure in place on V, laid out as
 * (nk, 1-hx:I+hx, 1-hy:J+hy).  Halo contents on entry are ignored except
 * where the reference would read them. */
int orc_filtering_procedure(const orc_cfg* c, double* V);

/* Same, on a compact (nk, I, J) array (x -> y; x == y allowed). */
int orc_filter_compact(const orc_cfg* c, const double* x, double* y);

/* Per-generation weight gradients: ga[g] = sum u_g * v_g with
 * u_g = B_g R_g Bz^T x and v_g = B_g R_g Bz^T gy (compact arrays). */
int orc_weight_grads(const orc_cfg* c, const double* x, const double* gy, double* ga);

/* Stage-level entry points on compact arrays, for adjoint-pair tests.
 * which: 0 = z forward Bz, 1 = z adjoint Bz^T,
 *        2 = horizontal forward (fill + vrbeta2), 3 = horizontal adjoint
 *            (vrbeta2t + fold), on a generation-g grid (g given by gen),
 *        4 = restriction R (g -> g+1; x is gen g, y is gen g+1),
 *        5 = prolongation P (g+1 -> g; x is gen g+1, y is gen g),
 *        6 = fast-filter horizontal forward (bocoy, rbeta y, bocox, rbeta x),
 *        7 = fast-filter horizontal adjoint (rbetaT x, bocoTx, rbetaT y,
 *            bocoTy), on a generation-g grid,
 *        8 = proc 2 line filters forward (boco_2d + dibeta, colors 1..3),
 *        9 = their adjoint (dibetat + bocoT_2d, colors 3..1),
 *       10 = one whole generation of proc 5 (filtering_lin3: adjoint side,
 *            weight a_gen, forward side; _g1 halo routines at gen 1). */
int orc_stage(const orc_cfg* c, int which, int gen, const double* x, double* y);

/* Setup values (for tests): rmom2_1, rmom2_2, exx (1D), exx (2D), ss1, ss2,
 * vertical reach, horizontal reach, and for the fast filters' line filter
 * exx, ss, reach.  Returns error if a reach exceeds a halo. */
int orc_setup_values(const orc_cfg* c, double out[11]);

/* Proc 2 (filtering_lin2_bckg) line filters, for tests: the three colors'
 * generators (dx, dy), integer half-spans h, formal half-spans hs and
 * dibeta weights fil[q*(ORC_DIB_NFIL+1) + i], i = 0..h (zero beyond). */
int orc_dibeta_values(const orc_cfg* c, int gen[6], int h[3], double hs[3], double fil[3 * (ORC_DIB_NFIL + 1)]);

/* The triad decomposition alone: asp = (A11, A22, A12) -> generators
 * lt = (dx0, dy0, dx1, dy1, dx2, dy2) and weights w. */
int orc_triad(const double asp[3], int lt[6], double w[3]);

/* The hexad decomposition: asp = (A11, A22, A33, A23, A31, A12) ->
 * generators lh[3*(c-1)..3*(c-1)+2] and weights w[c-1] for colors c = 1..7
 * (the hexad's own color null). */
int orc_hexad(const double asp[6], int lh[21], double w[7]);

/* ----------------------------------------------------------------------
 * Transfers between the analysis grid and the filter grid (the new map,
 * l_new_map: anal_to_filt_all2 / filt_to_anal_all2, mg_transfer.f90:154-203,
 * 339-464; offset interpolations mg_interpolate.f90:89-298, 634-960;
 * vertical l_vertical_*_spec2, mg_interpolate.f90:963-1044).
 * WORKA is (nka, nm0, mm0) with the level index fastest. */
typedef struct orc_xfer {
    int nm0, mm0;     /* analysis grid                                         */
    int nxpe, nype;   /* rank layout: nm = nm0/nxpe analysis points per rank   */
    int im, jm;       /* filter points per rank (im_filt, jm_filt)             */
    int hx, hy;       /* VALL halo widths                                      */
    int nkf, nka;     /* leading dims: filter km_all, analysis km_a_all         */
    int lm, lm_a, en; /* vertical: en = km3*n_ens blocks of lm_a / lm levels    */
    int order;        /* 3 = lsqr (default), 2 = quad, 1 = lin                  */
} orc_xfer;

/* anal_to_filt_all2: VALL (nkf, 1-hx:I+hx, 1-hy:J+hy) = 0, then the
 * adjoint interpolation of WORKA and bocoT_2d over the interpolation halo. */
int orc_anal_to_filt(const orc_xfer* c, const double* worka, double* vall);

/* filt_to_anal_all2: boco_2d fills VALL's halo (interpolation width), then
 * the direct interpolation into WORKA. */
int orc_filt_to_anal(const orc_xfer* c, double* vall, double* worka);

#ifdef __cplusplus
}
#endif
#endif
