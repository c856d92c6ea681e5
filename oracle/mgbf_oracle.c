/*
 * FP64 CPU oracle for the MGBF filtering pipeline -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates, on one global filter grid, the reference's CPU algorithm for
 * filtering_procedure(1), (6), the fast 1D+1D variants (3) and (8),
 * filtering_rad3 (4) and the line-filter procedures filtering_lin2_bckg (2),
 * filtering_lin3 (5) and filtering_lin2_ens (7).
 * Every routine below
 * names the reference routine (file:line, paths inside the reference project)
 * whose loops it follows.  The MPI halo exchange of the reference collapses
 * into the global-edge mirror/fold that mg_bocos applies at physical
 * boundaries; interior rank boundaries disappear because one array holds the
 * whole grid.  See mgbf_oracle.h for the parity status (unpinned).
 *
 * Only tests/, the smoke check and the benchmark's CPU-baseline leg use this.
 */
#include "mgbf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ arrays */

typedef struct {
    double* d;
    int nk, ilo, ihi, jlo, jhi;
} arr3;

static inline size_t a3i(const arr3* a, int k, int i, int j) {
    return (size_t)k + (size_t)a->nk * ((size_t)(i - a->ilo) +
                                        (size_t)(a->ihi - a->ilo + 1) * (size_t)(j - a->jlo));
}
#define A3(a, k, i, j) ((a).d[a3i(&(a), (k), (i), (j))])

static arr3 a3_alloc(int nk, int ilo, int ihi, int jlo, int jhi) {
    arr3 a;
    a.nk = nk; a.ilo = ilo; a.ihi = ihi; a.jlo = jlo; a.jhi = jhi;
    size_t n = (size_t)nk * (size_t)(ihi - ilo + 1) * (size_t)(jhi - jlo + 1);
    a.d = (double*)calloc(n ? n : 1, sizeof(double));
    return a;
}
static void a3_free(arr3* a) { free(a->d); a->d = NULL; }

/* Row parallelism.  Inside the k-split parallel region of
 * orc_filtering_procedure every thread runs the pipeline on its own level
 * range and the loops below stay serial.  Called outside any parallel region
 * (few levels per thread, the stage entry points, the weight gradients) the
 * loops marked ROWPAR split their rows over g_threads threads instead.  Each
 * row-parallel loop either writes whole rows of its output from inputs it
 * does not write, or (the two scatters vrbeta2t and adjoint4) is written in a
 * target-row form that adds every target's contributions in the order of the
 * literal loop; either way the results are bit-identical to the serial
 * literal loops. */
static int g_threads = 1;
#ifdef _OPENMP
#define ROWPAR (!omp_in_parallel() && g_threads > 1)
#define PRAGMA(x) _Pragma(#x)
#define ROW_FOR PRAGMA(omp parallel for schedule(static) if(ROWPAR) num_threads(g_threads))
static void set_threads(int n) { g_threads = n > 0 ? n : omp_get_max_threads(); }
#else
#define ROWPAR 0
#define ROW_FOR
static void set_threads(int n) { (void)n; g_threads = 1; }
#endif

/* Zero k-range [k0,k1) of every cell. */
static void a3_zero(arr3 a, int k0, int k1) {
    ROW_FOR
    for (int j = a.jlo; j <= a.jhi; ++j)
        for (int i = a.ilo; i <= a.ihi; ++i)
            for (int k = k0; k < k1; ++k) A3(a, k, i, j) = 0.0;
}
static void a3_copy(arr3 dst, arr3 src, int k0, int k1) {
    ROW_FOR
    for (int j = dst.jlo; j <= dst.jhi; ++j)
        for (int i = dst.ilo; i <= dst.ihi; ++i)
            for (int k = k0; k < k1; ++k) A3(dst, k, i, j) = A3(src, k, i, j);
}

static inline double ipow(double x, int p) {
    /* Fortran real**integer; p >= 0 */
    double r = 1.0;
    for (int t = 0; t < p; ++t) r *= x;
    return r;
}

/* ------------------------------------------------------------------ setup */

typedef struct {
    double rmom2_1, rmom2_2;
    double exx1;          /* el*rmom2_1 for the vertical filter          */
    double exx2, eyy2;    /* el*rmom2_2 for the horizontal filter        */
    double eyx2;          /* off-diagonal (zero: no anisotropy)          */
    double ss1, ss2;      /* inverse line sums                           */
    int reach1, reach2;
    double exxL, ssL;     /* fast filters' 1D horizontal line filter     */
    int reachL;
    double e3, ss3;       /* filtering_rad3's ball: el*rmom2_3, 1/sum    */
    int reach3;
    /* filtering_lin2_bckg's three line filters (colors): generator, integer
     * half-span, formal half-span and dibeta weights fil[0..h] */
    int ddx[3], ddy[3], dh[3];
    double dhs[3];
    double dfil[3][ORC_DIB_NFIL + 1];
    /* filtering_lin3's hexad (proc 5): for colors 1..7 the active slot (or
     * -1), per slot the generator, half-span and weights */
    int hslot[8];
    int hgen[6][3], hh[6];
    double hhs[6];
    double hfil[6][ORC_DIB_NFIL + 1];
} setup_t;

static const double EPS = 1.e-12;
static int dibeta_setup(const orc_cfg* c, setup_t* s);
static int hexad_setup(const orc_cfg* c, setup_t* s);

/* mg_parameter.f90:567-572 (rmom2), mg_intstate.f90:360-431 (pasp, cholaspect,
 * getlinesum), jp_pbfil.f90:74-107 (cholaspect1/2), 149-218 (getlinesum1/2). */
static int setup(const orc_cfg* c, setup_t* s) {
    double pee2 = 2.0 * c->p;
    s->rmom2_1 = 1.0 / sqrt(pee2 + 3.0);
    s->rmom2_2 = 1.0 / sqrt(pee2 + 4.0);
    /* cholaspect1: el = 1/sqrt(pasp1) */
    double el1 = 1.0 / sqrt(c->ampl01);
    /* cholaspect2 on diag(pasp02,pasp02): inv -> diag(1/pasp02); Cholesky ->
     * diag(sqrt(1/pasp02)), zero off-diagonal. */
    double el2 = sqrt(1.0 / c->ampl02);
    s->exx1 = el1 * s->rmom2_1;
    s->exx2 = el2 * s->rmom2_2;
    s->eyy2 = el2 * s->rmom2_2;
    s->eyx2 = 0.0;

    /* getlinesum1 (jp_pbfil.f90:149-180) with hx := hz */
    {
        double x = 1.0 / s->exx1;
        int gxl = (int)ceil(-x + EPS), gxm = (int)floor(x - EPS);
        if (c->l_vertical_filter && (gxl < -c->hz || gxm > c->hz)) return ORC_ERR_REACH;
        double sum = 0.0;
        for (int gx = gxl; gx <= gxm; ++gx) {
            double xx = gx;
            double rr = (xx * s->exx1) * (xx * s->exx1);
            sum += ipow(1.0 - rr, c->p);
        }
        s->ss1 = 1.0 / sum;
        s->reach1 = gxm;
    }
    /* getlinesum2 (jp_pbfil.f90:182-218) */
    {
        double sum = 0.0;
        double exx = s->exx2, eyy = s->eyy2, eyx = s->eyx2;
        double y = 1.0 / eyy;
        int gyl = (int)ceil(-y + EPS), gym = (int)floor(y - EPS);
        if (gyl < -c->hy || gym > c->hy) return ORC_ERR_REACH;
        int reach = 0;
        for (int gy = gyl; gy <= gym; ++gy) {
            double yy = gy, xc = -yy * eyx;
            double rrx = (yy * eyy) * (yy * eyy);
            double x = sqrt(1.0 - rrx);
            int gxl = (int)ceil((xc - x) / exx + EPS), gxm = (int)floor((xc + x) / exx - EPS);
            if (gxl < -c->hx || gxm > c->hx) return ORC_ERR_REACH;
            if (gxm > reach) reach = gxm;
            for (int gx = gxl; gx <= gxm; ++gx) {
                double xx = gx;
                double rr = rrx + (xx * exx - xc) * (xx * exx - xc);
                sum += ipow(1.0 - rr, c->p);
            }
        }
        s->ss2 = 1.0 / sum;
        s->reach2 = reach > gym ? reach : gym;
    }
    /* getlinesum1 on paspx / paspy (mg_intstate.f90:427-428): these aspects
     * skip cholaspect, so el = pasp02 itself (mg_intstate.f90:370-375). */
    {
        s->exxL = c->ampl02 * s->rmom2_1;
        double x = 1.0 / s->exxL;
        int gxl = (int)ceil(-x + EPS), gxm = (int)floor(x - EPS);
        int fast = c->proc == 3 || c->proc == 8;
        if (fast && (gxl < -c->hx || gxm > c->hx || gxl < -c->hy || gxm > c->hy)) return ORC_ERR_REACH;
        double sum = 0.0;
        for (int gx = gxl; gx <= gxm; ++gx) {
            double xx = gx, rr = (xx * s->exxL) * (xx * s->exxL);
            sum += ipow(1.0 - rr, c->p);
        }
        s->ssL = 1.0 / sum;
        s->reachL = gxm;
    }
    /* cholaspect3 (jp_pbfil.f90:109-126) on pasp3 = diag(pasp03) and
     * getlinesum3 (jp_pbfil.f90:220-268); rmom2_3 = 1/sqrt(2p+5). */
    {
        const double e = sqrt(1.0 / c->ampl03) * (1.0 / sqrt(pee2 + 5.0));
        s->e3 = e;
        double z = 1.0 / e;
        int gzl = (int)ceil(-z + EPS), gzm = (int)floor(z - EPS);
        int bad = gzl < -c->hz || gzm > c->hz;
        double sum = 0.0;
        for (int gz = gzl; gz <= gzm; ++gz) {
            double zz = gz, rry = (zz * e) * (zz * e), y = sqrt(1.0 - rry);
            int gyl = (int)ceil((0.0 - y) / e + EPS), gym = (int)floor((0.0 + y) / e - EPS);
            if (gyl < -c->hy || gym > c->hy) bad = 1;
            for (int gy = gyl; gy <= gym; ++gy) {
                double yy = gy, rrx = rry + (yy * e - 0.0) * (yy * e - 0.0), x = sqrt(1.0 - rrx);
                int gxl = (int)ceil((0.0 - x) / e + EPS), gxm = (int)floor((0.0 + x) / e - EPS);
                if (gxl < -c->hx || gxm > c->hx) bad = 1;
                for (int gx = gxl; gx <= gxm; ++gx) {
                    double xx = gx, rr = rrx + (xx * e - 0.0) * (xx * e - 0.0);
                    sum += ipow(1.0 - rr, c->p);
                }
            }
        }
        if (c->proc == 4 && bad) return ORC_ERR_REACH;
        s->ss3 = 1.0 / sum;
        s->reach3 = gzm;
    }
    if (c->proc == 2 || c->proc == 7) return dibeta_setup(c, s);
    if (c->proc == 5) {
        int rc = dibeta_setup(c, s);
        return rc ? rc : hexad_setup(c, s);
    }
    return ORC_OK;
}

/* ------------------------------------------ proc 2 line-filter setup */

/* Moment tables of inimomtab (jp_pbfil3.f90:378-457) for the beta filters of
 * integer half-span h = 1..nh: bnorm(h) = 1 / sum_i (1-(i/h)^2)^p and
 * bsprds(h) = sum_i i^2 (1-(i/h)^2)^p / sum_i (1-(i/h)^2)^p over i = -h..h.
 * The reference evaluates the continuum moments plus their Euler-Maclaurin
 * corrections, which for these polynomial weights are the exact sums. */
static void dib_moments(int p, double* bnorm, double* bsprd) {
    for (int h = 1; h <= ORC_DIB_NH; ++h) {
        double s0 = 0.0, s2 = 0.0;
        for (int i = -h; i <= h; ++i) {
            double z = (double)i / h, w = ipow(1.0 - z * z, p);
            s0 += w;
            s2 += (double)i * i * w;
        }
        bnorm[h] = 1.0 / s0;
        bsprd[h] = s2 / s0;
    }
}

/* hstform (jp_pbfil3.f90:1399-1430) of a spread^2 into the formal half-span
 * hs between two table entries, then blinfil (1463-1501): the weights
 * fil[0..h] of the two-beta filter of half-spans h = int(hs) and h+1. */
static int dib_weights(int p, double spread, const double* bnorm, const double* bsprd, int* h_out, double* hs_out,
                       double* f) {
    double hs = spread;
    int found = 0;
    if (hs >= 0.0)
        for (int h = 2; h <= ORC_DIB_NH && !found; ++h)
            if (bsprd[h] >= hs) {
                hs = h - (bsprd[h] - hs) / (bsprd[h] - bsprd[h - 1]);
                found = 1;
            }
    if (!found) return ORC_ERR_REACH;
    const int h = (int)hs, hp = h + 1;
    if (h < 1 || hp > ORC_DIB_NH || hp > ORC_DIB_NFIL) return ORC_ERR_REACH;
    const double whp = (hs - h) * bnorm[hp], wh = (hp - hs) * bnorm[h];
    for (int i = 0; i <= ORC_DIB_NFIL; ++i) f[i] = 0.0;
    for (int i = 0; i <= h; ++i) {
        double z = (double)i / hp;
        f[i] = whp * ipow(1.0 - z * z, p);
    }
    for (int i = 0; i < h; ++i) {
        double z = (double)i / h;
        f[i] += wh * ipow(1.0 - z * z, p);
    }
    *h_out = h;
    *hs_out = hs;
    return ORC_OK;
}

/* triad (jp_pbfil3.f90:573-624): resolve the aspect 3-vector (A11, A22, A12)
 * onto three integer line generators lt[q] with weights w[q] >= 0 (up to
 * -1e-14) such that A = sum_q w[q] lt[q] lt[q]^T.  Starts from the generators
 * (1,0), (0,1), (-1,-1); while the smallest weight is negative, flips and
 * recombines the generators and updates the projection rows. */
int orc_triad(const double asp[3], int lt_out[6], double w_out[3]) {
    int lt[3][2] = {{1, 0}, {0, 1}, {-1, -1}};
    int lu[3][3] = {{1, 0, -1}, {0, 1, -1}, {0, 0, 1}};  /* lu[col][row] */
    double w[3];
    for (int q = 0; q < 3; ++q) w[q] = asp[0] * lu[q][0] + asp[1] * lu[q][1] + asp[2] * lu[q][2];
    int it;
    for (it = 1; it <= 200; ++it) {
        int k = 0;
        for (int q = 1; q < 3; ++q)
            if (w[q] < w[k]) k = q;  /* first minimum */
        const double dw = 2.0 * w[k];
        if (dw >= -1.e-14) break;
        const int l = (k + 1) % 3, m = (l + 1) % 3;
        int dl[3];
        for (int r = 0; r < 3; ++r) dl[r] = 2 * lu[k][r];
        lt[l][0] = -lt[l][0]; lt[l][1] = -lt[l][1];
        lt[k][0] = -lt[l][0] - lt[m][0]; lt[k][1] = -lt[l][1] - lt[m][1];
        for (int q = 0; q < 3; ++q) {
            const int sg = q == k ? -1 : 1;
            for (int r = 0; r < 3; ++r) lu[q][r] += dl[r] * sg;
            w[q] += sg * dw;
        }
    }
    for (int q = 0; q < 3; ++q) {
        lt_out[2 * q] = lt[q][0]; lt_out[2 * q + 1] = lt[q][1];
        w_out[q] = w[q];
    }
    return it > 200 ? ORC_ERR_ARG : ORC_OK;
}

/* init_mg_line (mg_intstate.f90:436-480) for proc 2.  It runs after
 * def_mg_weights has replaced pasp2 = diag(mg_ampl02) by the Cholesky factor
 * of its inverse (mg_intstate.f90:385-388, 423), so the triad sees
 * (c, c, 0), c = 1/sqrt(mg_ampl02).  Each color's spread^2 then goes
 * through hstform (jp_pbfil3.f90:1399-1430: the formal half-span between
 * consecutive table entries) and blinfil (1463-1501: the weights of the
 * two-beta "dibeta" filter).  A spread beyond the table, a half-span the
 * table cannot hold, or a reach beyond the halo is an error here; the
 * reference prints and carries on (or reads outside its arrays). */
static int dibeta_setup(const orc_cfg* c, setup_t* s) {
    if (!c->mgbf_line) {
        /* init_mg_line did not run (mg_entrymod.f90:155-157): zero
         * generators, vdibeta2's copy branch for every color */
        for (int q = 0; q < 3; ++q) {
            s->ddx[q] = s->ddy[q] = s->dh[q] = 0;
            s->dhs[q] = 0.0;
            for (int i = 0; i <= ORC_DIB_NFIL; ++i) s->dfil[q][i] = i == 0 ? 1.0 : 0.0;
        }
        return ORC_OK;
    }
    double bnorm[ORC_DIB_NH + 1], bsprd[ORC_DIB_NH + 1];
    dib_moments(c->p, bnorm, bsprd);
    const double el = sqrt(1.0 / c->ampl02);
    const double asp[3] = {el, el, 0.0};
    int lt[6];
    double w[3];
    if (orc_triad(asp, lt, w)) return ORC_ERR_ARG;
    for (int q = 0; q < 3; ++q) {
        int rc = dib_weights(c->p, w[q], bnorm, bsprd, &s->dh[q], &s->dhs[q], s->dfil[q]);
        if (rc) return rc;
        s->ddx[q] = lt[2 * q]; s->ddy[q] = lt[2 * q + 1];
        if (s->dh[q] * abs(s->ddx[q]) > c->hx || s->dh[q] * abs(s->ddy[q]) > c->hy) return ORC_ERR_REACH;
    }
    return ORC_OK;
}

/* hexad (jp_pbfil3.f90:798-904): resolve the 3D aspect 6-vector
 * (A11, A22, A33, A23, A31, A12) onto the seven nonnull GF(8) "colors" of a
 * hexad (one of them, the hexad's own color, null): integer generators
 * lh[3*(c-1)..] and weights w[c-1], c = 1..7, with A = sum w l l^T.  The
 * iteration moves only the K-set of three generators (the others follow
 * from it) and applies a rank-1 update to the projection rows per step;
 * the default K-set and projections, the six K-set update matrices, the
 * step offsets, the sign pattern and the output color order are the
 * reference's tables, restated here. */
int orc_hexad(const double asp[6], int lh[21], double w7[7]) {
    static const int deflhex[7][3] = {{0, 0, 0}, {1, -1, 0}, {0, 1, -1}, {0, 0, 1}, {-1, 0, 1}, {0, 1, 0}, {1, 0, 0}};
    static const int deflui[7][6] = {{0, 0, 0, 0, 0, 0},  {0, 0, 0, 0, 0, -1}, {0, 0, 0, -1, 0, 0}, {0, 0, 1, 1, 1, 0},
                                     {0, 0, 0, 0, -1, 0}, {0, 1, 0, 1, 0, 1},  {1, 0, 0, 0, 1, 1}};
    /* M[d-1][c][r]: column c of the K-set update for step d = 1..6 */
    static const int mm[6][3][3] = {{{1, 1, -1}, {1, 0, 0}, {1, 0, -1}},   {{-1, 1, 0}, {-1, 1, 1}, {0, 1, 0}},
                                    {{0, -1, 1}, {1, -1, 0}, {1, 0, 0}},   {{0, 0, 1}, {0, -1, 1}, {1, -1, 1}},
                                    {{-1, 0, 1}, {0, 0, 1}, {-1, 1, 0}},   {{0, 1, 0}, {1, 0, -1}, {0, 1, -1}}};
    static const int ttriad[7] = {0, 5, 3, 3, 6, 5, 6};                                  /* index 1..6 */
    static const int sstriad[13] = {-1, -1, 1, -1, 1, 1, 1, -1, -1, 1, -1, 1, 1};        /* index -6..6 */
    static const int line[3] = {1, 2, 4};
    static const int jcol[7] = {7, 4, 6, 3, 5, 2, 1};
#define MOD7(a) ((((a) % 7) + 7) % 7)
    int lhex[7][3], lui[7][6], K[3][3];
    double wh[7];
    memcpy(lhex, deflhex, sizeof(lhex));
    memcpy(lui, deflui, sizeof(lui));
    int hcol = 0, kcol = 0;
    for (int q = 0; q < 7; ++q) {
        wh[q] = 0.0;
        for (int r = 0; r < 6; ++r) wh[q] += asp[r] * lui[q][r];
    }
    for (int i = 0; i < 3; ++i) memcpy(K[i], lhex[MOD7(hcol - line[i])], sizeof(K[i]));
    int it;
    for (it = 1; it <= 200; ++it) {
        kcol = 0;
        for (int q = 1; q < 7; ++q)
            if (wh[q] < wh[kcol]) kcol = q;
        const double dw = wh[kcol];
        if (dw >= -1.e-14) break;
        const int dcol = MOD7(kcol - hcol);
        hcol = kcol;
        const int L = MOD7(hcol + ttriad[dcol]);
        int Kn[3][3];
        for (int cc = 0; cc < 3; ++cc)
            for (int e = 0; e < 3; ++e) {
                int v = 0;
                for (int r = 0; r < 3; ++r) v += K[r][e] * mm[dcol - 1][cc][r];
                Kn[cc][e] = v;
            }
        memcpy(K, Kn, sizeof(K));
        int dl[6];
        for (int r = 0; r < 6; ++r) dl[r] = lui[hcol][r];
        for (int q = 0; q < 7; ++q) {
            const int sg = sstriad[q - L + 6];
            for (int r = 0; r < 6; ++r) lui[q][r] += dl[r] * sg;
            wh[q] += sg * dw;
        }
    }
    if (it > 200) return ORC_ERR_ARG;
    for (int i = 0; i < 3; ++i) {
        const int ip = (i + 1) % 3;
        for (int e = 0; e < 3; ++e) {
            lhex[MOD7(hcol - line[i])][e] = K[i][e];
            lhex[MOD7(hcol + line[i])][e] = K[i][e] - K[ip][e];
        }
    }
    for (int e = 0; e < 3; ++e) lhex[kcol][e] = 0;
    for (int i = 0; i < 7; ++i) {
        const int j = jcol[i] - 1;
        for (int e = 0; e < 3; ++e) lh[3 * j + e] = lhex[i][e];
        w7[j] = wh[i];
    }
#undef MOD7
    return ORC_OK;
}

/* init_mg_line's hextform (mg_intstate.f90:471; jp_pbfil3.f90:702-750) for
 * proc 5: pasp3 = diag(mg_ampl03) after cholaspect3 is diag(c3),
 * c3 = 1/sqrt(mg_ampl03); the hexad's six active colors in ascending order,
 * each spread^2 through the half-span transform and the two-beta weights. */
static int hexad_setup(const orc_cfg* c, setup_t* s) {
    for (int col = 0; col < 8; ++col) s->hslot[col] = -1;
    if (!c->mgbf_line) return ORC_OK;  /* qcols stay zero: every color copies */
    double bnorm[ORC_DIB_NH + 1], bsprd[ORC_DIB_NH + 1];
    dib_moments(c->p, bnorm, bsprd);
    const double c3 = sqrt(1.0 / c->ampl03);
    const double asp[6] = {c3, c3, c3, 0.0, 0.0, 0.0};
    int lh[21];
    double w7[7];
    if (orc_hexad(asp, lh, w7)) return ORC_ERR_ARG;
    int slot = 0;
    for (int col = 0; col < 8; ++col) s->hslot[col] = -1;
    for (int col = 1; col <= 7; ++col) {
        const int* g = &lh[3 * (col - 1)];
        if (g[0] == 0 && g[1] == 0 && g[2] == 0) continue;
        if (slot == 6) return ORC_ERR_ARG;
        s->hslot[col] = slot;
        for (int e = 0; e < 3; ++e) s->hgen[slot][e] = g[e];
        int rc = dib_weights(c->p, w7[col - 1], bnorm, bsprd, &s->hh[slot], &s->hhs[slot], s->hfil[slot]);
        if (rc) return rc;
        const int h = s->hh[slot];
        if (h * abs(g[0]) > c->hx || h * abs(g[1]) > c->hy || h * abs(g[2]) > c->hz) return ORC_ERR_REACH;
        ++slot;
    }
    return slot == 6 ? ORC_OK : ORC_ERR_ARG;  /* hextform: exactly six active lines */
}

int orc_dibeta_values(const orc_cfg* c, int gen[6], int h[3], double hs[3], double fil[3 * (ORC_DIB_NFIL + 1)]) {
    setup_t s;
    int rc = setup(c, &s);
    if (rc) return rc;
    if (c->proc != 2 && c->proc != 7 && (rc = dibeta_setup(c, &s))) return rc;
    for (int q = 0; q < 3; ++q) {
        gen[2 * q] = s.ddx[q]; gen[2 * q + 1] = s.ddy[q];
        h[q] = s.dh[q]; hs[q] = s.dhs[q];
        for (int i = 0; i <= ORC_DIB_NFIL; ++i) fil[q * (ORC_DIB_NFIL + 1) + i] = s.dfil[q][i];
    }
    return ORC_OK;
}

int orc_setup_values(const orc_cfg* c, double out[11]) {
    setup_t s;
    int rc = setup(c, &s);
    if (rc) return rc;
    out[0] = s.rmom2_1; out[1] = s.rmom2_2; out[2] = s.exx1; out[3] = s.exx2;
    out[4] = s.ss1; out[5] = s.ss2; out[6] = s.reach1; out[7] = s.reach2;
    out[8] = s.exxL; out[9] = s.ssL; out[10] = s.reachL;
    return ORC_OK;
}

/* --------------------------------------------------- horizontal beta filter */

/* vrbeta2 (jp_pbfil.f90:888-928): gather over the extended domain, output on
 * the interior, halo of the result zeroed; then a = b.  k-range [k0,k1). */
/* The disk of vrbeta2 / vrbeta2t: for every row gy its column range and
 * the weights frow = s*(1-rr)^p, computed by the reference's own formulas
 * (jp_pbfil.f90:909-924).  The stencil is the same at every point (uniform
 * aspect), so the table is built once per call; the sums below visit the
 * taps in the reference's order, so the results equal those of evaluating
 * the formulas at every point. */
typedef struct {
    int gyl, gym;
    int* gxl;     /* per row (index gy - gyl) */
    int* gxm;
    double** w;   /* w[row][gx - gxl[row]] */
} disk_t;

static disk_t disk_table(const setup_t* S, int p) {
    disk_t d;
    double exx = S->exx2, eyy = S->eyy2, eyx = S->eyx2, s = S->ss2;
    double y = 1.0 / eyy;
    d.gyl = (int)ceil(-y + EPS);
    d.gym = (int)floor(y - EPS);
    int n = d.gym - d.gyl + 1;
    d.gxl = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    d.gxm = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    d.w = (double**)malloc(sizeof(double*) * (size_t)(n > 0 ? n : 1));
    for (int gy = d.gyl; gy <= d.gym; ++gy) {
        int r = gy - d.gyl;
        double yy = gy, xc = -yy * eyx;
        double rrx = (yy * eyy) * (yy * eyy);
        double x = sqrt(1.0 - rrx);
        int gxl = (int)ceil((xc - x) / exx + EPS), gxm = (int)floor((xc + x) / exx - EPS);
        d.gxl[r] = gxl;
        d.gxm[r] = gxm;
        d.w[r] = (double*)malloc(sizeof(double) * (size_t)(gxm >= gxl ? gxm - gxl + 1 : 1));
        for (int gx = gxl; gx <= gxm; ++gx) {
            double xx = gx;
            double rr = rrx + (xx * exx - xc) * (xx * exx - xc);
            d.w[r][gx - gxl] = s * ipow(1.0 - rr, p);
        }
    }
    return d;
}

static void disk_free(disk_t* d) {
    for (int r = 0; r <= d->gym - d->gyl; ++r) free(d->w[r]);
    free(d->w);
    free(d->gxl);
    free(d->gxm);
}

static void vrbeta2(const setup_t* S, int p, arr3 a, arr3 b, int Lx, int Mx, int Ly, int My,
                    int k0, int k1, double* tb) {
    a3_zero(b, k0, k1);
    disk_t D = disk_table(S, p);
    const int par = ROWPAR;
#ifdef _OPENMP
#pragma omp parallel if(par) num_threads(g_threads)
#endif
    {
        double* tbl = par ? (double*)malloc(sizeof(double) * (size_t)a.nk) : tb;
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int iy = Ly; iy <= My; ++iy)
            for (int ix = Lx; ix <= Mx; ++ix) {
                for (int k = k0; k < k1; ++k) tbl[k] = 0.0;
                for (int gy = D.gyl; gy <= D.gym; ++gy) {
                    int jy = iy + gy, r = gy - D.gyl;
                    for (int gx = D.gxl[r]; gx <= D.gxm[r]; ++gx) {
                        int jx = ix + gx;
                        double frow = D.w[r][gx - D.gxl[r]];
                        const double* src = &A3(a, 0, jx, jy);
                        for (int k = k0; k < k1; ++k) tbl[k] += frow * src[k];
                    }
                }
                double* dst = &A3(b, 0, ix, iy);
                for (int k = k0; k < k1; ++k) dst[k] = tbl[k];
            }
        if (par) free(tbl);
    }
    disk_free(&D);
    a3_copy(a, b, k0, k1);
}

/* vrbeta2t (jp_pbfil.f90:1011-1050): scatter from the interior into the
 * extended domain (b starts at zero); then a = b. */
static void vrbeta2t(const setup_t* S, int p, arr3 a, arr3 b, int Lx, int Mx, int Ly, int My,
                     int k0, int k1) {
    a3_zero(b, k0, k1);
    disk_t D = disk_table(S, p);
    if (!ROWPAR) {
        for (int iy = Ly; iy <= My; ++iy)
            for (int ix = Lx; ix <= Mx; ++ix) {
                const double* ta = &A3(a, 0, ix, iy);
                for (int gy = D.gyl; gy <= D.gym; ++gy) {
                    int jy = iy + gy, r = gy - D.gyl;
                    for (int gx = D.gxl[r]; gx <= D.gxm[r]; ++gx) {
                        int jx = ix + gx;
                        double frow = D.w[r][gx - D.gxl[r]];
                        double* dst = &A3(b, 0, jx, jy);
                        for (int k = k0; k < k1; ++k) dst[k] += frow * ta[k];
                    }
                }
            }
    } else {
        /* target-row form: a thread owns the target rows jy and visits their
         * source rows iy = jy - gy in increasing order and the source
         * columns ix in increasing order, the order in which the literal
         * loop above adds into any one target */
        ROW_FOR
        for (int jy = Ly + D.gyl; jy <= My + D.gym; ++jy) {
            int iylo = jy - D.gym > Ly ? jy - D.gym : Ly, iyhi = jy - D.gyl < My ? jy - D.gyl : My;
            for (int iy = iylo; iy <= iyhi; ++iy) {
                int gy = jy - iy, r = gy - D.gyl;
                for (int ix = Lx; ix <= Mx; ++ix) {
                    const double* ta = &A3(a, 0, ix, iy);
                    for (int gx = D.gxl[r]; gx <= D.gxm[r]; ++gx) {
                        double frow = D.w[r][gx - D.gxl[r]];
                        double* dst = &A3(b, 0, ix + gx, jy);
                        for (int k = k0; k < k1; ++k) dst[k] += frow * ta[k];
                    }
                }
            }
        }
    }
    disk_free(&D);
    a3_copy(a, b, k0, k1);
}

/* ------------------------------------------------------ halo fill and fold */

/* boco_2d semantics at physical edges (mg_bocos.f90:225-377): y first on the
 * interior columns, then x on all rows including the y-halo rows;
 * half-sample mirror W(1-t) = W(t), W(M+t) = W(M+1-t). */
static void fill_h(arr3 W, int imax, int jmax, int nbx, int nby, int k0, int k1) {
    for (int j = 1; j <= nby; ++j)
        for (int i = 1; i <= imax; ++i)
            for (int k = k0; k < k1; ++k) {
                A3(W, k, i, -nby + j) = A3(W, k, i, nby + 1 - j);
            }
    for (int j = 1; j <= nby; ++j)
        for (int i = 1; i <= imax; ++i)
            for (int k = k0; k < k1; ++k) {
                A3(W, k, i, jmax + j) = A3(W, k, i, jmax + 1 - j);
            }
    for (int j = 1 - nby; j <= jmax + nby; ++j)
        for (int i = 1; i <= nbx; ++i)
            for (int k = k0; k < k1; ++k) {
                A3(W, k, -nbx + i, j) = A3(W, k, nbx + 1 - i, j);
            }
    for (int j = 1 - nby; j <= jmax + nby; ++j)
        for (int i = 1; i <= nbx; ++i)
            for (int k = k0; k < k1; ++k) {
                A3(W, k, imax + i, j) = A3(W, k, imax + 1 - i, j);
            }
}

/* bocoT_2d semantics at physical edges (mg_bocos.f90:929-1061): x first on
 * all rows, then y on the interior columns; halo values are left in place. */
static void fold_h(arr3 W, int imax, int jmax, int nbx, int nby, int k0, int k1) {
    for (int j = 1 - nby; j <= jmax + nby; ++j)
        for (int i = 1; i <= nbx; ++i)
            for (int k = k0; k < k1; ++k) A3(W, k, i, j) += A3(W, k, 1 - i, j);
    for (int j = 1 - nby; j <= jmax + nby; ++j)
        for (int i = 1; i <= nbx; ++i)
            for (int k = k0; k < k1; ++k)
                A3(W, k, imax - nbx + i, j) += A3(W, k, imax + 1 + nbx - i, j);
    for (int j = 1; j <= nby; ++j)
        for (int i = 1; i <= imax; ++i)
            for (int k = k0; k < k1; ++k) A3(W, k, i, j) += A3(W, k, i, 1 - j);
    for (int j = 1; j <= nby; ++j)
        for (int i = 1; i <= imax; ++i)
            for (int k = k0; k < k1; ++k)
                A3(W, k, i, jmax - nby + j) += A3(W, k, i, jmax + 1 + nby - j);
}

/* ------------------------------------------- fast filters: 1D line beta */

/* vrbeta1 / vrbeta1t (jp_pbfil.f90:856-885, 981-1009) applied to every
 * interior row (dir 0: along i, rbeta(km,hx,1,im,paspx,ssx,VALL(:,:,j))) or
 * every interior column (dir 1: along j, rbeta(km,hy,1,jm,paspy,ssy,
 * VALL(:,i,:))) of a generation array, as filtering_fast_bckg/_ens do
 * (mg_filtering.f90:825-997, 1316-1506).  Forward: gather over the line's
 * extended range, result on the interior, the line's halo zeroed.
 * Adjoint: scatter from the interior into the extended line (b = 0 first).
 * Either way the whole line, halo included, is overwritten (a = b). */
static void line_beta(const setup_t* S, int p, arr3 a, int I, int J, int hx, int hy, int dir, int adj, int k0,
                      int k1) {
    const int n = dir ? J : I, h = dir ? hy : hx, m = dir ? I : J;
    const int len = n + 2 * h;
    const int nk = k1 - k0;
    double* b = (double*)malloc(sizeof(double) * (size_t)nk * len);
    const double exx = S->exxL, s = S->ssL;
    const double x = 1.0 / exx;
    const int gxl = (int)ceil(-x + EPS), gxm = (int)floor(x - EPS);
#define LB(k, t) b[(size_t)((k) - k0) + (size_t)nk * (size_t)((t) + h - 1)]
#define LA(k, t) (*(dir ? &A3(a, k, line, t) : &A3(a, k, t, line)))
    for (int line = 1; line <= m; ++line) {
        for (size_t t = 0; t < (size_t)nk * len; ++t) b[t] = 0.0;
        for (int ix = 1; ix <= n; ++ix)
            for (int gx = gxl; gx <= gxm; ++gx) {
                int jx = ix + gx;
                double xx = gx, rr = (xx * exx) * (xx * exx);
                double frow = s * ipow(1.0 - rr, p);
                if (!adj)
                    for (int k = k0; k < k1; ++k) LB(k, ix) += frow * LA(k, jx);
                else
                    for (int k = k0; k < k1; ++k) LB(k, jx) += frow * LA(k, ix);
            }
        for (int t = 1 - h; t <= n + h; ++t)
            for (int k = k0; k < k1; ++k) LA(k, t) = LB(k, t);
    }
#undef LA
#undef LB
    free(b);
}

/* bocox / bocoy at physical edges (mg_bocos.f90:4044-4903): half-sample
 * mirror of the x halo on the interior rows only (dir 0), or of the y halo
 * on the interior columns only (dir 1); the corners are not written. */
static void fill_line(arr3 W, int imax, int jmax, int nb, int dir, int k0, int k1) {
    if (!dir) {
        for (int j = 1; j <= jmax; ++j)
            for (int i = 1; i <= nb; ++i)
                for (int k = k0; k < k1; ++k) {
                    A3(W, k, -nb + i, j) = A3(W, k, nb + 1 - i, j);
                    A3(W, k, imax + i, j) = A3(W, k, imax + 1 - i, j);
                }
    } else {
        for (int j = 1; j <= nb; ++j)
            for (int i = 1; i <= imax; ++i)
                for (int k = k0; k < k1; ++k) {
                    A3(W, k, i, jmax + j) = A3(W, k, i, jmax + 1 - j);
                    A3(W, k, i, -nb + j) = A3(W, k, i, nb + 1 - j);
                }
    }
}

/* bocoTx / bocoTy at physical edges (mg_bocos.f90:4906-5718): the transpose,
 * W(t) += W(1-t), W(M-nb+t) += W(M+nb+1-t) on the interior rows (dir 0) or
 * columns (dir 1); halo values stay in place. */
static void fold_line(arr3 W, int imax, int jmax, int nb, int dir, int k0, int k1) {
    if (!dir) {
        for (int j = 1; j <= jmax; ++j)
            for (int i = 1; i <= nb; ++i)
                for (int k = k0; k < k1; ++k) A3(W, k, i, j) += A3(W, k, 1 - i, j);
        for (int j = 1; j <= jmax; ++j)
            for (int i = 1; i <= nb; ++i)
                for (int k = k0; k < k1; ++k) A3(W, k, imax - nb + i, j) += A3(W, k, imax + nb + 1 - i, j);
    } else {
        for (int j = 1; j <= nb; ++j)
            for (int i = 1; i <= imax; ++i)
                for (int k = k0; k < k1; ++k) A3(W, k, i, j) += A3(W, k, i, 1 - j);
        for (int j = 1; j <= nb; ++j)
            for (int i = 1; i <= imax; ++i)
                for (int k = k0; k < k1; ++k) A3(W, k, i, jmax - nb + j) += A3(W, k, i, jmax + nb + 1 - j);
    }
}

/* The fast filters' horizontal adjoint for one generation
 * (mg_filtering.f90:859-906): rbetaT along x, bocoTx, rbetaT along y, bocoTy. */
static void fast_adjoint(const orc_cfg* c, const setup_t* S, arr3 U, int I, int J, int k0, int k1) {
    line_beta(S, c->p, U, I, J, c->hx, c->hy, 0, 1, k0, k1);
    fold_line(U, I, J, c->hx, 0, k0, k1);
    line_beta(S, c->p, U, I, J, c->hx, c->hy, 1, 1, k0, k1);
    fold_line(U, I, J, c->hy, 1, k0, k1);
}

/* ... and its forward (mg_filtering.f90:930-975): bocoy, rbeta along y,
 * bocox, rbeta along x. */
static void fast_forward(const orc_cfg* c, const setup_t* S, arr3 U, int I, int J, int k0, int k1) {
    fill_line(U, I, J, c->hy, 1, k0, k1);
    line_beta(S, c->p, U, I, J, c->hx, c->hy, 1, 0, k0, k1);
    fill_line(U, I, J, c->hx, 0, k0, k1);
    line_beta(S, c->p, U, I, J, c->hx, c->hy, 0, 0, k0, k1);
}

/* ------------------------------- proc 2: dibeta line filters by color */

/* vdibeta2 / vdibeta2t (jp_pbfil3.f90:1801-1837, 2345-2382) for color q on
 * a generation array, as filtering_lin2_bckg calls them
 * (mg_filtering.f90:683-822): interior points only, b = 0 first, then
 * a = b.  Forward: b(x) = fil0 a(x) + sum_t fil_t (a(x + t d) + a(x - t d)),
 * reading the filled halo; the halo of the result is zero.  Adjoint: the
 * scatter of the same weights from every interior point into the extended
 * array. */
static void dibeta_pass(const setup_t* S, int q, arr3 a, arr3 b, int I, int J, int adj, int k0, int k1) {
    a3_zero(b, k0, k1);
    const int dx = S->ddx[q], dy = S->ddy[q], h = S->dh[q];
    const double* f = S->dfil[q];
    for (int iy = 1; iy <= J; ++iy)
        for (int ix = 1; ix <= I; ++ix) {
            if (!adj) {
                double* dst = &A3(b, 0, ix, iy);
                const double* c0 = &A3(a, 0, ix, iy);
                for (int k = k0; k < k1; ++k) dst[k] = f[0] * c0[k];
                for (int t = 1; t <= h; ++t) {
                    const double* up = &A3(a, 0, ix + dx * t, iy + dy * t);
                    const double* dn = &A3(a, 0, ix - dx * t, iy - dy * t);
                    for (int k = k0; k < k1; ++k) dst[k] += f[t] * (up[k] + dn[k]);
                }
            } else {
                const double* at = &A3(a, 0, ix, iy);
                double* c0 = &A3(b, 0, ix, iy);
                for (int k = k0; k < k1; ++k) c0[k] += f[0] * at[k];
                for (int t = 1; t <= h; ++t) {
                    double* up = &A3(b, 0, ix + dx * t, iy + dy * t);
                    double* dn = &A3(b, 0, ix - dx * t, iy - dy * t);
                    for (int k = k0; k < k1; ++k) {
                        const double v = f[t] * at[k];
                        up[k] += v;
                        dn[k] += v;
                    }
                }
            }
        }
    a3_copy(a, b, k0, k1);
}

/* One generation of filtering_lin2_bckg's horizontal part: for colors 3, 2,
 * 1 the adjoint line filter and bocoT_2d; weighting; for colors 1, 2, 3
 * boco_2d and the forward line filter (mg_filtering.f90:725-797). */
static void lin2_adjoint(const orc_cfg* c, const setup_t* S, arr3 U, arr3 T, int I, int J, int k0, int k1) {
    for (int q = 2; q >= 0; --q) {
        dibeta_pass(S, q, U, T, I, J, 1, k0, k1);
        fold_h(U, I, J, c->hx, c->hy, k0, k1);
    }
}
static void lin2_forward(const orc_cfg* c, const setup_t* S, arr3 U, arr3 T, int I, int J, int k0, int k1) {
    for (int q = 0; q < 3; ++q) {
        fill_h(U, I, J, c->hx, c->hy, k0, k1);
        dibeta_pass(S, q, U, T, I, J, 0, k0, k1);
    }
}

/* ------------------------- proc 5: filtering_lin3's 3D line filters */

/* The 3D variables of a generation as filtering_lin3 holds them
 * (mg_filtering.f90:260-557): W(v, i, j, L), v < km3, with x/y halos and a
 * z halo of hz levels (stack_to_composite, mg_transfer.f90:206-234, puts
 * VALL((v-1)*lm+L, i, j) at L). */
typedef struct {
    double* d;
    int nv, I, J, lm, hx, hy, hz;
} w3_t;
static inline double* w3at(const w3_t* w, int v, int i, int j, int L) {
    const size_t ni = (size_t)w->I + 2 * w->hx, nj = (size_t)w->J + 2 * w->hy;
    return w->d + (size_t)v + (size_t)w->nv * ((size_t)(i + w->hx - 1) + ni * ((size_t)(j + w->hy - 1) +
                                                                              nj * (size_t)(L + w->hz - 1)));
}
#define W3(w, v, i, j, L) (*w3at(&(w), (v), (i), (j), (L)))

static void w3_from(w3_t w, arr3 U) {
    for (int L = 1; L <= w.lm; ++L)
        for (int j = 1 - w.hy; j <= w.J + w.hy; ++j)
            for (int i = 1 - w.hx; i <= w.I + w.hx; ++i)
                for (int v = 0; v < w.nv; ++v) W3(w, v, i, j, L) = A3(U, v * w.lm + L - 1, i, j);
}
static void w3_to(w3_t w, arr3 U) {
    for (int L = 1; L <= w.lm; ++L)
        for (int j = 1 - w.hy; j <= w.J + w.hy; ++j)
            for (int i = 1 - w.hx; i <= w.I + w.hx; ++i)
                for (int v = 0; v < w.nv; ++v) A3(U, v * w.lm + L - 1, i, j) = W3(w, v, i, j, L);
}

/* W(1-L) = W(1+L), W(lm+L) = W(lm-L), L = 1..hz, on every column */
static void w3_zmirror(w3_t w) {
    for (int L = 1; L <= w.hz; ++L)
        for (int j = 1 - w.hy; j <= w.J + w.hy; ++j)
            for (int i = 1 - w.hx; i <= w.I + w.hx; ++i)
                for (int v = 0; v < w.nv; ++v) {
                    W3(w, v, i, j, 1 - L) = W3(w, v, i, j, 1 + L);
                    W3(w, v, i, j, w.lm + L) = W3(w, v, i, j, w.lm - L);
                }
}

/* boco_3d at the physical edges, levels 1..lm: y on the interior columns
 * (north, then south), then x on every row (west, then east).  gh = 0 is
 * boco_3d_g1 (mg_bocos.f90:1425-1774), whose east edge is W(I+i) = W(I-i);
 * gh = 1 is boco_3d_gh (1777-2170): W(I+i) = W(I+1-i), and the z halo is
 * mirrored afterwards. */
static void boco3(w3_t w, int gh) {
    const int I = w.I, J = w.J;
    for (int L = 1; L <= w.lm; ++L)
        for (int j = 1; j <= w.hy; ++j)
            for (int i = 1; i <= I; ++i)
                for (int v = 0; v < w.nv; ++v) W3(w, v, i, J + j, L) = W3(w, v, i, J + 1 - j, L);
    for (int L = 1; L <= w.lm; ++L)
        for (int j = 1; j <= w.hy; ++j)
            for (int i = 1; i <= I; ++i)
                for (int v = 0; v < w.nv; ++v) W3(w, v, i, -w.hy + j, L) = W3(w, v, i, w.hy + 1 - j, L);
    for (int L = 1; L <= w.lm; ++L)
        for (int j = 1 - w.hy; j <= J + w.hy; ++j)
            for (int i = 1; i <= w.hx; ++i)
                for (int v = 0; v < w.nv; ++v) W3(w, v, -w.hx + i, j, L) = W3(w, v, w.hx + 1 - i, j, L);
    for (int L = 1; L <= w.lm; ++L)
        for (int j = 1 - w.hy; j <= J + w.hy; ++j)
            for (int i = 1; i <= w.hx; ++i)
                for (int v = 0; v < w.nv; ++v) W3(w, v, I + i, j, L) = W3(w, v, gh ? I + 1 - i : I - i, j, L);
    if (gh) w3_zmirror(w);
}

/* bocoT_3d at the physical edges: x on every row (west, then east), levels
 * 1..lm, then y on the interior columns (south, then north), then the z
 * halo folded into levels 2..hz+1 and lm-hz..lm-1 on every column.
 * gh = 0 is bocoT_3d_g1 (mg_bocos.f90:2173-2527), whose east and north
 * folds read W(I+hx-i) and W(J+hy-j): the edge column and row are added to
 * themselves and the outermost halo line is not folded.  gh = 1 is
 * bocoT_3d_gh (2530-2908) with W(I+1+hx-i) and W(J+1+hy-j). */
static void bocoT3(w3_t w, int gh) {
    const int I = w.I, J = w.J, hx = w.hx, hy = w.hy, o = gh ? 1 : 0;
    for (int L = 1; L <= w.lm; ++L)
        for (int j = 1 - hy; j <= J + hy; ++j)
            for (int i = 1; i <= hx; ++i)
                for (int v = 0; v < w.nv; ++v) W3(w, v, i, j, L) += W3(w, v, 1 - i, j, L);
    for (int L = 1; L <= w.lm; ++L)
        for (int j = 1 - hy; j <= J + hy; ++j)
            for (int i = 1; i <= hx; ++i)
                for (int v = 0; v < w.nv; ++v) W3(w, v, I - hx + i, j, L) += W3(w, v, I + o + hx - i, j, L);
    for (int L = 1; L <= w.lm; ++L)
        for (int j = 1; j <= hy; ++j)
            for (int i = 1; i <= I; ++i)
                for (int v = 0; v < w.nv; ++v) W3(w, v, i, j, L) += W3(w, v, i, 1 - j, L);
    for (int L = 1; L <= w.lm; ++L)
        for (int j = 1; j <= hy; ++j)
            for (int i = 1; i <= I; ++i)
                for (int v = 0; v < w.nv; ++v) W3(w, v, i, J - hy + j, L) += W3(w, v, i, J + o + hy - j, L);
    for (int L = 1; L <= w.hz; ++L) {
        for (int j = 1 - hy; j <= J + hy; ++j)
            for (int i = 1 - hx; i <= I + hx; ++i)
                for (int v = 0; v < w.nv; ++v) W3(w, v, i, j, 1 + L) += W3(w, v, i, j, 1 - L);
        for (int j = 1 - hy; j <= J + hy; ++j)
            for (int i = 1 - hx; i <= I + hx; ++i)
                for (int v = 0; v < w.nv; ++v) W3(w, v, i, j, w.lm - L) += W3(w, v, i, j, w.lm + L);
    }
}

/* vdibetax3 / vdibetax3t (jp_pbfil3.f90:1928-1977, 2475-2525) for color col
 * on the interior: b = 0 (z halo included), then a = b.  Where the point's
 * hexad has no line of this color, forward copies and adjoint adds the
 * value.  (The per-point slot counter of the reference is the same at
 * every point here: the aspect is uniform.) */
static void dib3(const setup_t* S, w3_t w, w3_t b, int col, int adj) {
    const size_t n = (size_t)w.nv * (w.I + 2 * w.hx) * (w.J + 2 * w.hy) * (w.lm + 2 * w.hz);
    memset(b.d, 0, sizeof(double) * n);
    const int q = S->hslot[col];
    for (int L = 1; L <= w.lm; ++L)
        for (int j = 1; j <= w.J; ++j)
            for (int i = 1; i <= w.I; ++i)
                for (int v = 0; v < w.nv; ++v) {
                    if (q < 0) {
                        W3(b, v, i, j, L) += W3(w, v, i, j, L);
                        continue;
                    }
                    const int dx = S->hgen[q][0], dy = S->hgen[q][1], dz = S->hgen[q][2];
                    const double* f = S->hfil[q];
                    if (!adj) {
                        double acc = f[0] * W3(w, v, i, j, L);
                        for (int t = 1; t <= S->hh[q]; ++t)
                            acc += f[t] * (W3(w, v, i + t * dx, j + t * dy, L + t * dz) +
                                           W3(w, v, i - t * dx, j - t * dy, L - t * dz));
                        W3(b, v, i, j, L) = acc;
                    } else {
                        const double at = W3(w, v, i, j, L);
                        W3(b, v, i, j, L) += f[0] * at;
                        for (int t = 1; t <= S->hh[q]; ++t) {
                            W3(b, v, i + t * dx, j + t * dy, L + t * dz) += f[t] * at;
                            W3(b, v, i - t * dx, j - t * dy, L - t * dz) += f[t] * at;
                        }
                    }
                }
    memcpy(w.d, b.d, sizeof(double) * n);
}

/* One generation of filtering_lin3 (mg_filtering.f90:285-535): the 2D
 * variables through proc 2's line filters; the 3D variables, adjoint side:
 * for colors 7..1 the z mirror, dibetat and bocoT_3d; weighting; forward
 * side: the z mirror once, then for colors 1..7 boco_3d and dibeta.
 * Generation 1 uses the _g1 halo routines, coarser ones the _gh ones. */
static void weight_gen(const orc_cfg* c, arr3 V, int I, int J, double a, double b, int k0, int k1);
static void lin3_generation(const orc_cfg* c, const setup_t* S, arr3 U, arr3 T, int I, int J, double a, double b,
                            int gh) {
    const int n3 = c->nzcol * c->lm;
    const size_t n = (size_t)(c->nzcol > 0 ? c->nzcol : 1) * (I + 2 * c->hx) * (J + 2 * c->hy) * (c->lm + 2 * c->hz);
    w3_t w = {(double*)calloc(n, sizeof(double)), c->nzcol, I, J, c->lm, c->hx, c->hy, c->hz};
    w3_t t = w;
    t.d = (double*)calloc(n, sizeof(double));
    if (c->nk > n3) lin2_adjoint(c, S, U, T, I, J, n3, c->nk);
    if (n3 > 0) {
        w3_from(w, U);
        for (int col = 7; col >= 1; --col) {
            w3_zmirror(w);
            dib3(S, w, t, col, 1);
            bocoT3(w, gh);
        }
        w3_to(w, U);
    }
    weight_gen(c, U, I, J, a, b, 0, c->nk);
    if (c->nk > n3) lin2_forward(c, S, U, T, I, J, n3, c->nk);
    if (n3 > 0) {
        w3_from(w, U);
        w3_zmirror(w);
        for (int col = 1; col <= 7; ++col) {
            boco3(w, gh);
            dib3(S, w, t, col, 0);
        }
        w3_to(w, U);
    }
    free(w.d);
    free(t.d);
}

/* ----------------------------------------------- filtering_rad3: 3D ball */

/* sup_vrbeta3 / sup_vrbeta3T (mg_filtering.f90:1923-2039) on the 3D
 * variables of a generation array, column by column (levels k = v*lm+L-1):
 * copy the column with its x/y halo, whole-sample mirror in L over hz
 * levels, vrbeta3 (gather, jp_pbfil.f90:930-977) or vrbeta3t (scatter from
 * the interior into the extended box, jp_pbfil.f90:1053-1100, then the L
 * fold), and copy back the INTERIOR only: the x/y halo of U keeps what it
 * held (the scatter's x/y-halo part is dropped). */
static void ball3(const orc_cfg* c, const setup_t* S, arr3 U, int I, int J, int adj) {
    const int lm = c->lm, hz = c->hz, hx = c->hx, hy = c->hy, p = c->p;
    const size_t ni = (size_t)I + 2 * hx, nj = (size_t)J + 2 * hy, nz = (size_t)lm + 2 * hz;
    double* W = (double*)malloc(sizeof(double) * ni * nj * nz);
    double* B = (double*)malloc(sizeof(double) * ni * nj * nz);
#define BX(a, i, j, L) a[((size_t)((L) + hz - 1) * nj + (size_t)((j) + hy - 1)) * ni + (size_t)((i) + hx - 1)]
    const double e = S->e3, s = S->ss3;
    const double z0 = 1.0 / e;
    const int gzl = (int)ceil(-z0 + EPS), gzm = (int)floor(z0 - EPS);
    for (int v = 0; v < c->nzcol; ++v) {
        for (int L = 1; L <= lm; ++L)
            for (int j = 1 - hy; j <= J + hy; ++j)
                for (int i = 1 - hx; i <= I + hx; ++i) BX(W, i, j, L) = A3(U, v * lm + L - 1, i, j);
        for (int L = 1; L <= hz; ++L)
            for (int j = 1 - hy; j <= J + hy; ++j)
                for (int i = 1 - hx; i <= I + hx; ++i) {
                    BX(W, i, j, 1 - L) = BX(W, i, j, 1 + L);
                    BX(W, i, j, lm + L) = BX(W, i, j, lm - L);
                }
        for (size_t t = 0; t < ni * nj * nz; ++t) B[t] = 0.0;
        for (int iz = 1; iz <= lm; ++iz)
            for (int iy = 1; iy <= J; ++iy)
                for (int ix = 1; ix <= I; ++ix) {
                    const double ta = BX(W, ix, iy, iz);
                    double tb = 0.0;
                    for (int gz = gzl; gz <= gzm; ++gz) {
                        const double zz = gz, rry = (zz * e) * (zz * e), y = sqrt(1.0 - rry);
                        const int gyl = (int)ceil((0.0 - y) / e + EPS), gym = (int)floor((0.0 + y) / e - EPS);
                        for (int gy = gyl; gy <= gym; ++gy) {
                            const double yy = gy, rrx = rry + (yy * e - 0.0) * (yy * e - 0.0), x = sqrt(1.0 - rrx);
                            const int gxl = (int)ceil((0.0 - x) / e + EPS), gxm = (int)floor((0.0 + x) / e - EPS);
                            for (int gx = gxl; gx <= gxm; ++gx) {
                                const double xx = gx, rr = rrx + (xx * e - 0.0) * (xx * e - 0.0);
                                const double frow = s * ipow(1.0 - rr, p);
                                if (adj) BX(B, ix + gx, iy + gy, iz + gz) += frow * ta;
                                else tb += frow * BX(W, ix + gx, iy + gy, iz + gz);
                            }
                        }
                    }
                    if (!adj) BX(B, ix, iy, iz) = tb;
                }
        if (adj)
            for (int L = 1; L <= hz; ++L)
                for (int j = 1 - hy; j <= J + hy; ++j)
                    for (int i = 1 - hx; i <= I + hx; ++i) {
                        BX(B, i, j, 1 + L) += BX(B, i, j, 1 - L);
                        BX(B, i, j, lm - L) += BX(B, i, j, lm + L);
                    }
        for (int L = 1; L <= lm; ++L)
            for (int j = 1; j <= J; ++j)
                for (int i = 1; i <= I; ++i) A3(U, v * lm + L - 1, i, j) = BX(B, i, j, L);
    }
#undef BX
    free(W);
    free(B);
}

static void weight_gen(const orc_cfg* c, arr3 V, int I, int J, double a, double b, int k0, int k1);

/* One generation of filtering_rad3 (mg_filtering.f90:123-257): the 2D
 * variables through vrbeta2t / vrbeta2, the 3D variables through the ball,
 * bocoT_2d / weighting / boco_2d over all levels in between. */
static void rad3_generation(const orc_cfg* c, const setup_t* S, arr3 U, arr3 tmp, int I, int J, double a, double b,
                            double* tb) {
    const int n3 = c->nzcol * c->lm, nk = c->nk;
    if (n3 < nk) vrbeta2t(S, c->p, U, tmp, 1, I, 1, J, n3, nk);
    if (n3 > 0) ball3(c, S, U, I, J, 1);
    fold_h(U, I, J, c->hx, c->hy, 0, nk);
    weight_gen(c, U, I, J, a, b, 0, nk);
    fill_h(U, I, J, c->hx, c->hy, 0, nk);
    if (n3 < nk) vrbeta2(S, c->p, U, tmp, 1, I, 1, J, n3, nk, tb);
    if (n3 > 0) ball3(c, S, U, I, J, 0);
}

/* ------------------------------------------------ restriction/prolongation */

/* def_offset_coef (mg_interpolate.f90:61-86) */
static const double PC[4] = {-9.0 / 128.0, 111.0 / 128.0, 29.0 / 128.0, -3.0 / 128.0};
static const double QC[4] = {-3.0 / 128.0, 29.0 / 128.0, 111.0 / 128.0, -9.0 / 128.0};
static const double AC[3] = {5.0 / 32.0, 30.0 / 32.0, -3.0 / 32.0};
static const double BC[3] = {-3.0 / 32.0, 30.0 / 32.0, 5.0 / 32.0};

/* adjoint (mg_generations.f90:1117-1187): P^T as a separable scatter from
 * F(1:im,1:jm) into W(-1:imL+2,-1:jmL+2); aux is (nk, 1:im, -1:jmL+2). */
static void adjoint4(arr3 F, arr3 W, arr3 aux, int im, int jm, int k0, int k1) {
    int imL = im / 2, jmL = jm / 2;
    a3_zero(aux, k0, k1);
    if (!ROWPAR) {
        for (int j = jm; j >= 2; j -= 2) {
            int jL = j / 2;
            for (int i = im; i >= 1; --i)
                for (int k = k0; k < k1; ++k) {
                    double f = A3(F, k, i, j);
                    A3(aux, k, i, jL + 2) += PC[3] * f;
                    A3(aux, k, i, jL + 1) += PC[2] * f;
                    A3(aux, k, i, jL) += PC[1] * f;
                    A3(aux, k, i, jL - 1) += PC[0] * f;
                }
        }
        for (int j = jm - 1; j >= 1; j -= 2) {
            int jL = j / 2;
            for (int i = im; i >= 1; --i)
                for (int k = k0; k < k1; ++k) {
                    double f = A3(F, k, i, j);
                    A3(aux, k, i, jL + 2) += QC[3] * f;
                    A3(aux, k, i, jL + 1) += QC[2] * f;
                    A3(aux, k, i, jL) += QC[1] * f;
                    A3(aux, k, i, jL - 1) += QC[0] * f;
                }
        }
    } else {
        /* target-row form of the two loops above: row r of aux takes the
         * even fine rows j = 2jL, jL = r+1 .. r-2 (decreasing, as j
         * decreases above), with weight PC[r-jL+1], then the odd rows
         * j = 2jL+1 in the same order with QC[r-jL+1] */
        ROW_FOR
        for (int r = -1; r <= jmL + 2; ++r) {
            for (int jL = r + 1; jL >= r - 2; --jL) {
                if (jL < 1 || jL > jmL) continue;
                const double c = PC[r - jL + 1];
                for (int i = im; i >= 1; --i)
                    for (int k = k0; k < k1; ++k) A3(aux, k, i, r) += c * A3(F, k, i, 2 * jL);
            }
            for (int jL = r + 1; jL >= r - 2; --jL) {
                if (jL < 0 || jL > jmL - 1) continue;
                const double c = QC[r - jL + 1];
                for (int i = im; i >= 1; --i)
                    for (int k = k0; k < k1; ++k) A3(aux, k, i, r) += c * A3(F, k, i, 2 * jL + 1);
            }
        }
    }
    a3_zero(W, k0, k1);
    ROW_FOR
    for (int jL = jmL + 2; jL >= -1; --jL) {
        for (int i = im - 1; i >= 1; i -= 2) {
            int iL = i / 2;
            for (int k = k0; k < k1; ++k) {
                double w = A3(aux, k, i, jL);
                A3(W, k, iL + 2, jL) += QC[3] * w;
                A3(W, k, iL + 1, jL) += QC[2] * w;
                A3(W, k, iL, jL) += QC[1] * w;
                A3(W, k, iL - 1, jL) += QC[0] * w;
            }
        }
        for (int i = im; i >= 2; i -= 2) {
            int iL = i / 2;
            for (int k = k0; k < k1; ++k) {
                double w = A3(aux, k, i, jL);
                A3(W, k, iL + 2, jL) += PC[3] * w;
                A3(W, k, iL + 1, jL) += PC[2] * w;
                A3(W, k, iL, jL) += PC[1] * w;
                A3(W, k, iL - 1, jL) += PC[0] * w;
            }
        }
    }
}

/* direct1 (mg_generations.f90:1190-1250): P as a separable gather from
 * W(-1:imL+2,-1:jmL+2) to F(1:im,1:jm); aux is (nk, 1:im, -1:jmL+2). */
static void direct4(arr3 W, arr3 F, arr3 aux, int im, int jm, int k0, int k1) {
    int jmL = jm / 2;
    ROW_FOR
    for (int jL = -1; jL <= jmL + 2; ++jL) {
        for (int i = 1; i <= im - 1; i += 2) {
            int iL = i / 2;
            for (int k = k0; k < k1; ++k)
                A3(aux, k, i, jL) = QC[0] * A3(W, k, iL - 1, jL) + QC[1] * A3(W, k, iL, jL) +
                                    QC[2] * A3(W, k, iL + 1, jL) + QC[3] * A3(W, k, iL + 2, jL);
        }
        for (int i = 2; i <= im; i += 2) {
            int iL = i / 2;
            for (int k = k0; k < k1; ++k)
                A3(aux, k, i, jL) = PC[0] * A3(W, k, iL - 1, jL) + PC[1] * A3(W, k, iL, jL) +
                                    PC[2] * A3(W, k, iL + 1, jL) + PC[3] * A3(W, k, iL + 2, jL);
        }
    }
    ROW_FOR
    for (int j = 1; j <= jm - 1; j += 2) {
        int jL = j / 2;
        for (int i = 1; i <= im; ++i)
            for (int k = k0; k < k1; ++k)
                A3(F, k, i, j) = QC[0] * A3(aux, k, i, jL - 1) + QC[1] * A3(aux, k, i, jL) +
                                 QC[2] * A3(aux, k, i, jL + 1) + QC[3] * A3(aux, k, i, jL + 2);
    }
    ROW_FOR
    for (int j = 2; j <= jm; j += 2) {
        int jL = j / 2;
        for (int i = 1; i <= im; ++i)
            for (int k = k0; k < k1; ++k)
                A3(F, k, i, j) = PC[0] * A3(aux, k, i, jL - 1) + PC[1] * A3(aux, k, i, jL) +
                                 PC[2] * A3(aux, k, i, jL + 1) + PC[3] * A3(aux, k, i, jL + 2);
    }
}

/* adjoint2 (mg_generations.f90:1253-1316): quadratic P^T into
 * W(0:imL+1,0:jmL+1); aux is (nk, 1:im, 0:jmL+1). */
static void adjoint3(arr3 F, arr3 W, arr3 aux, int im, int jm, int k0, int k1) {
    int jmL = jm / 2;
    a3_zero(aux, k0, k1);
    for (int j = jm; j >= 2; j -= 2) {
        int jL = j / 2;
        for (int i = im; i >= 1; --i)
            for (int k = k0; k < k1; ++k) {
                double f = A3(F, k, i, j);
                A3(aux, k, i, jL + 1) += BC[2] * f;
                A3(aux, k, i, jL) += BC[1] * f;
                A3(aux, k, i, jL - 1) += BC[0] * f;
            }
    }
    for (int j = jm - 1; j >= 1; j -= 2) {
        int jL = (j + 1) / 2;
        for (int i = im; i >= 1; --i)
            for (int k = k0; k < k1; ++k) {
                double f = A3(F, k, i, j);
                A3(aux, k, i, jL + 1) += AC[2] * f;
                A3(aux, k, i, jL) += AC[1] * f;
                A3(aux, k, i, jL - 1) += AC[0] * f;
            }
    }
    a3_zero(W, k0, k1);
    for (int jL = jmL + 1; jL >= 0; --jL) {
        for (int i = im - 1; i >= 1; i -= 2) {
            int iL = (i + 1) / 2;
            for (int k = k0; k < k1; ++k) {
                double w = A3(aux, k, i, jL);
                A3(W, k, iL + 1, jL) += AC[2] * w;
                A3(W, k, iL, jL) += AC[1] * w;
                A3(W, k, iL - 1, jL) += AC[0] * w;
            }
        }
        for (int i = im; i >= 2; i -= 2) {
            int iL = i / 2;
            for (int k = k0; k < k1; ++k) {
                double w = A3(aux, k, i, jL);
                A3(W, k, iL + 1, jL) += BC[2] * w;
                A3(W, k, iL, jL) += BC[1] * w;
                A3(W, k, iL - 1, jL) += BC[0] * w;
            }
        }
    }
}

/* direct2 (mg_generations.f90:1319-1374): quadratic P. */
static void direct3(arr3 W, arr3 F, arr3 aux, int im, int jm, int k0, int k1) {
    int jmL = jm / 2;
    for (int jL = 0; jL <= jmL + 1; ++jL) {
        for (int i = 1; i <= im - 1; i += 2) {
            int iL = (i + 1) / 2;
            for (int k = k0; k < k1; ++k)
                A3(aux, k, i, jL) = AC[0] * A3(W, k, iL - 1, jL) + AC[1] * A3(W, k, iL, jL) +
                                    AC[2] * A3(W, k, iL + 1, jL);
        }
        for (int i = 2; i <= im; i += 2) {
            int iL = i / 2;
            for (int k = k0; k < k1; ++k)
                A3(aux, k, i, jL) = BC[0] * A3(W, k, iL - 1, jL) + BC[1] * A3(W, k, iL, jL) +
                                    BC[2] * A3(W, k, iL + 1, jL);
        }
    }
    for (int j = 1; j <= jm - 1; j += 2) {
        int jL = (j + 1) / 2;
        for (int i = 1; i <= im; ++i)
            for (int k = k0; k < k1; ++k)
                A3(F, k, i, j) = AC[0] * A3(aux, k, i, jL - 1) + AC[1] * A3(aux, k, i, jL) +
                                 AC[2] * A3(aux, k, i, jL + 1);
    }
    for (int j = 2; j <= jm; j += 2) {
        int jL = j / 2;
        for (int i = 1; i <= im; ++i)
            for (int k = k0; k < k1; ++k)
                A3(F, k, i, j) = BC[0] * A3(aux, k, i, jL - 1) + BC[1] * A3(aux, k, i, jL) +
                                 BC[2] * A3(aux, k, i, jL + 1);
    }
}

/* ------------------------------------------------------------- vertical */

/* sup_vrbeta1_bck / sup_vrbeta1_ens (mg_filtering.f90:2154-2202, 2042-2091)
 * with vrbeta1 (jp_pbfil.f90:856-885): per (i,j), gather nz columns of lm
 * levels at offsets (k-1)*lm, whole-sample mirror by hz, filter, write back.
 * adj != 0 gives sup_vrbeta1T_* (mg_filtering.f90:2205-2262, 2094-2151) with
 * vrbeta1t (jp_pbfil.f90:981-1009) and the edge fold. */
static void vfilter(const orc_cfg* c, const setup_t* S, arr3 V, int adj) {
    const int lm = c->lm, hz = c->hz, nz = c->nzcol, p = c->p;
    const int ext = lm + 2 * hz;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(c->nthreads > 0 ? c->nthreads : omp_get_max_threads())
#endif
    for (int j = 1; j <= c->J; ++j) {
        double* W = (double*)malloc(sizeof(double) * (size_t)nz * ext);
        double* B = (double*)malloc(sizeof(double) * (size_t)nz * ext);
#define WZ(arr, k, L) arr[(size_t)(k) + (size_t)nz * (size_t)((L) + hz - 1)]
        for (int i = 1; i <= c->I; ++i) {
            for (int k = 0; k < nz; ++k)
                for (int L = 1; L <= lm; ++L) WZ(W, k, L) = A3(V, k * lm + L - 1, i, j);
            for (int L = 1; L <= hz; ++L)
                for (int k = 0; k < nz; ++k) {
                    WZ(W, k, 1 - L) = WZ(W, k, 1 + L);
                    WZ(W, k, lm + L) = WZ(W, k, lm - L);
                }
            for (size_t t = 0; t < (size_t)nz * ext; ++t) B[t] = 0.0;
            double exx = S->exx1, s = S->ss1;
            double x = 1.0 / exx;
            int gxl = (int)ceil(-x + EPS), gxm = (int)floor(x - EPS);
            if (!adj) {
                for (int ix = 1; ix <= lm; ++ix) {
                    for (int gx = gxl; gx <= gxm; ++gx) {
                        int jx = ix + gx;
                        double xx = gx, rr = (xx * exx) * (xx * exx);
                        double frow = s * ipow(1.0 - rr, p);
                        for (int k = 0; k < nz; ++k) WZ(B, k, ix) += frow * WZ(W, k, jx);
                    }
                }
            } else {
                for (int ix = 1; ix <= lm; ++ix) {
                    for (int gx = gxl; gx <= gxm; ++gx) {
                        int jx = ix + gx;
                        double xx = gx, rr = (xx * exx) * (xx * exx);
                        double frow = s * ipow(1.0 - rr, p);
                        for (int k = 0; k < nz; ++k) WZ(B, k, jx) += frow * WZ(W, k, ix);
                    }
                }
                for (int L = 1; L <= hz; ++L)
                    for (int k = 0; k < nz; ++k) {
                        WZ(B, k, 1 + L) += WZ(B, k, 1 - L);
                        WZ(B, k, lm - L) += WZ(B, k, lm + L);
                    }
            }
            for (int k = 0; k < nz; ++k)
                for (int L = 1; L <= lm; ++L) A3(V, k * lm + L - 1, i, j) = WZ(B, k, L);
        }
#undef WZ
        free(W);
        free(B);
    }
}

/* ------------------------------------------------------------- pipeline */

typedef struct {
    int I, J;
    arr3 H;     /* (nk, 1-hx:I+hx, 1-hy:J+hy) */
    arr3 tmp;   /* same shape, scratch for filters */
    arr3 INT;   /* coarse transfer (nk, -1:I/2+2, -1:J/2+2) */
    arr3 aux;   /* (nk, 1:I, -1:J/2+2) */
} gen_t;

static int check_cfg(const orc_cfg* c) {
    if (!c || c->I <= 0 || c->J <= 0 || c->nk <= 0 || c->gm < 1 || c->gm > ORC_MAX_GEN) return ORC_ERR_ARG;
    if (c->hx < 0 || c->hy < 0 || c->hz < 0 || c->p < 0) return ORC_ERR_ARG;
    if (c->proc != 1 && c->proc != 6 && c->proc != 3 && c->proc != 8 && c->proc != 4 && c->proc != 2 &&
        c->proc != 7 && c->proc != 5)
        return ORC_ERR_ARG;
    if (c->proc == 5) {
        if (c->nzcol < 0 || c->lm < 1 || (size_t)c->nzcol * c->lm > (size_t)c->nk) return ORC_ERR_ARG;
        if (c->nzcol > 0 && c->hz >= c->lm) return ORC_ERR_ARG;
        if (!(c->ampl03 > 0.0)) return ORC_ERR_ARG;
    }
    if (c->proc == 4) {
        if (c->nzcol < 0 || c->lm < 1 || (size_t)c->nzcol * c->lm > (size_t)c->nk) return ORC_ERR_ARG;
        if (c->nzcol > 0 && c->hz >= c->lm) return ORC_ERR_ARG;
        if (!(c->ampl03 > 0.0)) return ORC_ERR_ARG;
    }
    int d = 1 << (c->gm - 1);
    if (c->I % d || c->J % d) return ORC_ERR_DIV;
    if (c->gm > 1 && (c->I / d < 2 || c->J / d < 2)) return ORC_ERR_DIV;
    if (c->hx > c->I / d || c->hy > c->J / d) return ORC_ERR_DIV;
    if (c->l_vertical_filter) {
        if (c->lm < 1 || c->nzcol < 0 || (size_t)c->nzcol * c->lm > (size_t)c->nk) return ORC_ERR_ARG;
        if (c->nzcol > 0 && c->hz >= c->lm) return ORC_ERR_ARG;
    }
    return ORC_OK;
}

static void gens_alloc(const orc_cfg* c, gen_t* G) {
    for (int g = 0; g < c->gm; ++g) {
        int I = c->I >> g, J = c->J >> g;
        G[g].I = I; G[g].J = J;
        G[g].H = g ? a3_alloc(c->nk, 1 - c->hx, I + c->hx, 1 - c->hy, J + c->hy) : (arr3){0};
        G[g].tmp = a3_alloc(c->nk, 1 - c->hx, I + c->hx, 1 - c->hy, J + c->hy);
        G[g].INT = a3_alloc(c->nk, -1, I / 2 + 2, -1, J / 2 + 2);
        G[g].aux = a3_alloc(c->nk, 1, I, -1, J / 2 + 2);
    }
}
static void gens_free(const orc_cfg* c, gen_t* G) {
    for (int g = 0; g < c->gm; ++g) {
        if (g) a3_free(&G[g].H);
        a3_free(&G[g].tmp); a3_free(&G[g].INT); a3_free(&G[g].aux);
    }
}

/* Restriction g -> g+1 (upsending, mg_generations.f90:158-207 and 382-432;
 * lquart: upsending2*, 270-319, 497-547): adjoint + fold with halo 2 (1),
 * then the coarse interior becomes generation g+1 (upsend_all). */
static void restrict_gen(const orc_cfg* c, arr3 fine, gen_t* Gf, arr3 coarse, int k0, int k1) {
    int I = Gf->I, J = Gf->J, IL = I / 2, JL = J / 2;
    if (!c->lquart) {
        adjoint4(fine, Gf->INT, Gf->aux, I, J, k0, k1);
        fold_h(Gf->INT, IL, JL, 2, 2, k0, k1);
        ROW_FOR
        for (int j = 1; j <= JL; ++j)
            for (int i = 1; i <= IL; ++i)
                for (int k = k0; k < k1; ++k) A3(coarse, k, i, j) = A3(Gf->INT, k, i, j);
    } else {
        arr3 W = Gf->INT; /* view (0:IL+1, 0:JL+1) inside the (-1:IL+2) buffer */
        W.ilo = 0; W.ihi = IL + 1; W.jlo = 0; W.jhi = JL + 1;
        arr3 aux = Gf->aux; aux.jlo = 0; aux.jhi = JL + 1;
        adjoint3(fine, W, aux, I, J, k0, k1);
        fold_h(W, IL, JL, 1, 1, k0, k1);
        for (int j = 1; j <= JL; ++j)
            for (int i = 1; i <= IL; ++i)
                for (int k = k0; k < k1; ++k) A3(coarse, k, i, j) = A3(W, k, i, j);
    }
}

/* Prolongation and add g+1 -> g (downsending, mg_generations.f90:210-267,
 * 435-494; lquart: downsending2*): coarse interior copied into the transfer
 * array, halo 2 (1) filled, direct1 (direct2), result added to fine. */
static void prolong_add(const orc_cfg* c, arr3 coarse, gen_t* Gf, arr3 fine, int k0, int k1) {
    int I = Gf->I, J = Gf->J, IL = I / 2, JL = J / 2;
    arr3 W = Gf->INT, aux = Gf->aux;
    int nb = 2;
    if (c->lquart) { W.ilo = 0; W.ihi = IL + 1; W.jlo = 0; W.jhi = JL + 1; aux.jlo = 0; aux.jhi = JL + 1; nb = 1; }
    ROW_FOR
    for (int j = 1; j <= JL; ++j)
        for (int i = 1; i <= IL; ++i)
            for (int k = k0; k < k1; ++k) A3(W, k, i, j) = A3(coarse, k, i, j);
    fill_h(W, IL, JL, nb, nb, k0, k1);
    /* H_PROX / V_PROX live in tmp's interior */
    arr3 F = Gf->tmp;
    arr3 Fi = F; /* interior-only view for direct: reuse the full array */
    if (!c->lquart) direct4(W, Fi, aux, I, J, k0, k1);
    else direct3(W, Fi, aux, I, J, k0, k1);
    ROW_FOR
    for (int j = 1; j <= J; ++j)
        for (int i = 1; i <= I; ++i)
            for (int k = k0; k < k1; ++k) A3(fine, k, i, j) += A3(F, k, i, j);
}

/* weighting / weighting_helm / weighting_ens (mg_generations.f90:901-1052). */
static void weight_gen(const orc_cfg* c, arr3 V, int I, int J, double a, double b, int k0, int k1) {
    if (!c->lhelm || b == 0.0) {
        if (c->lhelm) {
            /* a*V - 0*(Laplacian): the Laplacian reads halo cells left by the
             * fold; they are finite, so the product is exactly zero. */
        }
        ROW_FOR
        for (int j = 1; j <= J; ++j)
            for (int i = 1; i <= I; ++i)
                for (int k = k0; k < k1; ++k) A3(V, k, i, j) *= a;
        return;
    }
    /* b != 0 is an extension (the reference fixes b = 0); the reference
     * would read stale fold halos, so fill a 1-wide mirror halo first. */
    fill_h(V, I, J, 1, 1, k0, k1);
    size_t n = (size_t)(k1 - k0) * I * J;
    double* out = (double*)malloc(sizeof(double) * (n ? n : 1));
    size_t t = 0;
    for (int j = 1; j <= J; ++j)
        for (int i = 1; i <= I; ++i)
            for (int k = k0; k < k1; ++k) {
                double v = A3(V, k, i, j);
                double lap = A3(V, k, i + 1, j) - 2 * v + A3(V, k, i - 1, j) + A3(V, k, i, j + 1) -
                             2 * v + A3(V, k, i, j - 1);
                out[t++] = a * v - b * lap;
            }
    t = 0;
    for (int j = 1; j <= J; ++j)
        for (int i = 1; i <= I; ++i)
            for (int k = k0; k < k1; ++k) A3(V, k, i, j) = out[t++];
    free(out);
}

static void horizontal_pipeline(const orc_cfg* c, const setup_t* S, arr3 V, gen_t* G, int k0, int k1) {
    const int gm = c->gm, hx = c->hx, hy = c->hy;
    const int filt1 = (c->proc == 1) || (c->proc == 2) || (c->proc == 3) || (c->proc == 4) || (c->proc == 5) ||
                      c->l_filt_g1;
    const int fast = c->proc == 3 || c->proc == 8;
    double* tb = (double*)malloc(sizeof(double) * (size_t)c->nk);
    /* up: V -> H_2 -> ... -> H_gm */
    for (int g = 0; g + 1 < gm; ++g) {
        arr3 fine = g ? G[g].H : V;
        restrict_gen(c, fine, &G[g], G[g + 1].H, k0, k1);
    }
    /* adjoint filter on all generations, fold, weight, fill, filter */
    for (int g = 0; g < gm; ++g) {
        arr3 U = g ? G[g].H : V;
        int I = G[g].I, J = G[g].J;
        if (g == 0 && !filt1) continue;
        if (c->proc == 4) {  /* whole columns: the caller runs one k-range */
            rad3_generation(c, S, U, G[g].tmp, I, J, c->a[g], c->b[g], tb);
            continue;
        }
        if (c->proc == 5) {  /* whole columns too */
            lin3_generation(c, S, U, G[g].tmp, I, J, c->a[g], c->b[g], g > 0);
            continue;
        }
        if (fast) {
            fast_adjoint(c, S, U, I, J, k0, k1);
            weight_gen(c, U, I, J, c->a[g], c->b[g], k0, k1);
            fast_forward(c, S, U, I, J, k0, k1);
            continue;
        }
        if (c->proc == 2 || c->proc == 7) {
            lin2_adjoint(c, S, U, G[g].tmp, I, J, k0, k1);
            weight_gen(c, U, I, J, c->a[g], c->b[g], k0, k1);
            lin2_forward(c, S, U, G[g].tmp, I, J, k0, k1);
            continue;
        }
        if (c->a[g] == 0.0 && c->b[g] == 0.0) {
            /* a zero-weighted generation filters to exact zeros (the weight
             * zeroes the interior, fill_h then every halo cell, and vrbeta2
             * of zeros is zero): skip its filters */
            a3_zero(U, k0, k1);
            continue;
        }
        vrbeta2t(S, c->p, U, G[g].tmp, 1, I, 1, J, k0, k1);
        fold_h(U, I, J, hx, hy, k0, k1);
        weight_gen(c, U, I, J, c->a[g], c->b[g], k0, k1);
        fill_h(U, I, J, hx, hy, k0, k1);
        vrbeta2(S, c->p, U, G[g].tmp, 1, I, 1, J, k0, k1, tb);
    }
    /* down: H_gm -> ... -> H_2 -> V */
    for (int g = gm - 1; g >= 1; --g) {
        arr3 fine = (g - 1) ? G[g - 1].H : V;
        prolong_add(c, G[g].H, &G[g - 1], fine, k0, k1);
    }
    free(tb);
}

int orc_filtering_procedure(const orc_cfg* c, double* Vd) {
    int rc = check_cfg(c);
    if (rc) return rc;
    set_threads(c->nthreads);
    setup_t S;
    rc = setup(c, &S);
    if (rc) return rc;
    arr3 V = {Vd, c->nk, 1 - c->hx, c->I + c->hx, 1 - c->hy, c->J + c->hy};
    /* rad3 and lin3 have no separate z filter */
    const int zfilt = c->proc != 4 && c->proc != 5 && c->l_vertical_filter && c->nzcol > 0;
    if (zfilt) vfilter(c, &S, V, 1);
    gen_t G[ORC_MAX_GEN];
    memset(G, 0, sizeof(G));
    gens_alloc(c, G);
    int nth = 1;
#ifdef _OPENMP
    nth = g_threads;
    if (nth > c->nk) nth = c->nk;
    if (c->proc == 4 || c->proc == 5) nth = 1;
    if ((c->proc == 1 || c->proc == 6) && c->nk < 16 * g_threads && g_threads > 1) {
        /* few levels per thread: the radial pipeline over all levels, its
         * loops split by rows (ROWPAR) instead of the levels by thread */
        horizontal_pipeline(c, &S, V, G, 0, c->nk);
    } else {
#pragma omp parallel num_threads(nth)
        {
            int t = omp_get_thread_num(), nt = omp_get_num_threads();
            int k0 = (int)((long long)c->nk * t / nt), k1 = (int)((long long)c->nk * (t + 1) / nt);
            if (k1 > k0) horizontal_pipeline(c, &S, V, G, k0, k1);
        }
    }
#else
    (void)nth;
    horizontal_pipeline(c, &S, V, G, 0, c->nk);
#endif
    gens_free(c, G);
    /* filtering_lin2_ens (proc 7) ends with the ADJOINT vertical filter
     * (sup_vrbeta1T_ens, mg_filtering.f90:1304), as the reference does */
    if (zfilt) vfilter(c, &S, V, c->proc == 7);
    return ORC_OK;
}

static double* to_halo(const orc_cfg* c, const double* x) {
    size_t ni = (size_t)c->I + 2 * c->hx, nj = (size_t)c->J + 2 * c->hy;
    double* V = (double*)calloc((size_t)c->nk * ni * nj, sizeof(double));
    if (!V) return NULL;
    arr3 a = {V, c->nk, 1 - c->hx, c->I + c->hx, 1 - c->hy, c->J + c->hy};
    ROW_FOR
    for (int j = 1; j <= c->J; ++j)
        for (int i = 1; i <= c->I; ++i)
            memcpy(&A3(a, 0, i, j), x + (size_t)c->nk * ((size_t)(i - 1) + (size_t)c->I * (j - 1)),
                   sizeof(double) * c->nk);
    return V;
}
static void from_halo(const orc_cfg* c, const double* V, double* y) {
    arr3 a = {(double*)V, c->nk, 1 - c->hx, c->I + c->hx, 1 - c->hy, c->J + c->hy};
    ROW_FOR
    for (int j = 1; j <= c->J; ++j)
        for (int i = 1; i <= c->I; ++i)
            memcpy(y + (size_t)c->nk * ((size_t)(i - 1) + (size_t)c->I * (j - 1)), &A3(a, 0, i, j),
                   sizeof(double) * c->nk);
}

int orc_filter_compact(const orc_cfg* c, const double* x, double* y) {
    int rc = check_cfg(c);
    if (rc) return rc;
    set_threads(c->nthreads);
    double* V = to_halo(c, x);
    if (!V) return ORC_ERR_ARG;
    rc = orc_filtering_procedure(c, V);
    if (!rc) from_halo(c, V, y);
    free(V);
    return rc;
}

/* u_g = B_g R_g Bz^T x for every generation, written into G[g] (gen 0 into V). */
static void half_chain(const orc_cfg* c, const setup_t* S, arr3 V, gen_t* G) {
    if (c->l_vertical_filter && c->nzcol > 0) vfilter(c, S, V, 1);
    const int filt1 = (c->proc == 1) || (c->proc == 2) || (c->proc == 3) || c->l_filt_g1;
    const int fast = c->proc == 3 || c->proc == 8;
    for (int g = 0; g + 1 < c->gm; ++g)
        restrict_gen(c, g ? G[g].H : V, &G[g], G[g + 1].H, 0, c->nk);
    for (int g = 0; g < c->gm; ++g) {
        if (g == 0 && !filt1) continue;
        arr3 U = g ? G[g].H : V;
        if (fast) {
            fast_adjoint(c, S, U, G[g].I, G[g].J, 0, c->nk);
            continue;
        }
        if (c->proc == 2 || c->proc == 7) {
            lin2_adjoint(c, S, U, G[g].tmp, G[g].I, G[g].J, 0, c->nk);
            continue;
        }
        vrbeta2t(S, c->p, U, G[g].tmp, 1, G[g].I, 1, G[g].J, 0, c->nk);
        fold_h(U, G[g].I, G[g].J, c->hx, c->hy, 0, c->nk);
    }
}

int orc_weight_grads(const orc_cfg* c, const double* x, const double* gy, double* ga) {
    int rc = check_cfg(c);
    if (rc) return rc;
    set_threads(c->nthreads);
    /* proc 4: its adjoint side is not the transpose of its forward side;
     * proc 7: Bz^T M Bz^T, so the gy chain would need Bz, not Bz^T */
    if (c->proc == 4 || c->proc == 5 || c->proc == 7) return ORC_ERR_ARG;
    setup_t S;
    rc = setup(c, &S);
    if (rc) return rc;
    double* Vx = to_halo(c, x);
    double* Vy = to_halo(c, gy);
    gen_t Gx[ORC_MAX_GEN], Gy[ORC_MAX_GEN];
    memset(Gx, 0, sizeof(Gx)); memset(Gy, 0, sizeof(Gy));
    gens_alloc(c, Gx); gens_alloc(c, Gy);
    arr3 ax = {Vx, c->nk, 1 - c->hx, c->I + c->hx, 1 - c->hy, c->J + c->hy};
    arr3 ay = {Vy, c->nk, 1 - c->hx, c->I + c->hx, 1 - c->hy, c->J + c->hy};
    half_chain(c, &S, ax, Gx);
    half_chain(c, &S, ay, Gy);
    const int filt1 = (c->proc == 1) || (c->proc == 2) || (c->proc == 3) || c->l_filt_g1;
    for (int g = 0; g < c->gm; ++g) {
        double s = 0.0;
        if (g == 0 && !filt1) { ga[g] = 0.0; continue; }
        arr3 U = g ? Gx[g].H : ax, W = g ? Gy[g].H : ay;
        for (int j = 1; j <= Gx[g].J; ++j)
            for (int i = 1; i <= Gx[g].I; ++i)
                for (int k = 0; k < c->nk; ++k) s += A3(U, k, i, j) * A3(W, k, i, j);
        ga[g] = s;
    }
    gens_free(c, Gx); gens_free(c, Gy);
    free(Vx); free(Vy);
    return ORC_OK;
}

int orc_stage(const orc_cfg* c, int which, int gen, const double* x, double* y) {
    int rc = check_cfg(c);
    if (rc) return rc;
    set_threads(c->nthreads);
    setup_t S;
    rc = setup(c, &S);
    if (rc) return rc;
    if (gen < 1 || gen > c->gm) return ORC_ERR_ARG;
    int I = c->I >> (gen - 1), J = c->J >> (gen - 1), nk = c->nk;
    if (which == 0 || which == 1) {
        orc_cfg cc = *c; cc.I = I; cc.J = J;
        double* V = to_halo(&cc, x);
        arr3 a = {V, nk, 1 - c->hx, I + c->hx, 1 - c->hy, J + c->hy};
        vfilter(&cc, &S, a, which == 1);
        from_halo(&cc, V, y);
        free(V);
        return ORC_OK;
    }
    if (which == 2 || which == 3) {
        orc_cfg cc = *c; cc.I = I; cc.J = J;
        double* V = to_halo(&cc, x);
        arr3 a = {V, nk, 1 - c->hx, I + c->hx, 1 - c->hy, J + c->hy};
        arr3 t = a3_alloc(nk, 1 - c->hx, I + c->hx, 1 - c->hy, J + c->hy);
        double* tb = (double*)malloc(sizeof(double) * nk);
        if (which == 2) {
            fill_h(a, I, J, c->hx, c->hy, 0, nk);
            vrbeta2(&S, c->p, a, t, 1, I, 1, J, 0, nk, tb);
        } else {
            vrbeta2t(&S, c->p, a, t, 1, I, 1, J, 0, nk);
            fold_h(a, I, J, c->hx, c->hy, 0, nk);
        }
        from_halo(&cc, V, y);
        free(tb); a3_free(&t); free(V);
        return ORC_OK;
    }
    if (which == 6 || which == 7) {
        orc_cfg cc = *c; cc.I = I; cc.J = J;
        double* V = to_halo(&cc, x);
        arr3 a = {V, nk, 1 - c->hx, I + c->hx, 1 - c->hy, J + c->hy};
        if (which == 6) fast_forward(c, &S, a, I, J, 0, nk);
        else fast_adjoint(c, &S, a, I, J, 0, nk);
        from_halo(&cc, V, y);
        free(V);
        return ORC_OK;
    }
    if (which == 10) {
        if (c->proc != 5) return ORC_ERR_ARG;
        orc_cfg cc = *c; cc.I = I; cc.J = J;
        double* V = to_halo(&cc, x);
        arr3 a = {V, nk, 1 - c->hx, I + c->hx, 1 - c->hy, J + c->hy};
        arr3 t = a3_alloc(nk, 1 - c->hx, I + c->hx, 1 - c->hy, J + c->hy);
        lin3_generation(c, &S, a, t, I, J, c->a[gen - 1], c->b[gen - 1], gen > 1);
        from_halo(&cc, V, y);
        a3_free(&t); free(V);
        return ORC_OK;
    }
    if (which == 8 || which == 9) {
        if (c->proc != 2 && c->proc != 7) return ORC_ERR_ARG;
        orc_cfg cc = *c; cc.I = I; cc.J = J;
        double* V = to_halo(&cc, x);
        arr3 a = {V, nk, 1 - c->hx, I + c->hx, 1 - c->hy, J + c->hy};
        arr3 t = a3_alloc(nk, 1 - c->hx, I + c->hx, 1 - c->hy, J + c->hy);
        if (which == 8) lin2_forward(c, &S, a, t, I, J, 0, nk);
        else lin2_adjoint(c, &S, a, t, I, J, 0, nk);
        from_halo(&cc, V, y);
        a3_free(&t); free(V);
        return ORC_OK;
    }
    if (which == 4 || which == 5) {
        if (gen >= c->gm) return ORC_ERR_ARG;
        gen_t Gf;
        memset(&Gf, 0, sizeof(Gf));
        Gf.I = I; Gf.J = J;
        Gf.tmp = a3_alloc(nk, 1, I, 1, J);
        Gf.INT = a3_alloc(nk, -1, I / 2 + 2, -1, J / 2 + 2);
        Gf.aux = a3_alloc(nk, 1, I, -1, J / 2 + 2);
        arr3 fine = a3_alloc(nk, 1, I, 1, J);
        arr3 coarse = a3_alloc(nk, 1, I / 2, 1, J / 2);
        if (which == 4) {
            memcpy(fine.d, x, sizeof(double) * (size_t)nk * I * J);
            restrict_gen(c, fine, &Gf, coarse, 0, nk);
            memcpy(y, coarse.d, sizeof(double) * (size_t)nk * (I / 2) * (J / 2));
        } else {
            memcpy(coarse.d, x, sizeof(double) * (size_t)nk * (I / 2) * (J / 2));
            prolong_add(c, coarse, &Gf, fine, 0, nk); /* fine starts at zero */
            memcpy(y, fine.d, sizeof(double) * (size_t)nk * I * J);
        }
        a3_free(&Gf.tmp); a3_free(&Gf.INT); a3_free(&Gf.aux); a3_free(&fine); a3_free(&coarse);
        return ORC_OK;
    }
    return ORC_ERR_ARG;
}

/* ------------------------------------------- analysis <-> filter transfers */

#define XF_IB 6 /* ib = jb = 6 (mg_parameter.f90:520-521): range of the xf table */

typedef struct {
    int ref;      /* first filter tap, rank-local 1-based index */
    double c[4];  /* weights of taps ref .. ref+order */
} xcoef;

/* lsqr_mg_coef (mg_interpolate.f90:89-298) along one axis of one rank:
 * lengthx = na (mg_parameter.f90:515-541), so dxa = 1, dxf = na/nf, both
 * grids offset by half a cell.  order 3: the blend of two quadratic
 * Lagrange interpolants (cx0..cx3, first tap iref); 2: quadratic (qx,
 * irefq); 1: linear (Lx, irefL). */
static void axis_coef(int na, int nf, int order, xcoef* out) {
    const double length = 1.0 * na;
    const double da = length / na, df = length / nf;
    const double a0 = da * 0.5, f0 = df * 0.5;
    for (int n = 1; n <= na; ++n) {
        const double x = a0 + da * (n - 1);
        int ifound = 1 - XF_IB;
        for (int i = 1 - XF_IB; i <= nf + XF_IB - 1; ++i)
            if (x < f0 + df * (i - 1)) { ifound = i; break; }
        xcoef* o = &out[n - 1];
        o->c[0] = o->c[1] = o->c[2] = o->c[3] = 0.0;
        if (order == 3) {
            const int i = ifound - 2;
            const double x1 = f0 + df * (i - 1), x2 = f0 + df * i, x3 = f0 + df * (i + 1), x4 = f0 + df * (i + 2);
            const double x1x = x1 - x, x2x = x2 - x, x3x = x3 - x, x4x = x4 - x;
            const double rx2x1 = 1. / (x2 - x1), rx3x1 = 1. / (x3 - x1);
            const double rx3x2 = 1. / (x3 - x2), rx4x2 = 1. / (x4 - x2), rx4x3 = 1. / (x4 - x3);
            const double cfl1 = x2x * x3x * rx2x1 * rx3x1;
            const double cfl2 = -(x1x * x3x * rx2x1 * rx3x2);
            const double cfl3 = x1x * x2x * rx3x1 * rx3x2;
            const double cll = x3x * rx3x2;
            const double cfr1 = x3x * x4x * rx3x2 * rx4x2;
            const double cfr2 = -(x2x * x4x * rx3x2 * rx4x3);
            const double cfr3 = x2x * x3x * rx4x2 * rx4x3;
            const double crr = -(x2x * rx3x2);
            o->ref = i;
            o->c[0] = cfl1 * cll;
            o->c[1] = cfl2 * cll + cfr1 * crr;
            o->c[2] = cfl3 * cll + cfr2 * crr;
            o->c[3] = cfr3 * crr;
        } else if (order == 2) {
            const int i = ifound - 1;
            const double x1 = f0 + df * (i - 1), x2 = f0 + df * i, x3 = f0 + df * (i + 1);
            const double x1_x = x1 - x, x2_x = x2 - x, x3_x = x3 - x;
            const double rx2x1 = 1. / (x2 - x1), rx3x1 = 1. / (x3 - x1), rx3x2 = 1. / (x3 - x2);
            o->ref = i;
            o->c[0] = x2_x * x3_x * rx2x1 * rx3x1;
            o->c[1] = -(x1_x * x3_x * rx2x1 * rx3x2);
            o->c[2] = x1_x * x2_x * rx3x1 * rx3x2;
        } else {
            const int i = ifound - 1;
            const double x1 = f0 + df * (i - 1), x2 = f0 + df * i;
            const double x1_x = x1 - x, x2_x = x2 - x;
            const double rx2x1 = 1. / (x2 - x1);
            o->ref = i;
            o->c[0] = x2_x * rx2x1;
            o->c[1] = -(x1_x * rx2x1);
        }
    }
}

static int xfer_check(const orc_xfer* c) {
    if (!c || c->nm0 <= 0 || c->mm0 <= 0 || c->nxpe <= 0 || c->nype <= 0 || c->im <= 0 || c->jm <= 0) return ORC_ERR_ARG;
    if (c->nm0 % c->nxpe || c->mm0 % c->nype) return ORC_ERR_ARG;
    if (c->order < 1 || c->order > 3 || c->hx < c->order || c->hy < c->order) return ORC_ERR_ARG;
    if (c->lm_a > c->lm && (c->lm_a != 2 * c->lm - 1 || (size_t)c->en * c->lm > (size_t)c->nkf ||
                            (size_t)c->en * c->lm_a > (size_t)c->nka))
        return ORC_ERR_ARG;
    if (c->lm_a <= c->lm && c->nka != c->nkf) return ORC_ERR_ARG;
    return ORC_OK;
}

/* filt_to_anal_all2 / filt_to_anal (mg_transfer.f90:184-203, 406-464):
 * boco_2d with the interpolation halo, lsqr/quad/lin_direct_offset
 * (mg_interpolate.f90:634-681, 750-795, 858-903), then
 * l_vertical_direct_spec2 (mg_interpolate.f90:1006-1044) when lm_a > lm. */
int orc_filt_to_anal(const orc_xfer* c, double* vall, double* worka) {
    int rc = xfer_check(c);
    if (rc) return rc;
    const int I = c->nxpe * c->im, J = c->nype * c->jm, nm = c->nm0 / c->nxpe, mm = c->mm0 / c->nype;
    const int ib = c->order, nt = c->order + 1, nk = c->nkf;
    arr3 V = {vall, nk, 1 - c->hx, I + c->hx, 1 - c->hy, J + c->hy};
    fill_h(V, I, J, ib, ib, 0, nk);
    xcoef* cx = (xcoef*)malloc(sizeof(xcoef) * nm);
    xcoef* cy = (xcoef*)malloc(sizeof(xcoef) * mm);
    axis_coef(nm, c->im, c->order, cx);
    axis_coef(mm, c->jm, c->order, cy);
    const int vert = c->lm_a > c->lm;
    double* work = vert ? (double*)malloc(sizeof(double) * (size_t)nk * c->nm0 * c->mm0) : worka;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int M = 1; M <= c->mm0; ++M) {
        const int rj = (M - 1) / mm;
        const xcoef* ky = &cy[M - 1 - rj * mm];
        const int j0 = rj * c->jm + ky->ref;
        double vx[4];
        for (int N = 1; N <= c->nm0; ++N) {
            const int ri = (N - 1) / nm;
            const xcoef* kx = &cx[N - 1 - ri * nm];
            const int i0 = ri * c->im + kx->ref;
            double* w = work + (size_t)nk * ((size_t)(N - 1) + (size_t)c->nm0 * (M - 1));
            for (int k = 0; k < nk; ++k) {
                for (int s = 0; s < nt; ++s) {
                    double v = kx->c[0] * A3(V, k, i0, j0 + s);
                    for (int t = 1; t < nt; ++t) v += kx->c[t] * A3(V, k, i0 + t, j0 + s);
                    vx[s] = v;
                }
                double r = ky->c[0] * vx[0];
                for (int s = 1; s < nt; ++s) r += ky->c[s] * vx[s];
                w[k] = r;
            }
        }
    }
    if (vert) {
        const size_t npts = (size_t)c->nm0 * c->mm0;
        for (size_t q = 0; q < npts; ++q) {
            const double* F = work + (size_t)nk * q;
            double* W = worka + (size_t)c->nka * q;
            for (int e = 0; e < c->en; ++e) {
                const int enm = e * c->lm_a, ekm = e * c->lm;
                int k = 1;
                for (int n = 1; n <= c->lm_a; n += 2) W[enm + n - 1] = F[ekm + k - 1], ++k;
                k = 1;
                for (int n = 2; n <= c->lm_a - 1; n += 2) W[enm + n - 1] = 0.5 * (F[ekm + k - 1] + F[ekm + k]), ++k;
            }
        }
        free(work);
    }
    free(cx);
    free(cy);
    return ORC_OK;
}

/* anal_to_filt_all2 / anal_to_filt (mg_transfer.f90:154-181, 339-403):
 * l_vertical_adjoint_spec2 (mg_interpolate.f90:963-1003) when lm_a > lm,
 * VALL = 0, lsqr/quad/lin_adjoint_offset (mg_interpolate.f90:684-747,
 * 798-855, 906-960), bocoT_2d with the interpolation halo (the halo keeps
 * its scattered values).  The ranks' scatters into each other's halos sum
 * into the one global array. */
int orc_anal_to_filt(const orc_xfer* c, const double* worka, double* vall) {
    int rc = xfer_check(c);
    if (rc) return rc;
    const int I = c->nxpe * c->im, J = c->nype * c->jm, nm = c->nm0 / c->nxpe, mm = c->mm0 / c->nype;
    const int ib = c->order, nt = c->order + 1, nk = c->nkf;
    const size_t npts = (size_t)c->nm0 * c->mm0;
    const double* work = worka;
    double* wbuf = NULL;
    if (c->lm_a > c->lm) {
        wbuf = (double*)calloc((size_t)nk * npts, sizeof(double));
        for (size_t q = 0; q < npts; ++q) {
            const double* W = worka + (size_t)c->nka * q;
            double* F = wbuf + (size_t)nk * q;
            for (int e = 0; e < c->en; ++e) {
                const int enm = e * c->lm_a, ekm = e * c->lm;
                int k = 1;
                for (int n = 2; n <= c->lm_a - 1; n += 2) {
                    F[ekm + k - 1] += 0.5 * W[enm + n - 1];
                    F[ekm + k] += 0.5 * W[enm + n - 1];
                    ++k;
                }
                k = 1;
                for (int n = 1; n <= c->lm_a; n += 2) F[ekm + k - 1] += W[enm + n - 1], ++k;
            }
        }
        work = wbuf;
    }
    arr3 V = {vall, nk, 1 - c->hx, I + c->hx, 1 - c->hy, J + c->hy};
    memset(vall, 0, sizeof(double) * (size_t)nk * (I + 2 * c->hx) * (size_t)(J + 2 * c->hy));
    xcoef* cx = (xcoef*)malloc(sizeof(xcoef) * nm);
    xcoef* cy = (xcoef*)malloc(sizeof(xcoef) * mm);
    axis_coef(nm, c->im, c->order, cx);
    axis_coef(mm, c->jm, c->order, cy);
    /* VX(nk, 1:nm0, 1-ib:J+ib) */
    arr3 VX = a3_alloc(nk, 1, c->nm0, 1 - ib, J + ib);
    a3_zero(VX, 0, nk);
    for (int M = 1; M <= c->mm0; ++M) {
        const int rj = (M - 1) / mm;
        const xcoef* ky = &cy[M - 1 - rj * mm];
        const int j0 = rj * c->jm + ky->ref;
        for (int N = 1; N <= c->nm0; ++N) {
            const double* w = work + (size_t)nk * ((size_t)(N - 1) + (size_t)c->nm0 * (M - 1));
            for (int s = 0; s < nt; ++s)
                for (int k = 0; k < nk; ++k) A3(VX, k, N, j0 + s) += w[k] * ky->c[s];
        }
    }
    for (int N = 1; N <= c->nm0; ++N) {
        const int ri = (N - 1) / nm;
        const xcoef* kx = &cx[N - 1 - ri * nm];
        const int i0 = ri * c->im + kx->ref;
        for (int j = 1 - ib; j <= J + ib; ++j)
            for (int t = 0; t < nt; ++t)
                for (int k = 0; k < nk; ++k) A3(V, k, i0 + t, j) += A3(VX, k, N, j) * kx->c[t];
    }
    fold_h(V, I, J, ib, ib, 0, nk);
    a3_free(&VX);
    free(cx);
    free(cy);
    free(wbuf);
    return ORC_OK;
}
