// FP64 setup of the filter tables; see mgbf_setup.hpp for the reference
// routines restated here.
#include "mgbf_setup.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <cstdlib>
#include <cstdio>

#include "../../include/mgbf.h"

namespace mgbf {

static double ipow(double x, int p) {
    double r = 1.0;
    for (int t = 0; t < p; ++t) r *= x;
    return r;
}

static double binom(int n, int k) {
    double r = 1.0;
    for (int t = 1; t <= k; ++t) r = r * (n - k + t) / t;
    return r;
}

int canonical_width(int R, int gy) {
    const long lim = (long)R * R + R - (long)gy * gy;
    int m = 0;
    while ((long)(m + 1) * (m + 1) <= lim) ++m;
    return m;
}

int build_hstencil(int p, double ampl02, int hx, int hy, HStencil& H, std::string& err) {
    if (!(ampl02 > 0.0)) {
        err = "mg_ampl02 must be positive";
        return MGBF_ERR_CONFIG;
    }
    const double rmom2_2 = 1.0 / std::sqrt(2.0 * p + 4.0);
    const double el = std::sqrt(1.0 / ampl02);  // cholaspect2 on diag(ampl02)
    const double exx = el * rmom2_2, eyy = el * rmom2_2, eyx = 0.0;
    H.p = p;
    H.exx = exx;
    H.eyy = eyy;
    // getlinesum2 (jp_pbfil.f90:182-218)
    const double y = 1.0 / eyy;
    const int gyl = (int)std::ceil(-y + kEps), gym = (int)std::floor(y - kEps);
    if (gyl < -hy || gym > hy) {
        err = "getlinesum2: filter reach " + std::to_string(std::max(-gyl, gym)) +
              " exceeds hy=" + std::to_string(hy);
        return MGBF_ERR_REACH;
    }
    std::vector<int> gxl(gym - gyl + 1 > 0 ? gym - gyl + 1 : 0), gxm(gxl.size());
    double sum = 0.0;
    int R = std::max(-gyl, gym);
    for (int gy = gyl; gy <= gym; ++gy) {
        const double yy = gy, xc = -yy * eyx;
        const double rrx = (yy * eyy) * (yy * eyy);
        const double x = std::sqrt(1.0 - rrx);
        const int lo = (int)std::ceil((xc - x) / exx + kEps), hi = (int)std::floor((xc + x) / exx - kEps);
        if (lo < -hx || hi > hx) {
            err = "getlinesum2: filter reach " + std::to_string(std::max(-lo, hi)) +
                  " exceeds hx=" + std::to_string(hx);
            return MGBF_ERR_REACH;
        }
        gxl[gy - gyl] = lo;
        gxm[gy - gyl] = hi;
        R = std::max(R, std::max(-lo, hi));
        for (int gx = lo; gx <= hi; ++gx) {
            const double xx = gx;
            const double rr = rrx + (xx * exx - xc) * (xx * exx - xc);
            sum += ipow(1.0 - rr, p);
        }
    }
    if (!(sum > 0.0)) {
        err = "getlinesum2: empty or degenerate stencil";
        return MGBF_ERR_CONFIG;
    }
    if (R > kMaxReach) {
        err = "horizontal reach " + std::to_string(R) + " exceeds the supported maximum " +
              std::to_string(kMaxReach);
        return MGBF_ERR_UNSUPPORTED;
    }
    const double s = 1.0 / sum;
    H.s = s;
    H.R = R;
    const int W = 2 * R + 1;
    H.mrow.assign(W, -1);
    H.w.assign((size_t)W * W, 0.0);
    bool symmetric = (gyl == -gym);
    for (int gy = gyl; gy <= gym; ++gy) {
        const int lo = gxl[gy - gyl], hi = gxm[gy - gyl];
        if (lo != -hi) symmetric = false;
        H.mrow[gy + R] = hi;
        const double yy = gy, xc = -yy * eyx;
        const double rrx = (yy * eyy) * (yy * eyy);
        for (int gx = lo; gx <= hi; ++gx) {
            const double xx = gx;
            const double rr = rrx + (xx * exx - xc) * (xx * exx - xc);
            H.w[(size_t)(gy + R) * W + (gx + R)] = s * ipow(1.0 - rr, p);  // frow
        }
    }
    if (!symmetric) {
        err = "radial support is not symmetric";
        return MGBF_ERR_CONFIG;
    }
    bool canon = (gyl == -R && gym == R);
    for (int gy = -R; gy <= R && canon; ++gy)
        if (H.mrow[gy + R] != canonical_width(R, std::abs(gy))) canon = false;
    H.canonical = canon && p <= kMaxMomP;
    H.mom = HMomCoefs<double>{};
    if (H.canonical) {
        // Row gy of the disk: w = s (A - u)^p with A = 1 - (e gy)^2,
        // u = (e gx)^2 = sum_q C(p,q) A^(p-q) (-u)^q: the kernel keeps
        // T'_q = C(p,q) (-1)^q sum u^q a and evaluates Horner in A; s is
        // applied at the store (HMomArgs::scale).
        const int PQ = p + 1;
        for (int gy = 0; gy <= R; ++gy) H.mom.coef[gy * PQ] = 1.0 - (gy * eyy) * (gy * eyy);
        for (int m = 0; m <= R; ++m) {
            const double u = (m * exx) * (m * exx);
            for (int q = 0; q <= p; ++q)
                H.mom.upow[m * PQ + q] = binom(p, q) * ((q & 1) ? -1.0 : 1.0) * ipow(u, q);
        }
    }
    return MGBF_OK;
}

int build_zstencil(int p, double ampl01, int hz, int lm, bool need, ZStencil& Z, std::string& err) {
    if (!(ampl01 > 0.0)) {
        err = "mg_ampl01 must be positive";
        return MGBF_ERR_CONFIG;
    }
    const double rmom2_1 = 1.0 / std::sqrt(2.0 * p + 3.0);
    const double el = 1.0 / std::sqrt(ampl01);  // cholaspect1
    const double exx = el * rmom2_1;
    const double x = 1.0 / exx;
    const int gxl = (int)std::ceil(-x + kEps), gxm = (int)std::floor(x - kEps);
    // getlinesum1 (jp_pbfil.f90:149-180), called unconditionally in
    // def_mg_weights (mg_intstate.f90:429)
    if (gxl < -hz || gxm > hz) {
        err = "getlinesum1: filter reach " + std::to_string(std::max(-gxl, gxm)) +
              " exceeds hz=" + std::to_string(hz);
        return MGBF_ERR_REACH;
    }
    double sum = 0.0;
    for (int gx = gxl; gx <= gxm; ++gx) {
        const double xx = gx;
        sum += ipow(1.0 - (xx * exx) * (xx * exx), p);
    }
    const double s = 1.0 / sum;
    const int mz = std::max(-gxl, gxm);
    if (need && mz > kMaxZReach) {
        err = "vertical reach " + std::to_string(mz) + " exceeds the supported maximum " +
              std::to_string(kMaxZReach);
        return MGBF_ERR_UNSUPPORTED;
    }
    Z.lm = lm;
    Z.mz = mz;
    Z.exx = exx;
    Z.s = s;
    Z.wz.assign(2 * mz + 1, 0.0);
    for (int gx = gxl; gx <= gxm; ++gx) {
        const double xx = gx;
        Z.wz[gx + mz] = s * ipow(1.0 - (xx * exx) * (xx * exx), p);  // frow of vrbeta1
    }
    if (!need) return MGBF_OK;
    if (mz > lm - 1) {
        err = "vertical reach " + std::to_string(mz) + " needs lm >= " + std::to_string(mz + 1);
        return MGBF_ERR_CONFIG;
    }
    const int bw = 2 * mz + 1;
    Z.fwd.assign((size_t)lm * bw, 0.0);
    Z.adj.assign((size_t)lm * bw, 0.0);
    // forward: W(1-L) = W(1+L), W(lm+L) = W(lm-L) (whole-sample mirror,
    // mg_filtering.f90:2178-2181), then b(L) = sum_g w(g) W(L+g)
    for (int L = 0; L < lm; ++L)
        for (int g = gxl; g <= gxm; ++g) {
            int q = L + g;
            if (q < 0) q = -q;
            if (q > lm - 1) q = 2 * (lm - 1) - q;
            Z.fwd[(size_t)L * bw + (q - L) + mz] += Z.wz[g + mz];
        }
    for (int L = 0; L < lm; ++L)
        for (int d = -mz; d <= mz; ++d) {
            const int r = L + d;
            if (r < 0 || r >= lm) continue;
            Z.adj[(size_t)L * bw + d + mz] = Z.fwd[(size_t)r * bw + (-d) + mz];
        }
    // M = Bz Bz^T: M(L, L+e) = sum_k Bz(L, k) Bz(L+e, k)
    Z.mmz = std::min(2 * mz, lm - 1);
    const int mw = 2 * Z.mmz + 1;
    Z.mm.assign((size_t)lm * mw, 0.0);
    for (int L = 0; L < lm; ++L)
        for (int e = -Z.mmz; e <= Z.mmz; ++e) {
            const int L2 = L + e;
            if (L2 < 0 || L2 >= lm) continue;
            double acc = 0.0;
            for (int k = std::max(0, std::max(L, L2) - mz); k <= std::min(lm - 1, std::min(L, L2) + mz); ++k)
                acc += Z.fwd[(size_t)L * bw + (k - L) + mz] * Z.fwd[(size_t)L2 * bw + (k - L2) + mz];
            Z.mm[(size_t)L * mw + e + Z.mmz] = acc;
        }
    return MGBF_OK;
}

int build_interp(int nf, bool quart, Interp1D& T, std::string& err) {
    // def_offset_coef (mg_interpolate.f90:61-86)
    static const double PC[4] = {-9.0 / 128.0, 111.0 / 128.0, 29.0 / 128.0, -3.0 / 128.0};
    static const double QC[4] = {-3.0 / 128.0, 29.0 / 128.0, 111.0 / 128.0, -9.0 / 128.0};
    static const double AC[3] = {5.0 / 32.0, 30.0 / 32.0, -3.0 / 32.0};
    static const double BC[3] = {-3.0 / 32.0, 30.0 / 32.0, 5.0 / 32.0};
    if (nf % 2) {
        err = "generation size " + std::to_string(nf) + " is odd";
        return MGBF_ERR_DIVISIBILITY;
    }
    const int nc = nf / 2;
    const int nt = quart ? 3 : 4;
    if (nc < (quart ? 1 : 2)) {
        err = "coarse generation size " + std::to_string(nc) + " too small for the interpolation halo";
        return MGBF_ERR_DIVISIBILITY;
    }
    T.nf = nf;
    T.nc = nc;
    T.ntap = nt;
    T.pidx.assign((size_t)nf * nt, 0);
    T.pw.assign((size_t)nf * nt, 0.0);
    std::vector<double> P((size_t)nf * nc, 0.0);
    for (int i = 1; i <= nf; ++i) {
        int iL;
        const double* cf;
        if (!quart) {  // direct1 (mg_generations.f90:1190-1250)
            iL = i / 2;
            cf = (i % 2) ? QC : PC;
        } else {  // direct2 (mg_generations.f90:1319-1374)
            if (i % 2) { iL = (i + 1) / 2; cf = AC; }
            else { iL = i / 2; cf = BC; }
        }
        for (int t = 0; t < nt; ++t) {
            int c = iL - 1 + t;             // coarse index with halo 2 (1)
            if (c < 1) c = 1 - c;           // boco_2d half-sample mirror
            if (c > nc) c = 2 * nc + 1 - c;
            T.pidx[(size_t)(i - 1) * nt + t] = c - 1;
            T.pw[(size_t)(i - 1) * nt + t] = cf[t];
            P[(size_t)(i - 1) * nc + (c - 1)] += cf[t];
        }
    }
    T.rw.assign((size_t)nc * 8, 0.0);
    for (int c = 0; c < nc; ++c)
        for (int f = 0; f < nf; ++f) {
            const double v = P[(size_t)f * nc + c];
            if (v == 0.0) continue;
            const int a = f - (2 * c - 3);
            if (a < 0 || a >= 8) {
                err = "restriction stencil wider than 8";
                return MGBF_ERR_CONFIG;
            }
            T.rw[(size_t)c * 8 + a] = v;
        }
    return MGBF_OK;
}

// getlinesum1 (jp_pbfil.f90:149-180) and the vrbeta1 weights
// (jp_pbfil.f90:856-885) for el = paspx = paspy = pasp02.
// Beta filters of integer half-span m = 1..nh: normalisation and spread^2
// (the corrected moments of inimomtab, jp_pbfil3.f90:378-457, are these
// exact sums).
static void dib_table(int p, double* norm, double* spread) {
    for (int m = 1; m <= kDibNH; ++m) {
        double s0 = 0.0, s2 = 0.0;
        for (int i = -m; i <= m; ++i) {
            const double u = 1.0 - (double(i) / m) * (double(i) / m);
            const double w = std::pow(u, p);
            s0 += w;
            s2 += double(i) * i * w;
        }
        norm[m] = 1.0 / s0;
        spread[m] = s2 / s0;
    }
}

// hstform (jp_pbfil3.f90:1399-1430): spread^2 -> formal half-span hs between
// the table entries around it; blinfil (1463-1501): the weights fil[0..h] of
// the two-beta filter of half-spans h = int(hs) and h + 1.  False when the
// spread is beyond the table.
static bool dib_weights(int p, double s2, const double* norm, const double* spread, int& h_out, double& hs_out,
                        double* fil) {
    double hs = -1.0;
    if (s2 >= 0.0)
        for (int m = 2; m <= kDibNH; ++m)
            if (spread[m] >= s2) {
                hs = m - (spread[m] - s2) / (spread[m] - spread[m - 1]);
                break;
            }
    const int h = hs < 0.0 ? 0 : int(hs), hp = h + 1;
    if (hs < 0.0 || h < 1 || hp > kDibNH || hp > kDibNFil) return false;
    const double whp = (hs - h) * norm[hp], wh = (hp - hs) * norm[h];
    for (int i = 0; i <= kDibNFil; ++i) fil[i] = 0.0;
    for (int i = 0; i <= h; ++i) {
        const double u = 1.0 - (double(i) / hp) * (double(i) / hp);
        fil[i] = whp * std::pow(u, p);
    }
    for (int i = 0; i < h; ++i) {
        const double u = 1.0 - (double(i) / h) * (double(i) / h);
        fil[i] += wh * std::pow(u, p);
    }
    h_out = h;
    hs_out = hs;
    return true;
}

int build_dstencil(int p, double ampl02, int hx, int hy, DStencil& out, std::string& err) {
    out = DStencil{};
    if (!(ampl02 > 0.0) || p < 1) {
        err = "line filters need mg_ampl02 > 0 and p >= 1";
        return MGBF_ERR_CONFIG;
    }
    double norm[kDibNH + 1], spread[kDibNH + 1];
    dib_table(p, norm, spread);
    // triad of (A11, A22, A12): generators g[q], projections lu[q] (rows of
    // the inverse basis), weights w[q] = A . lu[q]
    const double c = std::sqrt(1.0 / ampl02);
    const double A[3] = {c, c, 0.0};
    int g[3][2] = {{1, 0}, {0, 1}, {-1, -1}};
    int lu[3][3] = {{1, 0, -1}, {0, 1, -1}, {0, 0, 1}};
    double w[3];
    for (int q = 0; q < 3; ++q) w[q] = A[0] * lu[q][0] + A[1] * lu[q][1] + A[2] * lu[q][2];
    bool done = false;
    for (int it = 0; it < 200 && !done; ++it) {
        int k = 0;
        for (int q = 1; q < 3; ++q)
            if (w[q] < w[k]) k = q;
        const double dw = 2.0 * w[k];
        if (dw >= -1e-14) {
            done = true;
            break;
        }
        const int l = (k + 1) % 3, m = (l + 1) % 3;
        int d2[3];
        for (int r = 0; r < 3; ++r) d2[r] = 2 * lu[k][r];
        for (int e = 0; e < 2; ++e) {
            g[l][e] = -g[l][e];
            g[k][e] = -g[l][e] - g[m][e];
        }
        for (int q = 0; q < 3; ++q) {
            const int sg = q == k ? -1 : 1;
            for (int r = 0; r < 3; ++r) lu[q][r] += sg * d2[r];
            w[q] += sg * dw;
        }
    }
    if (!done) {
        err = "triad: the aspect tensor did not resolve into three line filters";
        return MGBF_ERR_CONFIG;
    }
    for (int q = 0; q < 3; ++q) {
        int h = 0;
        double hs = 0.0;
        if (!dib_weights(p, w[q], norm, spread, h, hs, out.fil[q])) {
            err = "line filter spread^2 " + std::to_string(w[q]) + " (mg_ampl02) is beyond the moment table (nh = " +
                  std::to_string(kDibNH) + ")";
            return MGBF_ERR_REACH;
        }
        out.dx[q] = g[q][0]; out.dy[q] = g[q][1]; out.h[q] = h; out.hs[q] = hs;
        if (h * std::abs(g[q][0]) > hx || h * std::abs(g[q][1]) > hy) {
            err = "line filter " + std::to_string(q + 1) + " reaches " + std::to_string(h) + " steps of (" +
                  std::to_string(g[q][0]) + "," + std::to_string(g[q][1]) + "), beyond the halo hx=" +
                  std::to_string(hx) + ", hy=" + std::to_string(hy);
            return MGBF_ERR_REACH;
        }
    }
    out.ok = true;
    return MGBF_OK;
}

// The hexad of a 3D aspect (jp_pbfil3.f90:798-904).  The seven nonzero
// elements of GF(8) index the colors; a hexad is a set of six of them whose
// generators span the aspect with non-negative weights, the seventh (its
// own color, hcol) being null.  The iteration keeps three K-set generators
// (the colors hcol - 1, hcol - 2, hcol - 4), derives the other three as
// differences of consecutive ones, and while a weight is negative moves the
// null color there, transforms the K-set by one of six unimodular matrices
// (chosen by the step hcol_new - hcol_old) and applies a rank-one update
// with the sign pattern of the new color's lines to the projection rows.
// The starting generators and projections, the six matrices, the step
// offsets, the sign pattern and the output color order are the reference's
// tables (they decide which generators the filters use and in what order,
// which changes the result).  Returns false if 200 steps do not settle.
static bool hexad(const double A[6], int gen[7][3], double wgt[7]) {
    static const int l0[7][3] = {{0, 0, 0}, {1, -1, 0}, {0, 1, -1}, {0, 0, 1}, {-1, 0, 1}, {0, 1, 0}, {1, 0, 0}};
    static const int u0[7][6] = {{0, 0, 0, 0, 0, 0},  {0, 0, 0, 0, 0, -1}, {0, 0, 0, -1, 0, 0}, {0, 0, 1, 1, 1, 0},
                                 {0, 0, 0, 0, -1, 0}, {0, 1, 0, 1, 0, 1},  {1, 0, 0, 0, 1, 1}};
    static const int mk[6][3][3] = {{{1, 1, -1}, {1, 0, 0}, {1, 0, -1}},  {{-1, 1, 0}, {-1, 1, 1}, {0, 1, 0}},
                                    {{0, -1, 1}, {1, -1, 0}, {1, 0, 0}},  {{0, 0, 1}, {0, -1, 1}, {1, -1, 1}},
                                    {{-1, 0, 1}, {0, 0, 1}, {-1, 1, 0}},  {{0, 1, 0}, {1, 0, -1}, {0, 1, -1}}};
    static const int step_off[7] = {0, 5, 3, 3, 6, 5, 6};
    static const int sign[13] = {-1, -1, 1, -1, 1, 1, 1, -1, -1, 1, -1, 1, 1};  // offset -6..6
    static const int lines[3] = {1, 2, 4};
    static const int out_color[7] = {7, 4, 6, 3, 5, 2, 1};
    auto md7 = [](int a) { return ((a % 7) + 7) % 7; };
    int L[7][3], U[7][6], K[3][3];
    std::memcpy(L, l0, sizeof(L));
    std::memcpy(U, u0, sizeof(U));
    double w[7];
    for (int q = 0; q < 7; ++q) {
        w[q] = 0.0;
        for (int r = 0; r < 6; ++r) w[q] += A[r] * U[q][r];
    }
    int hcol = 0, kcol = 0;
    for (int i = 0; i < 3; ++i) std::memcpy(K[i], L[md7(hcol - lines[i])], sizeof(K[i]));
    bool done = false;
    for (int it = 0; it < 200; ++it) {
        kcol = 0;
        for (int q = 1; q < 7; ++q)
            if (w[q] < w[kcol]) kcol = q;
        const double dw = w[kcol];
        if (dw >= -1e-14) {
            done = true;
            break;
        }
        const int d = md7(kcol - hcol);
        hcol = kcol;
        const int lc = md7(hcol + step_off[d]);
        int Kn[3][3];
        for (int c = 0; c < 3; ++c)
            for (int e = 0; e < 3; ++e) {
                int v = 0;
                for (int r = 0; r < 3; ++r) v += K[r][e] * mk[d - 1][c][r];
                Kn[c][e] = v;
            }
        std::memcpy(K, Kn, sizeof(K));
        int du[6];
        for (int r = 0; r < 6; ++r) du[r] = U[hcol][r];
        for (int q = 0; q < 7; ++q) {
            const int sg = sign[q - lc + 6];
            for (int r = 0; r < 6; ++r) U[q][r] += sg * du[r];
            w[q] += sg * dw;
        }
    }
    if (!done) return false;
    for (int i = 0; i < 3; ++i)
        for (int e = 0; e < 3; ++e) {
            L[md7(hcol - lines[i])][e] = K[i][e];
            L[md7(hcol + lines[i])][e] = K[i][e] - K[(i + 1) % 3][e];
        }
    for (int e = 0; e < 3; ++e) L[kcol][e] = 0;
    for (int i = 0; i < 7; ++i) {
        const int c = out_color[i] - 1;
        for (int e = 0; e < 3; ++e) gen[c][e] = L[i][e];
        wgt[c] = w[i];
    }
    return true;
}

int build_xstencil(int p, double ampl03, int hx, int hy, int hz, bool line, XStencil& out, std::string& err) {
    out = XStencil{};
    if (!line) {  // init_mg_line did not run: the colors' slots stay empty, every color copies
        out.ok = true;
        return MGBF_OK;
    }
    if (!(ampl03 > 0.0) || p < 1) {
        err = "3D line filters need mg_ampl03 > 0 and p >= 1";
        return MGBF_ERR_CONFIG;
    }
    double norm[kDibNH + 1], spread[kDibNH + 1];
    dib_table(p, norm, spread);
    const double c3 = std::sqrt(1.0 / ampl03);  // cholaspect3 of diag(mg_ampl03)
    const double A[6] = {c3, c3, c3, 0.0, 0.0, 0.0};
    int gen[7][3];
    double w[7];
    if (!hexad(A, gen, w)) {
        err = "hexad: the 3D aspect did not resolve into six line filters";
        return MGBF_ERR_CONFIG;
    }
    int slot = 0;
    for (int col = 1; col <= 7; ++col) {
        const int* g = gen[col - 1];
        if (g[0] == 0 && g[1] == 0 && g[2] == 0) continue;
        if (slot == 6) {
            err = "hexad: more than six active colors";
            return MGBF_ERR_CONFIG;
        }
        out.slot[col] = slot;
        for (int e = 0; e < 3; ++e) out.g[slot][e] = g[e];
        if (!dib_weights(p, w[col - 1], norm, spread, out.h[slot], out.hs[slot], out.fil[slot])) {
            err = "3D line filter spread^2 " + std::to_string(w[col - 1]) +
                  " (mg_ampl03) is beyond the moment table (nh = " + std::to_string(kDibNH) + ")";
            return MGBF_ERR_REACH;
        }
        const int h = out.h[slot];
        if (h * std::abs(g[0]) > hx || h * std::abs(g[1]) > hy || h * std::abs(g[2]) > hz) {
            err = "3D line filter of color " + std::to_string(col) + " reaches " + std::to_string(h) + " steps of (" +
                  std::to_string(g[0]) + "," + std::to_string(g[1]) + "," + std::to_string(g[2]) +
                  "), beyond the halo (hx, hy, hz)";
            return MGBF_ERR_REACH;
        }
        ++slot;
    }
    if (slot != 6) {  // hextform wants exactly six active lines
        err = "hexad: " + std::to_string(slot) + " active colors instead of six";
        return MGBF_ERR_CONFIG;
    }
    out.ok = true;
    return MGBF_OK;
}

int build_lstencil(int p, double ampl02, int hx, int hy, LStencil& out, std::string& err) {
    if (!(ampl02 > 0.0)) {
        err = "mg_ampl02 must be positive";
        return MGBF_ERR_CONFIG;
    }
    out = LStencil{};
    out.p = p;
    out.exx = ampl02 * (1.0 / std::sqrt(2.0 * p + 3.0));
    const double x = 1.0 / out.exx;
    const int lo = (int)std::ceil(-x + kEps), hi = (int)std::floor(x - kEps);
    if (lo < -hx || hi > hx || lo < -hy || hi > hy) {
        err = "getlinesum1 on paspx/paspy: reach " + std::to_string(std::max(-lo, hi)) + " exceeds hx/hy";
        return MGBF_ERR_REACH;
    }
    double sum = 0.0;
    for (int g = lo; g <= hi; ++g) {
        const double rr = (g * out.exx) * (g * out.exx);
        sum += std::pow(1.0 - rr, p);
    }
    out.s = 1.0 / sum;
    out.R = hi;
    out.w.resize(hi + 1);
    for (int g = 0; g <= hi; ++g) {
        const double rr = (g * out.exx) * (g * out.exx);
        out.w[g] = out.s * std::pow(1.0 - rr, p);
    }
    return MGBF_OK;
}

int build_bstencil(int p, double ampl03, int hx, int hy, int hz, BStencil& out, std::string& err) {
    out = BStencil{};
    if (!(ampl03 > 0.0)) {
        err = "mg_ampl03 must be positive";
        return MGBF_ERR_CONFIG;
    }
    const double e = std::sqrt(1.0 / ampl03) * (1.0 / std::sqrt(2.0 * p + 5.0));
    const double z = 1.0 / e;
    const int gzl = (int)std::ceil(-z + kEps), gzm = (int)std::floor(z - kEps);
    if (gzl < -hz || gzm > hz) {
        err = "getlinesum3: filter reach becomes too large for hz";
        return MGBF_ERR_REACH;
    }
    double sum = 0.0;
    std::vector<double> raw;
    for (int gz = gzl; gz <= gzm; ++gz) {
        const double rry = (gz * e) * (gz * e), y = std::sqrt(1.0 - rry);
        const int gyl = (int)std::ceil((0.0 - y) / e + kEps), gym = (int)std::floor((0.0 + y) / e - kEps);
        if (gyl < -hy || gym > hy) {
            err = "getlinesum3: filter reach becomes too large for hy";
            return MGBF_ERR_REACH;
        }
        for (int gy = gyl; gy <= gym; ++gy) {
            const double rrx = rry + (gy * e - 0.0) * (gy * e - 0.0), x = std::sqrt(1.0 - rrx);
            const int gxl = (int)std::ceil((0.0 - x) / e + kEps), gxm = (int)std::floor((0.0 + x) / e - kEps);
            if (gxl < -hx || gxm > hx) {
                err = "getlinesum3: filter reach becomes too large for hx";
                return MGBF_ERR_REACH;
            }
            for (int gx = gxl; gx <= gxm; ++gx) {
                const double rr = rrx + (gx * e - 0.0) * (gx * e - 0.0);
                const double v = std::pow(1.0 - rr, p);
                sum += v;
                raw.push_back(v);
                out.taps.insert(out.taps.end(), {gx, gy, gz, 0});
            }
        }
    }
    out.e = e;
    out.s = 1.0 / sum;
    out.R = gzm;
    for (double v : raw) out.w.push_back(out.s * v);
    const int nw = 2 * out.R + 1;
    for (size_t e = 0; e < out.w.size(); ++e) {
        const int gx = out.taps[4 * e], gy = out.taps[4 * e + 1], gz = out.taps[4 * e + 2];
        const size_t nr = out.rows.size() / 2;
        if (nr == 0 || out.rows[2 * nr - 2] != gy || out.rows[2 * nr - 1] != gz) {
            out.rows.insert(out.rows.end(), {gy, gz});
            out.rw.resize(out.rw.size() + nw, 0.0);
        }
        out.rw[out.rw.size() - nw + gx + out.R] = out.w[e];
    }
    return MGBF_OK;
}

void build_xfer_axis(int na, int nf, int nranks, int order, XferAxis& out) {
    constexpr int ib = 6;  // xf table range 1-ib .. nf+ib (mg_parameter.f90:520-521)
    const double length = 1.0 * na;
    const double da = length / na, df = length / nf;
    const double a0 = da * 0.5, f0 = df * 0.5;
    std::vector<int> lref(na);
    std::vector<double> lc(4 * (size_t)na, 0.0);
    for (int n = 1; n <= na; ++n) {
        const double x = a0 + da * (n - 1);
        int ifound = 1 - ib;
        for (int i = 1 - ib; i <= nf + ib - 1; ++i)
            if (x < f0 + df * (i - 1)) {
                ifound = i;
                break;
            }
        double* c = &lc[4 * (size_t)(n - 1)];
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
            lref[n - 1] = i;
            c[0] = cfl1 * cll;
            c[1] = cfl2 * cll + cfr1 * crr;
            c[2] = cfl3 * cll + cfr2 * crr;
            c[3] = cfr3 * crr;
        } else if (order == 2) {
            const int i = ifound - 1;
            const double x1 = f0 + df * (i - 1), x2 = f0 + df * i, x3 = f0 + df * (i + 1);
            const double x1_x = x1 - x, x2_x = x2 - x, x3_x = x3 - x;
            const double rx2x1 = 1. / (x2 - x1), rx3x1 = 1. / (x3 - x1), rx3x2 = 1. / (x3 - x2);
            lref[n - 1] = i;
            c[0] = x2_x * x3_x * rx2x1 * rx3x1;
            c[1] = -(x1_x * x3_x * rx2x1 * rx3x2);
            c[2] = x1_x * x2_x * rx3x1 * rx3x2;
        } else {
            const int i = ifound - 1;
            const double x1 = f0 + df * (i - 1), x2 = f0 + df * i;
            const double x1_x = x1 - x, x2_x = x2 - x;
            const double rx2x1 = 1. / (x2 - x1);
            lref[n - 1] = i;
            c[0] = x2_x * rx2x1;
            c[1] = -(x1_x * rx2x1);
        }
    }
    out = XferAxis{};
    out.order = order;
    const int ntot = na * nranks, nft = nf * nranks, ne = nft + 2 * order;
    out.ref.resize(ntot);
    out.c.resize(4 * (size_t)ntot);
    std::vector<std::vector<std::pair<int, double>>> lists(ne);
    for (int r = 0; r < nranks; ++r)
        for (int n = 0; n < na; ++n) {
            const int N = r * na + n;
            out.ref[N] = r * nf + lref[n] - 1;  // global, 0-based
            for (int t = 0; t < 4; ++t) out.c[4 * (size_t)N + t] = lc[4 * (size_t)n + t];
            for (int t = 0; t <= order; ++t) {
                const int e = out.ref[N] + t + order;
                if (e >= 0 && e < ne) lists[e].push_back({N, lc[4 * (size_t)n + t]});
            }
        }
    out.off.assign(ne + 1, 0);
    for (int e = 0; e < ne; ++e) {
        out.off[e + 1] = out.off[e] + (int)lists[e].size();
        for (auto& pr : lists[e]) {
            out.src.push_back(pr.first);
            out.w.push_back(pr.second);
        }
    }
}

int check_other_reaches(int p, double ampl02, double ampl03, int hx, int hy, int hz, std::string& err) {
    // getlinesum(hx,1,im,paspx,ssx) / (hy,...,paspy,ssy): paspx = pasp02 is
    // used without cholaspect (mg_intstate.f90:370-375,427-428).
    const double rmom2_1 = 1.0 / std::sqrt(2.0 * p + 3.0);
    {
        const double exx = ampl02 * rmom2_1;
        const double x = 1.0 / exx;
        const int lo = (int)std::ceil(-x + kEps), hi = (int)std::floor(x - kEps);
        if (lo < -hx || hi > hx || lo < -hy || hi > hy) {
            err = "getlinesum1 on paspx/paspy: reach " + std::to_string(std::max(-lo, hi)) +
                  " exceeds hx/hy";
            return MGBF_ERR_REACH;
        }
    }
    // getlinesum3 on pasp3 = diag(ampl03) after cholaspect3.
    if (ampl03 > 0.0) {
        const double rmom2_3 = 1.0 / std::sqrt(2.0 * p + 5.0);
        const double e = std::sqrt(1.0 / ampl03) * rmom2_3;
        const double z = 1.0 / e;
        const int hi = (int)std::floor(z - kEps);
        if (hi > hz || hi > hy || hi > hx) {
            err = "getlinesum3 on pasp3: reach " + std::to_string(hi) + " exceeds hx/hy/hz";
            return MGBF_ERR_REACH;
        }
    }
    return MGBF_OK;
}

}  // namespace mgbf
