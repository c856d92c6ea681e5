// FP64 host-side setup of the MGBF filter tables.
//
// Restates the reference's setup arithmetic (all FP64, as in the reference):
//   rmom2_k            mg_parameter.f90:567-572
//   cholaspect1/2      jp_pbfil.f90:74-107 (diagonal aspect tensors)
//   paspx / paspy      mg_intstate.f90:370-375, 427-428 (no cholaspect)
//   getlinesum1/2      jp_pbfil.f90:149-218 (support and normalisation)
//   vrbeta1/2 weights  jp_pbfil.f90:856-928 (frow = s*(1-rr)^p)
//   def_offset_coef    mg_interpolate.f90:61-86
// and turns them into the tables the kernels consume: banded z matrices
// (with the whole-sample mirror and edge fold folded in), the radial
// support table, dense radial weights, moment coefficients, and
// restriction/prolongation index/weight rows with the half-sample mirror
// folded in.
#pragma once
#include <string>
#include <vector>

#include "mgbf_kernels.cuh"

namespace mgbf {

constexpr double kEps = 1.e-12;  // jp_pbfil.f90: eps in getlinesum / rbeta

struct HStencil {
    int p = 2;
    double exx = 0, eyy = 0, s = 0;
    int R = 0;                  // reach: max |gx|, |gy| in the support
    std::vector<int> mrow;      // 2R+1 row half-widths (-1: empty row)
    std::vector<double> w;      // (2R+1)^2 dense weights (zero outside)
    bool canonical = false;     // support == disk of radius R + 1/2
    HMomCoefs<double> mom{};    // moment coefficients (valid if canonical)
};

// The fast filters' (procs 3 and 8) 1D horizontal line beta: vrbeta1 along
// x and y with paspx = paspy = pasp02 taken WITHOUT cholaspect
// (mg_intstate.f90:370-375), so exx = mg_ampl02 * rmom2_1.
struct LStencil {
    int p = 2;
    double exx = 0, s = 0;
    int R = 0;                  // reach: taps -R..R
    std::vector<double> w;      // R+1 normalised weights s*(1-(g exx)^2)^p, g = 0..R
};

// filtering_lin2_bckg's three line filters ("colors"), as init_mg_line sets
// them up (mg_intstate.f90:436-480; jp_pbfil3.f90:378-457, 573-624,
// 1399-1501): the triad decomposition of the Cholesky factor of the inverse
// aspect, (c, c, 0) with c = 1/sqrt(mg_ampl02), into integer generators
// (dx, dy) and spreads^2; each spread^2 -> formal half-span hs between two
// integer beta filters -> the dibeta weights fil[0..h].
constexpr int kDibNH = 6;             // moment-table size nh (mg_parameter.f90:562)
constexpr int kDibNFil = kDibNH + 2;  // nfil (mg_parameter.f90:563)
struct DStencil {
    bool ok = false;
    int dx[3] = {0, 0, 0}, dy[3] = {0, 0, 0}, h[3] = {0, 0, 0};
    double hs[3] = {0, 0, 0};
    double fil[3][kDibNFil + 1] = {};
};

// filtering_lin3's 3D line filters (procedure 5) as init_mg_line sets them
// up (mg_intstate.f90:465-477; jp_pbfil3.f90:657-934): the hexad
// decomposition of the Cholesky factor of the inverse 3D aspect, (c3, c3, c3,
// 0, 0, 0) with c3 = 1/sqrt(mg_ampl03), into seven colors; per color the
// active slot (or -1: the color copies), and per slot the generator
// (dx, dy, dz), half-span h and dibeta weights fil[0..h].
struct XStencil {
    bool ok = false;
    int slot[8] = {-1, -1, -1, -1, -1, -1, -1, -1};  // by color 1..7 (index 0 unused)
    int g[6][3] = {};
    int h[6] = {};
    double hs[6] = {};
    double fil[6][kDibNFil + 1] = {};
};

// filtering_rad3's 3D ball: vrbeta3 (jp_pbfil.f90:930-977) with el from
// cholaspect3 of pasp3 = diag(mg_ampl03) (jp_pbfil.f90:109-126), normalised
// by getlinesum3 (jp_pbfil.f90:220-268); taps in the reference's gz, gy, gx
// loop order.
struct BStencil {
    int R = -1;                 // reach in every direction (-1: none)
    double e = 0, s = 0;
    std::vector<int> taps;      // (gx, gy, gz, 0) per tap
    std::vector<double> w;      // normalised weight per tap
    // the same taps grouped in rows along x: (gy, gz) per row, in tap order,
    // and 2R+1 weights per row for gx = -R..R (zero where the ball has no tap)
    std::vector<int> rows;
    std::vector<double> rw;
};

struct ZStencil {
    int lm = 0, mz = 0;
    double exx = 0, s = 0;
    std::vector<double> wz;     // 2mz+1 tap weights
    std::vector<double> fwd;    // lm x (2mz+1) band of Bz
    std::vector<double> adj;    // lm x (2mz+1) band of Bz^T
    // M = Bz Bz^T (symmetric, half-width mmz = min(2mz, lm-1)), lm x (2mmz+1):
    // the whole vertical filtering of a column when it is applied in one pass
    int mmz = 0;
    std::vector<double> mm;
};

struct Interp1D {
    int nf = 0, nc = 0, ntap = 4;
    std::vector<double> rw;     // nc x 8 restriction weights, fine f = 2c-3+a
    std::vector<int> pidx;      // nf x ntap coarse indices (mirrored)
    std::vector<double> pw;     // nf x ntap prolongation weights
};

// One axis of the analysis <-> filter transfer, global over nranks ranks:
// per analysis point the first filter tap (global, 0-based; may lie in the
// mirror halo) and 4 weights (order+1 used).  lsqr_mg_coef
// (mg_interpolate.f90:89-298) on each rank's local grid, lengthx = na
// (mg_parameter.f90:515-541).
struct XferAxis {
    int order = 3;
    std::vector<int> ref;     // na * nranks
    std::vector<double> c;    // 4 per point
    // adjoint lists over the extended filter index e = ref + t + order,
    // e in [0, nf*nranks + 2*order): offsets, source analysis index, weight
    std::vector<int> off, src;
    std::vector<double> w;
};
void build_xfer_axis(int na, int nf, int nranks, int order, XferAxis& out);

// Returns 0 or an MGBF_ERR_* code with a message in err.
int build_hstencil(int p, double ampl02, int hx, int hy, HStencil& out, std::string& err);
int build_zstencil(int p, double ampl01, int hz, int lm, bool need_mirror, ZStencil& out,
                   std::string& err);
int build_interp(int nf, bool quart, Interp1D& out, std::string& err);
int build_lstencil(int p, double ampl02, int hx, int hy, LStencil& out, std::string& err);
int build_dstencil(int p, double ampl02, int hx, int hy, DStencil& out, std::string& err);
int build_bstencil(int p, double ampl03, int hx, int hy, int hz, BStencil& out, std::string& err);
// line = mgbf_line: without it init_mg_line never runs and every color copies.
int build_xstencil(int p, double ampl03, int hx, int hy, int hz, bool line, XStencil& out, std::string& err);

// Reach checks def_mg_weights performs for the other filters of the
// reference (getlinesum on paspx/paspy, mg_intstate.f90:427-428, which skip
// cholaspect; getlinesum3 on pasp3, mg_intstate.f90:431).
int check_other_reaches(int p, double ampl02, double ampl03, int hx, int hy, int hz,
                        std::string& err);

// Canonical row half-width of a disk of radius R + 1/2.
int canonical_width(int R, int gy);

// Sets the calling thread's mgbf_last_error() message (no heap use) and
// returns code.
int report_error(int code, const char* msg);

}  // namespace mgbf
