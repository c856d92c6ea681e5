// Internal interface between the host orchestration (mgbf_capi.cpp) and the
// sm_103a kernels (mgbf_kernels.cu, mgbf_hbeta.cu).  Plain C++ types only.
//
// Field views: element (k, i, j) of a generation field lives at
//   p + k + si*i + sj*j        (k, i, j 0-based; k stride is always 1)
// Views produced for a horizontal filter carry an x halo of `hx` mirrored
// columns on each side (columns -hx..-1 and I..I+hx-1 are readable).
#pragma once
#include <cuda.h>

#include <cstdint>

namespace mgbf {

enum class DType : int { F64 = 0, F32 = 1, BF16 = 2 };

struct View {
    void* p = nullptr;
    long long si = 0, sj = 0;
};

// Maximum horizontal reach handled by the kernels and maximum power p of the
// moment kernel.
constexpr int kMaxReach = 32;
constexpr int kMaxMomP = 4;
constexpr int kMaxZReach = 16;  // vertical reach handled by the z kernel

// Polls of an mbarrier before a TMA-fed kernel gives up on a row (the
// copy engine normally delivers a row within a few hundred polls).  The
// drain of a block's own copies after such a failure always uses this
// default, whatever limit the waits ran with.
constexpr int kDefaultWaitPolls = 1 << 20;

struct ZArgs {
    View in, out;
    int nk, I, J;
    int lm, nzk;        // levels per column, number of z-filtered leading entries (nzcol*lm)
    int mz;             // half bandwidth
    const void* band;   // lm x (2mz+1) weights (accumulation type), device
    int mirror_hx;      // write a mirrored x halo of this width (0: none)
};

// 1D line beta of the fast filters along x (dir 0: i, stride si) or y
// (dir 1: j, stride sj) of an interior (nk, I, J) view, half-sample mirror
// at both ends: out = scale * sum_{|d|<=R} w[|d|] in(mirror(t+d)).
constexpr int kMaxLineReach = 64;
struct LineArgs {
    View in, out;
    int nk, I, J;
    int dir;
    int R;
    double w[kMaxLineReach + 1];  // w[0..R], already normalised
    double scale;
    // float copies (made by launch_line): converting FP64 in every thread
    // would load the small FP64 pipe
    float wf[kMaxLineReach + 1];
    float scalef;
};

// Analysis <-> filter grid transfers (mgbf_xfer.cu).
struct XferDirectArgs {
    View in, out;      // in: filter field (interior origin), out: analysis field
    int nk, I, J, nm0, mm0;
    int order;         // 3 lsqr (4 taps), 2 quad, 1 lin
    const int* rx;     // first filter tap per analysis column (0-based, may leave [0, I))
    const int* ry;
    const void* cx;    // 4 weights per analysis column (accumulation type)
    const void* cy;
    int max_strip_rows;  // filter rows needed by 8 consecutive analysis rows (0: unknown)
};
struct XferGatherArgs {
    View in, out;
    int nk, na, nb;    // targets: na x nb points
    int dir;           // 0: list over the first point index (sources along in.si); 1: over the second (in.sj)
    const int* off;    // list offsets per target, size n+1
    const int* src;    // source index per entry
    const void* w;     // weight per entry (accumulation type)
    int out_a0, out_b0;  // output view coordinate = target index - out_*0
};
// anal_to_filt's two gathers in one kernel: per block one filter row b, a
// tile of target columns and a group of levels; the y gather of the tile's
// analysis columns goes to shared memory, the x gather reads it from there.
struct XferFusedArgs {
    View in;             // analysis field (k, c, r)
    View out;            // extended filter array, origin at the first interior point
    int nk;              // levels (multiple of 4)
    int IE, JE;          // targets: IE x JE extended filter points
    int ib;              // output coordinate = target index - ib
    int ta;              // target columns per tile
    int lanes;           // 4-level lanes per level group
    int ncmax;           // analysis columns of the widest tile (shared memory rows)
    const int *offx, *srcx, *offy, *srcy;
    const void *wx, *wy;  // FP32 weights
    const int* tile_c0;  // first analysis column per tile
    const int* tile_nc;  // analysis columns per tile
};
struct XferVertArgs {
    View in, out;
    int nkf, nka, lm, en;  // en blocks of lm filter / 2lm-1 analysis levels
    int adjoint;           // 0: filter -> analysis levels, 1: the transpose
    int na, nb, a0, b0;    // points a0 .. a0+na-1, b0 .. b0+nb-1 (view coordinates)
};

// filtering_rad3's 3D ball (mgbf_rad3.cu) on the ncol*lm leading levels.
struct BallArgs {
    View in, out;
    View prev;          // adjoint, generation 1: the caller's halo to fold (has_prev)
    int ncol, lm, I, J;
    int adjoint, has_prev, hx, hy;
    int ntaps;
    const int4* taps;   // (gx, gy, gz, 0) per tap
    const void* w;      // weight per tap (accumulation type)
    int R, nrows;       // reach; rows of taps along x
    const int2* rows;   // (gy, gz) per row
    const void* rw;     // 2R+1 weights per row (accumulation type)
    double scale;
    float scalef;       // set by launch_ball
};

// One color of filtering_lin2_bckg's line filters (jp_pbfil3.f90:1801-1837
// vdibeta2, 2345-2382 vdibeta2t) on a generation: generator (dx, dy),
// half-span h, symmetric weights fil[0..h].  Forward: boco_2d's mirror fill
// as an index reflection, then the gather on the interior.  Adjoint: the
// scatter from the interior followed by bocoT_2d (fold widths hx, hy), as a
// gather over the target's mirror images.
struct DibArgs {
    View in, out;
    int nk, I, J;
    int dx, dy, h;
    int hx, hy;
    int adjoint;
    double fil[9];
    float filf[9];      // set by launch_dibeta
    double scale;
    float scalef;       // set by launch_dibeta
};

// filtering_lin3's 3D part on one generation (mgbf_lin3.cu).  w, t: work
// arrays W(v, i, j, L) with halos hx, hy, hz, level index fastest,
// element (v, i, j, L) at (L+hz) + (lm+2hz)*(v + nv*((i+hx) + (I+2hx)*(j+hy))).
constexpr int kMaxL3Span = 8;  // dibeta half-span limit (nfil)
enum Lin3Op : int { kL3From = 0, kL3To, kL3DibFwd, kL3DibAdj, kL3FoldX, kL3FoldY, kL3FoldZ, kL3FillY, kL3FillX,
                    kL3ZMirror, kL3HaloZero };
struct Lin3Args {
    View in, out;            // generation buffers (k = v*lm + L, i, j): kL3From reads in, kL3To writes out
    void* w;                 // the array a stage works on
    void* t;                 // dibeta output
    int nv, lm, I, J, hx, hy, hz;
    int gh;                  // 0: generation 1 halo forms (boco_3d_g1, bocoT_3d_g1), 1: coarser
    int dx, dy, dz, h;       // dibeta generator and half-span
    double fil[kMaxL3Span + 1];
    float filf[kMaxL3Span + 1];  // set by launch_lin3
    double scale;            // kL3To: multiplies the output
};

struct RestrictArgs {
    View fine, coarse;
    int nk, If, Jf;     // fine interior sizes; coarse = If/2, Jf/2
    const void* wx;     // Ic x 8 weights for fine columns 2c-3 .. 2c+4
    const void* wy;     // Jc x 8
    int mirror_hx;      // x halo width to mirror into the coarse view
};

// Generation 1's vertical adjoint filter fused with its restriction:
// zout = Bz^T fine (with a mirrored x halo of mirror_z columns), coarse =
// R zout.  band: lm x (2mz+1) adjoint band (accumulation type); levels past
// nzk are copied.
struct ZRestrictArgs {
    RestrictArgs r;      // fine = the caller's field, coarse = generation 2
    View zout;           // generation 1
    int mirror_z;
    const void* band;
    int lm, nzk, mz;
    const void* tmap = nullptr;  // host CUtensorMap of the fine field: levels x If x Jf (box: see zrestrict_box)
    int* status = nullptr;       // device status word: set to 1 when a bounded wait runs out
    int max_polls = kDefaultWaitPolls;
    int write_zout = 1;          // 0 with nzk == 0: restriction only (generation 1 neither filtered nor written)
};

struct ProlongArgs {
    View coarse, base, out;  // out = base + P(coarse); out may equal base
    int nk, If, Jf;          // fine interior sizes
    int ntap;                // 4 (cubic offset stencil) or 3 (quadratic)
    const int* ix;           // If x ntap coarse column indices (reflected)
    const void* wxp;         // If x ntap weights
    const int* iy;           // Jf x ntap
    const void* wyp;         // Jf x ntap
    int has_base;
};

// Fused last prolongation (generation 2 -> 1) and vertical forward filter:
// y = Bz (base + P coarse).  Blocks cover whole z columns.
struct ProlongZArgs {
    ProlongArgs p;      // coarse = generation 2, base = generation 1, out = y
    const void* band;   // lm x (2mz+1) forward band
    int lm, nzk, mz;
    const void* tmap = nullptr;  // host CUtensorMap of the coarse field (box: see prolongz_box), or null
    int* status = nullptr;       // device status word: set to 1 when a bounded wait runs out
    int max_polls = kDefaultWaitPolls;
};

struct HDirectArgs {
    View in, out;
    int nk, I, J;
    int R;                   // reach
    const int* mrow;         // 2R+1 row half-widths (-1: empty row), device
    const void* w;           // (2R+1)^2 weights, device
    int mirror_hx;
    double scale;            // multiplies every output (generation weight)
};

template <typename A>
struct HMomCoefs {
    A coef[(kMaxReach + 1) * (kMaxMomP + 1)];  // coef[gy*(P+1)] = A(gy) = 1 - (e gy)^2
    A upow[(kMaxReach + 1) * (kMaxMomP + 1)];  // upow[m*(P+1)+q] = C(P,q) (-1)^q (e m)^(2q)
};

struct HMomArgs {
    View in, out;
    int nk, I, J;
    int rows;                // output rows per block (<= 0: all rows)
    int mirror_hx;
    int halo;                // x padding of the input view (readable columns -halo..I+halo-1)
    double scale;            // multiplies every output (normalisation s x generation weight)
    const void* tmap;        // host copy of a 3D TMA tensor map of the input buffer, or null
    int* status;             // device status word: set to 1 when a bounded wait runs out
    int variant = 0;         // FP32 kernels: 0 TMA two-row, 1 TMA one-row, 2 cp.async staged,
                             // 3 TMA two rows per barrier filtered one after the other
    int max_polls = kDefaultWaitPolls;  // polls of a row's barrier before the block gives up
    // 1: the input view has no x halo (halo = 0; the TMA map covers columns
    // 0..I-1, I >= R) and edge tiles take the half-sample mirror of their
    // out-of-range columns in shared memory.  Single-row TMA kernel only.
    int mirror_in = 0;
};

constexpr int kHMomVariants = 4;

// Tile columns of the TMA moment kernel for reach R (box = 64 levels x this
// many columns x 1 row); the host encodes tensor maps with this box.
constexpr int hmom_tma_tx(int R) { return R <= 12 ? 2 : 1; }
constexpr int hmom_tma_cols(int R) { return 4 * hmom_tma_tx(R) + 2 * R; }

// Reaches with a compiled moment kernel (p = 2).
#define MGBF_HMOM_REACHES(X) X(4) X(5) X(6) X(8) X(10) X(12) X(16) X(24)
// the same list in two halves, instantiated by separate translation units
#define MGBF_HMOM_REACHES_A(X) X(4) X(5) X(6) X(8)
#define MGBF_HMOM_REACHES_B(X) X(10) X(12) X(16) X(24)

// Columns per thread of the moment kernel for reach R, chosen to keep the
// ring of output rows and the input row segment in registers.
constexpr int hmom_tx_for(int elem_bytes, int R) {
    return elem_bytes == 8 ? (R <= 8 ? 2 : 1) : (R <= 12 ? 4 : 2);
}

struct DotArgs {
    View a, b;
    int nk, I, J;
    double* out;             // device accumulator (one double)
};

// Launchers; return 0 or a cudaError_t value.
int launch_zfilter(DType t, const ZArgs& a, void* stream);
int launch_restrict(DType t, const RestrictArgs& a, void* stream);
// TMA box of the fused generation-1 restriction for a group: lv levels per
// block (0: the fused kernel does not cover the group -- FP64, or z columns
// of lm levels that divide neither 128 nor 96, or a vertical reach mz above
// 8), and the box the tensor map of the fine field must be encoded with:
// `levels` x `cols` x 1 row (the levels padding grows with mz).
struct ZrBox {
    int lv = 0, levels = 0, cols = 0;
};
ZrBox zrestrict_box(DType t, int lm, int nzk, int mz);
// Returns -1 (nothing launched) when the shape does not fit: no box, no
// tensor map or status word, levels not a multiple of 4, unaligned views or
// vertical reach above 8; the caller then runs Bz^T and the restriction apart.
int launch_zrestrict(DType t, const ZRestrictArgs& a, void* stream);
int launch_prolong(DType t, const ProlongArgs& a, void* stream);
// Coarse-field TMA box of the fused last prolongation for a group: lv
// levels per block (0: no TMA form -- FP64, or z columns of lm levels that
// divide neither 128 nor 96) and the staged coarse columns; the tensor map of
// the coarse field is encoded with a box of lv x cols x 1 row.
struct PzBox {
    int lv = 0, cols = 0;
};
PzBox prolongz_box(DType t, int lm, int ntap);
// Returns -1 when the shape is outside the fused kernels' limits (lm > 256 or
// vertical reach > 8); the caller then runs prolongation and z filter apart.
// The TMA-fed kernel runs when a tensor map and status word are given and the
// shape fits it; otherwise the shared-memory kernels.
int launch_prolong_z(DType t, const ProlongZArgs& a, void* stream);
int launch_hdirect(DType t, const HDirectArgs& a, void* stream);
int launch_mirror_x(DType t, View v, int nk, int I, int J, int hx, void* stream);
int launch_copy(DType t, View in, View out, int nk, int I, int J, int mirror_hx, void* stream);
int launch_line(DType t, const LineArgs& a, void* stream);
int launch_ball(DType t, const BallArgs& a, void* stream);
int launch_dibeta(DType t, const DibArgs& a, void* stream);
int launch_lin3(DType t, const Lin3Args& a, int op, void* stream);
int launch_rad3_halo(DType t, View out, View src, int nk, int n3, int I, int J, int hx, int hy, void* stream);
int launch_xfer_direct(DType t, const XferDirectArgs& a, void* stream);
int launch_xfer_gather(DType t, const XferGatherArgs& a, void* stream);
// FP32 / BF16 with 16-byte aligned 4-level vectors; returns -1 (nothing
// launched) when the shape does not fit, so the caller runs the two gathers.
int launch_xfer_a2f_fused(DType t, const XferFusedArgs& a, void* stream);
int launch_xfer_fold(DType t, View v, int nk, int I, int J, int b, void* stream);
int launch_xfer_fill(DType t, View v, int nk, int I, int J, int b, void* stream);
int launch_xfer_vert(DType t, const XferVertArgs& a, void* stream);
int launch_zero_halo_edges(DType t, View v, int nk, int I, int J, int hx, int hy, void* stream);
int launch_zero_halo(DType t, View v, int nk, int I, int J, int hx, int hy, void* stream);
int launch_dot(DType t, const DotArgs& a, void* stream);

// Moment kernel: returns -1 if no instantiation matches (R, p); the caller
// then uses the direct kernel.  coefs are in double; converted internally.
bool hmom_available(DType t, int R, int p);
int launch_hmom(DType t, int R, int p, const HMomArgs& a, const HMomCoefs<double>& c,
                void* stream);

// Persistent radial side: the generations of one variable group in one
// launch of k_hmom_persist (the single-row TMA pipeline, tile after tile).
// Each segment is one generation: its HMomArgs (views, sizes, rows per
// block, scale, mirror, status, poll limit; tmap and variant unused) and,
// filled in by the launcher, its tile grid and first tile.  queue: one int
// of device memory the launcher zeroes before the launch.
constexpr int kMaxPersistSegs = 8;
struct HMomSeg {
    HMomArgs a;
    int nkb = 0, nstrip = 0, nrowb = 0, first = 0;
};
struct HMomPersistArgs {
    HMomSeg seg[kMaxPersistSegs];
    int nseg = 0, ntiles = 0;
    int* queue = nullptr;
    int blocks_per_sm = 0;  // resident blocks per SM the launch asks for (capped by occupancy; <= 0: all that fit)
};
struct HMomMaps {
    CUtensorMap m[kMaxPersistSegs];  // TMA map of each segment's input buffer (box as k_hmom_tma)
};
// Returns -1 (nothing launched) for FP64, reaches without a moment kernel,
// or views the TMA pipeline cannot take; the caller then launches per
// generation.
int launch_hmom_persist(DType t, int R, int p, const HMomPersistArgs& pa, const HMomMaps& maps,
                        const HMomCoefs<double>& c, void* stream);

}  // namespace mgbf
