// Learned orbit surrogate: network layout, normalisation and kernel entry points.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>

#include "bhr.h"

#include "kernels.cuh"
#include "march.cuh"

namespace bhr {
namespace surr {

constexpr int kH = 64;     // hidden width
constexpr int kIn = 3;     // (log r_cam, transform of b / sqrt(27), orbit coordinate sigma)
constexpr int kOut = 2;    // (scaled polar-angle residual, capture logit)
constexpr int kLd = 72;    // bf16 row stride of weight / activation tiles in shared memory

// Flat FP32 parameter block (master weights); W[o][i] row-major.
constexpr int kW1 = 0;               // [64][3]
constexpr int kB1 = kW1 + kH * kIn;  // [64]
constexpr int kW2 = kB1 + kH;        // [64][64]
constexpr int kB2 = kW2 + kH * kH;   // [64]
constexpr int kW3 = kB2 + kH;        // [64][64]
constexpr int kB3 = kW3 + kH * kH;   // [64]
constexpr int kW4 = kB3 + kH;        // [2][64]
constexpr int kB4 = kW4 + kOut * kH; // [2]
constexpr int kNParams = kB4 + kOut; // 8706
// training gradients: each warp adds its tile's gradients into copy (warp % kGradCopies) of the
// buffer, which spreads the global atomics over as many addresses; Adam sums the copies and
// zeroes them for the next step
constexpr int kGradCopies = 32;

// Input normalisation and the trained range (stored with the weights).
struct Norm {
    float rc_lo, rc_hi;   // trained camera radii
    float b_max;          // trained impact parameters [0, b_max]
    float t_eps;          // b transform: t = sign(beta) ln(1 + |beta| / t_eps)
    float t_scale;        // x2 = t * t_scale
    float y_scale;        // polar-angle residual = y * y_scale
    float band;           // |b - sqrt(27)| below this falls back to the integrator
    float ue;             // exit u of the training orbits (1 / escape radius)
};

struct TrainSample {      // one training sample (16 bytes) + label
    float x1, x2, sigma, y;
};

// label: 0 escaped (y valid), 1 captured, 2 unusable (budget)
cudaError_t launch_orbit_data(uint64_t seed, int64_t n_orbits, int k_per_orbit, const Norm& nrm, double step_frac,
                              TrainSample* X, int8_t* lab, unsigned long long* stats, int grid, cudaStream_t st);
cudaError_t launch_train_step(const float* params, const TrainSample* X, const int8_t* lab, int64_t n_samples,
                              const int64_t* idx, int batch, uint64_t seed, float w_u, float w_c, float* grads,
                              float* loss, int grid, cudaStream_t st);
cudaError_t launch_adam(float* params, float* grads, float* m, float* v, int step, float lr, float beta1,
                        float beta2, float eps, cudaStream_t st);
// wait_cycles <= 0: the default completion-wait limit; withhold: the timeout self-test
cudaError_t launch_mlp_infer(const float* params, const float4* q, float2* out, int n, int* status, int grid,
                             cudaStream_t st, long long wait_cycles = 0, bool withhold = false);

// The exit query of a ray, (x1, x2, sigma at the exit) for an escaping orbit and (x1, x2, 1) for a
// captured one, depends on the view (x1) and on x2 alone: per view it is tabulated on
// kExitTableN points of x2 for each half (0: captured, beta < 0; 1: escaping) and read back by
// linear interpolation. Entry i of a half holds points i and i + 1 (one 16-byte load).
constexpr int kExitTableN = 2048;
// A view's exit table, in float4 entries (N = kExitTableN points per half):
//   [0, N)          captured half: entry i = (y, capture logit) of points i and i + 1
//   escaping half, over the points x2_i = tab_lo[1] + i tab_h[1]:
//   kExitPsi  + j   the escape direction's angle in the orbital plane (from e1 = the camera
//                   direction towards e2) minus pi at points j .. j + 3 (cubic interpolation)
//   kExitPhi0 + j   the angle from the camera to the exit, points j .. j + 3
//   kExitIc   + j   the angle from the camera to the turning point, points j .. j + 3
//   kExitRange + m  the disk's angle range from the turning point (Ilo, Ihi) of points m, m + 1
//   kExitU2   + m   (u2_m, u2_{m+1}, logit_m, logit_{m+1}): the turning point and capture logit
//   kExitPsiB, kExitPhi0B   the tolerance escape's second regime (below)
// The tolerance escape of the SHADER and CPU rules exits at u_e = min(1 / rEscMin, u_tol(b)); the
// two branches meet with a kink at b = b_kink, which cubic interpolation would smear. So psi and
// phi0 are tabulated for each branch over the whole range (kExitPsi / kExitPhi0: the exit at
// rEscMin, kExitPsiB / kExitPhi0B: at u_tol(b)), and a ray reads the branch its b lies on.
constexpr int kExitPsi = kExitTableN, kExitPhi0 = 2 * kExitTableN, kExitIc = 3 * kExitTableN;
constexpr int kExitRange = 4 * kExitTableN, kExitU2 = 5 * kExitTableN;
constexpr int kExitPsiB = 6 * kExitTableN, kExitPhi0B = 7 * kExitTableN;
constexpr int kExitTabEntries = 8 * kExitTableN;
// Rays this many table spacings below the x2 of the camera's tangential ray (b = r_cam /
// sqrt(1 - 2 / r_cam), whose turning point is the camera) go to the fallback march: the angle to
// the turning point has a square-root end there, which the cubic interpolation does not follow.
constexpr float kTangentMargin = 10.0f;
// The crossing query of an escaping orbit, (x1, x2, sigma_k), is a function of (x2, sigma) per
// view: tabulated on kCrossNx points of x2 (the escaping half's range) by kCrossNs of sigma in
// [-1, 1], read by bilinear interpolation. Cell (i, j) holds its four corners (one 16-byte load).
constexpr int kCrossNx = 256, kCrossNs = 64;
constexpr int kCrossCells = (kCrossNx - 1) * (kCrossNs - 1);

// View constants in double for the impact parameter near the photon sphere (the direction of a
// pixel and its angle from the hole, as the FP32 setup computes them, in FP64)
struct Fp64Cam {
    double inv_w2, inv_h2;  // 2 / width, 2 / height
    double aspect_d;        // width / height
    double rhat_d[3];       // camera direction from the float camera position
    double b_scale_d;       // r_cam / sqrt(1 - 2 / r_cam)
};
struct SurrView {
    DevView view;
    Rule rule;
    Norm norm;
    float x1;  // network input 1 of this view (scaled log r_cam)
    float uc;  // 1 / r_cam
    float u_esc_min;  // 1 / rEscMin of the tolerance escape (SHADER and CPU rules)
    float b_kink;     // tolerance escape: b where the exit moves from rEscMin to u_tol(b)
    float x2_lim;     // x2 above which rays fall back (kTangentMargin spacings below the tangential ray)
    const float4* exit_table;  // the view's exit table (kExitTabEntries float4, layout above)
    float tab_lo[2], tab_h[2], tab_inv_h[2];  // x2 of a half's first point, spacing, 1 / spacing
    const float4* cross_table;  // [kCrossCells] y at the cell's corners (i, j), (i, j+1), (i+1, j), (i+1, j+1)
    float cx_h, cx_inv_h;       // the cross table's x2 spacing (first point tab_lo[1]) and its inverse
    float b_scale;          // r_cam / sqrt(1 - 2 / r_cam): b = b_scale sin(angle from the radial direction)
    // the pixel direction of blackhole.frag:68-72 before its normalisation, an affine function
    // of the pixel: (i - i_mid) dir_i + (j - j_mid) dir_j + dir_0 (from the image's centre, so
    // that the terms stay near unit size)
    float dir_i[3], dir_j[3], dir_0[3];
    int32_t i_mid, j_mid;
    Fp64Cam fc;             // the FP64 impact parameter near the photon sphere
    // the rays of the view's photon-sphere band that the band march takes (bit ray % 32 of word
    // ray / 32; they are skipped here), or nullptr when no band march runs
    const uint32_t* band_mask;
};
// The band march: the rays of the fallback band (|b - sqrt 27| < band) found before the pass by
// k_band_list and marched by the integrator beside it. Per view a list of at most kBandCap rays;
// rays beyond it go the fallback list's way.
constexpr int kBandCap = 1 << 15;
// The row search's constants of a view (rhat the camera direction; R, U, B the camera basis'
// columns), in float: the rows' quadratics lose nothing that two pixels of margin do not cover.
struct BandRows {
    float c_out, c_in;      // cos^2 of the angles from the hole at b_hi and b_lo (b range with margin)
    float a, rhU, rhB;      // rhat . R, rhat . U, rhat . B
    float RR, RU, RB;       // R . R, R . U, R . B
    float UU, UB, BB;       // U . U, U . B, B . B
};
struct BandView {
    DevView view;
    Fp64Cam fc;
    BandRows q;
    uint32_t* mask;   // the view's band mask (ceil(rays / 32) words, zeroed before the launch)
    int* list;        // the view's band list (kBandCap rays)
    int32_t row0;     // first row of this view in the launch's row numbering
    int32_t rows;     // rows searched (0: the view's band is not searched, see bhr::surr::band_rows)
};
struct BandBatch {
    int32_t nviews, total_rows;
    Rule rule;
    float band;       // the fallback band |b - sqrt 27| < band
    WorkQueue* qb;    // qb[2 v].fb_count: rays in view v's band list
    BandView v[kMaxViews];
};
// The learned surrogate's tables of up to kTabMaxViews views, built by one launch on the tensor
// cores (surrogate.cu k_tables): per view its exit table (escaping half: one tile of 128 points
// per branch of the rule's exit; captured half) and crossing table, 128-row tiles of network
// queries, each tile through the tcgen05 network (tc_mlp.cuh mlp_tile_l1f).
constexpr int kTabMaxViews = 64;
struct TabView {
    float x1, uc, u_esc_min, esc_tol, b_kink, two_over_r3, disk_inner, disk_outer;
    int32_t tol;    // the tolerance escape (SHADER and CPU rules): two exit branches
    int32_t tile0;  // the view's first tile in the launch
    float4* exit_table;
    float4* cross_table;
};
struct TabBatch {
    int32_t nviews, ntiles;
    Norm norm;
    float tab_lo[2], tab_h[2], cx_h;
    TabView v[kTabMaxViews];
};
// tiles of one view: kExitTableN / 128 per exit branch, kExitTableN / 128 captured, the crossing cells' rows
constexpr int kTabTilesExit = kExitTableN / 128, kTabTilesCross = kCrossNx * kCrossNs / 128;
inline int tab_tiles(bool tol) { return kTabTilesExit * (tol ? 3 : 2) + kTabTilesCross; }
// Builds the batch's tables; *status becomes 1 if a tensor-core completion wait ran out (the
// tables are then NaN where it did).
cudaError_t launch_tables(const TabBatch& b, const float* params, int* status, int grid, cudaStream_t st);
// Resident blocks per SM of the surrogate pass (its grid: SMs x this), per variant as measured:
// the learned pass 2% faster with four than with three, the closed-form pass 5% slower.
constexpr int surr_blocks_per_sm(bool net) { return net ? 4 : 3; }
// The surrogate pass of one view (net: the learned variant, which reads the crossing table;
// otherwise the converged closed form).
cudaError_t launch_surrogate_trace(const SurrView& sv, WorkQueue* q, int* fb_list, int grid, bool net,
                                   cudaStream_t st);
// Finds every view's band rays (search rows from bhr::surr::band_rows) into their band lists and
// masks: one warp per searched row.
cudaError_t launch_band_list(const BandBatch& b, cudaStream_t st);
// The row search of a view's band: the b range [b_lo, b_hi] as cos^2 of the angle from the hole
// (c_out at b_hi, c_in at b_lo) and the rows' quadratic coefficients, and whether the view's
// pixel rows cut that cone in bounded intervals (the hole within 85 degrees of the view axis less
// the cone's angle). Views that fail it have no band march: their band rays take the fallback list.
bool band_rows(const bhr_view& v, const Fp64Cam& fc, double b_lo, double b_hi, BandRows* q);
// Fills the view's exit table for the non-learned variant (the converged closed form, no network).
cudaError_t launch_exit_table_cf(const SurrView& sv, float4* table, cudaStream_t st);
// x2 ranges of the two halves: captured beta in [-1, -band / sqrt 27], escaping in
// [band / sqrt 27, b_max / sqrt 27 - 1].
inline void exit_table_range(const Norm& nm, float lo[2], float h[2]) {
    const double s27 = 5.196152422706632;
    auto x2 = [&](double beta) {
        return (beta < 0 ? -1.0 : 1.0) * std::log1p(std::fabs(beta) / double(nm.t_eps)) * double(nm.t_scale);
    };
    const double b0 = double(nm.band) / s27;
    const double ends[2][2] = {{x2(-1.0), x2(-b0)}, {x2(b0), x2(double(nm.b_max) / s27 - 1.0)}};
    for (int s = 0; s < 2; ++s) {
        lo[s] = float(ends[s][0]);
        h[s] = float((ends[s][1] - ends[s][0]) / double(kExitTableN - 1));
    }
}
int train_smem_bytes();
// Whether the surrogate with normalisation nm answers view v (otherwise *why says what is missing):
// lensed rays (no far mode), the thin disk or none, and the CONFIG rule at the trained exit
// radius, or the SHADER or CPU rule's tolerance escape.
bool supports_view(const Norm& nm, const bhr_view& v, std::string* why);
// The surrogate's normalisation and device (for the context that serves BHR_METHOD_SURROGATE).
Norm norm_of(const bhr_surrogate* s);
int device_of(const bhr_surrogate* s);

}  // namespace surr
}  // namespace bhr
