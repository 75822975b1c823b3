// Host-side scan geometry for the distance-driven operators.
//
// A plan is built once per options vector (and dtype) and holds, per view:
//   * the branch (image rows are the integration lines when |cos| dominates,
//     columns otherwise) and the detector-order flip, decided exactly as the
//     reference does (src/fan_ed_kernel.cu:61-77);
//   * the D+1 detector-cell boundaries projected onto the view's axis
//     (x-axis for row lines, y-axis for column lines), evaluated in fp64 with
//     the reference's formulas (src/fan_ed_kernel.cu:78-95,
//     src/fan_ea_kernel.cu:72-84, src/para_kernel.cu:52-60), in increasing
//     order, plus the cell widths (fp64 differences);
//   * per-detector normalisation factors;
//   * an approximate inverse of the boundary map (axis coordinate -> fractional
//     cell index) used to seed the cell search in the image-side gather;
// and per (view, line) the affine map from pixel-edge index k to the axis,
// axis = alpha + sigma * k, evaluated in fp64 from the rounded source position.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace ctgb {

enum Scan { kFanED = 0, kFanEA = 1, kPara = 2 };

struct HostGeom {
  int V = 0, D = 0, W = 0, H = 0, L = 0, scan = 0, dtype = 0;
  // option values after rounding to the data type
  double views = 0, dets = 0, width = 0, height = 0, dImg = 0, dDet = 0, Ang0 = 0, dAng = 0, s2r = 0,
         d2r = 0, binshift = 0;
  std::vector<int32_t> flags;  // V: bit0 row lines (x-branch), bit1 flipped detector order
  std::vector<double> src;     // V*2: source x, y (fan)
  std::vector<double> db;      // V*(D+1): cell boundaries on the axis, increasing
  std::vector<double> wd;      // V*D: cell widths db[d+1]-db[d]
  std::vector<double> fq;      // V*D: A / A^T factor (fan dImg/(cbar*w), para dImg/dDet)
  std::vector<double> fbt;     // V*D: extra B^T factor (EA: dImg/cbar), 1 otherwise
  std::vector<double> lp;      // V*L*2: alpha, sigma (pixel edge k of a line maps to alpha + sigma*k)
  std::vector<double> inv;     // V*5: guess u = x*P0/(P1+x*P2) (atan for EA), cell = P3+P4*u
  std::vector<double> wpre;    // D: fbp detector pre-weight, applied as (y * wpre[k]) * wscale
  double wscale = 1.0;
  std::vector<double> taps;    // 2D-1: RL ramp taps (src/fan_ed_kernel.cu:926-943)
  std::vector<double> taps_lo; // 2D-1: fp64 tap minus the stored one (fp32 plans), else 0
  double dfilt = 0.0;          // tap spacing of the ramp filter (virtual bin, or dDet)
  std::vector<double> options; // the options vector the geometry was built from
  double x0 = 0, y0 = 0;       // left image edge x, bottom image edge y
};

// Parse the reference's options vector and build the geometry. dtype 0 = fp32,
// 1 = fp64. Returns false and sets `err` on invalid options.
bool build_geometry(const double* options, int n_options, int dtype, HostGeom& g, std::string& err);

// fbp filter windows: the reference's Ram-Lak (RL) kernel, Shepp-Logan, and RL
// under a Hann window (its exact discrete form, [1/4, 1/2, 1/4] * RL).
enum FilterWindow { kRamLak = 0, kSheppLogan = 1, kHann = 2 };

// Ramp filter taps (2D-1, offsets -(D-1)..D-1) of `window` into g.taps /
// g.taps_lo, for the plan's dtype. ea_exact (equal-angle fans only) multiplies
// each tap by (n dDet / sin(n dDet))^2, the factor that makes the RL kernel
// exact on equiangular samples. RamLak without ea_exact reproduces the
// reference's taps; the others have no counterpart in it.
bool filter_taps(HostGeom& g, int window, bool ea_exact, std::string& err);

}  // namespace ctgb
