// Host-side scan geometry (see geometry.h). The view angle is formed in the
// data type exactly as the reference forms it (src/fan_ed_kernel.cu:61), so the
// branch and flip decisions are the reference's; everything continuous after
// that (source position, boundaries, widths, line maps, normalisation) is
// evaluated in fp64, which makes the tables the FP64 evaluation of the
// reference's formulas. The kernels consume them as (hi, lo) pairs.
#include "geometry.h"

#include <cmath>
#include <limits>

namespace ctgb {

namespace {

template <class T> inline T map_x(T sx, T sy, T dx, T dy) { return (sx * dy - sy * dx) / (dy - sy); }
template <class T> inline T map_y(T sx, T sy, T dx, T dy) { return (sy * dx - sx * dy) / (dx - sx); }

template <class T>
bool build(const double* o, int n, HostGeom& g, std::string& err) {
  if (n < 9) { err = "options vector needs at least 9 entries"; return false; }
  const double st = o[n - 1];
  if (!(st == 0.0 || st == 1.0 || st == 2.0)) { err = "scan_type (last option) must be 0, 1 or 2"; return false; }
  g.scan = (int)st;
  if (g.scan != kPara && n < 12) { err = "fan-beam options vector needs 12 entries"; return false; }
  for (int i = 0; i < 4; ++i) {
    if (!(o[i] >= 1.0) || o[i] != std::floor(o[i]) || o[i] > 65536.0) {
      err = "views, dets, width and height must be positive integers";
      return false;
    }
  }
  const T views = (T)o[0], dets = (T)o[1], width = (T)o[2], height = (T)o[3];
  const T dImg = (T)o[4], dDet = (T)o[5], Ang0 = (T)o[6], dAng = (T)o[7];
  T s2r = 0, d2r = 0, binshift;
  if (g.scan == kPara) {
    binshift = (T)o[8];
  } else {
    s2r = (T)o[8]; d2r = (T)o[9]; binshift = (T)o[10];
  }
  if (!(dImg > 0) || !(dDet > 0)) { err = "dImg and dDet must be positive"; return false; }
  if (g.scan != kPara && !(s2r > 0 && s2r + d2r > 0)) { err = "s2r must be positive"; return false; }
  g.V = (int)o[0]; g.D = (int)o[1]; g.W = (int)o[2]; g.H = (int)o[3];
  g.L = g.H > g.W ? g.H : g.W;
  g.views = views; g.dets = dets; g.width = width; g.height = height; g.dImg = dImg; g.dDet = dDet;
  g.Ang0 = Ang0; g.dAng = dAng; g.s2r = s2r; g.d2r = d2r; g.binshift = binshift;
  const int V = g.V, D = g.D, L = g.L;
  g.flags.assign(V, 0);
  g.src.assign((size_t)V * 2, 0.0);
  g.db.assign((size_t)V * (D + 1), 0.0);
  g.wd.assign((size_t)V * D, 0.0);
  g.fq.assign((size_t)V * D, 0.0);
  g.fbt.assign((size_t)V * D, 1.0);
  g.lp.assign((size_t)V * L * 2, 0.0);
  g.inv.assign((size_t)V * 5, 0.0);

  const double PI = std::acos(-1.0);
  const double x0 = -(double)width / 2 * (double)dImg;   // left image edge (src/fan_ed_kernel.cu:107)
  const double y0 = -(double)height / 2 * (double)dImg;  // bottom image edge (src/fan_ed_kernel.cu:196)
  g.x0 = x0; g.y0 = y0;
  // virtual detector pitch / shift (src/fan_ed_kernel.cu:68-69)
  const double virdDet = (double)s2r / ((double)s2r + (double)d2r) * (double)dDet;
  const double virshift = (double)s2r / ((double)s2r + (double)d2r) * (double)binshift;
  const double R = (double)s2r;
  double max_half_x = std::fabs(x0), max_half_y = std::fabs(y0);

  std::vector<double> cosb(D + 1);
  for (int v = 0; v < V; ++v) {
    // idxview * dAng + Ang0 in the data type (src/fan_ed_kernel.cu:61); nvcc's
    // default FMA contraction makes it one fused multiply-add
    const double ang = (double)std::fma((T)v, dAng, Ang0);
    const bool xb = std::fabs(ang - std::round(ang / PI) * PI) * 4 / PI <= 1;
    const double e2 = (ang - std::floor(ang / 2 / PI) * 2 * PI) * 4 / PI;
    const bool flip = e2 >= 3 && e2 < 7;
    const double c = std::cos(ang), s = std::sin(ang);
    g.flags[v] = (xb ? 1 : 0) | (flip ? 2 : 0);
    const double sx = -s * (double)s2r, sy = c * (double)s2r;
    g.src[2 * v] = sx; g.src[2 * v + 1] = sy;
    if (g.scan != kPara) {
      // the source must stay outside the image along the integration lines
      if ((xb && std::fabs(sy) <= max_half_y) || (!xb && std::fabs(sx) <= max_half_x)) {
        err = "source lies inside the image field of view";
        return false;
      }
    }
    const double e = flip ? -1.0 : 1.0;
    double* dbv = &g.db[(size_t)v * (D + 1)];
    for (int b = 0; b <= D; ++b) {
      const double tb = flip ? ((double)dets / 2 - b) : (b - (double)dets / 2);
      double val;
      if (g.scan == kFanED) {
        const double sdet = tb * virdDet + virshift;
        const double detx = sdet * c, dety = sdet * s;
        val = xb ? map_x(sx, sy, detx, dety) : map_y(sx, sy, detx, dety);
      } else if (g.scan == kFanEA) {
        const double beta = tb * (double)dDet + (double)binshift + ang;
        val = xb ? sx + std::sin(beta) / std::cos(beta) * sy : sy + std::cos(beta) / std::sin(beta) * sx;
      } else {
        val = (tb * (double)dDet + (double)binshift) / (xb ? c : s);
      }
      dbv[b] = val;
    }
    for (int b = 0; b < D; ++b) {
      if (!(dbv[b + 1] > dbv[b])) {
        err = "detector boundaries are not strictly increasing on the projection axis";
        return false;
      }
      g.wd[(size_t)v * D + b] = dbv[b + 1] - dbv[b];
    }
    if (g.scan != kPara) {
      for (int b = 0; b <= D; ++b) {
        const double u = dbv[b];
        cosb[b] = xb ? std::fabs(sy) / std::sqrt((u - sx) * (u - sx) + sy * sy)
                     : std::fabs(sx) / std::sqrt((u - sy) * (u - sy) + sx * sx);
      }
      for (int d = 0; d < D; ++d) {
        const double cbar = (cosb[d + 1] + cosb[d]) / 2;
        g.fq[(size_t)v * D + d] = (double)dImg / (cbar * g.wd[(size_t)v * D + d]);
        if (g.scan == kFanEA) g.fbt[(size_t)v * D + d] = (double)dImg / cbar;
      }
    } else {
      for (int d = 0; d < D; ++d) g.fq[(size_t)v * D + d] = (double)dImg / (double)dDet;
    }
    // per-line affine pixel-edge maps
    const int nl = xb ? g.H : g.W;
    for (int l = 0; l < nl; ++l) {
      double alpha, sigma;
      if (xb) {
        const double i0y = ((double)height / 2 - l - 0.5) * (double)dImg;
        if (g.scan != kPara) {
          const double den = i0y - sy;
          alpha = (sx * i0y - sy * (double)x0) / den;
          sigma = -sy * (double)dImg / den;
        } else {
          alpha = s / c * i0y + (double)x0;
          sigma = (double)dImg;
        }
      } else {
        const double i0x = (l - (double)width / 2 + 0.5) * (double)dImg;
        if (g.scan != kPara) {
          const double den = i0x - sx;
          alpha = (sy * i0x - sx * (double)y0) / den;
          sigma = -sx * (double)dImg / den;
        } else {
          alpha = (double)y0 + c / s * i0x;
          sigma = (double)dImg;
        }
      }
      if (!(sigma > 0)) { err = "degenerate pixel projection (source inside the image?)"; return false; }
      double* q = &g.lp[((size_t)v * L + l) * 2];
      q[0] = alpha; q[1] = sigma;
    }
    // inverse boundary map seed
    double* P = &g.inv[(size_t)v * 5];
    if (g.scan == kPara) {
      P[0] = xb ? c : s; P[1] = 1.0; P[2] = 0.0;
      P[3] = D / 2.0 - e * (double)binshift / (double)dDet;
      P[4] = e / (double)dDet;
    } else {
      P[0] = xb ? c : s; P[1] = R; P[2] = xb ? s : -c;
      if (g.scan == kFanED) {
        P[3] = D / 2.0 - e * virshift / virdDet;
        P[4] = e * R / virdDet;
      } else {
        P[3] = D / 2.0 - e * (double)binshift / (double)dDet;
        P[4] = e / (double)dDet;
      }
    }
  }

  // FBP detector pre-weight and ramp taps (src/fan_ed_kernel.cu:1349-1366,
  // src/fan_ea_kernel.cu:1075-1090, src/para_kernel.cu:823-833)
  g.wpre.assign(D, 1.0);
  T dfilt = dDet;
  if (g.scan == kFanED) {
    const T vd = dDet * s2r / (s2r + d2r);
    for (int k = 0; k < D; ++k) {
      T t = (-dets / 2 + (T)0.5) + (T)k;
      T r = t * vd;
      r = r * r;
      g.wpre[k] = (double)(s2r / std::sqrt(s2r * s2r + r));
    }
    dfilt = vd;
    g.wscale = (double)vd;
  } else if (g.scan == kFanEA) {
    for (int k = 0; k < D; ++k) {
      T t = (-dets / 2 + (T)0.5) + (T)k;
      T r = std::cos(t * dDet);
      g.wpre[k] = (double)(r * s2r * dDet);
    }
  } else {
    for (int k = 0; k < D; ++k) g.wpre[k] = (double)dDet;
  }
  // The taps are the reference's values in T. In fp32 the filter also applies
  // the remainder to the fp64 taps: the RL kernel's response nearly cancels on
  // smooth rows, so the fp32 rounding of the taps alone moves an equal-angle
  // reconstruction by ~1e-5 relative.
  g.dfilt = (double)dfilt;
  g.taps.assign(2 * D - 1, 0.0);
  g.taps_lo.assign(2 * D - 1, 0.0);
  const double df = (double)dfilt;
  for (int j = 0; j < 2 * D - 1; ++j) {
    const int x = j - D + 1;
    double exact = 0.0;
    if (std::abs(x) % 2 == 1) {
      exact = -1 / (PI * PI * x * x * df * df);
      g.taps[j] = (double)(T)exact;
    } else if (x == 0) {
      exact = 1 / (4 * df * df);
      g.taps[j] = (double)(T)(1 / (4 * dfilt * dfilt));
    }
    if (sizeof(T) == 4) g.taps_lo[j] = exact - g.taps[j];
  }
  return true;
}

}  // namespace

// RL kernel value at integer offset x for tap spacing d (src/fan_ed_kernel.cu:926-943)
static double rl_tap(long x, double d) {
  const double PI = std::acos(-1.0);
  if (x == 0) return 1 / (4 * d * d);
  if (std::labs(x) % 2 == 1) return -1 / (PI * PI * (double)x * (double)x * d * d);
  return 0.0;
}

bool filter_taps(HostGeom& g, int window, bool ea_exact, std::string& err) {
  if (window < kRamLak || window > kHann) {
    err = "filter window must be 0 (Ram-Lak), 1 (Shepp-Logan) or 2 (Hann)";
    return false;
  }
  if (ea_exact && g.scan != kFanEA) {
    err = "the exact equal-angle kernel applies to equal-angle fan beams (scan_type 1) only";
    return false;
  }
  const int D = g.D;
  const double d = g.dfilt;
  if (window == kRamLak && !ea_exact) {  // the reference's taps, as built with the plan
    HostGeom fresh;
    std::string e;
    if (!build_geometry(g.options.data(), (int)g.options.size(), g.dtype, fresh, e)) {
      err = e;
      return false;
    }
    g.taps = fresh.taps;
    g.taps_lo = fresh.taps_lo;
    return true;
  }
  const double PI = std::acos(-1.0);
  g.taps.assign(2 * D - 1, 0.0);
  g.taps_lo.assign(2 * D - 1, 0.0);
  for (int j = 0; j < 2 * D - 1; ++j) {
    const long x = j - D + 1;
    double h;
    if (window == kSheppLogan) h = -2 / (PI * PI * d * d * (4.0 * (double)x * (double)x - 1.0));
    else if (window == kHann) h = 0.25 * rl_tap(x - 1, d) + 0.5 * rl_tap(x, d) + 0.25 * rl_tap(x + 1, d);
    else h = rl_tap(x, d);
    if (ea_exact && x != 0) {
      const double gam = (double)x * d;
      const double f = gam / std::sin(gam);
      h *= f * f;
    }
    const double hi = g.dtype == 0 ? (double)(float)h : h;
    g.taps[j] = hi;
    g.taps_lo[j] = g.dtype == 0 ? h - hi : 0.0;
  }
  return true;
}

bool build_geometry(const double* options, int n_options, int dtype, HostGeom& g, std::string& err) {
  g = HostGeom();
  g.dtype = dtype;
  if (options && n_options > 0) g.options.assign(options, options + n_options);
  if (dtype == 0) return build<float>(options, n_options, g, err);
  if (dtype == 1) return build<double>(options, n_options, g, err);
  err = "dtype must be 0 (float32) or 1 (float64)";
  return false;
}

}  // namespace ctgb
