// CPU oracle for CTLIB's distance-driven operators. TEST INFRASTRUCTURE ONLY:
// the tests, the smoke check and the CPU-baseline leg of the benchmark link it as
// the checker. The product path (ctlib_gb300) never calls it.
//
// It restates the arithmetic of the reference kernels in plain C++17 (OpenMP over
// views / image lines), one two-pointer merge per (view, image line) over the
// full detector row:
//   fan equal-distance  src/fan_ed_kernel.cu:8-21 (map_x, map_y, cweight),
//                       :24-254 (prj), :257-499 (prj_t), :502-705 (bprj_t),
//                       :708-923 (bprj), :926-943 (rlfilter), :1333-1382 (fbp)
//   fan equal-angle     src/fan_ea_kernel.cu:8-20, :23-240, :243-472, :475-698,
//                       :701-901, :904-921, :1059-1107
//   parallel beam       src/para_kernel.cu:8-170, :173-336, :339-499, :502-663,
//                       :666-683, :809-849
// Type promotions follow the reference (scalar_t vs double per expression), so
// the float instantiation tracks the reference's fp32 rounding; the double
// instantiation with `f32ang` keeps the fp32 view angles (hence the same
// branch / flip decisions) and is the FP64 oracle for fp32 inputs.
//
// Parity pin: tests/golden/ holds outputs of the reference's own kernel source,
// executed on the CPU by oracle/ref_emu; tests/test_oracle_golden.py checks this
// file against them.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum Op { OP_PRJ = 0, OP_PRJ_T = 1, OP_BPRJ = 2, OP_BPRJ_T = 3, OP_FBP = 4, OP_RAMP = 5, OP_BPRJ_SV = 6 };
enum Scan { FAN_ED = 0, FAN_EA = 1, PARA = 2 };

template <class T>
struct Opts {
  int V, D, W, H, scan;
  T views, dets, width, height, dImg, dDet, Ang0, dAng, s2r, d2r, binshift;
};

// Options vector semantics (src/ctlib.cpp:18, src/fan_ed_kernel.cu:1165-1175,
// src/para_kernel.cu:687-695): scan_type is the last entry; parallel reads
// binshift from index 8.
template <class T>
bool parse(const double* o, int n, Opts<T>& p) {
  if (n < 9) return false;
  p.scan = (int)o[n - 1];
  if (p.scan < 0 || p.scan > 2) return false;
  if (p.scan != PARA && n < 12) return false;
  p.V = (int)o[0]; p.D = (int)o[1]; p.W = (int)o[2]; p.H = (int)o[3];
  p.views = (T)o[0]; p.dets = (T)o[1]; p.width = (T)o[2]; p.height = (T)o[3];
  p.dImg = (T)o[4]; p.dDet = (T)o[5]; p.Ang0 = (T)o[6]; p.dAng = (T)o[7];
  if (p.scan == PARA) {
    p.binshift = (T)o[8]; p.s2r = 0; p.d2r = 0;
  } else {
    p.s2r = (T)o[8]; p.d2r = (T)o[9]; p.binshift = (T)o[10];
  }
  return p.V > 0 && p.D > 0 && p.W > 0 && p.H > 0;
}

template <class T> inline T map_x(T sx, T sy, T dx, T dy) { return (sx * dy - sy * dx) / (dy - sy); }
template <class T> inline T map_y(T sx, T sy, T dx, T dy) { return (sy * dx - sx * dy) / (dx - sx); }

template <class T>
struct View {
  bool xb = true, flip = false;
  double ang = 0, c = 1, s = 0;
  T sx = 0, sy = 0;
  std::vector<T> db;    // D+1 detector boundaries on the common axis, increasing
  std::vector<T> cbar;  // fan: mean cosine of the two boundary rays per detector
};

// View angle idxview * dAng + Ang0 in the data type (src/fan_ed_kernel.cu:61).
// nvcc's default --fmad=true contracts this expression into one fused
// multiply-add, so it is evaluated as an FMA here.
template <class T>
double view_angle(const Opts<T>& o, int v, bool f32ang) {
  if (f32ang) return (double)std::fma((float)v, (float)o.dAng, (float)o.Ang0);
  return (double)std::fma((T)v, o.dAng, o.Ang0);
}

template <class T>
View<T> make_view(const Opts<T>& o, int v, bool f32ang) {
  View<T> w;
  const double PI = std::acos(-1.0);
  const double ang = view_angle(o, v, f32ang);
  w.ang = ang;
  w.xb = std::fabs(ang - std::round(ang / PI) * PI) * 4 / PI <= 1;
  const double e2 = (ang - std::floor(ang / 2 / PI) * 2 * PI) * 4 / PI;
  w.flip = e2 >= 3 && e2 < 7;
  w.c = std::cos(ang);
  w.s = std::sin(ang);
  const int D = o.D;
  w.db.resize(D + 1);
  if (o.scan != PARA) {
    w.sx = (T)(-w.s * (double)o.s2r);
    w.sy = (T)(w.c * (double)o.s2r);
  }
  // virtual-detector pitch and shift are scalar_t expressions widened to double
  const double virdDet = (double)(o.s2r / (o.s2r + o.d2r) * o.dDet);
  const double virshift = (double)(o.s2r / (o.s2r + o.d2r) * o.binshift);
  for (int b = 0; b <= D; ++b) {
    const T tb = w.flip ? (o.dets / 2 - (T)b) : ((T)b - o.dets / 2);
    T val;
    if (o.scan == FAN_ED) {
      const double sdet = (double)tb * virdDet + virshift;
      const T detx = (T)(sdet * w.c), dety = (T)(sdet * w.s);
      val = w.xb ? map_x(w.sx, w.sy, detx, dety) : map_y(w.sx, w.sy, detx, dety);
    } else if (o.scan == FAN_EA) {
      const double beta = (double)(tb * o.dDet + o.binshift) + ang;
      val = w.xb ? (T)((double)w.sx + std::sin(beta) / std::cos(beta) * (double)w.sy)
                 : (T)((double)w.sy + std::cos(beta) / std::sin(beta) * (double)w.sx);
    } else {
      const T num = tb * o.dDet + o.binshift;
      val = (T)((double)num / (w.xb ? w.c : w.s));
    }
    w.db[b] = val;
  }
  if (o.scan != PARA) {
    std::vector<T> cosb(D + 1);
    for (int b = 0; b <= D; ++b) {
      const T u = w.db[b];
      cosb[b] = w.xb ? std::fabs(w.sy) / std::sqrt((u - w.sx) * (u - w.sx) + w.sy * w.sy)
                     : std::fabs(w.sx) / std::sqrt((u - w.sy) * (u - w.sy) + w.sx * w.sx);
    }
    w.cbar.resize(D);
    for (int d = 0; d < D; ++d) w.cbar[d] = (cosb[d + 1] + cosb[d]) / 2;
  }
  return w;
}

// Geometry of one image line in one view: the N+1 pixel boundaries projected
// onto the view's axis, and the pixel centres (for the backprojector weights).
template <class T>
struct Line {
  int N;
  std::vector<T> pb, cx, cy;
};

template <class T>
void make_line(const Opts<T>& o, const View<T>& w, int line, Line<T>& L) {
  const bool fan = o.scan != PARA;
  if (w.xb) {  // line = image row, walk along +x
    const int N = o.W;
    L.N = N;
    L.pb.resize(N + 1); L.cx.resize(N); L.cy.resize(N);
    const T i0y = (T)(((double)(o.height / 2 - (T)line) - 0.5) * (double)o.dImg);
    const T x0 = -o.width / 2 * o.dImg;
    T pstart = 0;
    if (!fan) pstart = (T)(w.s / w.c * (double)i0y + (double)x0);
    for (int k = 0; k <= N; ++k) {
      const T xk = x0 + (T)k * o.dImg;
      L.pb[k] = fan ? map_x(w.sx, w.sy, xk, i0y) : (T)(pstart + (T)k * o.dImg);
      if (k > 0) { L.cx[k - 1] = xk - o.dImg / 2; L.cy[k - 1] = i0y; }
    }
  } else {  // line = image column, walk along +y (image row H-1-k)
    const int N = o.H;
    L.N = N;
    L.pb.resize(N + 1); L.cx.resize(N); L.cy.resize(N);
    const T i0x = (T)(((double)((T)line - o.width / 2) + 0.5) * (double)o.dImg);
    const T y0 = -o.height / 2 * o.dImg;
    T pstart = 0;
    if (!fan) pstart = (T)((double)y0 + w.c / w.s * (double)i0x);
    for (int k = 0; k <= N; ++k) {
      const T yk = y0 + (T)k * o.dImg;
      L.pb[k] = fan ? map_y(w.sx, w.sy, i0x, yk) : (T)(pstart + (T)k * o.dImg);
      if (k > 0) { L.cx[k - 1] = i0x; L.cy[k - 1] = yk - o.dImg / 2; }
    }
  }
}

// Merge of two increasing boundary lists; f(k, d, len) for every overlap of
// pixel k with detector d of positive length.
template <class T, class F>
inline void merge(const T* pb, int N, const T* db, int D, F&& f) {
  int k = 0, d = 0;
  while (k < N && pb[k + 1] <= db[0]) ++k;
  while (d < D && db[d + 1] <= pb[0]) ++d;
  while (k < N && d < D) {
    const T lo = std::max(pb[k], db[d]);
    const T pe = pb[k + 1], de = db[d + 1];
    const T hi = std::min(pe, de);
    if (hi > lo) f(k, d, hi - lo);
    if (pe < de) ++k;
    else if (de < pe) ++d;
    else { ++k; ++d; }
  }
}

template <class T>
inline size_t pix_index(const Opts<T>& o, bool xb, int line, int k) {
  return xb ? (size_t)line * o.W + k : (size_t)(o.H - 1 - k) * o.W + line;
}

// backprojector pixel weight: U^2 weight (ED, src/fan_ed_kernel.cu:18-21),
// squared source distance (EA, divides; src/fan_ea_kernel.cu:18-20)
template <class T>
inline T cweight_ed(T sx, T sy, T x, T y, T r) {
  T d = (sx * x + sy * y) / r;
  return r * r / ((r - d) * (r - d));
}
template <class T>
inline T cweight_ea(T sx, T sy, T x, T y) {
  return (sx - x) * (sx - x) + (sy - y) * (sy - y);
}

// detector-side operators (A and B^T): one sinogram row per (slice, view)
template <class T>
void det_gather(const Opts<T>& o, const std::vector<View<T>>& views, bool transpose_b,
                int B, const T* img, T* out) {
  const int V = o.V, D = o.D;
  const T dinterval = o.dImg / o.dDet;
#pragma omp parallel
  {
    std::vector<T> acc(D);
    Line<T> L;
#pragma omp for collapse(2) schedule(dynamic, 4)
    for (int b = 0; b < B; ++b) {
      for (int v = 0; v < V; ++v) {
        const View<T>& w = views[v];
        const T* x = img + (size_t)b * o.H * o.W;
        std::fill(acc.begin(), acc.end(), (T)0);
        const int nlines = w.xb ? o.H : o.W;
        for (int line = 0; line < nlines; ++line) {
          make_line(o, w, line, L);
          const T* pb = L.pb.data();
          if (!transpose_b) {
            if (o.scan == PARA) {
              merge(pb, L.N, w.db.data(), D, [&](int k, int d, T len) {
                acc[d] += len * x[pix_index(o, w.xb, line, k)] * dinterval;
              });
            } else {
              merge(pb, L.N, w.db.data(), D, [&](int k, int d, T len) {
                acc[d] += len * x[pix_index(o, w.xb, line, k)] / (w.db[d + 1] - w.db[d]);
              });
            }
          } else {
            merge(pb, L.N, w.db.data(), D, [&](int k, int d, T len) {
              const T val = x[pix_index(o, w.xb, line, k)];
              if (o.scan == PARA) {
                acc[d] += len * val / o.dImg;
              } else {
                const T pw = pb[k + 1] - pb[k];
                if (o.scan == FAN_ED)
                  acc[d] += len * val / pw * cweight_ed(w.sx, w.sy, L.cx[k], L.cy[k], o.s2r);
                else
                  acc[d] += len * val / pw / cweight_ea(w.sx, w.sy, L.cx[k], L.cy[k]);
              }
            });
          }
        }
        T* y = out + ((size_t)b * V + v) * D;
        for (int d = 0; d < D; ++d) {
          T r = acc[d];
          if (o.scan != PARA && (!transpose_b || o.scan == FAN_EA)) {
            // A: x dImg / mean cosine (src/fan_ed_kernel.cu:146-157);
            // EA B^T carries the same factor (src/fan_ea_kernel.cu:590-607)
            r *= o.dImg;
            r /= w.cbar[d];
          }
          y[w.flip ? D - 1 - d : d] = r;
        }
      }
    }
  }
}

// image-side operators (A^T and B): every image line gathers over the views of
// its branch, so each output pixel is written by one thread
template <class T>
void pix_gather(const Opts<T>& o, const std::vector<View<T>>& views, bool backproj,
                int B, const T* sino, T* img, bool per_view = false) {
  // per_view: B x V x H x W output, one image per view with no sum over views
  // (backprojection_sv, src/fan_ed_kernel.cu:946-1161 writes
  // image[channel][view][row][col])
  const int V = o.V, D = o.D;
  const T dinterval = o.dImg / o.dDet;
  std::vector<int> xv, yv;
  for (int v = 0; v < V; ++v) (views[v].xb ? xv : yv).push_back(v);
  std::memset(img, 0, sizeof(T) * (size_t)B * (per_view ? V : 1) * o.H * o.W);
  for (int pass = 0; pass < 2; ++pass) {
    const std::vector<int>& vl = pass == 0 ? xv : yv;
    const int nlines = pass == 0 ? o.H : o.W;
#pragma omp parallel
    {
      std::vector<T> q(D), tmp;
      Line<T> L;
#pragma omp for collapse(2) schedule(dynamic, 2)
      for (int b = 0; b < B; ++b) {
        for (int line = 0; line < nlines; ++line) {
          for (int v : vl) {
            T* x = img + ((size_t)b * (per_view ? V : 1) + (per_view ? v : 0)) * o.H * o.W;
            const View<T>& w = views[v];
            const T* y = sino + ((size_t)b * V + v) * D;
            for (int d = 0; d < D; ++d) {
              T val = y[w.flip ? D - 1 - d : d];
              if (!backproj) {
                if (o.scan == PARA) {
                  q[d] = val;  // multiplied by dinterval per segment
                } else {
                  // src/fan_ed_kernel.cu:343-357: y * dImg / cbar / width
                  val *= o.dImg;
                  val /= w.cbar[d];
                  val /= (w.db[d + 1] - w.db[d]);
                  q[d] = val;
                }
              } else {
                q[d] = val;
              }
            }
            make_line(o, w, line, L);
            const T* pb = L.pb.data();
            if (!backproj) {
              merge(pb, L.N, w.db.data(), D, [&](int k, int d, T len) {
                T c = o.scan == PARA ? len * q[d] * dinterval : len * q[d];
                x[pix_index(o, w.xb, line, k)] += c;
              });
            } else {
              tmp.assign(L.N, (T)0);
              std::vector<char> hit(L.N, 0);
              merge(pb, L.N, w.db.data(), D, [&](int k, int d, T len) {
                if (o.scan == PARA) tmp[k] += len * q[d] / o.dImg;
                else tmp[k] += len * q[d] / (pb[k + 1] - pb[k]);
                hit[k] = 1;
              });
              for (int k = 0; k < L.N; ++k) {
                if (!hit[k]) continue;
                T c = tmp[k];
                if (o.scan == FAN_ED) c *= cweight_ed(w.sx, w.sy, L.cx[k], L.cy[k], o.s2r);
                else if (o.scan == FAN_EA) c /= cweight_ea(w.sx, w.sy, L.cx[k], L.cy[k]);
                x[pix_index(o, w.xb, line, k)] += c;
              }
            }
          }
        }
      }
    }
  }
}

// RL ramp taps, length 2D-1 (src/fan_ed_kernel.cu:926-943)
template <class T>
void ramp_taps(int D, T d, T* h) {
  const double PI = std::acos(-1.0);
  for (int j = 0; j < 2 * D - 1; ++j) {
    const int x = j - D + 1;
    if (std::abs(x) % 2 == 1)
      h[j] = (T)(-1 / (PI * PI * x * x * (double)d * (double)d));
    else if (x == 0)
      h[j] = 1 / (4 * d * d);
    else
      h[j] = 0;
  }
}

// fbp filter selected for the oracle's fbp (tests only): window 0 Ram-Lak (the
// reference), 1 Shepp-Logan, 2 Ram-Lak under a Hann window; ea_exact scales the
// taps by (n d / sin(n d))^2 (equal-angle fans). The variants restate published
// kernels in fp64: Shepp & Logan (1974), h(n) = -2 / (pi^2 d^2 (4 n^2 - 1)); the
// Hann window as its discrete convolution [1/4, 1/2, 1/4] with Ram-Lak; the
// equiangular fan-beam kernel of Kak & Slaney (ch. 3), (gamma / sin gamma)^2
// times the ramp kernel.
static int g_window = 0, g_ea_exact = 0;

static double rl_tap64(long x, double d) {
  const double PI = std::acos(-1.0);
  if (x == 0) return 1 / (4 * d * d);
  if (std::labs(x) % 2 == 1) return -1 / (PI * PI * (double)x * (double)x * d * d);
  return 0.0;
}

template <class T>
void filter_taps(int D, T d, T* h) {
  if (g_window == 0 && !g_ea_exact) {
    ramp_taps(D, d, h);
    return;
  }
  const double PI = std::acos(-1.0), dd = (double)d;
  for (int j = 0; j < 2 * D - 1; ++j) {
    const long x = j - D + 1;
    double v;
    if (g_window == 1) v = -2 / (PI * PI * dd * dd * (4.0 * (double)x * (double)x - 1.0));
    else if (g_window == 2) v = 0.25 * rl_tap64(x - 1, dd) + 0.5 * rl_tap64(x, dd) + 0.25 * rl_tap64(x + 1, dd);
    else v = rl_tap64(x, dd);
    if (g_ea_exact && x != 0) {
      const double gam = (double)x * dd;
      v *= (gam / std::sin(gam)) * (gam / std::sin(gam));
    }
    h[j] = (T)v;
  }
}

// FBP: detector pre-weight, RL filtering as a zero-padded linear convolution
// along the detector axis (fp64 accumulation), backprojection, x dAng/2
// (src/fan_ed_kernel.cu:1333-1382, src/fan_ea_kernel.cu:1059-1107,
//  src/para_kernel.cu:809-849)
template <class T>
void fbp(const Opts<T>& o, const std::vector<View<T>>& views, int B, const T* sino, T* img) {
  const int V = o.V, D = o.D;
  std::vector<T> wgt(D);
  T dfilt;
  if (o.scan == FAN_ED) {
    const T virdDet = o.dDet * o.s2r / (o.s2r + o.d2r);
    for (int k = 0; k < D; ++k) {
      T t = (-o.dets / 2 + (T)0.5) + (T)k;
      T r = t * virdDet;
      r = r * r;
      r = o.s2r / std::sqrt(o.s2r * o.s2r + r);
      wgt[k] = r;
    }
    dfilt = virdDet;
  } else if (o.scan == FAN_EA) {
    for (int k = 0; k < D; ++k) {
      T t = (-o.dets / 2 + (T)0.5) + (T)k;
      T r = std::cos(t * o.dDet);
      wgt[k] = r * o.s2r * o.dDet;
    }
    dfilt = o.dDet;
  } else {
    for (int k = 0; k < D; ++k) wgt[k] = o.dDet;
    dfilt = o.dDet;
  }
  std::vector<T> h(2 * D - 1);
  filter_taps(D, dfilt, h.data());
  std::vector<T> filt((size_t)B * V * D);
#pragma omp parallel
  {
    std::vector<T> row(D);
#pragma omp for collapse(2) schedule(static)
    for (int b = 0; b < B; ++b)
      for (int v = 0; v < V; ++v) {
        const T* y = sino + ((size_t)b * V + v) * D;
        for (int k = 0; k < D; ++k) {
          T r = y[k] * wgt[k];
          if (o.scan == FAN_ED) r = r * (o.dDet * o.s2r / (o.s2r + o.d2r));
          row[k] = r;
        }
        T* out = filt.data() + ((size_t)b * V + v) * D;
        for (int k = 0; k < D; ++k) {
          double s = 0;
          for (int m = 0; m < D; ++m) s += (double)row[m] * (double)h[m - k + D - 1];
          out[k] = (T)s;
        }
      }
  }
  pix_gather(o, views, true, B, filt.data(), img);
  const size_t n = (size_t)B * o.H * o.W;
  for (size_t i = 0; i < n; ++i) {
    T r = img[i] * o.dAng;
    img[i] = r / 2;
  }
}

template <class T>
int run(int op, const double* opts, int nopts, bool f32ang, int B, const void* in, void* out) {
  Opts<T> o;
  if (!parse(opts, nopts, o)) return 1;
  if (op == OP_RAMP) {
    ramp_taps(o.D, o.scan == FAN_ED ? o.dDet * o.s2r / (o.s2r + o.d2r) : o.dDet, (T*)out);
    return 0;
  }
  std::vector<View<T>> views(o.V);
#pragma omp parallel for schedule(static)
  for (int v = 0; v < o.V; ++v) views[v] = make_view(o, v, f32ang);
  const T* x = (const T*)in;
  T* y = (T*)out;
  switch (op) {
    case OP_PRJ: det_gather(o, views, false, B, x, y); break;
    case OP_BPRJ_T: det_gather(o, views, true, B, x, y); break;
    case OP_PRJ_T: pix_gather(o, views, false, B, x, y); break;
    case OP_BPRJ: pix_gather(o, views, true, B, x, y); break;
    case OP_FBP: fbp(o, views, B, x, y); break;
    case OP_BPRJ_SV:
      if (o.scan != FAN_ED) return 3;  // the reference defines it for equal-distance fans only
      pix_gather(o, views, true, B, x, y, true);
      break;
    default: return 2;
  }
  return 0;
}

}  // namespace

extern "C" {

// mode 0: fp32 data and arithmetic (mirrors the reference's fp32 instantiation)
// mode 1: fp64 data and arithmetic (mirrors the reference's fp64 instantiation)
// mode 2: fp64 arithmetic on fp32 options: view angles rounded as in fp32, so
//         branch and flip decisions match the fp32 path (the FP64 oracle)
int oracle_run(int op, const double* opts, int nopts, int mode, int batch, const void* in,
               void* out, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  if (mode == 0) return run<float>(op, opts, nopts, true, batch, in, out);
  if (mode == 1) return run<double>(op, opts, nopts, false, batch, in, out);
  if (mode == 2) {
    // fp32 inputs come with an fp32 options tensor: round the values first
    std::vector<double> o32(opts, opts + nopts);
    for (double& x : o32) x = (double)(float)x;
    return run<double>(op, o32.data(), nopts, true, batch, in, out);
  }
  return 3;
}

// filter of the oracle's fbp (see filter_taps); returns 1 on a bad window
int oracle_set_filter(int window, int ea_exact) {
  if (window < 0 || window > 2) return 1;
  g_window = window;
  g_ea_exact = ea_exact != 0;
  return 0;
}

// per-view branch (1 = image rows are the lines) and flip flags, for tests
int oracle_view_flags(const double* opts, int nopts, int mode, int* xbranch, int* flip) {
  Opts<double> o;
  if (!parse(opts, nopts, o)) return 1;
  for (int v = 0; v < o.V; ++v) {
    View<double> w;
    if (mode == 1) {
      Opts<double> od = o;
      w = make_view(od, v, false);
    } else {
      Opts<float> of;
      parse(opts, nopts, of);
      View<float> wf = make_view(of, v, true);
      w.xb = wf.xb; w.flip = wf.flip;
    }
    xbranch[v] = w.xb;
    flip[v] = w.flip;
  }
  return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
