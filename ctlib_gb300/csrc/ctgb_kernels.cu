// Distance-driven CT operators for GB300 (sm_103a) behind the C ABI in ctgb.h.
//
// Every operator is an atomic-free gather over the overlap of two increasing
// boundary lists on a common axis (per view: D+1 detector-cell boundaries;
// per view and image line: W+1 or H+1 pixel edges, affine in the edge index):
//
//   detector gather (A, B^T): one thread per (view, detector cell) walks all
//     image lines of its view; per line it maps its two cell boundaries into
//     pixel-edge coordinates (one FMA each) and sums the 1-3 overlapped pixels.
//     A CTA is 8 consecutive views x 32 consecutive cells, so the 8 warps read
//     nearly the same pixels of the same line and share them through L1.
//   image gather (A^T, B): one thread per pixel walks all views; per view it
//     maps its two pixel edges onto the axis, seeds the detector cell from a
//     closed-form inverse of the boundary map, corrects it against the stored
//     boundaries and sums the 1-3 overlapped cells. A CTA is a 32 x 8 pixel
//     tile, whose footprint per view is ~40 consecutive cells.
//
// Slices are processed SB at a time per thread (geometry computed once, SB
// fused multiply-adds per overlap); inputs are first re-laid out so that the
// SB values of one pixel / cell are one vector load. Sums over lines and views
// use blocked Kahan compensation (plain fp32 within a block of 16, compensated
// across blocks). The RL ramp filter of fbp is a direct convolution with the
// odd-tap structure of the RL kernel, fused with the detector pre-weight.
//
// Reference semantics followed: src/fan_ed_kernel.cu:24-943,
// src/fan_ea_kernel.cu:23-921, src/para_kernel.cu:8-683 (weights, flip and
// branch rules, Q3 factor of equal-angle B^T at src/fan_ea_kernel.cu:590-607).

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "ctgb.h"
#include "geometry.h"

namespace ctgb {

// ----------------------------------------------------------------------------
// errors
// ----------------------------------------------------------------------------
static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CTGB_CUDA(call)                                                                  \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) return fail(CTGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// ----------------------------------------------------------------------------
// device plan
// ----------------------------------------------------------------------------
template <class T>
struct DevPlan {
  int V, D, W, H, L, scan;
  T dImg, s2r, x0, y0, dAng, wscale;
  const int* flags;   // V
  const T* src;       // V*2
  const T* db;        // V*(D+1)
  const T* fq;        // V*D
  const T* fbt;       // V*D
  const T* lp;        // V*L*4
  const float* inv;   // V*5
  const T* rowc;      // H: row centre y
  const T* colc;      // W: column centre x
  const T* wpre;      // D
  const T* taps;      // 2D-1
};

template <class T>
struct VecT;
template <>
struct VecT<float> { using v4 = float4; using v2 = float2; };
template <>
struct VecT<double> { using v4 = double4; using v2 = double2; };

template <class T, int SB>
__device__ __forceinline__ void load_vec(const T* __restrict__ p, T (&v)[SB]) {
  if constexpr (sizeof(T) == 4 && SB % 4 == 0) {
#pragma unroll
    for (int i = 0; i < SB / 4; ++i) {
      float4 x = __ldg(reinterpret_cast<const float4*>(p) + i);
      v[4 * i] = x.x; v[4 * i + 1] = x.y; v[4 * i + 2] = x.z; v[4 * i + 3] = x.w;
    }
  } else if constexpr (SB % 2 == 0) {
    using V2 = typename VecT<T>::v2;
#pragma unroll
    for (int i = 0; i < SB / 2; ++i) {
      V2 x = __ldg(reinterpret_cast<const V2*>(p) + i);
      v[2 * i] = x.x; v[2 * i + 1] = x.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < SB; ++i) v[i] = __ldg(p + i);
  }
}

template <class T, int SB>
__device__ __forceinline__ void store_vec(T* p, const T (&v)[SB]) {
  if constexpr (sizeof(T) == 4 && SB % 4 == 0) {
#pragma unroll
    for (int i = 0; i < SB / 4; ++i)
      reinterpret_cast<float4*>(p)[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
  } else if constexpr (SB % 2 == 0) {
    using V2 = typename VecT<T>::v2;
#pragma unroll
    for (int i = 0; i < SB / 2; ++i) {
      V2 x; x.x = v[2 * i]; x.y = v[2 * i + 1];
      reinterpret_cast<V2*>(p)[i] = x;
    }
  } else {
#pragma unroll
    for (int i = 0; i < SB; ++i) p[i] = v[i];
  }
}

// Kahan fold of a block partial into (sum, comp); the partial is reset.
template <class T, int SB>
__device__ __forceinline__ void kahan_fold(T (&sum)[SB], T (&comp)[SB], T (&blk)[SB]) {
#pragma unroll
  for (int s = 0; s < SB; ++s) {
    T y = blk[s] - comp[s];
    T t = sum[s] + y;
    comp[s] = (t - sum[s]) - y;
    sum[s] = t;
    blk[s] = T(0);
  }
}

enum Kind { kA = 0, kBt = 1, kAt = 2, kB = 3 };
constexpr int kFoldEvery = 16;

// ----------------------------------------------------------------------------
// layout kernels
// ----------------------------------------------------------------------------
// image [B][H][W] -> rows [G][H][W][SB] and columns [G][W][H][SB] (k from the
// bottom row), zero-padded to G*SB slices
template <class T, int SB>
__global__ void k_layout_image(const T* __restrict__ img, T* __restrict__ imx, T* __restrict__ imy, int B,
                               int H, int W, int G) {
  const size_t n = (size_t)G * H * W;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % W);
    const int r = (int)((i / W) % H);
    const int g = (int)(i / ((size_t)W * H));
    T v[SB];
#pragma unroll
    for (int s = 0; s < SB; ++s) {
      const int b = g * SB + s;
      v[s] = b < B ? img[((size_t)b * H + r) * W + c] : T(0);
    }
    store_vec<T, SB>(imx + i * SB, v);
    if (imy) store_vec<T, SB>(imy + (((size_t)g * W + c) * H + (H - 1 - r)) * SB, v);
  }
}

// sinogram [B][V][D] (external detector order) -> [G][V][D][SB] (internal,
// increasing-boundary order), times an optional per-(view, cell) factor
template <class T, int SB>
__global__ void k_layout_sino(const T* __restrict__ y, T* __restrict__ q, const int* __restrict__ flags,
                              const T* __restrict__ f, int B, int V, int D, int G) {
  const size_t n = (size_t)G * V * D;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int d = (int)(i % D);
    const int v = (int)((i / D) % V);
    const int g = (int)(i / ((size_t)D * V));
    const int de = (flags[v] & 2) ? D - 1 - d : d;
    const T fac = f ? f[(size_t)v * D + d] : T(1);
    T val[SB];
#pragma unroll
    for (int s = 0; s < SB; ++s) {
      const int b = g * SB + s;
      val[s] = b < B ? y[((size_t)b * V + v) * D + de] * fac : T(0);
    }
    store_vec<T, SB>(q + i * SB, val);
  }
}

// ----------------------------------------------------------------------------
// backprojector pixel weights
// ----------------------------------------------------------------------------
// U^2 weight (src/fan_ed_kernel.cu:18-21)
template <class T>
__device__ __forceinline__ T cweight_ed(T sx, T sy, T x, T y, T r) {
  const T d = (sx * x + sy * y) / r;
  return r * r / ((r - d) * (r - d));
}
// squared source distance (src/fan_ea_kernel.cu:18-20), used as a divisor
template <class T>
__device__ __forceinline__ T dist2_ea(T sx, T sy, T x, T y) {
  return (sx - x) * (sx - x) + (sy - y) * (sy - y);
}

// ----------------------------------------------------------------------------
// detector gather: A (kind kA) and B^T (kind kBt)
// ----------------------------------------------------------------------------
template <class T, int SB, int KIND>
__global__ void __launch_bounds__(256) k_det_gather(DevPlan<T> P, const T* __restrict__ imx,
                                                    const T* __restrict__ imy, T* __restrict__ out, int B) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int d = blockIdx.x * 32 + lane;
  const int v = blockIdx.y * 8 + warp;
  const int g = blockIdx.z;
  if (v >= P.V || d >= P.D) return;
  const int fl = P.flags[v];
  const bool xb = fl & 1;
  const T* dbv = P.db + (size_t)v * (P.D + 1);
  const T dlo = dbv[d], dhi = dbv[d + 1];
  const int nlines = xb ? P.H : P.W;
  const int N = xb ? P.W : P.H;
  const T* base = xb ? imx + (size_t)g * P.H * P.W * SB : imy + (size_t)g * P.W * P.H * SB;
  const T* lpv = P.lp + (size_t)v * P.L * 4;
  T sx = T(0), sy = T(0);
  if (KIND == kBt && P.scan != kPara) { sx = P.src[2 * v]; sy = P.src[2 * v + 1]; }

  T sum[SB], comp[SB], blk[SB];
#pragma unroll
  for (int s = 0; s < SB; ++s) { sum[s] = T(0); comp[s] = T(0); blk[s] = T(0); }

  for (int l = 0; l < nlines; ++l) {
    const T sigma = lpv[4 * l + 1], beta = lpv[4 * l + 2], gam = lpv[4 * l + 3];
    const T tlo = fma(dlo, gam, beta), thi = fma(dhi, gam, beta);
    const T a = tlo > T(0) ? tlo : T(0);
    const T b = thi < T(N) ? thi : T(N);
    if (a < b) {
      const int k0 = (int)floor(a);
      int k1 = (int)ceil(b);
      if (k1 > N) k1 = N;
      const T* row = base + (size_t)l * N * SB;
      T lc = T(0);
      if (KIND == kBt && P.scan != kPara) lc = xb ? P.rowc[l] : P.colc[l];
      for (int k = k0; k < k1; ++k) {
        const T lo = a > T(k) ? a : T(k);
        const T hi = b < T(k + 1) ? b : T(k + 1);
        T w = hi - lo;
        if (KIND == kA) {
          w *= sigma;
        } else if (P.scan == kFanED) {
          const T pc = fma(T(k) + T(0.5), P.dImg, xb ? P.x0 : P.y0);
          w *= xb ? cweight_ed(sx, sy, pc, lc, P.s2r) : cweight_ed(sx, sy, lc, pc, P.s2r);
        } else if (P.scan == kFanEA) {
          const T pc = fma(T(k) + T(0.5), P.dImg, xb ? P.x0 : P.y0);
          w /= xb ? dist2_ea(sx, sy, pc, lc) : dist2_ea(sx, sy, lc, pc);
        }
        T u[SB];
        load_vec<T, SB>(row + (size_t)k * SB, u);
#pragma unroll
        for (int s = 0; s < SB; ++s) blk[s] = fma(w, u[s], blk[s]);
      }
    }
    if ((l % kFoldEvery) == kFoldEvery - 1) kahan_fold<T, SB>(sum, comp, blk);
  }
  kahan_fold<T, SB>(sum, comp, blk);
  T f = T(1);
  if (KIND == kA) f = P.fq[(size_t)v * P.D + d];
  else if (P.scan == kFanEA) f = P.fbt[(size_t)v * P.D + d];
  const int de = (fl & 2) ? P.D - 1 - d : d;
#pragma unroll
  for (int s = 0; s < SB; ++s) {
    const int bb = g * SB + s;
    if (bb < B) out[((size_t)bb * P.V + v) * P.D + de] = sum[s] * f;
  }
}

// ----------------------------------------------------------------------------
// image gather: A^T (kind kAt) and B (kind kB)
// ----------------------------------------------------------------------------
template <class T, int SB, int KIND>
__global__ void __launch_bounds__(256) k_pix_gather(DevPlan<T> P, const T* __restrict__ q, T* __restrict__ img,
                                                    int B, T out_mul, T out_div) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c = blockIdx.x * 32 + lane;
  const int r = blockIdx.y * 8 + warp;
  const int g = blockIdx.z;
  if (c >= P.W || r >= P.H) return;
  const T* qg = q + (size_t)g * P.V * P.D * SB;
  // pixel centre (for the backprojector weights)
  const T pcx = fma(T(c) + T(0.5), P.dImg, P.x0);
  const T pcy = P.rowc[r];

  T sum[SB], comp[SB], blk[SB];
#pragma unroll
  for (int s = 0; s < SB; ++s) { sum[s] = T(0); comp[s] = T(0); blk[s] = T(0); }

  for (int v = 0; v < P.V; ++v) {
    const int fl = P.flags[v];
    const bool xb = fl & 1;
    const int line = xb ? r : c;
    const int k = xb ? c : P.H - 1 - r;
    const T* lpl = P.lp + ((size_t)v * P.L + line) * 4;
    const T alpha = lpl[0], sigma = lpl[1];
    const T xlo = fma(sigma, T(k), alpha);
    const T xhi = fma(sigma, T(k + 1), alpha);
    // seed the cell index from the closed-form inverse of the boundary map
    const float* iv = P.inv + (size_t)v * 5;
    const float xf = (float)xlo;
    float u = xf * iv[0] / fmaf(xf, iv[2], iv[1]);
    if (P.scan == kFanEA) u = atanf(u);
    const float cb = fmaf(iv[4], u, iv[3]);
    const int D = P.D;
    int d = cb < 0.f ? 0 : (cb >= (float)(D - 1) ? D - 1 : (int)cb);
    const T* dbv = P.db + (size_t)v * (D + 1);
    while (d > 0 && xlo < dbv[d]) --d;
    while (d < D - 1 && dbv[d + 1] <= xlo) ++d;
    T vacc[SB];
    if (KIND == kB) {
#pragma unroll
      for (int s = 0; s < SB; ++s) vacc[s] = T(0);
    }
    T lob = dbv[d];
    const T* qv = qg + (size_t)v * D * SB;
    for (; d < D; ++d) {
      const T hib = dbv[d + 1];
      const T lo = xlo > lob ? xlo : lob;
      const T hi = xhi < hib ? xhi : hib;
      if (lo >= xhi) break;
      if (hi > lo) {
        const T w = hi - lo;
        T qq[SB];
        load_vec<T, SB>(qv + (size_t)d * SB, qq);
        if (KIND == kAt) {
#pragma unroll
          for (int s = 0; s < SB; ++s) blk[s] = fma(w, qq[s], blk[s]);
        } else {
#pragma unroll
          for (int s = 0; s < SB; ++s) vacc[s] = fma(w, qq[s], vacc[s]);
        }
      }
      if (hib >= xhi) break;
      lob = hib;
    }
    if (KIND == kB) {
      T wv;
      if (P.scan == kFanED) {
        wv = cweight_ed(P.src[2 * v], P.src[2 * v + 1], pcx, pcy, P.s2r) / sigma;
      } else if (P.scan == kFanEA) {
        wv = T(1) / (dist2_ea(P.src[2 * v], P.src[2 * v + 1], pcx, pcy) * sigma);
      } else {
        wv = T(1) / P.dImg;
      }
#pragma unroll
      for (int s = 0; s < SB; ++s) blk[s] = fma(vacc[s], wv, blk[s]);
    }
    if ((v % kFoldEvery) == kFoldEvery - 1) kahan_fold<T, SB>(sum, comp, blk);
  }
  kahan_fold<T, SB>(sum, comp, blk);
#pragma unroll
  for (int s = 0; s < SB; ++s) {
    const int bb = g * SB + s;
    if (bb < B) img[((size_t)bb * P.H + r) * P.W + c] = sum[s] * out_mul / out_div;
  }
}

// ----------------------------------------------------------------------------
// fbp ramp filter: q[g][v][d][s] = sum_m pre(y)[m] * h[m - k + D - 1], k = ext(d)
// One CTA per (slice group, view); each thread produces 8 outputs of one parity
// for one slice: outputs k0, k0+2, ..., k0+14 only meet taps of odd offset (the
// even non-zero offsets of the RL kernel are zero), plus the centre tap.
// ----------------------------------------------------------------------------
template <class T, int SB>
__global__ void __launch_bounds__(256) k_ramp_filter(DevPlan<T> P, const T* __restrict__ y, T* __restrict__ q,
                                                     int B) {
  extern __shared__ unsigned char smem_raw[];
  T* taps = reinterpret_cast<T*>(smem_raw);          // 2D-1
  T* rows = taps + (2 * P.D - 1 + 1);                 // SB x D
  const int v = blockIdx.x, g = blockIdx.y, D = P.D;
  for (int j = threadIdx.x; j < 2 * D - 1; j += blockDim.x) taps[j] = P.taps[j];
  for (int i = threadIdx.x; i < SB * D; i += blockDim.x) {
    const int s = i / D, m = i % D;
    const int bb = g * SB + s;
    T val = T(0);
    if (bb < B) val = (y[((size_t)bb * P.V + v) * D + m] * P.wpre[m]) * P.wscale;
    rows[s * D + m] = val;
  }
  __syncthreads();
  const int chunks = (D + 15) / 16;               // 16 outputs (8 per parity) per chunk
  const int items = SB * 2 * chunks;
  const bool flip = P.flags[v] & 2;
  T* qv = q + ((size_t)g * P.V + v) * D * SB;
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    const int s = it % SB;
    const int par = (it / SB) & 1;
    const int ch = it / (2 * SB);
    const int k0 = ch * 16 + par;
    const T* row = rows + s * D;
    T acc[8];
    T win[8];
    // window: win[i] = h(m - k0 - 2i) for the current input m (opposite parity)
    int m = 1 - par;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      acc[i] = T(0);
      const int off = m - k0 - 2 * i;  // odd
      const int ti = off + D - 1;
      win[i] = (ti >= 0 && ti < 2 * D - 1) ? taps[ti] : T(0);
    }
    for (; m < D; m += 2) {
      const T xm = row[m];
#pragma unroll
      for (int i = 0; i < 8; ++i) acc[i] = fma(xm, win[i], acc[i]);
#pragma unroll
      for (int i = 7; i > 0; --i) win[i] = win[i - 1];
      const int ti = m + 2 - k0 + D - 1;
      win[0] = (ti >= 0 && ti < 2 * D - 1) ? taps[ti] : T(0);
    }
    const T h0 = taps[D - 1];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int k = k0 + 2 * i;
      if (k < D) {
        const T val = fma(h0, row[k], acc[i]);
        const int di = flip ? D - 1 - k : k;
        qv[(size_t)di * SB + s] = val;
      }
    }
  }
}

// ----------------------------------------------------------------------------
// plan
// ----------------------------------------------------------------------------
}  // namespace ctgb

struct ctgb_plan {
  ctgb::HostGeom geom;
  int device = 0;
  int dtype = 0;
  void* dev = nullptr;  // one allocation holding all tables
  ctgb::DevPlan<float> pf{};
  ctgb::DevPlan<double> pd{};
};

namespace ctgb {

template <class T>
static int upload(ctgb_plan* p) {
  const HostGeom& g = p->geom;
  const int V = g.V, D = g.D, L = g.L;
  // table sizes in elements of T
  std::vector<std::pair<const std::vector<double>*, size_t>> parts;
  std::vector<double> rowc(g.H), colc(g.W);
  for (int r = 0; r < g.H; ++r) rowc[r] = (double)(T)(((double)((T)(g.height / 2) - (T)r) - 0.5) * g.dImg);
  for (int c = 0; c < g.W; ++c) colc[c] = (double)(T)(((double)((T)c - (T)(g.width / 2)) + 0.5) * g.dImg);
  const std::vector<const std::vector<double>*> tabs = {&g.src, &g.db, &g.fq, &g.fbt, &g.lp,
                                                        &rowc, &colc, &g.wpre, &g.taps};
  size_t off = 0;
  std::vector<size_t> offs;
  auto align = [](size_t x) { return (x + 31) & ~(size_t)31; };
  for (auto* t : tabs) { offs.push_back(off); off = align(off + t->size() * sizeof(T)); }
  const size_t off_flags = off; off = align(off + (size_t)V * sizeof(int));
  const size_t off_inv = off; off = align(off + (size_t)V * 5 * sizeof(float));
  std::vector<unsigned char> host(off, 0);
  for (size_t i = 0; i < tabs.size(); ++i) {
    T* dst = reinterpret_cast<T*>(host.data() + offs[i]);
    for (size_t j = 0; j < tabs[i]->size(); ++j) dst[j] = (T)(*tabs[i])[j];
  }
  std::memcpy(host.data() + off_flags, g.flags.data(), (size_t)V * sizeof(int));
  float* invf = reinterpret_cast<float*>(host.data() + off_inv);
  for (size_t j = 0; j < g.inv.size(); ++j) invf[j] = (float)g.inv[j];
  CTGB_CUDA(cudaSetDevice(p->device));
  CTGB_CUDA(cudaMalloc(&p->dev, off));
  CTGB_CUDA(cudaMemcpy(p->dev, host.data(), off, cudaMemcpyHostToDevice));
  unsigned char* b = static_cast<unsigned char*>(p->dev);
  DevPlan<T> P{};
  P.V = V; P.D = D; P.W = g.W; P.H = g.H; P.L = L; P.scan = g.scan;
  P.dImg = (T)g.dImg; P.s2r = (T)g.s2r; P.x0 = (T)g.x0; P.y0 = (T)g.y0; P.dAng = (T)g.dAng;
  P.wscale = (T)g.wscale;
  P.src = reinterpret_cast<const T*>(b + offs[0]);
  P.db = reinterpret_cast<const T*>(b + offs[1]);
  P.fq = reinterpret_cast<const T*>(b + offs[2]);
  P.fbt = reinterpret_cast<const T*>(b + offs[3]);
  P.lp = reinterpret_cast<const T*>(b + offs[4]);
  P.rowc = reinterpret_cast<const T*>(b + offs[5]);
  P.colc = reinterpret_cast<const T*>(b + offs[6]);
  P.wpre = reinterpret_cast<const T*>(b + offs[7]);
  P.taps = reinterpret_cast<const T*>(b + offs[8]);
  P.flags = reinterpret_cast<const int*>(b + off_flags);
  P.inv = reinterpret_cast<const float*>(b + off_inv);
  if constexpr (sizeof(T) == 4) p->pf = P; else p->pd = P;
  return CTGB_OK;
}

// slices per thread: float up to 16, double up to 4
static int slices_per_thread(int dtype, int batch) {
  const int cap = dtype == 0 ? 16 : 4;
  int sb = 1;
  while (sb < batch && sb < cap) sb *= 2;
  return sb;
}

static size_t esize(int dtype) { return dtype == 0 ? 4 : 8; }

static size_t workspace_bytes(const ctgb_plan* p, int op, int batch) {
  const HostGeom& g = p->geom;
  const int sb = slices_per_thread(p->dtype, batch);
  const size_t G = (size_t)((batch + sb - 1) / sb);
  const size_t es = esize(p->dtype);
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  if (op == CTGB_OP_PROJECTION || op == CTGB_OP_BACKPROJECTION_T)
    return 2 * al(G * g.H * g.W * sb * es);
  return al(G * g.V * g.D * sb * es);
}

template <class T, int SB>
static int run_op(const ctgb_plan* p, const DevPlan<T>& P, int op, const void* in, void* out, int batch,
                  void* ws, cudaStream_t st) {
  const int G = (batch + SB - 1) / SB;
  const HostGeom& g = p->geom;
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const T* x = static_cast<const T*>(in);
  T* y = static_cast<T*>(out);
  if (op == CTGB_OP_PROJECTION || op == CTGB_OP_BACKPROJECTION_T) {
    T* imx = static_cast<T*>(ws);
    T* imy = reinterpret_cast<T*>(static_cast<unsigned char*>(ws) + al((size_t)G * g.H * g.W * SB * sizeof(T)));
    const size_t n = (size_t)G * g.H * g.W;
    const int tb = 256;
    const int nb = (int)std::min<size_t>((n + tb - 1) / tb, 152 * 16);
    k_layout_image<T, SB><<<nb, tb, 0, st>>>(x, imx, imy, batch, g.H, g.W, G);
    dim3 grid((g.D + 31) / 32, (g.V + 7) / 8, G);
    if (op == CTGB_OP_PROJECTION)
      k_det_gather<T, SB, kA><<<grid, 256, 0, st>>>(P, imx, imy, y, batch);
    else
      k_det_gather<T, SB, kBt><<<grid, 256, 0, st>>>(P, imx, imy, y, batch);
  } else {
    T* qb = static_cast<T*>(ws);
    if (op == CTGB_OP_FBP) {
      const size_t smem = ((size_t)2 * g.D + (size_t)SB * g.D) * sizeof(T);
      if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_ramp_filter<T, SB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return fail(CTGB_ERR_CUDA, std::string("ramp filter smem: ") + cudaGetErrorString(e));
      }
      k_ramp_filter<T, SB><<<dim3(g.V, G), 256, smem, st>>>(P, x, qb, batch);
    } else {
      const size_t n = (size_t)G * g.V * g.D;
      const int tb = 256;
      const int nb = (int)std::min<size_t>((n + tb - 1) / tb, 152 * 16);
      k_layout_sino<T, SB><<<nb, tb, 0, st>>>(x, qb, P.flags, op == CTGB_OP_PROJECTION_T ? P.fq : nullptr,
                                             batch, g.V, g.D, G);
    }
    dim3 grid((g.W + 31) / 32, (g.H + 7) / 8, G);
    if (op == CTGB_OP_PROJECTION_T)
      k_pix_gather<T, SB, kAt><<<grid, 256, 0, st>>>(P, qb, y, batch, T(1), T(1));
    else if (op == CTGB_OP_BACKPROJECTION)
      k_pix_gather<T, SB, kB><<<grid, 256, 0, st>>>(P, qb, y, batch, T(1), T(1));
    else
      k_pix_gather<T, SB, kB><<<grid, 256, 0, st>>>(P, qb, y, batch, P.dAng, T(2));
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(CTGB_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return CTGB_OK;
}

static int dispatch(const ctgb_plan* p, int op, const void* in, void* out, int batch, void* ws, size_t wsb,
                    void* stream) {
  if (!p) return fail(CTGB_ERR_INVALID, "null plan");
  if (batch < 0) return fail(CTGB_ERR_INVALID, "negative batch");
  if (batch == 0) return CTGB_OK;
  if (!in || !out) return fail(CTGB_ERR_INVALID, "null input or output pointer");
  const size_t need = workspace_bytes(p, op, batch);
  if (need > 0 && (!ws || wsb < need))
    return fail(CTGB_ERR_WORKSPACE, "workspace too small: need " + std::to_string(need) + " bytes");
  if ((reinterpret_cast<uintptr_t>(ws) & 255) != 0) return fail(CTGB_ERR_INVALID, "workspace must be 256-byte aligned");
  int cur = -1;
  CTGB_CUDA(cudaGetDevice(&cur));
  if (cur != p->device) CTGB_CUDA(cudaSetDevice(p->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int sb = slices_per_thread(p->dtype, batch);
  int rc;
  if (p->dtype == 0) {
    switch (sb) {
      case 1: rc = run_op<float, 1>(p, p->pf, op, in, out, batch, ws, st); break;
      case 2: rc = run_op<float, 2>(p, p->pf, op, in, out, batch, ws, st); break;
      case 4: rc = run_op<float, 4>(p, p->pf, op, in, out, batch, ws, st); break;
      case 8: rc = run_op<float, 8>(p, p->pf, op, in, out, batch, ws, st); break;
      default: rc = run_op<float, 16>(p, p->pf, op, in, out, batch, ws, st); break;
    }
  } else {
    switch (sb) {
      case 1: rc = run_op<double, 1>(p, p->pd, op, in, out, batch, ws, st); break;
      case 2: rc = run_op<double, 2>(p, p->pd, op, in, out, batch, ws, st); break;
      default: rc = run_op<double, 4>(p, p->pd, op, in, out, batch, ws, st); break;
    }
  }
  if (cur != p->device && cur >= 0) cudaSetDevice(cur);
  return rc;
}

}  // namespace ctgb

// ----------------------------------------------------------------------------
// C ABI
// ----------------------------------------------------------------------------
extern "C" {

int ctgb_version(void) { return 1; }

const char* ctgb_last_error(void) { return ctgb::g_err.c_str(); }

int ctgb_plan_create(ctgb_plan** plan, const double* options, int n_options, int dtype, int device) {
  using namespace ctgb;
  if (!plan || !options) return fail(CTGB_ERR_INVALID, "null plan or options pointer");
  *plan = nullptr;
  auto* p = new ctgb_plan();
  std::string err;
  if (!build_geometry(options, n_options, dtype, p->geom, err)) {
    delete p;
    return fail(CTGB_ERR_INVALID, err);
  }
  p->device = device;
  p->dtype = dtype;
  int rc = dtype == 0 ? upload<float>(p) : upload<double>(p);
  if (rc != CTGB_OK) {
    if (p->dev) cudaFree(p->dev);
    delete p;
    return rc;
  }
  *plan = p;
  return CTGB_OK;
}

int ctgb_plan_destroy(ctgb_plan* plan) {
  if (!plan) return CTGB_OK;
  if (plan->dev) {
    int cur = -1;
    cudaGetDevice(&cur);
    cudaSetDevice(plan->device);
    cudaFree(plan->dev);
    if (cur >= 0) cudaSetDevice(cur);
  }
  delete plan;
  return CTGB_OK;
}

int ctgb_plan_info(const ctgb_plan* p, int* views, int* dets, int* width, int* height, int* scan_type,
                   int* dtype) {
  if (!p) return ctgb::fail(CTGB_ERR_INVALID, "null plan");
  if (views) *views = p->geom.V;
  if (dets) *dets = p->geom.D;
  if (width) *width = p->geom.W;
  if (height) *height = p->geom.H;
  if (scan_type) *scan_type = p->geom.scan;
  if (dtype) *dtype = p->dtype;
  return CTGB_OK;
}

size_t ctgb_workspace_size(const ctgb_plan* plan, int op, int batch) {
  if (!plan || batch <= 0 || op < 0 || op > 4) return 0;
  return ctgb::workspace_bytes(plan, op, batch);
}

int ctgb_projection(const ctgb_plan* p, const void* image, void* sino, int batch, void* ws, size_t wsb,
                    void* stream) {
  return ctgb::dispatch(p, CTGB_OP_PROJECTION, image, sino, batch, ws, wsb, stream);
}
int ctgb_projection_t(const ctgb_plan* p, const void* sino, void* image, int batch, void* ws, size_t wsb,
                      void* stream) {
  return ctgb::dispatch(p, CTGB_OP_PROJECTION_T, sino, image, batch, ws, wsb, stream);
}
int ctgb_backprojection(const ctgb_plan* p, const void* sino, void* image, int batch, void* ws, size_t wsb,
                        void* stream) {
  return ctgb::dispatch(p, CTGB_OP_BACKPROJECTION, sino, image, batch, ws, wsb, stream);
}
int ctgb_backprojection_t(const ctgb_plan* p, const void* image, void* sino, int batch, void* ws, size_t wsb,
                          void* stream) {
  return ctgb::dispatch(p, CTGB_OP_BACKPROJECTION_T, image, sino, batch, ws, wsb, stream);
}
int ctgb_fbp(const ctgb_plan* p, const void* sino, void* image, int batch, void* ws, size_t wsb, void* stream) {
  return ctgb::dispatch(p, CTGB_OP_FBP, sino, image, batch, ws, wsb, stream);
}

long ctgb_geometry_query(const double* options, int n_options, int dtype, int what, double* out, size_t n_out) {
  ctgb::HostGeom g;
  std::string err;
  if (!ctgb::build_geometry(options, n_options, dtype, g, err)) {
    ctgb::fail(CTGB_ERR_INVALID, err);
    return -1;
  }
  std::vector<double> flags(g.flags.begin(), g.flags.end());
  const std::vector<double>* src = nullptr;
  switch (what) {
    case 0: src = &flags; break;
    case 1: src = &g.db; break;
    case 2: src = &g.fq; break;
    case 3: src = &g.lp; break;
    case 4: src = &g.inv; break;
    case 5: src = &g.wpre; break;
    case 6: src = &g.taps; break;
    default: ctgb::fail(CTGB_ERR_INVALID, "unknown geometry table"); return -1;
  }
  if (out) {
    const size_t n = std::min(n_out, src->size());
    std::memcpy(out, src->data(), n * sizeof(double));
  }
  return (long)src->size();
}

}  // extern "C"
