// Distance-driven CT operators for GB300 (sm_103a) behind the C ABI in ctgb.h.
//
// Every operator is an atomic-free gather over the overlap of two increasing
// boundary lists on a common axis (per view: D+1 detector-cell boundaries;
// per view and image line: W+1 or H+1 pixel edges, affine in the edge index):
//
//   detector gather (A, B^T): one thread per (view, detector cell) walks all
//     image lines of its view; per line it maps its two cell boundaries into
//     pixel-edge coordinates (one FMA each) and sums the 1-3 overlapped pixels.
//     A CTA is 4 or 8 consecutive views x 32 consecutive cells, so its warps
//     read nearly the same pixels of the same line and share them through L1.
//   image gather (A^T, B): one thread per pixel (or 2-4 pixel rows) walks all
//     views; per view it maps its lower pixel edge onto the axis, seeds the
//     detector cell (a per-tile quadratic of the closed-form inverse of the
//     boundary map), confirms or corrects it against the stored boundaries and
//     sums the 1-3 overlapped cells. A CTA is a 32-column pixel tile whose
//     footprint per view is a few dozen consecutive cells, staged by a producer
//     warp into a shared-memory ring with TMA bulk copies.
//
// Slices are processed SB at a time per thread (geometry computed once, SB
// fused multiply-adds per overlap); inputs are first re-laid out so that the
// SB values of one pixel / cell are one vector load. Sums over lines and views
// use blocked Kahan compensation (plain fp32 within a block of 32, compensated
// across blocks). The RL ramp filter of fbp is a direct convolution with the
// odd-tap structure of the RL kernel, fused with the detector pre-weight.
//
// Reference semantics followed: src/fan_ed_kernel.cu:24-943,
// src/fan_ea_kernel.cu:23-921, src/para_kernel.cu:8-683 (weights, flip and
// branch rules, Q3 factor of equal-angle B^T at src/fan_ea_kernel.cu:590-607).

#include <cuda.h>  // driver types only (CUcontext, CUresult); no libcuda link
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>
#include <vector>

#include "ctgb.h"
#include "ctgb_internal.h"
#include "geometry.h"

namespace ctgb {

// ----------------------------------------------------------------------------
// errors
// ----------------------------------------------------------------------------
static thread_local std::string g_err;

int fail(int code, const std::string& msg) {
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
// Coordinates are kept exact to ~1e-7 relative in fp32 by carrying every large
// quantity as an unevaluated (hi, lo) pair built from the fp64 plan, and by
// taking all differences that matter (cell boundary minus pixel edge) between
// nearby numbers only: the detector gather anchors each cell boundary to the
// integer pixel index it falls in and keeps the fraction, the image gather
// anchors each pixel edge to the cell it falls in and keeps the offset. A and
// A^T then evaluate the same overlaps to fp32 rounding, which keeps them
// adjoint to ~1e-7 and within ~1e-7 of the fp64 evaluation.
template <class T>
struct DevPlan {
  int V, D, W, H, L, scan;
  int Dp;             // padded_cells(D): row stride of cell records and sinogram planes
  int even_taps;      // fbp filter with non-zero even offsets (windowed kernels), besides the centre
  unsigned long long wait_ns;  // limit of each bounded wait in the staged image gather
  T dImg, s2r, dAng, wscale;
  // at least 1.5 units in the last place of the largest cell boundary (4 used):
  // db_hi[d+1] - db_hi[d] and w[d] differ by less, so an edge with
  // xs - db_hi[d] < w[d] - ub_margin lies below db_hi[d+1]
  T ub_margin;
  const int* flags;   // V
  const T* wsrc;      // V*2   weight source: equal-distance fans (sx, sy) / s2r^2, equal-angle (sx, sy)
  const T* db2;       // V*(D+1)*2  cell boundaries (hi, lo)
  const T* rec;       // V*Dp*4 cell records (db hi, db lo, width, next cell's width); zero past D
  const T* wd;        // V*D   cell widths
  const T* fq;        // V*D   A / A^T factor
  const T* fbt;       // V*D   EA B^T factor
  const T* lg;        // V*L*4 (1/sigma hi, 1/sigma lo, floor(beta), beta - floor(beta)), beta = -alpha/sigma
  const T* ls;        // V*L   sigma
  const T* lp;        // V*L*4 (alpha hi, alpha lo, sigma hi, sigma lo), hi parts on a common grid
  const float* inv;   // V*5   cell-index seed
  const T* rowc;      // H: row centre y
  const T* colc;      // W: column centre x
  const T* wpre;      // D
  const T* taps;      // 2D-1
  const T* tapl;      // 2D-1  fp64 taps minus taps (fp32 plans)
};

// Cells per row of the cell records and sinogram planes: D plus two padding
// cells (zero width, zero samples), rounded up to a multiple of 4. The image
// gather's straight-line steps read up to two cells past the pixel's first one
// without a range check; past D they read a padding cell, whose overlap is 0.
__host__ __device__ __forceinline__ int padded_cells(int D) { return (D + 2 + 3) & ~3; }

template <class T>
struct VecT;
template <>
struct VecT<float> { using v2 = float2; };
template <>
struct VecT<double> { using v2 = double2; };

template <class T>
struct Quad {
  T x, y, z, w;
};

template <class T>
__device__ __forceinline__ Quad<T> ld4(const T* p) {
  if constexpr (sizeof(T) == 4) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(p));
    return {a.x, a.y, a.z, a.w};
  } else {
    const double2 a = __ldg(reinterpret_cast<const double2*>(p));
    const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
    return {a.x, a.y, b.x, b.y};
  }
}

// SB slice values of one pixel / cell are stored as NQ planes of QW values;
// consecutive pixels (cells) of one plane are contiguous, so the lanes of a
// warp, which own consecutive cells (pixels), read contiguous vectors.
template <int SB>
struct Planes {
  static constexpr int QW = SB >= 4 ? 4 : SB;
  static constexpr int NQ = SB / QW;
};

template <class T, int QW>
__device__ __forceinline__ void load_q(const T* __restrict__ p, T* v) {
  if constexpr (sizeof(T) == 4 && QW == 4) {
    const float4 x = __ldg(reinterpret_cast<const float4*>(p));
    v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
  } else if constexpr (QW >= 2) {
    using V2 = typename VecT<T>::v2;
#pragma unroll
    for (int i = 0; i < QW / 2; ++i) {
      const V2 x = __ldg(reinterpret_cast<const V2*>(p) + i);
      v[2 * i] = x.x; v[2 * i + 1] = x.y;
    }
  } else {
    v[0] = __ldg(p);
  }
}

template <class T, int QW>
__device__ __forceinline__ void store_q(T* p, const T* v) {
  if constexpr (sizeof(T) == 4 && QW == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  } else if constexpr (QW >= 2) {
    using V2 = typename VecT<T>::v2;
#pragma unroll
    for (int i = 0; i < QW / 2; ++i) {
      V2 x; x.x = v[2 * i]; x.y = v[2 * i + 1];
      reinterpret_cast<V2*>(p)[i] = x;
    }
  } else {
    p[0] = v[0];
  }
}

// Round-to-nearest multiply / add that the compiler never contracts into an
// FMA: the two-product and two-sum steps below are exact only if the product
// and the sums they correct are the rounded ones.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
// correctly rounded 1/x (the value of T(1) / x)
__device__ __forceinline__ float rcp_rn(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rcp_rn(double x) { return __drcp_rn(x); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// Kahan fold of a block partial into a (sum, comp) pair kept in shared memory:
// the pair is touched once per kFoldEvery lines / views, so it need not hold
// registers; layout [2][SB][nt] (nt threads adding) keeps the accesses
// conflict-free. The partial is reset.
template <class T, int SB>
__device__ __forceinline__ void kahan_fold_smem(T* acc, T (&blk)[SB], int nt) {
  const int t = threadIdx.x;
#pragma unroll
  for (int s = 0; s < SB; ++s) {
    T* sum = acc + (size_t)s * nt + t;
    T* comp = acc + (size_t)(SB + s) * nt + t;
    const T y = sub_rn(blk[s], *comp);
    const T tt = add_rn(*sum, y);
    *comp = sub_rn(sub_rn(tt, *sum), y);
    *sum = tt;
    blk[s] = T(0);
  }
}

template <class T, int SB>
__device__ __forceinline__ void kahan_init_smem(T* acc, int nt) {
#pragma unroll
  for (int s = 0; s < 2 * SB; ++s) acc[(size_t)s * nt + threadIdx.x] = T(0);
}

enum Kind { kA = 0, kBt = 1, kAt = 2, kB = 3 };
constexpr int kFoldEvery = 32;
// Straight-line pixels per cell (cells per pixel) before the remainder loop: U
// = 3 or 2 per operator (ctgb_plan_set_unroll), 3 unless tuned.



// ----------------------------------------------------------------------------
// L2 warm-up of plan tables
// ----------------------------------------------------------------------------
// The gathers read per-view / per-line tables with little reuse per CTA; after
// an L2 flush their first touches go to HBM one dependent load at a time. The
// layout kernel that runs right before each gather asks the TMA unit to pull
// those tables into L2 with bulk prefetches of 64 KB (no registers, no smem).
struct PrefetchList {
  const void* ptr[6];
  unsigned long long bytes[6];
  int n;
};
constexpr unsigned kPrefetchChunk = 64u << 10;

__device__ __forceinline__ void l2_prefetch_bulk(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// CTA b (thread 0) prefetches chunk b, b + gridDim.x, ... of the concatenated
// list, visiting only its own chunks (a handful of steps, so the warp holding
// thread 0 is not held back from its share of the layout work)
__device__ __forceinline__ void prefetch_tables(const PrefetchList& L) {
  if (threadIdx.x != 0) return;
  unsigned long long first = 0;  // global index of table t's first chunk
  unsigned long long c = blockIdx.x;
  for (int t = 0; t < L.n; ++t) {
    const unsigned long long nb = L.bytes[t];
    const unsigned long long nch = (nb + kPrefetchChunk - 1) / kPrefetchChunk;
    for (; c < first + nch; c += gridDim.x) {
      const unsigned long long off = (c - first) * kPrefetchChunk;
      unsigned len = (unsigned)((nb - off) < kPrefetchChunk ? (nb - off) : kPrefetchChunk);
      len &= ~15u;  // bulk prefetch sizes are multiples of 16 bytes
      if (len) l2_prefetch_bulk(static_cast<const unsigned char*>(L.ptr[t]) + off, len);
    }
    first += nch;
  }
}

// ----------------------------------------------------------------------------
// layout kernels
// ----------------------------------------------------------------------------
// Pixel-blocked line layout of the detector gather: a line is a run of blocks
// of 8 pixels, each block holding the block's NQ planes of 8 x QW values, so the
// planes of pixel k lie at fixed offsets (qd * 8 * QW) from blk_off(k) and the
// lanes of a warp, which read consecutive pixels, still read whole 128-byte
// lines. With one plane (SB = 1) the layout is the plain row [N].
template <int SB>
__host__ __device__ __forceinline__ int blk_off(int k) {
  constexpr int QW = Planes<SB>::QW, NQ = Planes<SB>::NQ;
  return ((k >> 3) * NQ * 8 + (k & 7)) * QW;
}
__host__ __device__ __forceinline__ int round8(int n) { return (n + 7) & ~7; }

// image [B][H][W] -> row lines [G][H][blocked W] and column lines [G][W][blocked
// H] (column walk index k = H-1-row), zero-padded to G*SB slices; a line holds
// round8(N) * SB values
template <class T, int SB>
__global__ void k_layout_image(const T* __restrict__ img, T* __restrict__ imx, T* __restrict__ imy, int B,
                               int H, int W, int G, PrefetchList pf) {
  constexpr int QW = Planes<SB>::QW, NQ = Planes<SB>::NQ;
  prefetch_tables(pf);
  const size_t sx = (size_t)round8(W) * SB, sy = (size_t)round8(H) * SB;
  const int rows = G * NQ * H;  // (g, qd, r), r fastest; a CTA walks the columns of one row
  for (int row = blockIdx.x; row < rows; row += gridDim.x) {
    const int r = row % H, qd = (row / H) % NQ, g = row / (H * NQ);
    T* ox = imx + ((size_t)g * H + r) * sx + qd * 8 * QW;
    T* oy = imy + (size_t)g * W * sy + blk_off<SB>(H - 1 - r) + qd * 8 * QW;
    for (int c = threadIdx.x; c < W; c += blockDim.x) {
      T v[QW];
#pragma unroll
      for (int j = 0; j < QW; ++j) {
        const int b = g * SB + qd * QW + j;
        v[j] = b < B ? img[((size_t)b * H + r) * W + c] : T(0);
      }
      store_q<T, QW>(ox + blk_off<SB>(c), v);
      store_q<T, QW>(oy + (size_t)c * sy, v);
    }
  }
}

// sinogram [B][V][D] (external detector order) -> [G][V][NQ][Dp][QW]
// (increasing-boundary order, zero past D), times an optional per-(view, cell)
// factor
template <class T, int SB>
__global__ void k_layout_sino(const T* __restrict__ y, T* __restrict__ q, const int* __restrict__ flags,
                              const T* __restrict__ f, int B, int V, int D, int Dp, int G, PrefetchList pf) {
  constexpr int QW = Planes<SB>::QW, NQ = Planes<SB>::NQ;
  prefetch_tables(pf);
  const int rows = G * V * NQ;  // (g, v, qd), qd fastest; a CTA walks the cells of one row
  for (int row = blockIdx.x; row < rows; row += gridDim.x) {
    const int qd = row % NQ, v = (row / NQ) % V, g = row / (NQ * V);
    const bool flip = flags[v] & 2;
    T* out = q + (size_t)row * Dp * QW;
    for (int d = threadIdx.x; d < Dp; d += blockDim.x) {
      T val[QW];
      if (d < D) {
        const int de = flip ? D - 1 - d : d;
        const T fac = f ? f[(size_t)v * D + d] : T(1);
#pragma unroll
        for (int j = 0; j < QW; ++j) {
          const int b = g * SB + qd * QW + j;
          val[j] = b < B ? y[((size_t)b * V + v) * D + de] * fac : T(0);
        }
      } else {
#pragma unroll
        for (int j = 0; j < QW; ++j) val[j] = T(0);
      }
      store_q<T, QW>(out + (size_t)d * QW, val);
    }
  }
}

// ----------------------------------------------------------------------------
// backprojector pixel weights
// ----------------------------------------------------------------------------
// The sums of two products are written as one explicit FMA over one rounded
// product: left to the compiler, which product it fuses can differ between
// inlined copies, and every copy (staged or global view, one or more pixels per
// thread, any schedule) must give the same weight bit for bit.
// U^2 weight (src/fan_ed_kernel.cu:18-21): r^2 / (r - d)^2, d = (sx x + sy y) / r
// the pixel's distance along the source direction. Written 1 / t^2 with
// t = 1 - (sx / r^2) x - (sy / r^2) y, where (nx, ny) = (sx, sy) / r^2 comes per
// view from the plan (wsrc, formed in fp64), so that one division is left for
// the caller to fold with its other divisors.
template <class T>
__device__ __forceinline__ T ued_base(T nx, T ny, T x, T y) {
  return T(1) - fma(nx, x, mul_rn(ny, y));
}
// squared source distance (src/fan_ea_kernel.cu:18-20), used as a divisor
template <class T>
__device__ __forceinline__ T dist2_ea(T sx, T sy, T x, T y) {
  const T ex = sx - x, ey = sy - y;
  return fma(ex, ex, mul_rn(ey, ey));
}

// ----------------------------------------------------------------------------
// detector gather: A (kind kA) and B^T (kind kBt)
// ----------------------------------------------------------------------------
// Thread = (view v, cell d), SB slices. Per line: the cell's lower boundary in
// pixel-edge units is u = db*(1/sigma) + beta; it is split into an integer
// anchor k and a fraction f computed from exact products (two-product via FMA),
// and the cell spans [f, f + w/sigma) pixels from k on.
// Residual epilogue of the data-term gradient (RES): r = A x - y for the
// measured sinogram y (B x V x D), written to `res` (same layout, may be null)
// and, times the A^T factor fq, straight into the image gather's input layout
// q[G][V][NQ][Dp][QW] (increasing-boundary cell order), so A^T(Ax - y) needs no
// separate subtraction or re-layout of the sinogram.
template <class T>
struct ResidualOut {
  const T* y;
  T* res;
  T* q;
};

template <class T, int SB, int KIND, int U, bool RES = false, bool PLAIN = false>
__device__ __forceinline__ void det_gather_cell(const DevPlan<T>& P, int v, int d, int g, const T* __restrict__ imx,
                                                const T* __restrict__ imy, size_t sx_line, size_t sy_line,
                                                T* __restrict__ out, int B, ResidualOut<T> ro = {}) {
  // row lines of slice group g start at imx + g*H*sx_line, column lines at
  // imy + g*W*sy_line; a line is pixel-blocked (blk_off)
  constexpr int QW = Planes<SB>::QW, NQ = Planes<SB>::NQ;
  const int fl = P.flags[v];
  const bool xb = fl & 1;
  const int nlines = xb ? P.H : P.W;
  const int N = xb ? P.W : P.H;
  const size_t stride = xb ? sx_line : sy_line;
  const T* base = xb ? imx + (size_t)g * P.H * sx_line : imy + (size_t)g * P.W * sy_line;
  const size_t bi = ((size_t)v * (P.D + 1) + d) * 2;
  const T Dh = P.db2[bi], Dl = P.db2[bi + 1];
  const T wcell = P.wd[(size_t)v * P.D + d];
  const T* lgv = P.lg + (size_t)v * P.L * 4;
  const T* lsv = P.ls + (size_t)v * P.L;
  T sx = T(0), sy = T(0);
  if (KIND == kBt && P.scan != kPara) { sx = P.wsrc[2 * v]; sy = P.wsrc[2 * v + 1]; }
  const T pc0 = xb ? P.colc[0] : P.rowc[P.H - 1];  // centre of pixel k = 0 along the walk

  extern __shared__ unsigned char det_smem[];
  T* acc = reinterpret_cast<T*>(det_smem);  // [2][SB][blockDim]: running sum, compensation
  kahan_init_smem<T, SB>(acc, blockDim.x);
  T blk[SB];
#pragma unroll
  for (int s = 0; s < SB; ++s) blk[s] = T(0);

  auto G4n = ld4<T>(lgv);
  T sign = lsv[0];
  for (int l = 0; l < nlines; ++l) {
    const auto G4 = G4n;
    const T sig = sign;
    if (l + 1 < nlines) {  // next line's map, loaded while this line is walked
      G4n = ld4<T>(lgv + 4 * (l + 1));
      sign = lsv[l + 1];
    }
    const T ph = mul_rn(Dh, G4.x);
    const T pl = fma(Dh, G4.x, -ph);
    const T corr = add_rn(fma(Dl, G4.x, fma(Dh, G4.y, pl)), G4.w);
    const T kaf = floor(add_rn(add_rn(ph, G4.z), corr));
    T f = add_rn(sub_rn(ph, sub_rn(kaf, G4.z)), corr);
    int k = (int)kaf;
    if (f < T(0)) { f += T(1); --k; }
    T a = f;
    T b = fma(wcell, G4.x, f);
    if (k < 0) {  // cell starts left of the image: move to pixel 0
      const T sh = T(-k);
      a -= sh;
      b -= sh;
      k = 0;
    }
    if (k >= N || b <= T(0)) {
      if (!PLAIN && (l % kFoldEvery) == kFoldEvery - 1) kahan_fold_smem<T, SB>(acc, blk, blockDim.x);
      continue;
    }
    // pixels past the line's end take no weight: with b clamped to N - k their
    // overlaps come out <= 0 (the clamp is exact, N - k is an integer)
    b = fmin(b, T(N - k));
    const T* row = base + (size_t)l * stride;
    T lc = T(0);
    if (KIND == kBt && P.scan != kPara) lc = xb ? P.rowc[l] : P.colc[l];
    // weight of pixel kk (overlap ov in pixel units, ov >= 0)
    auto weight = [&](T ov, int kk) {
      T w = ov;
      if (KIND == kA) {
        w *= sig;
      } else if (P.scan == kFanED) {
        const T pc = fma(T(kk), P.dImg, pc0);
        const T t = xb ? ued_base(sx, sy, pc, lc) : ued_base(sx, sy, lc, pc);
        w /= t * t;
      } else if (P.scan == kFanEA) {
        const T pc = fma(T(kk), P.dImg, pc0);
        w /= xb ? dist2_ea(sx, sy, pc, lc) : dist2_ea(sx, sy, lc, pc);
      }
      return w;
    };
    // first U pixels straight-line: all overlaps, then all loads, then all
    // FMAs (steps past the cell or the line get weight 0 on a clamped, valid
    // pixel), so the loads of one line are in flight together. The overlap of
    // pixel k+j is min(b-j, 1) - max(a-j, 0); a < 2, so from j = 2 on the
    // second term is 0.
    T wj[U];
    int oj[U];
#pragma unroll
    for (int j = 0; j < U; ++j) {
      const T hi = fmin(b - T(j), T(1));
      const T ov = j < 2 ? hi - fmax(a - T(j), T(0)) : hi;
      const int kk = min(k + j, N - 1);
      oj[j] = blk_off<SB>(kk);
      // 0 where the pixel is not reached (A: a max instead of a compare and a
      // select; B^T keeps the select, which measured faster around its division)
      if (KIND == kA) wj[j] = weight(fmax(ov, T(0)), kk);
      else wj[j] = ov > T(0) ? weight(ov, kk) : T(0);
    }
#pragma unroll
    for (int qd = 0; qd < NQ; ++qd) {
      T u[U][QW];
#pragma unroll
      for (int j = 0; j < U; ++j) load_q<T, QW>(row + oj[j] + qd * 8 * QW, u[j]);
#pragma unroll
      for (int j = 0; j < U; ++j)
#pragma unroll
        for (int i = 0; i < QW; ++i) blk[qd * QW + i] = fma(wj[j], u[j][i], blk[qd * QW + i]);
    }
    // rare: a cell wider than U - 1 pixels
    for (int j = U; b - T(j) > T(0); ++j) {
      const T ov = fmin(b - T(j), T(1));
      const T w = weight(ov, k + j);
      const T* px = row + blk_off<SB>(k + j);
#pragma unroll
      for (int qd = 0; qd < NQ; ++qd) {
        T u[QW];
        load_q<T, QW>(px + qd * 8 * QW, u);
#pragma unroll
        for (int i = 0; i < QW; ++i) blk[qd * QW + i] = fma(w, u[i], blk[qd * QW + i]);
      }
    }
    if (!PLAIN && (l % kFoldEvery) == kFoldEvery - 1) kahan_fold_smem<T, SB>(acc, blk, blockDim.x);
  }
  kahan_fold_smem<T, SB>(acc, blk, blockDim.x);
  T fac = T(1);
  if (KIND == kA) fac = P.fq[(size_t)v * P.D + d];
  else if (P.scan == kFanEA) fac = P.fbt[(size_t)v * P.D + d];
  const int de = (fl & 2) ? P.D - 1 - d : d;
  if constexpr (RES) {
    constexpr int QW = Planes<SB>::QW, NQ = Planes<SB>::NQ;
#pragma unroll
    for (int qd = 0; qd < NQ; ++qd) {
      T vals[QW];
#pragma unroll
      for (int i = 0; i < QW; ++i) {
        const int s = qd * QW + i, bb = g * SB + s;
        T r = T(0);
        if (bb < B) {
          const size_t e = ((size_t)bb * P.V + v) * P.D + de;
          // rounded as projection's output, then the subtraction (no contraction)
          r = sub_rn(mul_rn(acc[(size_t)s * blockDim.x + threadIdx.x], fac), ro.y[e]);
          if (ro.res) ro.res[e] = r;
        }
        vals[i] = mul_rn(r, fac);
      }
      T* qrow = ro.q + (((size_t)g * P.V + v) * NQ + qd) * P.Dp * QW;
      store_q<T, QW>(qrow + (size_t)d * QW, vals);
      if (d == P.D - 1) {  // the row's padding cells
#pragma unroll
        for (int i = 0; i < QW; ++i) vals[i] = T(0);
        for (int dd = P.D; dd < P.Dp; ++dd) store_q<T, QW>(qrow + (size_t)dd * QW, vals);
      }
    }
  } else {
#pragma unroll
    for (int s = 0; s < SB; ++s) {
      const int bb = g * SB + s;
      if (bb < B) out[((size_t)bb * P.V + v) * P.D + de] = acc[(size_t)s * blockDim.x + threadIdx.x] * fac;
    }
  }
}

// Register cap: 96 for the two-step fp32 kernels, where holding a whole line's
// loads in flight beats the extra warps (2.53 against 2.79 ms for A on the
// 16-slice fan-ED 512 batch); 72 for the three-step and fp64 ones.
template <class T, int U>
constexpr int det_max_regs() { return (sizeof(T) == 4 && U == 2) ? 96 : 72; }

template <class T, int SB, int KIND, int U, bool RES = false, bool PLAIN = false>
__global__ void __maxnreg__((det_max_regs<T, U>())) k_det_gather(DevPlan<T> P, const T* __restrict__ imx,
                                                    const T* __restrict__ imy, T* __restrict__ out, int B,
                                                    ResidualOut<T> ro) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int d = blockIdx.x * 32 + lane;
  const int v = blockIdx.y * (blockDim.x >> 5) + warp;
  if (v >= P.V || d >= P.D) return;
  det_gather_cell<T, SB, KIND, U, RES, PLAIN>(P, v, d, blockIdx.z, imx, imy, (size_t)round8(P.W) * SB,
                                       (size_t)round8(P.H) * SB, out, B, ro);
}

// ----------------------------------------------------------------------------
// mbarrier and bulk-copy primitives (PTX, sm_90 and later)
// ----------------------------------------------------------------------------
// Every wait is bounded: after the plan's wait limit (DevPlan::wait_ns, 1 s by
// default) of polling it gives up, the kernel counts the event in
// g_wait_timeouts and falls back to global loads, so a stalled copy can never
// hang the GPU. A limit of 0 makes a wait give up unless its phase has already
// completed at the first try (ctgb_plan_set_wait_limit: the fallback path on
// demand, for tests). The producer's final drain of copies in flight always
// allows kWaitLimitNs, whatever the plan's limit.
constexpr unsigned long long kWaitLimitNs = 1000000000ull;  // 1 s
__device__ unsigned long long g_wait_timeouts;

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// wait for the completion of the phase of parity `parity`; false if it did not
// complete within `limit_ns` (0: only the first try)
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  if (limit_ns == 0) return false;
  const unsigned long long t0 = global_ns();
  for (unsigned i = 1; i < (1u << 30); ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 0 && global_ns() - t0 > limit_ns) break;
  }
  return false;
}
// global -> shared bulk copy (TMA), completion counted in bytes on `bar`;
// both addresses 16-byte aligned, size a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ int ld_volatile(const int& x) { return *reinterpret_cast<const volatile int*>(&x); }
__device__ __forceinline__ void report_timeout(int* bad) {
  *reinterpret_cast<volatile int*>(bad) = 1;
  atomicAdd(&g_wait_timeouts, 1ull);
}

// ----------------------------------------------------------------------------
// image gather: A^T (kind kAt) and B (kind kB)
// ----------------------------------------------------------------------------
// Thread = pixel (r, c), SB slices, loop over views. Per view the pixel's lower
// edge x = alpha + sigma*k is formed as an unevaluated pair (an exact high part
// from grid-aligned line maps, and a low part), its cell d is seeded and
// confirmed (or corrected) against the stored boundaries, and the offset
// a = x - db[d] is taken between the two nearby pairs; the cells then follow by
// widths.
//
// Cells are read through records rec[d] = (db_hi[d], db_lo[d], w[d],
// w[d+1]) and sinogram planes q[qd][d][QW] with plane stride qs; `rec` and
// `q` point at cell `base`; the search stays in [dlo, dhi), and the straight-
// line steps read at most two padding cells past it. The same code runs on a
// shared-memory window of the cells (SM, seeded per tile) and on the global
// tables (seeded by the closed form), with identical arithmetic past the seed.

template <class T, bool SM>
__device__ __forceinline__ Quad<T> ldrec(const T* p) {
  if constexpr (!SM) {
    return ld4<T>(p);
  } else if constexpr (sizeof(T) == 4) {
    const float4 a = *reinterpret_cast<const float4*>(p);
    return {a.x, a.y, a.z, a.w};
  } else {
    const double2 a = reinterpret_cast<const double2*>(p)[0];
    const double2 b = reinterpret_cast<const double2*>(p)[1];
    return {a.x, a.y, b.x, b.y};
  }
}

template <class T, int QW, bool SM>
__device__ __forceinline__ void ldq(const T* __restrict__ p, T* v) {
  if constexpr (!SM) {
    load_q<T, QW>(p, v);
  } else if constexpr (sizeof(T) == 4 && QW == 4) {
    const float4 x = *reinterpret_cast<const float4*>(p);
    v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
  } else if constexpr (QW >= 2) {
    using V2 = typename VecT<T>::v2;
#pragma unroll
    for (int i = 0; i < QW / 2; ++i) {
      const V2 x = reinterpret_cast<const V2*>(p)[i];
      v[2 * i] = x.x; v[2 * i + 1] = x.y;
    }
  } else {
    v[0] = p[0];
  }
}

// Per-view constants of the closed-form inverse of the boundary map:
// u = x*a / (x*c + b) (atan'ed for equal-angle fans), cell = e*u + d.
struct Seed {
  float a, b, c, d, e;
};
__device__ __forceinline__ Seed load_seed(const float* p) { return {p[0], p[1], p[2], p[3], p[4]}; }

// fp32 cell coordinate of axis coordinate x (cell d spans [d, d + 1)), unclamped
__device__ __forceinline__ float seed_coord(int scan, float xf, const Seed& sd) {
  float u = __fdividef(xf * sd.a, fmaf(xf, sd.c, sd.b));
  if (scan == kFanEA) u = atanf(u);
  return fmaf(sd.e, u, sd.d);
}

// fp32 seed of the cell holding axis coordinate x, clamped to [dlo, dhi) (the
// conversion saturates, and maps NaN to 0)
__device__ __forceinline__ int seed_cell(int scan, float xf, const Seed& sd, int dlo, int dhi) {
  return min(max(__float2int_rz(seed_coord(scan, xf, sd)), dlo), dhi - 1);
}

// Seed of a staged view: the cell coordinate as a quadratic in x, interpolating
// the closed form at the ends and the middle of the tile's edge range. Over the
// few dozen cells a tile spans the map is nearly linear, so the quadratic lands
// within a small fraction of a cell; like the closed form it only starts the
// search, so it changes no result.
struct QuadSeed {
  float c0, c1, c2;  // cell = c0 + c1 x + c2 x^2
};
__device__ __forceinline__ int seed_cell(int, float xf, const QuadSeed& sd, int dlo, int dhi) {
  return min(max(__float2int_rz(fmaf(xf, fmaf(xf, sd.c2, sd.c1), sd.c0)), dlo), dhi - 1);
}

// Where one view meets one pixel: the pixel's first U cells (offsets oj from
// `base`, overlap weights ov) and the state the remainder loop resumes from.
template <class T, int U>
struct CellSpan {
  int d;     // first cell after the straight-line ones
  T a, b;    // pixel edges relative to cell d's lower boundary
  T wv;      // backprojector view weight
  T ov[U];
  int oj[U];
};

// Geometry of one view for one pixel (lower edge index k on its line, line
// map A4): exact edge, seeded and corrected cell search, U straight-line
// overlaps. Cells past the pixel get weight 0; the straight-line steps may run
// up to U - 1 cells past dhi, onto the zero-width padding cells of the tables
// (or of a staged window, which always holds them when it reaches D).
template <class T, int KIND, int U, bool SM, class SeedT>
__device__ __forceinline__ void pix_geom(const DevPlan<T>& P, const Quad<T>& A4, T kf, const SeedT& sd, T sx, T sy,
                                         T pcx, T pcy, const T* __restrict__ rec, int base, int dlo, int dhi,
                                         CellSpan<T, U>& cs) {
  // x = alpha + sigma*k as (xs, xl): the line map's high parts lie on a grid
  // that makes alpha_hi + sigma_hi*k exact for every edge of the line
  const T xs = fma(A4.z, kf, A4.x);
  const T xl = fma(A4.w, kf, A4.y);
  // The cell: db_hi[d] <= xs < db_hi[d+1], d in [dlo, dhi), then one cell back
  // if the offset of the edge into it, taken between the two nearby pairs, is
  // negative. The seed is almost always that cell with a non-negative offset,
  // which one test confirms (conservatively: an edge within ub_margin of the
  // upper boundary takes the search); otherwise the search walks from the seed.
  // A record carries the next cell's width (w1) instead of its boundary.
  int d = seed_cell(P.scan, (float)xs, sd, dlo, dhi);
  Quad<T> rd = ldrec<T, SM>(rec + (d - base) * 4);
  const T off = sub_rn(xs, rd.x);
  T a = add_rn(off, sub_rn(xl, rd.y));
  T w0 = rd.z, w1 = rd.w;
  if (!(rd.x <= xs && off < rd.z - P.ub_margin && a >= T(0))) {
    while (d > dlo && xs < rd.x) {
      --d;
      rd = ldrec<T, SM>(rec + (d - base) * 4);
    }
    while (d < dhi - 1 && rec[(d + 1 - base) * 4] <= xs) {  // db_hi[d+1]; none after a step down
      ++d;
      rd = ldrec<T, SM>(rec + (d - base) * 4);
    }
    a = add_rn(sub_rn(xs, rd.x), sub_rn(xl, rd.y));
    w0 = rd.z;
    w1 = rd.w;
    if (a < T(0) && d > dlo) {
      --d;
      w1 = w0;
      w0 = rec[(d - base) * 4 + 2];
      a += w0;
    }
  }
  const T sig = A4.z + A4.w;
  T b = a + sig;
  // backprojector view weight of this pixel (U^2 / sigma, 1 / (L^2 sigma),
  // 1 / dImg), folded into each cell's overlap weight
  T wv = T(1);
  if (KIND == kB) {
    if (P.scan == kFanED) {
      const T t = ued_base(sx, sy, pcx, pcy);
      wv = rcp_rn(t * t * sig);
    }
    else if (P.scan == kFanEA) wv = rcp_rn(dist2_ea(sx, sy, pcx, pcy) * sig);
    else wv = rcp_rn(P.dImg);
  }
#pragma unroll
  for (int j = 0; j < U; ++j) {
    cs.oj[j] = d + j - base;
    const T w = j == 0 ? w0 : (j == 1 ? w1 : rec[cs.oj[j] * 4 + 2]);
    const T ov = fmax(fmin(b, w) - fmax(a, T(0)), T(0));
    cs.ov[j] = KIND == kB ? ov * wv : ov;
    a -= w;
    b -= w;
  }
  cs.d = d + U;
  cs.a = a;
  cs.b = b;
  cs.wv = wv;
}

// The sums of one view's span into blk: U straight-line cells, then the rare
// remainder (cells past the U-th one that the pixel still reaches)
template <class T, int SB, int KIND, int U, bool SM>
__device__ __forceinline__ void pix_accum(const CellSpan<T, U>& cs, const T* __restrict__ rec,
                                          const T* __restrict__ qv, int qs, int base, int dhi, T (&blk)[SB]) {
  constexpr int QW = Planes<SB>::QW, NQ = Planes<SB>::NQ;
#pragma unroll
  for (int qd = 0; qd < NQ; ++qd) {
    T qq[U][QW];
#pragma unroll
    for (int j = 0; j < U; ++j) ldq<T, QW, SM>(qv + (qd * qs + cs.oj[j]) * QW, qq[j]);
#pragma unroll
    for (int j = 0; j < U; ++j)
#pragma unroll
      for (int i = 0; i < QW; ++i) blk[qd * QW + i] = fma(cs.ov[j], qq[j][i], blk[qd * QW + i]);
  }
  T a = cs.a, b = cs.b;
  if (!(b > T(0))) return;
  for (int d = cs.d; b > T(0) && d < dhi; ++d) {
    const T w = rec[(d - base) * 4 + 2];
    T ov = fmin(b, w) - fmax(a, T(0));
    if (ov > T(0)) {
      if (KIND == kB) ov *= cs.wv;
#pragma unroll
      for (int qd = 0; qd < NQ; ++qd) {
        T qq[QW];
        ldq<T, QW, SM>(qv + (qd * qs + (d - base)) * QW, qq);
#pragma unroll
        for (int i = 0; i < QW; ++i) blk[qd * QW + i] = fma(ov, qq[i], blk[qd * QW + i]);
      }
    }
    a -= w;
    b -= w;
  }
}

// one view's contribution to one pixel, accumulated into blk
template <class T, int SB, int KIND, int U, bool SM, class SeedT>
__device__ __forceinline__ void pix_view(const DevPlan<T>& P, const Quad<T>& A4, T kf, const SeedT& sd, T sx, T sy,
                                         T pcx, T pcy, const T* __restrict__ rec, const T* __restrict__ qv, int qs,
                                         int base, int dlo, int dhi, T (&blk)[SB]) {
  CellSpan<T, U> cs;
  pix_geom<T, KIND, U, SM>(P, A4, kf, sd, sx, sy, pcx, pcy, rec, base, dlo, dhi, cs);
  pix_accum<T, SB, KIND, U, SM>(cs, rec, qv, qs, base, dhi, blk);
}

// view v of pixel (r, c), everything read from the global tables; q planes of
// view v start at qv with stride qs
template <class T, int SB, int KIND, int U>
__device__ __forceinline__ void pix_view_global(const DevPlan<T>& P, int v, int r, int c, const T* __restrict__ qv,
                                                int qs, T pcx, T pcy, T (&blk)[SB]) {
  const bool xb = P.flags[v] & 1;
  const int k = xb ? c : P.H - 1 - r;
  const Quad<T> A4 = ld4<T>(P.lp + ((size_t)v * P.L + (xb ? r : c)) * 4);
  pix_view<T, SB, KIND, U, false>(P, A4, T(k), load_seed(P.inv + (size_t)v * 5), P.wsrc[2 * v], P.wsrc[2 * v + 1], pcx,
                                  pcy, P.rec + (size_t)v * P.Dp * 4, qv, qs, 0, 0, P.D, blk);
}

// Parts per tile of the staged image gather: a tile's views are split into
// consecutive parts of at least 128 views, up to 8, each part its own CTA.
// Shorter CTAs fill the last wave of a grid that is only a few waves deep (one
// 512^2 slice of 1152 views is 2048 CTAs, 3.4 waves of 608 resident ones).
// Small images (at most 2^17 pixels) have few tiles, so their views split
// finer, into parts of at least 40 views (one 256^2 slice is 128 tiles of
// 32 x 16 pixels: with 360 views, 1024 CTAs instead of 256). Each part writes
// its scaled sum to its own partial image and k_combine_parts adds the parts
// in order, from zero, so the result does not depend on which CTA finishes
// first. The split depends on the plan alone (views and image size), never on
// the batch or the schedule, so every schedule gives the same result bit for
// bit; the ragged path sums the same parts in the same order and matches too.
__host__ __device__ __forceinline__ int view_split(int views, long long pixels) {
  if (pixels <= (1 << 17)) return views < 80 ? 1 : min(8, views / 40);
  return views < 256 ? 1 : (views >= 1024 ? 8 : views / 128);
}

// Staged image gather. A CTA is a 32 x (R * PX) pixel tile plus one producer
// warp: R consumer warps, lane = column, and warp w owns rows w, w + R, ...,
// w + (PX - 1) R, so that the per-view costs of a warp (barrier, slot header,
// loop) are shared by PX pixels where few slices leave them poorly shared
// (PX = 2 up to 8 slices per thread). For each view the producer finds
// the tile's cell footprint from its four corner pixel edges (exact extremes:
// along a line the edges grow with k, and across lines each edge moves
// monotonically because the source lies outside the image), and when it fits
// the slot's window of cells it copies the cell records, the q planes of those
// cells and the tile's line maps into a ring of kSlots<T, SB> shared-memory slots with TMA bulk
// copies. Consumers then read only shared memory; a view whose footprint does
// not fit is read from the global tables instead (same arithmetic, same
// result). The window carries a margin of two cells on each side, so every cell
// a pixel can reach (including the seed correction and the step back when the
// offset is negative) lies inside it.
// pixel rows per consumer thread of the staged image gather: 2 up to 8 slices
// per thread, where the per-view costs are shared by few slices (A^T of one
// 512^2 slice, 1152 views: 2.10 to 1.65 ms, 4 rows 1.90 ms; of 8 slices: 2.25
// to 1.95 ms); 1 for 16 slices, whose 32 sums do not fit 72 registers (2 rows
// spill: 3.14 against 2.62 ms)
template <int SB>
constexpr int kPixRows = SB <= 8 ? 2 : 1;

template <class T, int SB>
struct PixSlot {
  // cells per staged view window (multiple of 4): one- and two-slice slots are
  // small, so they take the wider footprints of the taller pixel-blocked tiles
  static constexpr int kWin = SB <= 2 ? 128 : 64;
  static constexpr int kQBytes = SB * kWin * (int)sizeof(T);    // NQ planes x kWin cells x QW
  static constexpr int kRecBytes = kWin * 4 * (int)sizeof(T);   // kWin records
  static constexpr int kLpBytes = 32 * 4 * (int)sizeof(T);      // up to 32 line maps
  static constexpr int kBytes = kQBytes + kRecBytes + kLpBytes;
};

// CTAs per SM of the staged image gather: four at one to four fp32 slices per
// thread, whose sums fit 56 registers and whose small slots leave room for four
// CTAs' rings (more warps to hide the shared-memory latency of an issue-bound
// loop; A^T of 2 and 4 512^2 slices: 1.05 -> 0.88 and 1.13 -> 1.05 ms); three
// otherwise (72 registers).
template <class T, int SB>
constexpr int kPixCtas = (sizeof(T) == 4 && SB <= 4) ? 4 : 3;

// Views in flight per CTA: as many slots as fit beside the Kahan sums of 8 row
// warps with kPixCtas CTAs per SM (228 KB of shared memory per SM, less 2 KB per
// CTA for the static arrays and the per-CTA reserve: 74 KB of dynamic shared
// memory each at three CTAs, 55 KB at four), at most 16. The ring has to cover
// the time from a slot's release by the slowest row warp to its refill
// landing; the few-slice slots are small, so those rings get deep (fp32: 16
// slots for one slice per thread, 15 with four pixel rows; 13 and 10 for two
// slices; 15 for four, 11 for eight, 7 for sixteen).
template <class T, int SB, int PX = kPixRows<SB>>
constexpr int kSlots = [] {
  constexpr int acc = 2 * PX * SB * 256 * (int)sizeof(T);
  constexpr int budget = 228 * 1024 / kPixCtas<T, SB> - 2048;
  constexpr int n = (budget - acc - 1024) / PixSlot<T, SB>::kBytes;
  return n > 16 ? 16 : (n < 4 ? 4 : n);
}();

// SV: single-view backprojection (src/fan_ed_kernel.cu:946-1161): each view's
// sum goes to its own image, img[slice][view][row][col], with no sum over views.
//
// nsplit: blockIdx.z = slice group * nsplit + part, and part p takes views
// [V*p/nsplit, V*(p+1)/nsplit). Summing operators use view_split(V, W*H) parts:
// with one, the CTA writes the output; with more, part p writes its scaled sum
// to partial image p of `parts` ([nsplit][B][H][W]) and k_combine_parts adds
// them. SV writes every view's image directly, so it takes any number of parts
// and no partial images.
//
// The CTA's work, (bx, by, bz) standing for its block index: k_pix_gather runs
// it over a regular grid, k_rag_pix_gather over a task list of several slices.
template <class T, int SB, int KIND, int U, bool SV, int PX, bool PLAIN>
__device__ __forceinline__ void pix_gather_cta(const DevPlan<T>& P, const T* __restrict__ q, T* __restrict__ img,
                                               T* __restrict__ parts, int B, T out_mul, T out_div, int nsplit,
                                               int bx, int by, int bz) {
  constexpr int QW = Planes<SB>::QW, NQ = Planes<SB>::NQ;
  using S = PixSlot<T, SB>;
  constexpr int kWin = S::kWin;
  constexpr int kSlots = ctgb::kSlots<T, SB, PX>;
  static_assert(NQ + 2 <= 32, "one producer lane per copy");
  __shared__ __align__(8) unsigned long long s_full[kSlots], s_empty[kSlots];
  // slot header: (window cell count or -1, flags, first line, seed c0) and seed
  // (c1, c2); the source position for the backprojector
  __shared__ int4 s_hdr[kSlots];
  __shared__ float2 s_qsd[kSlots];
  __shared__ T s_src[kSlots][2];
  __shared__ int s_bad;
  extern __shared__ __align__(16) unsigned char pix_smem[];
  const int R = (int)(blockDim.x >> 5) - 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int CT = 32 * R;                     // consumer threads
  T* acc = reinterpret_cast<T*>(pix_smem);  // [2][PX * SB][CT]: running sum, compensation
  unsigned char* slots = pix_smem + (size_t)2 * PX * SB * CT * sizeof(T);
  const int c0 = bx * 32, r0 = by * R * PX;
  const int part = bz % nsplit, g = bz / nsplit;
  const int V = P.V, D = P.D, Dp = P.Dp;
  const int vbeg = (int)((long long)V * part / nsplit), vend = (int)((long long)V * (part + 1) / nsplit);
  const int NV = vend - vbeg;  // views of this CTA; the slot of view vbeg + u is u % kSlots
  const T* qg = q + (size_t)g * V * Dp * SB;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kSlots; ++i) {
      mbar_init(&s_full[i], 1);
      mbar_init(&s_empty[i], R);
    }
    s_bad = 0;
    mbar_init_fence();
  }
  __syncthreads();

  if (warp == R) {  // producer
    const int c1 = min(c0 + 32, P.W) - 1, r1 = min(r0 + R * PX, P.H) - 1;
    // Per-view inputs of the window search, loaded for view vb + lane one batch
    // of 32 views ahead so that their latency overlaps the copies of the batch
    // before; the search itself (seed, then the bracketing boundaries) costs
    // one more dependent load, usually without correction steps.
    struct ViewIn {
      int fl;
      Seed sd;
      T sx, sy;
      Quad<T> A4[2];
    };
    auto load_in = [&](int v, ViewIn& in) {
      in.fl = 0;
      if (v >= vend) return;
      in.fl = P.flags[v];
      in.sd = load_seed(P.inv + (size_t)v * 5);
      in.sx = P.wsrc[2 * v];
      in.sy = P.wsrc[2 * v + 1];
      const bool xb = in.fl & 1;
      in.A4[0] = ld4<T>(P.lp + ((size_t)v * P.L + (xb ? r0 : c0)) * 4);
      in.A4[1] = ld4<T>(P.lp + ((size_t)v * P.L + (xb ? r1 : c1)) * 4);
    };
    // window start of view v, or -1 if the tile's footprint does not fit; qs:
    // the view's quadratic seed over the tile's edge range
    auto window = [&](int v, const ViewIn& in, int& l0, int& nl, QuadSeed& qs) {
      if (v >= vend) return -1;
      const bool xb = in.fl & 1;
      int ka, kb;
      if (xb) { ka = c0; kb = c1 + 1; l0 = r0; nl = r1 - r0 + 1; }
      else { ka = P.H - 1 - r1; kb = P.H - r0; l0 = c0; nl = c1 - c0 + 1; }
      const T* db2v = P.db2 + (size_t)v * (D + 1) * 2;
      T xs[4];
      int d[4];
      T lo_b[4], hi_b[4];
      // the corner edges' seeds, kept for the quadratic: the extremes of the
      // edge range are corner edges
      float xlo = 0.f, xhi = 0.f, flo = 0.f, fhi = 0.f;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const Quad<T>& A4 = in.A4[e & 1];
        xs[e] = add_rn(A4.x, mul_rn(A4.z, T((e & 2) ? kb : ka)));
        const float xf = (float)xs[e], fe = seed_coord(P.scan, xf, in.sd);
        if (e == 0 || xf < xlo) { xlo = xf; flo = fe; }
        if (e == 0 || xf > xhi) { xhi = xf; fhi = fe; }
        d[e] = (int)fminf(fmaxf(fe, 0.f), (float)(D - 1));
        lo_b[e] = db2v[2 * d[e]];
        hi_b[e] = db2v[2 * d[e] + 2];
      }
      int dmin = D, dmax = -1;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        int dd = d[e];
        if (dd > 0 && xs[e] < lo_b[e]) {
          do --dd; while (dd > 0 && xs[e] < db2v[2 * dd]);
        } else if (dd < D - 1 && hi_b[e] <= xs[e]) {
          do ++dd; while (dd < D - 1 && db2v[2 * dd + 2] <= xs[e]);
        }
        dmin = min(dmin, dd);
        dmax = max(dmax, dd);
      }
      {  // quadratic through the ends and the middle of [xlo, xhi]
        const float h = 0.5f * (xhi - xlo), xm = xlo + h;
        const float fm = seed_coord(P.scan, xm, in.sd), ih = __fdividef(0.5f, h);
        const float s1 = (fhi - flo) * ih, s2 = ((fhi - fm) - (fm - flo)) * ih * __fdividef(1.f, h);
        qs.c2 = s2;
        qs.c1 = fmaf(-2.f * s2, xm, s1);
        qs.c0 = fmaf(fmaf(s2, xm, -s1), xm, fm);
      }
      // two cells of margin, or up to the second padding cell past D
      const int lo = max(0, dmin - 2) & ~3;
      const int hi = min(D + 1, dmax + 2);
      return hi < lo + kWin ? lo : -1;
    };
    ViewIn cur, nxt;
    QuadSeed qsd{0.f, 0.f, 0.f};
    int ws, l0 = 0, nl = 0;
    load_in(vbeg + lane, cur);
    ws = window(vbeg + lane, cur, l0, nl, qsd);
    // Views issued so far (header written and the slot's full barrier armed).
    // Before use u of a slot the producer waits until the consumers released
    // use u - 1 (empty) and until use u - 1's copies landed (full), so at most
    // one phase of each full barrier is ever pending. Once a wait has run out
    // (here or in a consumer, s_bad), the producer issues nothing more: no
    // header, arrive or copy, since an arrive on a phase still waiting for its
    // bytes would exceed that phase's expected count.
    // Views go out in rounds of kRound: the lanes of a round's views wait for
    // their slots, write their headers and arm their full barriers side by
    // side, then kCopies lanes per view issue its copies, so that a round costs
    // the serial steps of one view. (One view per step left the row warps
    // waiting for their slots 28% of the time at 16 slices per thread: the
    // producer, one warp among the SM's busy row warps, could not keep the
    // ring ahead.)
    constexpr int kCopies = NQ + 2;
    constexpr int kRound = [] {
      int r = 4;
      if (32 / kCopies < r) r = 32 / kCopies;
      if (kSlots / 2 < r) r = kSlots / 2;
      return r;
    }();
    static_assert(kRound >= 1 && kRound * kCopies <= 32, "one lane per copy of a round");
    int issued = 0;
    for (int ub = 0; ub < NV; ub += 32) {
      load_in(vbeg + ub + 32 + lane, nxt);  // in flight during this batch's copies
      const int nv = min(32, NV - ub);
      const int slot_m = (ub + lane) % kSlots, use_m = (ub + lane) / kSlots;  // this lane's view
      const bool staged_m = ws >= 0;
      int j = 0;
      for (; j < nv; j += kRound) {
        const int ng = min(kRound, nv - j);
        const bool mine = lane >= j && lane < j + ng;
        int go = 1;
        if (mine) {
          if (ld_volatile(s_bad)) {
            go = 0;
          } else if (use_m > 0 && !(mbar_wait(&s_empty[slot_m], (use_m - 1) & 1, P.wait_ns) &&
                                    mbar_wait(&s_full[slot_m], (use_m - 1) & 1, P.wait_ns))) {
            report_timeout(&s_bad);
            go = 0;
          }
        }
        if (!__all_sync(0xffffffffu, go)) break;
        if (mine) {
          // staged: the window's cell count and the quadratic seed shifted to
          // window-relative cells, so that consumers index the slot directly
          s_hdr[slot_m] = make_int4(staged_m ? min(kWin, D - ws) : -1, cur.fl, l0, __float_as_int(qsd.c0 - (float)ws));
          s_qsd[slot_m] = make_float2(qsd.c1, qsd.c2);
          s_src[slot_m][0] = cur.sx;
          s_src[slot_m][1] = cur.sy;
        }
        __syncwarp();
        if (mine) {
          if (staged_m) {
            const int ncell = min(kWin, Dp - ws);
            mbar_arrive_expect_tx(&s_full[slot_m],
                                  (unsigned)((ncell * (NQ * QW + 4) + nl * 4) * (int)sizeof(T)));
          } else {
            mbar_arrive(&s_full[slot_m]);
          }
        }
        issued += ng;
        __syncwarp();
        // copy c of the round's view g on lane g * kCopies + c
        const int g = lane / kCopies, c = lane - g * kCopies;
        const int src = j + min(g, ng - 1);
        const int wsg = __shfl_sync(0xffffffffu, ws, src);
        const int l0g = __shfl_sync(0xffffffffu, l0, src);
        const int nlg = __shfl_sync(0xffffffffu, nl, src);
        if (g < ng && wsg >= 0) {
          const int ug = ub + j + g, vg = vbeg + ug, slot = ug % kSlots;
          const int ncell = min(kWin, Dp - wsg);
          unsigned char* sl = slots + (size_t)slot * S::kBytes;
          if (c < NQ)
            bulk_g2s(sl + (size_t)c * kWin * QW * sizeof(T), qg + (((size_t)vg * NQ + c) * Dp + wsg) * QW,
                     (unsigned)(ncell * QW * sizeof(T)), &s_full[slot]);
          else if (c == NQ)
            bulk_g2s(sl + S::kQBytes, P.rec + ((size_t)vg * Dp + wsg) * 4, (unsigned)(ncell * 4 * sizeof(T)),
                     &s_full[slot]);
          else
            bulk_g2s(sl + S::kQBytes + S::kRecBytes, P.lp + ((size_t)vg * P.L + l0g) * 4,
                     (unsigned)(nlg * 4 * sizeof(T)), &s_full[slot]);
        }
      }
      if (j < nv) break;  // stopped after a timeout
      cur = nxt;
      ws = window(vbeg + ub + 32 + lane, cur, l0, nl, qsd);
    }
    // Normally the consumers wait on every phase issued. After a timeout, wait
    // for the last issued phase of every slot (the only one that can still be
    // pending), so that no copy is still landing in this CTA's shared memory
    // when the producer returns; this drain always allows kWaitLimitNs. A copy
    // is issued only with in-bounds source and destination (window start
    // clamped to [0, Dp), byte counts from the copied range), so on a working
    // GPU it lands within microseconds and the drain ends at once. Should the
    // drain itself run out, the event is counted once more and the producer
    // returns; the consumers finish on global loads, and a copy still in flight
    // could then land in shared memory that a later CTA on the same SM owns.
    if (lane == 0 && ld_volatile(s_bad)) {
      for (int i = 0; i < kSlots && i < issued; ++i) {
        const int last = i + ((issued - 1 - i) / kSlots) * kSlots;
        if (!mbar_wait(&s_full[i], (last / kSlots) & 1, kWaitLimitNs)) report_timeout(&s_bad);
      }
    }
    return;
  }

  // consumers: pixels (r[p], c), p < PX; acc holds [PX][2][SB][CT]
  const int c = c0 + lane;
  int rp[PX];
  bool act[PX];
  T pcy[PX], kf_row[PX];
  bool any = false;
#pragma unroll
  for (int p = 0; p < PX; ++p) {
    rp[p] = r0 + warp + p * R;
    kf_row[p] = T(P.H - 1 - rp[p]);
    act[p] = c < P.W && rp[p] < P.H;
    pcy[p] = act[p] ? P.rowc[rp[p]] : T(0);
    any = any || act[p];
  }
  const T pcx = any ? P.colc[c] : T(0);
  T blk[PX][SB];
#pragma unroll
  for (int p = 0; p < PX; ++p) {
    kahan_init_smem<T, SB>(acc + (size_t)p * 2 * SB * CT, CT);
#pragma unroll
    for (int s = 0; s < SB; ++s) blk[p][s] = T(0);
  }
  const T kf_col = T(c);  // the pixel's edge index on row lines; on column lines it is H - 1 - r
  int slot = 0;
  unsigned phase = 0;
  for (int u = 0; u < NV; ++u) {
    const int v = vbeg + u;
    bool ok = false;
    if (!ld_volatile(s_bad)) {
      ok = mbar_wait(&s_full[slot], phase, P.wait_ns);
      if (!ok) report_timeout(&s_bad);
    }
    if (SV) {
#pragma unroll
      for (int p = 0; p < PX; ++p)
#pragma unroll
        for (int s = 0; s < SB; ++s) blk[p][s] = T(0);
    }
    if (any) {
      const int4 h0 = ok ? s_hdr[slot] : make_int4(-1, 0, 0, 0);
      if (h0.x >= 0) {
        const float2 h1 = s_qsd[slot];
        const QuadSeed sd{__int_as_float(h0.w), h1.x, h1.y};
        const bool xb = h0.y & 1;
        const unsigned char* sl = slots + slot * S::kBytes;
        const T* sq = reinterpret_cast<const T*>(sl);
        const T* srec = reinterpret_cast<const T*>(sl + S::kQBytes);
        const T* slp = reinterpret_cast<const T*>(sl + S::kQBytes + S::kRecBytes);
        T sx = T(0), sy = T(0);
        if (KIND == kB) { sx = s_src[slot][0]; sy = s_src[slot][1]; }
#pragma unroll
        for (int p = 0; p < PX; ++p) {
          if (PX > 1 && !act[p]) continue;
          const Quad<T> A4 = ldrec<T, true>(slp + ((xb ? rp[p] : c) - h0.z) * 4);
          pix_view<T, SB, KIND, U, true>(P, A4, xb ? kf_col : kf_row[p], sd, sx, sy, pcx, pcy[p], srec, sq, kWin,
                                         0, 0, h0.x, blk[p]);
        }
      } else {
#pragma unroll
        for (int p = 0; p < PX; ++p) {
          if (PX > 1 && !act[p]) continue;
          pix_view_global<T, SB, KIND, U>(P, v, rp[p], c, qg + (size_t)v * NQ * Dp * QW, Dp, pcx, pcy[p], blk[p]);
        }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&s_empty[slot]);
    if (++slot == kSlots) {
      slot = 0;
      phase ^= 1u;
    }
    if (SV) {
#pragma unroll
      for (int p = 0; p < PX; ++p) {
        if (!act[p]) continue;
#pragma unroll
        for (int s = 0; s < SB; ++s) {
          const int bb = g * SB + s;
          if (bb < B) img[(((size_t)bb * V + v) * P.H + rp[p]) * P.W + c] = blk[p][s];
        }
      }
    } else if (!PLAIN && (u % kFoldEvery) == kFoldEvery - 1) {
#pragma unroll
      for (int p = 0; p < PX; ++p) kahan_fold_smem<T, SB>(acc + (size_t)p * 2 * SB * CT, blk[p], CT);
    }
  }
  if constexpr (!SV) {
#pragma unroll
    for (int p = 0; p < PX; ++p) {
      T* ap = acc + (size_t)p * 2 * SB * CT;
      kahan_fold_smem<T, SB>(ap, blk[p], CT);
      if (!act[p]) continue;
#pragma unroll
      for (int s = 0; s < SB; ++s) {
        const int bb = g * SB + s;
        if (bb >= B) continue;
        const T val = ap[(size_t)s * CT + threadIdx.x] * out_mul / out_div;
        T* base = nsplit == 1 ? img : parts + (size_t)part * B * P.H * P.W;
        base[((size_t)bb * P.H + rp[p]) * P.W + c] = val;
      }
    }
  }
}

template <class T, int SB, int KIND, int U, bool SV = false, int PX = 1, bool PLAIN = false>
__global__ void __launch_bounds__(288, (kPixCtas<T, SB>)) k_pix_gather(DevPlan<T> P, const T* __restrict__ q,
                                                       T* __restrict__ img, T* __restrict__ parts, int B,
                                                       T out_mul, T out_div, int nsplit) {
  pix_gather_cta<T, SB, KIND, U, SV, PX, PLAIN>(P, q, img, parts, B, out_mul, out_div, nsplit, blockIdx.x, blockIdx.y,
                                                blockIdx.z);
}

// Sum of the view parts of the staged image gather: out[i] = ((0 + p_0[i]) +
// p_1[i]) + ..., in part order (the order the ragged path adds its parts in).
template <class T>
__global__ void __launch_bounds__(256) k_combine_parts(const T* __restrict__ parts, T* __restrict__ out, size_t n,
                                                       int nparts) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  if constexpr (sizeof(T) == 4) {
    if ((n & 3) == 0) {
      const size_t n4 = n / 4;
      const float4* p4 = reinterpret_cast<const float4*>(parts);
      float4* o4 = reinterpret_cast<float4*>(out);
      for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += stride) {
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int p = 0; p < nparts; ++p) {
          const float4 v = __ldcs(p4 + (size_t)p * n4 + i);
          s.x = __fadd_rn(s.x, v.x); s.y = __fadd_rn(s.y, v.y);
          s.z = __fadd_rn(s.z, v.z); s.w = __fadd_rn(s.w, v.w);
        }
        o4[i] = s;
      }
      return;
    }
  }
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    T s = T(0);
    for (int p = 0; p < nparts; ++p) s = add_rn(s, parts[(size_t)p * n + i]);
    out[i] = s;
  }
}

// ----------------------------------------------------------------------------
// fbp ramp filter: q[g][v][d][s] = sum_m pre(y)[m] * h[m - k + D - 1], k = ext(d)
// One CTA per (slice group, view); each thread produces 8 outputs of one parity
// for one slice: outputs k0, k0+2, ..., k0+14 only meet taps of odd offset (the
// even non-zero offsets of the RL kernel are zero), plus the centre tap.
// ----------------------------------------------------------------------------
// Called by every thread of the CTA; `smem` holds ramp_smem_elems(D, SB)
// elements. In fp32 the taps are pairs (taps, tapl) and the low parts are summed
// separately.
//
// Shared-memory layout. A warp's threads produce outputs whose tap indices are
// 16 apart, and its slices' input rows lie D apart; stored plainly, the taps
// would be read 8 ways and, for D a multiple of 32, the rows 16 ways onto one
// bank. Tap index t (padded by kTapPad zero taps on both sides, so no index the
// loop forms needs a range check) sits at word t + t / 32, and the rows have an
// odd stride D + 1: both then spread over the banks.
constexpr int kTapPad = 32;
__host__ __device__ __forceinline__ int tap_slot(int t) { return t + (t >> 5); }
__host__ __device__ __forceinline__ size_t ramp_smem_elems(int D, int SB) {
  const int ntap = 2 * D - 1 + 2 * kTapPad;  // padded tap indices 0 .. ntap-1
  return 2 * (size_t)tap_slot(ntap) + (size_t)SB * (D + 1);
}

template <class T, int SB, bool PLAIN = false>
__device__ __forceinline__ void ramp_filter_view(const DevPlan<T>& P, int v, int g, const T* __restrict__ y,
                                                 T* __restrict__ q, int qs, int B, T* smem) {
  constexpr bool kLo = sizeof(T) == 4;
  const int D = P.D;
  const int ntap = 2 * D - 1 + 2 * kTapPad;
  T* taps = smem;                       // tap index t at taps[tap_slot(t + kTapPad)]
  T* tapl = taps + tap_slot(ntap);      // the same for the low parts
  T* rows = tapl + tap_slot(ntap);      // SB rows of stride D + 1
  const int rs = D + 1;
  __syncthreads();  // smem may still be read by a previous task of this CTA
  for (int j = threadIdx.x; j < ntap; j += blockDim.x) {
    const int t = j - kTapPad;
    const bool in = t >= 0 && t < 2 * D - 1;
    taps[tap_slot(j)] = in ? P.taps[t] : T(0);
    tapl[tap_slot(j)] = (kLo && in) ? P.tapl[t] : T(0);
  }
  for (int i = threadIdx.x; i < SB * D; i += blockDim.x) {
    const int s = i / D, m = i % D;
    const int bb = g * SB + s;
    T val = T(0);
    if (bb < B) val = (y[((size_t)bb * P.V + v) * D + m] * P.wpre[m]) * P.wscale;
    rows[s * rs + m] = val;
  }
  __syncthreads();
  const int chunks = (D + 15) / 16;               // 16 outputs (8 per parity) per chunk
  const int items = SB * 2 * chunks;
  const bool flip = P.flags[v] & 2;
  T* qv = q + ((size_t)g * P.V + v) * qs * SB;
  for (int i = threadIdx.x; i < SB * (qs - D); i += blockDim.x)  // row padding
    qv[((size_t)(i / Planes<SB>::QW / (qs - D)) * qs + D + (i / Planes<SB>::QW) % (qs - D)) * Planes<SB>::QW +
       i % Planes<SB>::QW] = T(0);
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    const int s = it % SB;
    const int par = (it / SB) & 1;
    const int ch = it / (2 * SB);
    const int k0 = ch * 16 + par;
    const T* row = rows + s * rs;
    // blocks of 16 taps are summed plainly (part) and folded into acc with
    // Kahan compensation (comp): the ramp filter cancels strongly, so the
    // far, small taps must not be added straight onto the large running sum;
    // the low parts of the taps go to their own plain sum (plo)
    T acc[8], comp[8], part[8], plo[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      acc[i] = T(0);
      comp[i] = T(0);
      part[i] = T(0);
      plo[i] = T(0);
    }
    int step = 0;
    // one pass over the inputs m = m0, m0+2, ...: window win[i] = h(m - k0 - 2i)
    auto pass = [&](int m0) {
      // tap indices run from -15 (first window of the last chunk, k0 <= D) to 2D (last new
      // tap), inside the kTapPad zero margins
      T win[8], wlo[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int ts = tap_slot(m0 - k0 - 2 * i + D - 1 + kTapPad);
        win[i] = taps[ts];
        wlo[i] = tapl[ts];
      }
      int m = m0;
      // blocks of 8 steps: at a block's start win[i] holds tap(base + m - 2i)
      // (base = D - 1 - k0); the block loads nw[j] = tap(base + m + 2(j + 1)), and
      // step t of the block gives output i the tap base + m + 2(t - i), which is
      // win[i - t] for t <= i and nw[t - i - 1] otherwise: fixed registers, no
      // window shifts. Same FMAs, same order and fold points as one step at a
      // time below.
      for (; m + 14 < D; m += 16, step += 8) {
        T nw[8], nl[8], xv[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int ts = tap_slot(m + 2 * (j + 1) - k0 + D - 1 + kTapPad);
          nw[j] = taps[ts];
          nl[j] = tapl[ts];
          xv[j] = row[m + 2 * j];
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) {
#pragma unroll
          for (int i = 0; i < 8; ++i) part[i] = fma(xv[t], t <= i ? win[i - t] : nw[t - i - 1], part[i]);
          if constexpr (kLo) {
#pragma unroll
            for (int i = 0; i < 8; ++i) plo[i] = fma(xv[t], t <= i ? wlo[i - t] : nl[t - i - 1], plo[i]);
          }
          if (!PLAIN && ((step + t) & 15) == 15) {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              const T y = sub_rn(part[i], comp[i]);
              const T tt = add_rn(acc[i], y);
              comp[i] = sub_rn(sub_rn(tt, acc[i]), y);
              acc[i] = tt;
              part[i] = T(0);
            }
          }
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          win[i] = nw[7 - i];
          wlo[i] = nl[7 - i];
        }
      }
      for (; m < D; m += 2, ++step) {
        const T xm = row[m];
#pragma unroll
        for (int i = 0; i < 8; ++i) part[i] = fma(xm, win[i], part[i]);
        if constexpr (kLo) {
#pragma unroll
          for (int i = 0; i < 8; ++i) plo[i] = fma(xm, wlo[i], plo[i]);
        }
#pragma unroll
        for (int i = 7; i > 0; --i) {
          win[i] = win[i - 1];
          wlo[i] = wlo[i - 1];
        }
        const int ts = tap_slot(m + 2 - k0 + D - 1 + kTapPad);
        win[0] = taps[ts];
        wlo[0] = tapl[ts];
        if (!PLAIN && (step & 15) == 15) {
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const T y = sub_rn(part[i], comp[i]);
            const T t = add_rn(acc[i], y);
            comp[i] = sub_rn(sub_rn(t, acc[i]), y);
            acc[i] = t;
            part[i] = T(0);
          }
        }
      }
    };
    pass(1 - par);                // odd offsets: the only non-zero ones of the RL kernel besides 0
    if (P.even_taps) pass(par);   // windowed kernels: even offsets, the centre tap included
#pragma unroll
    for (int i = 0; i < 8; ++i) acc[i] = add_rn(acc[i], sub_rn(part[i], comp[i]));
    const T h0 = taps[tap_slot(D - 1 + kTapPad)], h0l = tapl[tap_slot(D - 1 + kTapPad)];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int k = k0 + 2 * i;
      if (k < D) {
        T val;
        if (P.even_taps) {
          val = acc[i];
          if constexpr (kLo) val = add_rn(val, plo[i]);
        } else {
          val = fma(h0, row[k], acc[i]);
          if constexpr (kLo) val = add_rn(val, fma(h0l, row[k], plo[i]));
        }
        const int di = flip ? D - 1 - k : k;
        qv[((size_t)(s / Planes<SB>::QW) * qs + di) * Planes<SB>::QW + (s % Planes<SB>::QW)] = val;
      }
    }
  }
}

template <class T, int SB, bool PLAIN = false>
__global__ void __launch_bounds__(256) k_ramp_filter(DevPlan<T> P, const T* __restrict__ y, T* __restrict__ q,
                                                     int B) {
  extern __shared__ unsigned char smem_raw[];
  ramp_filter_view<T, SB, PLAIN>(P, blockIdx.x, blockIdx.y, y, q, P.Dp, B, reinterpret_cast<T*>(smem_raw));
}

// ----------------------------------------------------------------------------
// plan
// ----------------------------------------------------------------------------
}  // namespace ctgb

struct ctgb_plan {
  ctgb::HostGeom geom;
  int device = 0;
  int dtype = 0;
  // per-operator schedule: cap on slices per thread (0 = default) and warps
  // per CTA of the gather kernel (8 or 4)
  int sb_cap[6] = {0, 0, 0, 0, 0, 0};
  int warps[6] = {8, 8, 8, 8, 8, 8};
  // straight-line steps of the gather loop (3 or 2; 2 is built for fp32 with
  // 4 or more slices per thread, other widths always use 3)
  int unroll[6] = {3, 3, 3, 3, 3, 3};
  // one plain fp32 running sum per output instead of compensated sums
  // (ctgb_plan_set_summation; fp32 plans, the five operators only)
  bool plain = false;
  // optional events recorded right before and after each gather kernel on the
  // launch stream (ctgb_plan_set_kernel_events), to time that kernel alone
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
  int sms = 152;        // multiprocessors of the plan's device
  void* dev = nullptr;  // one allocation holding all tables
  ctgb::DevPlan<float> pf{};
  ctgb::DevPlan<double> pd{};
};

namespace ctgb {

// Line map x(k) = alpha + sigma*k of a line with K pixels, split for a type of
// `digits` significant bits into (alpha_hi, alpha_lo, sigma_hi, sigma_lo). The
// high parts are rounded to multiples of one power of two qg, chosen so that
// every value alpha_hi + sigma_hi*k (k = 0 .. K, the line's pixel edges) is a
// multiple of qg below 2^digits qg in magnitude: that sum is then exact in the
// type and the image gather forms it with one FMA. The low parts are the
// remainders (at most qg/2 each), summed by a second FMA to ~2^-38 of the
// coordinate in fp32. The device table stores each part rounded to the type.
static void split_line_map(double alpha, double sigma, int K, int digits, double* out) {
  const double M = std::max({std::fabs(alpha), std::fabs(alpha + sigma * K), sigma * K});
  const double qg = std::ldexp(1.0, std::ilogb(M) + 2 - digits);
  const double ah = std::nearbyint(alpha / qg) * qg, sh = std::nearbyint(sigma / qg) * qg;
  out[0] = ah;
  out[1] = alpha - ah;
  out[2] = sh;
  out[3] = sigma - sh;
}

template <class T>
static int upload(ctgb_plan* p) {
  const HostGeom& g = p->geom;
  const int V = g.V, D = g.D, L = g.L;
  auto split_hi = [](double x) { return (double)(T)x; };
  // tables in elements of T, each built in double and rounded once
  std::vector<double> db2((size_t)V * (D + 1) * 2), lg((size_t)V * L * 4, 0.0), ls((size_t)V * L, 1.0),
      lp((size_t)V * L * 4, 0.0), rowc(g.H), colc(g.W);
  for (size_t i = 0; i < g.db.size(); ++i) {
    const double hi = split_hi(g.db[i]);
    db2[2 * i] = hi;
    db2[2 * i + 1] = g.db[i] - hi;
  }
  const int Dp = padded_cells(D);
  std::vector<double> rec((size_t)V * Dp * 4, 0.0);
  for (int v = 0; v < V; ++v)
    for (int d = 0; d < D; ++d) {
      double* e = &rec[((size_t)v * Dp + d) * 4];
      const size_t b = (size_t)v * (D + 1) + d;
      e[0] = db2[2 * b];
      e[1] = db2[2 * b + 1];
      e[2] = g.wd[(size_t)v * D + d];
      e[3] = d + 1 < D ? g.wd[(size_t)v * D + d + 1] : 0.0;  // the padding cell's width past D
    }
  for (size_t i = 0; i < (size_t)V * L; ++i) {
    const double alpha = g.lp[2 * i], sigma = g.lp[2 * i + 1];
    if (!(sigma > 0)) continue;  // unused line slot (lines = min(H, W) for this view)
    const double gam = 1.0 / sigma, beta = -alpha / sigma;
    const double gh = split_hi(gam), bi = std::floor(beta);
    lg[4 * i] = gh; lg[4 * i + 1] = gam - gh; lg[4 * i + 2] = bi; lg[4 * i + 3] = beta - bi;
    ls[i] = sigma;
    split_line_map(alpha, sigma, (g.flags[i / L] & 1) ? g.W : g.H, std::numeric_limits<T>::digits, &lp[4 * i]);
  }
  for (int r = 0; r < g.H; ++r) rowc[r] = (g.height / 2 - r - 0.5) * g.dImg;
  for (int c = 0; c < g.W; ++c) colc[c] = (c - g.width / 2 + 0.5) * g.dImg;
  // the backprojector weights' source table: equal-distance fans need the source
  // position only divided by s2r^2 (ued_base), formed here in fp64
  std::vector<double> wsrc = g.src;
  if (g.scan == kFanED)
    for (double& x : wsrc) x /= (double)g.s2r * (double)g.s2r;
  const std::vector<const std::vector<double>*> tabs = {&wsrc, &db2, &g.wd, &g.fq, &g.fbt, &lg, &ls, &lp,
                                                        &rowc, &colc, &g.wpre, &g.taps, &g.taps_lo, &rec};
  size_t off = 0;
  std::vector<size_t> offs;
  auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
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
  CTGB_CUDA(cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device));
  CTGB_CUDA(cudaMalloc(&p->dev, off));
  CTGB_CUDA(cudaMemcpy(p->dev, host.data(), off, cudaMemcpyHostToDevice));
  unsigned char* b = static_cast<unsigned char*>(p->dev);
  DevPlan<T> P{};
  P.V = V; P.D = D; P.W = g.W; P.H = g.H; P.L = L; P.scan = g.scan;
  P.dImg = (T)g.dImg; P.s2r = (T)g.s2r; P.dAng = (T)g.dAng; P.wscale = (T)g.wscale;
  {
    double m = 0.0;
    for (const double x : g.db) m = std::max(m, std::fabs(x));
    for (const double x : g.wd) m = std::max(m, std::fabs(x));
    P.ub_margin = (T)std::ldexp(4.0, std::ilogb(m) + 1 - std::numeric_limits<T>::digits);
  }
  P.wsrc = reinterpret_cast<const T*>(b + offs[0]);
  P.db2 = reinterpret_cast<const T*>(b + offs[1]);
  P.wd = reinterpret_cast<const T*>(b + offs[2]);
  P.fq = reinterpret_cast<const T*>(b + offs[3]);
  P.fbt = reinterpret_cast<const T*>(b + offs[4]);
  P.lg = reinterpret_cast<const T*>(b + offs[5]);
  P.ls = reinterpret_cast<const T*>(b + offs[6]);
  P.lp = reinterpret_cast<const T*>(b + offs[7]);
  P.rowc = reinterpret_cast<const T*>(b + offs[8]);
  P.colc = reinterpret_cast<const T*>(b + offs[9]);
  P.wpre = reinterpret_cast<const T*>(b + offs[10]);
  P.taps = reinterpret_cast<const T*>(b + offs[11]);
  P.tapl = reinterpret_cast<const T*>(b + offs[12]);
  P.rec = reinterpret_cast<const T*>(b + offs[13]);
  P.Dp = Dp;
  P.wait_ns = kWaitLimitNs;
  P.flags = reinterpret_cast<const int*>(b + off_flags);
  P.inv = reinterpret_cast<const float*>(b + off_inv);
  if constexpr (sizeof(T) == 4) p->pf = P; else p->pd = P;
  return CTGB_OK;
}

// slices per thread: float up to 16, double up to 4, or the tuned cap
static int slices_per_thread(int dtype, int batch, int tuned_cap = 0) {
  int cap = dtype == 0 ? 16 : 4;
  if (tuned_cap > 0 && tuned_cap < cap) cap = tuned_cap;
  int sb = 1;
  while (sb < batch && sb < cap) sb *= 2;
  return sb;
}

static size_t esize(int dtype) { return dtype == 0 ? 4 : 8; }

// partial images of the staged image gather's view parts (none for one part
// or for single-view backprojection, which writes each view's image directly)
static size_t pix_parts_bytes(const HostGeom& g, int op, int batch, size_t es) {
  const int np = view_split(g.V, (long long)g.W * g.H);
  if (np == 1 || op == CTGB_OP_BACKPROJECTION_SV) return 0;
  return ((size_t)np * batch * g.H * g.W * es + 255) & ~(size_t)255;
}

static size_t workspace_bytes(const ctgb_plan* p, int op, int batch) {
  const HostGeom& g = p->geom;
  const int sb = slices_per_thread(p->dtype, batch, p->sb_cap[op]);
  const size_t G = (size_t)((batch + sb - 1) / sb);
  const size_t es = esize(p->dtype);
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  if (op == CTGB_OP_PROJECTION || op == CTGB_OP_BACKPROJECTION_T)
    return al(G * g.H * (size_t)round8(g.W) * sb * es) + al(G * g.W * (size_t)round8(g.H) * sb * es);
  return al(G * g.V * (size_t)padded_cells(g.D) * sb * es) + pix_parts_bytes(g, op, batch, es);
}

// two straight-line steps are instantiated for every fp32 width (the autotuner
// picks them per operator and batch; fp64 keeps three)
template <class T, int SB>
constexpr bool kTwoStep = sizeof(T) == 4;

// plain-summation variants (no Kahan folds) are instantiated for fp32 with three
// straight-line steps only: they serve error studies, not speed; for fp64 the
// flag names the default kernels, so no extra fp64 code is built
template <class T>
constexpr bool kPlainBuilt = sizeof(T) == 4;

// bytes of the image line planes of the detector gather, and of the sinogram
// planes of the image gather, for G slice groups of SB slices
static size_t det_planes_bytes(const HostGeom& g, size_t G, int sb, size_t es) {
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  return al(G * g.H * (size_t)round8(g.W) * sb * es) + al(G * g.W * (size_t)round8(g.H) * sb * es);
}
static size_t pix_planes_bytes(const HostGeom& g, size_t G, int sb, size_t es) {
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  return al(G * g.V * (size_t)padded_cells(g.D) * sb * es);
}

// The data-term gradient groups slices as projection_t does (both gathers read
// planes of the same grouping); its workspace holds both plane sets.
static int gradient_sb(const ctgb_plan* p, int batch) {
  return slices_per_thread(p->dtype, batch, p->sb_cap[CTGB_OP_PROJECTION_T]);
}
static size_t gradient_workspace_bytes(const ctgb_plan* p, int batch) {
  const int sb = gradient_sb(p, batch);
  const size_t G = (size_t)((batch + sb - 1) / sb);
  return det_planes_bytes(p->geom, G, sb, esize(p->dtype)) + pix_planes_bytes(p->geom, G, sb, esize(p->dtype)) +
         pix_parts_bytes(p->geom, CTGB_OP_PROJECTION_T, batch, esize(p->dtype));
}

// Image re-layout + detector gather: A or B^T of x into y, or (RES) A's residual
// against ro.y for the data-term gradient. `sched` is the operator whose
// schedule (warps per CTA, straight-line steps) is used.
template <class T, int SB, bool RES>
static int launch_det(const ctgb_plan* p, const DevPlan<T>& P, int op, int sched, const T* x, T* y, int batch,
                      void* ws, cudaStream_t st, ResidualOut<T> ro = {}) {
  const int G = (batch + SB - 1) / SB;
  const HostGeom& g = p->geom;
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  T* imx = static_cast<T*>(ws);
  T* imy = reinterpret_cast<T*>(static_cast<unsigned char*>(ws) + al((size_t)G * g.H * round8(g.W) * SB * sizeof(T)));
  const int tb = 256;
  const int nb = (int)std::min<size_t>((size_t)G * Planes<SB>::NQ * g.H, 152 * 16);
  PrefetchList pf{};
  const size_t VL = (size_t)g.V * g.L, VD = (size_t)g.V * g.D;
  pf.ptr[0] = P.lg; pf.bytes[0] = VL * 4 * sizeof(T);
  pf.ptr[1] = P.ls; pf.bytes[1] = VL * sizeof(T);
  pf.ptr[2] = P.db2; pf.bytes[2] = (VD + g.V) * 2 * sizeof(T);
  pf.ptr[3] = P.wd; pf.bytes[3] = VD * sizeof(T);
  pf.ptr[4] = op == CTGB_OP_BACKPROJECTION_T ? P.fbt : P.fq; pf.bytes[4] = VD * sizeof(T);
  pf.n = 5;
  k_layout_image<T, SB><<<nb, tb, 0, st>>>(x, imx, imy, batch, g.H, g.W, G, pf);
  const int wpc = p->warps[sched];
  dim3 grid((g.D + 31) / 32, (g.V + wpc - 1) / wpc, G);
  const size_t acc_smem = (size_t)2 * SB * 32 * wpc * sizeof(T);
  const bool two = kTwoStep<T, SB> && p->unroll[sched] == 2;
  constexpr int U2 = kTwoStep<T, SB> ? 2 : 3;
  auto launch = [&](auto kern) {
    if (p->ev_start) cudaEventRecord(p->ev_start, st);
    kern<<<grid, 32 * wpc, acc_smem, st>>>(P, imx, imy, y, batch, ro);
    if (p->ev_stop) cudaEventRecord(p->ev_stop, st);
  };
  const bool plain = !RES && kPlainBuilt<T> && p->plain;
  if (RES || op == CTGB_OP_PROJECTION) {
    if (plain) launch(k_det_gather<T, SB, kA, 3, false, kPlainBuilt<T>>);
    else if (two) launch(k_det_gather<T, SB, kA, U2, RES>);
    else launch(k_det_gather<T, SB, kA, 3, RES>);
  } else {
    if (plain) launch(k_det_gather<T, SB, kBt, 3, false, kPlainBuilt<T>>);
    else if (two) launch(k_det_gather<T, SB, kBt, U2>);
    else launch(k_det_gather<T, SB, kBt, 3>);
  }
  return CTGB_OK;
}

template <class T, int SB, int PX>
static int launch_pix_rows(const ctgb_plan* p, const DevPlan<T>& P, int op, int sched, T* y, int batch, const T* qb,
                           T* parts, int nsplit, cudaStream_t st);

// Four pixel rows per consumer thread are built for one or two fp32 slices per
// thread: they share each warp's per-view costs between twice the pixels of
// two rows, and are taken when the grid still fills two waves (16 x 16 tiles x
// 8 view parts for one 512^2 slice of 1152 views: A^T 0.97 -> 0.85 ms), not on
// small images (parallel 256^2, 360 views: 128 CTAs, 0.14 -> 0.18 ms).
template <class T, int SB>
constexpr bool kWideBuilt = sizeof(T) == 4 && SB <= 2;

// Staged image gather (A^T, B, fbp's backprojection, single-view B) from the
// sinogram planes qb; unless `planes_ready`, qb is first filled from x (re-layout,
// or the ramp filter for fbp). `parts` holds the partial images of the view
// parts (pix_parts_bytes), which k_combine_parts sums into y.
template <class T, int SB>
static int launch_pix(const ctgb_plan* p, const DevPlan<T>& P, int op, int sched, const T* x, T* y, int batch,
                      T* qb, T* parts, bool planes_ready, cudaStream_t st) {
  const int G = (batch + SB - 1) / SB;
  const HostGeom& g = p->geom;
  const bool plain = kPlainBuilt<T> && p->plain && op != CTGB_OP_BACKPROJECTION_SV;
  if (!planes_ready && op == CTGB_OP_FBP) {
    const size_t smem = ramp_smem_elems(g.D, SB) * sizeof(T);
    auto ramp = plain ? k_ramp_filter<T, SB, kPlainBuilt<T>> : k_ramp_filter<T, SB>;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(ramp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return fail(CTGB_ERR_CUDA, std::string("ramp filter smem: ") + cudaGetErrorString(e));
    }
    // one thread per work item (8 outputs of one parity and slice) up to 256:
    // a one-slice row of 736 bins is 92 items, which a 256-thread CTA would
    // leave mostly idle
    const int items = SB * 2 * ((g.D + 15) / 16);
    const int nt = std::min(256, std::max(32, (items + 31) / 32 * 32));
    ramp<<<dim3(g.V, G), nt, smem, st>>>(P, x, qb, batch);
  } else if (!planes_ready) {
    const int tb = 256;
    const int nb = (int)std::min<size_t>((size_t)G * g.V * Planes<SB>::NQ, 152 * 16);
    PrefetchList pf{};
    const size_t VL = (size_t)g.V * g.L;
    pf.ptr[0] = P.lp; pf.bytes[0] = VL * 4 * sizeof(T);
    pf.ptr[1] = P.rec; pf.bytes[1] = (size_t)g.V * P.Dp * 4 * sizeof(T);
    pf.ptr[2] = P.db2; pf.bytes[2] = ((size_t)g.V * g.D + g.V) * 2 * sizeof(T);
    pf.n = 3;
    k_layout_sino<T, SB><<<nb, tb, 0, st>>>(x, qb, P.flags, op == CTGB_OP_PROJECTION_T ? P.fq : nullptr, batch,
                                           g.V, g.D, P.Dp, G, pf);
  }
  // single-view backprojection writes each view's image on its own, so its views
  // split over any number of CTAs with no adds: 8 parts shorten the CTAs of a
  // grid that is only ~2 waves deep (7.62 to 6.85 ms for 16 x 512^2, 1152 views)
  const int nsplit = op == CTGB_OP_BACKPROJECTION_SV ? std::min(8, g.V) : view_split(g.V, (long long)g.W * g.H);
  if constexpr (kWideBuilt<T, SB>) {
    const int wpc = p->warps[sched];
    const long long ctas = (long long)((g.W + 31) / 32) * ((g.H + 4 * wpc - 1) / (4 * wpc)) * G * nsplit;
    if (ctas >= 2LL * p->sms * kPixCtas<T, SB>)
      return launch_pix_rows<T, SB, 4>(p, P, op, sched, y, batch, qb, parts, nsplit, st);
  }
  return launch_pix_rows<T, SB, kPixRows<SB>>(p, P, op, sched, y, batch, qb, parts, nsplit, st);
}

// The staged image gather at PX pixel rows per consumer thread, then the sum
// of its view parts.
template <class T, int SB, int PX>
static int launch_pix_rows(const ctgb_plan* p, const DevPlan<T>& P, int op, int sched, T* y, int batch, const T* qb,
                           T* parts, int nsplit, cudaStream_t st) {
  const int G = (batch + SB - 1) / SB;
  const HostGeom& g = p->geom;
  const bool plain = kPlainBuilt<T> && p->plain && op != CTGB_OP_BACKPROJECTION_SV;
  const int wpc = p->warps[sched];  // consumer warps (PX pixel rows each) + one producer warp
  dim3 grid((g.W + 31) / 32, (g.H + wpc * PX - 1) / (wpc * PX), G);
  const int nt = 32 * (wpc + 1);
  const size_t smem =
      (size_t)2 * PX * SB * (32 * wpc) * sizeof(T) + (size_t)kSlots<T, SB, PX> * PixSlot<T, SB>::kBytes;
  auto launch = [&](auto kern, T mul, T div) -> int {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return fail(CTGB_ERR_CUDA, std::string("image gather smem: ") + cudaGetErrorString(e));
    const bool sv = op == CTGB_OP_BACKPROJECTION_SV;
    if (p->ev_start) cudaEventRecord(p->ev_start, st);
    kern<<<dim3(grid.x, grid.y, grid.z * nsplit), nt, smem, st>>>(P, qb, y, parts, batch, mul, div, nsplit);
    if (p->ev_stop) cudaEventRecord(p->ev_stop, st);
    if (nsplit > 1 && !sv) {
      const size_t n = (size_t)batch * g.H * g.W;
      const int cb = (int)std::min<size_t>((n / 4 + 255) / 256, 152 * 8);
      k_combine_parts<T><<<std::max(cb, 1), 256, 0, st>>>(parts, y, n, nsplit);
    }
    return CTGB_OK;
  };
  constexpr int U2 = kTwoStep<T, SB> ? 2 : 3;
  const bool two = kTwoStep<T, SB> && p->unroll[sched] == 2;
  constexpr bool PL = kPlainBuilt<T>;
  if (plain) {
    if (op == CTGB_OP_PROJECTION_T) return launch(k_pix_gather<T, SB, kAt, 3, false, PX, PL>, T(1), T(1));
    if (op == CTGB_OP_BACKPROJECTION) return launch(k_pix_gather<T, SB, kB, 3, false, PX, PL>, T(1), T(1));
    return launch(k_pix_gather<T, SB, kB, 3, false, PX, PL>, P.dAng, T(2));
  }
  if (op == CTGB_OP_BACKPROJECTION_SV)
    return two ? launch(k_pix_gather<T, SB, kB, U2, true, PX>, T(1), T(1))
               : launch(k_pix_gather<T, SB, kB, 3, true, PX>, T(1), T(1));
  if (op == CTGB_OP_PROJECTION_T)
    return two ? launch(k_pix_gather<T, SB, kAt, U2, false, PX>, T(1), T(1))
               : launch(k_pix_gather<T, SB, kAt, 3, false, PX>, T(1), T(1));
  if (op == CTGB_OP_BACKPROJECTION)
    return two ? launch(k_pix_gather<T, SB, kB, U2, false, PX>, T(1), T(1))
               : launch(k_pix_gather<T, SB, kB, 3, false, PX>, T(1), T(1));
  return two ? launch(k_pix_gather<T, SB, kB, U2, false, PX>, P.dAng, T(2))
             : launch(k_pix_gather<T, SB, kB, 3, false, PX>, P.dAng, T(2));
}

template <class T, int SB>
static int run_op(const ctgb_plan* p, const DevPlan<T>& P, int op, const void* in, void* out, int batch,
                  void* ws, cudaStream_t st) {
  const T* x = static_cast<const T*>(in);
  T* y = static_cast<T*>(out);
  int rc;
  if (op == CTGB_OP_PROJECTION || op == CTGB_OP_BACKPROJECTION_T)
    rc = launch_det<T, SB, false>(p, P, op, op, x, y, batch, ws, st);
  else
    rc = launch_pix<T, SB>(p, P, op, op, x, y, batch, static_cast<T*>(ws),
                           reinterpret_cast<T*>(static_cast<unsigned char*>(ws) +
                                                pix_planes_bytes(p->geom, (batch + SB - 1) / SB, SB, sizeof(T))),
                           false, st);
  if (rc != CTGB_OK) return rc;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(CTGB_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return CTGB_OK;
}

// Data-term gradient A^T(Ax - y): image re-layout, detector gather writing the
// residual straight into the image gather's planes (and optionally to `res`),
// image gather. The workspace holds both plane sets; the detector gather uses
// projection's schedule, the image gather projection_t's.
template <class T, int SB>
static int run_gradient(const ctgb_plan* p, const DevPlan<T>& P, const T* x, const T* y, T* res, T* grad, int batch,
                        void* ws, cudaStream_t st) {
  const size_t G = (size_t)((batch + SB - 1) / SB);
  unsigned char* w = static_cast<unsigned char*>(ws);
  const size_t det_b = det_planes_bytes(p->geom, G, SB, sizeof(T));
  T* qb = reinterpret_cast<T*>(w + det_b);
  T* parts = reinterpret_cast<T*>(w + det_b + pix_planes_bytes(p->geom, G, SB, sizeof(T)));
  int rc = launch_det<T, SB, true>(p, P, CTGB_OP_PROJECTION, CTGB_OP_PROJECTION, x, nullptr, batch, ws, st,
                                   ResidualOut<T>{y, res, qb});
  if (rc == CTGB_OK)
    rc = launch_pix<T, SB>(p, P, CTGB_OP_PROJECTION_T, CTGB_OP_PROJECTION_T, nullptr, grad, batch, qb, parts, true,
                           st);
  if (rc != CTGB_OK) return rc;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(CTGB_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return CTGB_OK;
}

static int dispatch(const ctgb_plan* p, int op, const void* in, void* out, int batch, void* ws, size_t wsb,
                    void* stream) {
  if (!p) return fail(CTGB_ERR_INVALID, "null plan");
  if (batch < 0) return fail(CTGB_ERR_INVALID, "negative batch");
  if (op == CTGB_OP_BACKPROJECTION_SV && p->geom.scan != kFanED)
    return fail(CTGB_ERR_INVALID, "backprojection_sv is defined for equal-distance fan beams (scan_type 0) only");
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
  const int sb = slices_per_thread(p->dtype, batch, p->sb_cap[op]);
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

static int dispatch_gradient(const ctgb_plan* p, const void* image, const void* sino, void* res, void* grad,
                             int batch, void* ws, size_t wsb, void* stream) {
  if (!p) return fail(CTGB_ERR_INVALID, "null plan");
  if (batch < 0) return fail(CTGB_ERR_INVALID, "negative batch");
  if (batch == 0) return CTGB_OK;
  if (!image || !sino || !grad) return fail(CTGB_ERR_INVALID, "null image, sinogram or gradient pointer");
  const size_t need = gradient_workspace_bytes(p, batch);
  if (!ws || wsb < need) return fail(CTGB_ERR_WORKSPACE, "workspace too small: need " + std::to_string(need) + " bytes");
  if ((reinterpret_cast<uintptr_t>(ws) & 255) != 0) return fail(CTGB_ERR_INVALID, "workspace must be 256-byte aligned");
  int cur = -1;
  CTGB_CUDA(cudaGetDevice(&cur));
  if (cur != p->device) CTGB_CUDA(cudaSetDevice(p->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int sb = gradient_sb(p, batch);
  int rc;
  if (p->dtype == 0) {
    const float* x = static_cast<const float*>(image);
    const float* y = static_cast<const float*>(sino);
    float* r = static_cast<float*>(res);
    float* gr = static_cast<float*>(grad);
    switch (sb) {
      case 1: rc = run_gradient<float, 1>(p, p->pf, x, y, r, gr, batch, ws, st); break;
      case 2: rc = run_gradient<float, 2>(p, p->pf, x, y, r, gr, batch, ws, st); break;
      case 4: rc = run_gradient<float, 4>(p, p->pf, x, y, r, gr, batch, ws, st); break;
      case 8: rc = run_gradient<float, 8>(p, p->pf, x, y, r, gr, batch, ws, st); break;
      default: rc = run_gradient<float, 16>(p, p->pf, x, y, r, gr, batch, ws, st); break;
    }
  } else {
    const double* x = static_cast<const double*>(image);
    const double* y = static_cast<const double*>(sino);
    double* r = static_cast<double*>(res);
    double* gr = static_cast<double*>(grad);
    switch (sb) {
      case 1: rc = run_gradient<double, 1>(p, p->pd, x, y, r, gr, batch, ws, st); break;
      case 2: rc = run_gradient<double, 2>(p, p->pd, x, y, r, gr, batch, ws, st); break;
      default: rc = run_gradient<double, 4>(p, p->pd, x, y, r, gr, batch, ws, st); break;
    }
  }
  if (cur != p->device && cur >= 0) cudaSetDevice(cur);
  return rc;
}

// ----------------------------------------------------------------------------
// ragged batches: slices with their own plans, one persistent launch per stage
// ----------------------------------------------------------------------------
// Each stage's work is a host-built task list, longest tasks first; persistent
// CTAs (as many as fit at once) walk it with a grid stride and read the plan of
// the task's slice from a device array. Slice pointers travel as a by-value
// kernel parameter, so a run needs no host-to-device copy and can be captured in
// a CUDA graph. One slice per plan entry: the gathers run with one slice per
// thread, and a slice's row lines are its own image (no re-layout needed).
constexpr int kMaxRagged = 128;

template <class T>
struct RaggedIO {
  const T* in[kMaxRagged];
  T* out[kMaxRagged];
};

// every slice's device plan, passed by value as one kernel parameter (23.5 KB
// for fp32 plans, 25.6 KB for fp64, of the 32 KB a launch may carry): a CTA
// reads its slice's geometry from the constant bank, as a per-slice launch
// reads its own plan
template <class T>
struct RaggedPlans {
  DevPlan<T> p[kMaxRagged];
};

struct RTask {
  int slice, a, b;
};

// one CTA of the staged image gather: tile column bx, tile row by, view part
struct RPixTask {
  int slice, bx, by, part;
};

// tile rows per CTA of the ragged image gather: 8 row warps of kRagPX pixel rows
constexpr int kRagPixWarps = 8;
// views per CTA (one warp each) of the ragged detector gather
constexpr int kRagDetWarps = 8;
// pixel rows per consumer thread of a ragged tile: four, as a one-slice call
// takes on large images (the ragged launch's task list always fills the GPU;
// one launch per stage on 96 mixed slices: 169 -> 157 ms against two rows)
constexpr int kRagPX = 4;
constexpr int kRagPixRows = kRagPixWarps * kRagPX;

template <class T>
__global__ void __launch_bounds__(256) k_rag_transpose(const __grid_constant__ RaggedPlans<T> rp,
                                                       const RTask* __restrict__ tasks, int ntasks,
                                                       const __grid_constant__ RaggedIO<T> io, unsigned char* ws,
                                                       const size_t* __restrict__ off) {
  __shared__ T tile[32][33];
  for (int t = blockIdx.x; t < ntasks; t += gridDim.x) {
    const RTask tk = tasks[t];
    const int H = rp.p[tk.slice].H, W = rp.p[tk.slice].W;
    const T* img = io.in[tk.slice];
    T* imy = reinterpret_cast<T*>(ws + off[tk.slice]);
    const int r0 = tk.a * 32, c0 = tk.b * 32;
    __syncthreads();
    for (int i = threadIdx.x; i < 1024; i += blockDim.x) {
      const int rr = i >> 5, cc = i & 31, r = r0 + rr, c = c0 + cc;
      tile[rr][cc] = (r < H && c < W) ? img[(size_t)r * W + c] : T(0);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 1024; i += blockDim.x) {
      const int cc = i >> 5, rr = i & 31, r = r0 + rr, c = c0 + cc;
      if (r < H && c < W) imy[(size_t)c * H + (H - 1 - r)] = tile[rr][cc];
    }
  }
}

// The detector gather of a per-slice call with one slice per thread (two
// straight-line pixels in fp32, three in fp64; the step count never changes
// results), each CTA walking the task list; the slice's plan is read in place
// from the constant bank.
template <class T, int KIND>
__global__ void __launch_bounds__(256) k_rag_det_gather(const __grid_constant__ RaggedPlans<T> rp,
                                                        const RTask* __restrict__ tasks, int ntasks,
                                                        const __grid_constant__ RaggedIO<T> io, unsigned char* ws,
                                                        const size_t* __restrict__ off) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int t = blockIdx.x; t < ntasks; t += gridDim.x) {
    const RTask tk = tasks[t];
    const DevPlan<T>& P = rp.p[tk.slice];
    const int v = tk.a * (blockDim.x >> 5) + warp, d = tk.b * 32 + lane;
    if (v < P.V && d < P.D)
      det_gather_cell<T, 1, KIND, kTwoStep<T, 1> ? 2 : 3>(P, v, d, 0, io.in[tk.slice],
                                                          reinterpret_cast<const T*>(ws + off[tk.slice]),
                                                          (size_t)P.W, (size_t)P.H, io.out[tk.slice], 1);
  }
}

template <class T, bool SCALE>
__global__ void __launch_bounds__(256) k_rag_sino_rows(const __grid_constant__ RaggedPlans<T> rp,
                                                       const RTask* __restrict__ tasks, int ntasks,
                                                       const __grid_constant__ RaggedIO<T> io, unsigned char* ws,
                                                       const size_t* __restrict__ off) {
  for (int t = blockIdx.x; t < ntasks; t += gridDim.x) {
    const RTask tk = tasks[t];
    const DevPlan<T>& P = rp.p[tk.slice];
    const int v = tk.a, D = P.D;
    const bool flip = P.flags[v] & 2;
    const T* y = io.in[tk.slice] + (size_t)v * D;
    T* q = reinterpret_cast<T*>(ws + off[tk.slice]) + (size_t)v * P.Dp;
    for (int d = threadIdx.x; d < P.Dp; d += blockDim.x) {
      T val = T(0);
      if (d < D) {
        val = y[flip ? D - 1 - d : d];
        if (SCALE) val *= P.fq[(size_t)v * D + d];
      }
      q[d] = val;
    }
  }
}

// The staged image gather of k_pix_gather (one slice per thread, two pixel
// rows, two straight-line cells in fp32, three in fp64; the step count never
// changes results), each CTA one task of the task list: the
// same arithmetic, view parts and fold points as a per-slice call, so the
// results are the same bit for bit. Sinogram planes [V][Dp] per slice at
// off_q, partial images [parts][H][W] at off_parts.
template <class T, int KIND>
__global__ void __launch_bounds__(32 * (kRagPixWarps + 1), (kPixCtas<T, 1>))
    k_rag_pix_gather(const __grid_constant__ RaggedPlans<T> rp, const RPixTask* __restrict__ tasks,
                     const __grid_constant__ RaggedIO<T> io, unsigned char* ws, const size_t* __restrict__ off_q,
                     const size_t* __restrict__ off_parts, int fbp_scale) {
  const RPixTask t = tasks[blockIdx.x];
  const DevPlan<T>& P = rp.p[t.slice];
  pix_gather_cta<T, 1, KIND, kTwoStep<T, 1> ? 2 : 3, false, kRagPX, false>(
      P, reinterpret_cast<const T*>(ws + off_q[t.slice]), io.out[t.slice],
      reinterpret_cast<T*>(ws + off_parts[t.slice]), 1, fbp_scale ? P.dAng : T(1), fbp_scale ? T(2) : T(1),
      view_split(P.V, (long long)P.W * P.H), t.bx, t.by, t.part);
}

// k_combine_parts over the slices whose views were split: task (slice, chunk
// of kCombineChunk pixels)
constexpr int kCombineChunk = 4096;
template <class T>
__global__ void __launch_bounds__(256) k_rag_combine(const __grid_constant__ RaggedPlans<T> rp,
                                                     const RTask* __restrict__ tasks, int ntasks,
                                                     const __grid_constant__ RaggedIO<T> io, unsigned char* ws,
                                                     const size_t* __restrict__ off_parts) {
  for (int t = blockIdx.x; t < ntasks; t += gridDim.x) {
    const RTask tk = tasks[t];
    const DevPlan<T>& P = rp.p[tk.slice];
    const size_t n = (size_t)P.H * P.W;
    const int np = view_split(P.V, (long long)P.W * P.H);
    const T* parts = reinterpret_cast<const T*>(ws + off_parts[tk.slice]);
    const size_t end = min(n, (size_t)(tk.a + 1) * kCombineChunk);
    for (size_t i = (size_t)tk.a * kCombineChunk + threadIdx.x; i < end; i += blockDim.x) {
      T s = T(0);
      for (int p = 0; p < np; ++p) s = add_rn(s, parts[(size_t)p * n + i]);
      io.out[tk.slice][i] = s;
    }
  }
}

template <class T>
__global__ void __launch_bounds__(256) k_rag_ramp(const __grid_constant__ RaggedPlans<T> rp,
                                                  const RTask* __restrict__ tasks, int ntasks,
                                                  const __grid_constant__ RaggedIO<T> io, unsigned char* ws,
                                                  const size_t* __restrict__ off) {
  extern __shared__ unsigned char smem_raw[];
  for (int t = blockIdx.x; t < ntasks; t += gridDim.x) {
    const RTask tk = tasks[t];
    const DevPlan<T>& P = rp.p[tk.slice];
    ramp_filter_view<T, 1>(P, tk.a, 0, io.in[tk.slice], reinterpret_cast<T*>(ws + off[tk.slice]), P.Dp, 1,
                           reinterpret_cast<T*>(smem_raw));
  }
}

// ----------------------------------------------------------------------------
// projection without any allocation
// ----------------------------------------------------------------------------
// Scratch for ctgb_projection_noalloc lives in this module's own static device
// memory instead of a caller-provided buffer. Its size is fixed: every GPU on
// which this library's kernels are loaded reserves these bytes until process
// exit. Host code only knows the array through cudaGetSymbolAddress (the name
// itself is a host-side stand-in, not a device address). The device address is
// looked up with the device current, once per device and CUDA context: the
// cache is keyed on the context's process-unique ID (cuCtxGetId), so a context
// torn down and created again (cudaDeviceReset) gets a fresh lookup instead of
// a dead address.
constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;  // 64 MiB
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mu;
struct NoAllocEntry {
  unsigned long long ctx_id;  // 0: not looked up yet (context IDs start at 1)
  void* ptr;
};
static NoAllocEntry g_noalloc_dev[256] = {};

// ID of the calling thread's current context, through the driver entry point
// (the library links only the CUDA runtime, so it loads where no driver is)
static int current_context_id(unsigned long long* id) {
  using CtxGetId = CUresult (*)(CUcontext, unsigned long long*);
  static CtxGetId fn = nullptr;
  if (!fn) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    const cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !f)
      return fail(CTGB_ERR_CUDA, std::string("cuCtxGetId entry point: ") + cudaGetErrorString(e));
    fn = reinterpret_cast<CtxGetId>(f);
  }
  const CUresult r = fn(nullptr, id);
  if (r != CUDA_SUCCESS) return fail(CTGB_ERR_CUDA, "cuCtxGetId failed with driver error " + std::to_string((int)r));
  return CTGB_OK;
}

// Device address of the scratch array on `device`, which must be current.
static int noalloc_scratch(int device, void** out) {
  if (device < 0 || device >= 256) return fail(CTGB_ERR_INVALID, "device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  unsigned long long ctx = 0;
  int rc = current_context_id(&ctx);
  if (rc != CTGB_OK) return rc;
  NoAllocEntry& ent = g_noalloc_dev[device];
  if (ent.ctx_id != ctx || !ent.ptr) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(CTGB_ERR_CUDA, std::string("scratch symbol address: ") + cudaGetErrorString(e));
    ent.ptr = ptr;
    ent.ctx_id = ctx;
  }
  *out = ent.ptr;
  return CTGB_OK;
}

static int projection_noalloc(const ctgb_plan* p, const void* image, void* sino, int batch, void* stream) {
  if (!p) return fail(CTGB_ERR_INVALID, "null plan");
  if (batch <= 0) return batch == 0 ? CTGB_OK : fail(CTGB_ERR_INVALID, "negative batch");
  const size_t need = workspace_bytes(p, CTGB_OP_PROJECTION, batch);
  if (need > kNoAllocScratchBytes)
    return fail(CTGB_ERR_WORKSPACE, "ctgb_projection_noalloc: batch of " + std::to_string(batch) + " needs " +
                                        std::to_string(need) + " scratch bytes, above the fixed " +
                                        std::to_string(kNoAllocScratchBytes) +
                                        "-byte static buffer; use ctgb_projection with a caller workspace");
  int cur = -1;
  CTGB_CUDA(cudaGetDevice(&cur));
  if (cur != p->device) CTGB_CUDA(cudaSetDevice(p->device));
  void* ws = nullptr;
  int rc = noalloc_scratch(p->device, &ws);
  // Nothing left in the array by an earlier call (possibly of another plan,
  // with other line lengths) needs clearing: the layout kernel writes every
  // element the detector gather reads, and the gather clamps its pixel index
  // to N - 1, so it never reads the padding columns of a line (round8(N) - N
  // of them), which the layout kernel leaves as they were.
  if (rc == CTGB_OK) rc = dispatch(p, CTGB_OP_PROJECTION, image, sino, batch, ws, kNoAllocScratchBytes, stream);
  if (cur != p->device && cur >= 0) cudaSetDevice(cur);
  return rc;
}

struct RaggedStage {
  const void* tasks = nullptr;  // device: RTask, or RPixTask for the image gather
  int n = 0;
  int grid = 0;
};

}  // namespace ctgb

struct ctgb_ragged {
  int n = 0, device = 0, maxD = 0, dtype = 0;
  void* dev = nullptr;
  void* host_plans = nullptr;  // every slice's DevPlan<T> (RaggedPlans<T>), passed by value to the kernels
  const size_t* off_img = nullptr;    // per slice: transposed image in the workspace
  const size_t* off_sino = nullptr;   // per slice: sinogram planes [V][Dp] in the workspace
  const size_t* off_parts = nullptr;  // per slice: partial images of the view parts
  size_t ws_img = 0, ws_sino = 0;
  size_t pix_smem = 0;
  ctgb::RaggedStage transpose, detg, rows, pixg, ramp, combine;
};

namespace ctgb {

template <class T>
static const DevPlan<T>& plan_of(const ctgb_plan* p) {
  if constexpr (sizeof(T) == 4) return p->pf; else return p->pd;
}

static void free_host_plans(ctgb_ragged* r) {
  if (r->dtype == 0) delete static_cast<RaggedPlans<float>*>(r->host_plans);
  else delete static_cast<RaggedPlans<double>*>(r->host_plans);
  r->host_plans = nullptr;
}

template <class T>
static int ragged_build(ctgb_ragged* r, const ctgb_plan* const* plans, int n) {
  std::vector<DevPlan<T>> dp(n);
  std::vector<size_t> oi(n), os(n), opt(n);
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  // task lists, each entry with its length for the longest-first order
  std::vector<std::pair<long, RTask>> tr, dg, rw, rp, cb;
  std::vector<std::pair<long, RPixTask>> pg;
  auto* hp = new RaggedPlans<T>();
  r->host_plans = hp;
  const size_t es = sizeof(T);
  for (int i = 0; i < n; ++i) {
    const HostGeom& g = plans[i]->geom;
    dp[i] = plan_of<T>(plans[i]);
    hp->p[i] = dp[i];
    const int Dp = dp[i].Dp;
    const int np = view_split(g.V, (long long)g.W * g.H);
    oi[i] = r->ws_img;
    r->ws_img += al((size_t)g.H * g.W * es);
    os[i] = r->ws_sino;
    r->ws_sino += al((size_t)g.V * Dp * es);
    opt[i] = r->ws_sino;
    if (np > 1) r->ws_sino += al((size_t)np * g.H * g.W * es);
    if (g.D > r->maxD) r->maxD = g.D;
    const long lines = g.H > g.W ? g.H : g.W;
    for (int a = 0; a < (g.H + 31) / 32; ++a)
      for (int b = 0; b < (g.W + 31) / 32; ++b) tr.push_back({1, {i, a, b}});
    for (int a = 0; a < (g.V + kRagDetWarps - 1) / kRagDetWarps; ++a)
      for (int b = 0; b < (g.D + 31) / 32; ++b) dg.push_back({lines, {i, a, b}});
    for (int a = 0; a < g.V; ++a) {
      rw.push_back({g.D, {i, a, 0}});
      rp.push_back({(long)g.D * g.D, {i, a, 0}});
    }
    // a CTA's time grows with its views (a part's) and its pixels per thread
    const long pix_len = (long)(g.V / np) * 64;
    for (int part = 0; part < np; ++part)
      for (int by = 0; by < (g.H + kRagPixRows - 1) / kRagPixRows; ++by)
        for (int bx = 0; bx < (g.W + 31) / 32; ++bx) pg.push_back({pix_len, {i, bx, by, part}});
    if (np > 1)
      for (int a = 0; a < (int)(((size_t)g.H * g.W + kCombineChunk - 1) / kCombineChunk); ++a)
        cb.push_back({np, {i, a, 0}});
  }
  // longest tasks first (stable, so a slice's tasks stay together)
  auto by_len = [](const auto& x, const auto& y) { return x.first > y.first; };
  for (auto* v : {&tr, &dg, &rw, &rp, &cb}) std::stable_sort(v->begin(), v->end(), by_len);
  std::stable_sort(pg.begin(), pg.end(), by_len);
  const size_t b_off = al(sizeof(size_t) * n);
  std::vector<std::pair<std::vector<unsigned char>, size_t>> lists;  // bytes, entries
  auto pack = [&](const auto& v) {
    using E = typename std::decay_t<decltype(v)>::value_type::second_type;
    std::vector<unsigned char> b(sizeof(E) * v.size());
    for (size_t k = 0; k < v.size(); ++k) std::memcpy(b.data() + k * sizeof(E), &v[k].second, sizeof(E));
    lists.push_back({std::move(b), v.size()});
  };
  pack(tr); pack(dg); pack(rw); pack(pg); pack(rp); pack(cb);
  size_t total = 3 * b_off;
  for (auto& l : lists) total += al(l.first.size() ? l.first.size() : 1);
  std::vector<unsigned char> host(total, 0);
  size_t o = 0;
  auto put = [&](const void* src, size_t bytes, size_t span) {
    if (bytes) std::memcpy(host.data() + o, src, bytes);
    const size_t at = o;
    o += span;
    return at;
  };
  const size_t o_oi = put(oi.data(), sizeof(size_t) * n, b_off);
  const size_t o_os = put(os.data(), sizeof(size_t) * n, b_off);
  const size_t o_op = put(opt.data(), sizeof(size_t) * n, b_off);
  size_t o_stage[6];
  for (int k = 0; k < 6; ++k)
    o_stage[k] = put(lists[k].first.data(), lists[k].first.size(), al(lists[k].first.size() ? lists[k].first.size() : 1));
  CTGB_CUDA(cudaMalloc(&r->dev, total));
  CTGB_CUDA(cudaMemcpy(r->dev, host.data(), total, cudaMemcpyHostToDevice));
  unsigned char* base = static_cast<unsigned char*>(r->dev);
  r->off_img = reinterpret_cast<const size_t*>(base + o_oi);
  r->off_sino = reinterpret_cast<const size_t*>(base + o_os);
  r->off_parts = reinterpret_cast<const size_t*>(base + o_op);
  RaggedStage* st[6] = {&r->transpose, &r->detg, &r->rows, &r->pixg, &r->ramp, &r->combine};
  r->pix_smem =
      (size_t)2 * kRagPX * 1 * (32 * kRagPixWarps) * es + (size_t)kSlots<T, 1, kRagPX> * PixSlot<T, 1>::kBytes;
  for (const void* f : {(const void*)k_rag_pix_gather<T, kAt>, (const void*)k_rag_pix_gather<T, kB>})
    CTGB_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)r->pix_smem));
  const size_t ramp_smem = ramp_smem_elems(r->maxD, 1) * es;
  if (ramp_smem > 48 * 1024)
    CTGB_CUDA(cudaFuncSetAttribute((const void*)k_rag_ramp<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)ramp_smem));
  // one CTA per task in every stage: the block scheduler hands tasks out in
  // list order (longest first) as CTAs finish, which balances the stage; a
  // persistent grid walking the list with a fixed stride left some CTAs with
  // far more work than others
  for (int i = 0; i < 6; ++i) {
    st[i]->tasks = base + o_stage[i];
    st[i]->n = (int)lists[i].second;
    st[i]->grid = st[i]->n;
  }
  return CTGB_OK;
}

template <class T>
static int ragged_run_t(const ctgb_ragged* r, int op, const void* const* in, void* const* out, void* ws,
                        void* stream) {
  RaggedIO<T> io{};
  for (int i = 0; i < r->n; ++i) {
    if (!in[i] || !out[i]) return fail(CTGB_ERR_INVALID, "null slice pointer");
    io.in[i] = static_cast<const T*>(in[i]);
    io.out[i] = static_cast<T*>(out[i]);
  }
  const RaggedPlans<T>& hp = *static_cast<const RaggedPlans<T>*>(r->host_plans);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* w = static_cast<unsigned char*>(ws);
  auto rt = [](const RaggedStage& s) { return static_cast<const RTask*>(s.tasks); };
  if (op == CTGB_OP_PROJECTION || op == CTGB_OP_BACKPROJECTION_T) {
    k_rag_transpose<T><<<r->transpose.grid, 256, 0, st>>>(hp, rt(r->transpose), r->transpose.n, io, w,
                                                          r->off_img);
    const int nt = 32 * kRagDetWarps;
    const size_t acc_smem = (size_t)2 * nt * sizeof(T);
    if (op == CTGB_OP_PROJECTION)
      k_rag_det_gather<T, kA><<<r->detg.grid, nt, acc_smem, st>>>(hp, rt(r->detg), r->detg.n, io, w,
                                                                  r->off_img);
    else
      k_rag_det_gather<T, kBt><<<r->detg.grid, nt, acc_smem, st>>>(hp, rt(r->detg), r->detg.n, io, w,
                                                                   r->off_img);
  } else {
    if (op == CTGB_OP_FBP) {
      const size_t smem = ramp_smem_elems(r->maxD, 1) * sizeof(T);
      // one slice per task: 2 * ceil(D / 16) work items, 46 to 128 for rows of
      // 368 to 1024 bins
      k_rag_ramp<T><<<r->ramp.grid, 128, smem, st>>>(hp, rt(r->ramp), r->ramp.n, io, w, r->off_sino);
    } else if (op == CTGB_OP_PROJECTION_T) {
      k_rag_sino_rows<T, true><<<r->rows.grid, 256, 0, st>>>(hp, rt(r->rows), r->rows.n, io, w, r->off_sino);
    } else {
      k_rag_sino_rows<T, false><<<r->rows.grid, 256, 0, st>>>(hp, rt(r->rows), r->rows.n, io, w, r->off_sino);
    }
    const RPixTask* pt = static_cast<const RPixTask*>(r->pixg.tasks);
    const int nt = 32 * (kRagPixWarps + 1);
    if (op == CTGB_OP_PROJECTION_T)
      k_rag_pix_gather<T, kAt><<<r->pixg.grid, nt, r->pix_smem, st>>>(hp, pt, io, w, r->off_sino, r->off_parts, 0);
    else
      k_rag_pix_gather<T, kB><<<r->pixg.grid, nt, r->pix_smem, st>>>(hp, pt, io, w, r->off_sino, r->off_parts,
                                                                     op == CTGB_OP_FBP ? 1 : 0);
    if (r->combine.n > 0)
      k_rag_combine<T><<<r->combine.grid, 256, 0, st>>>(hp, rt(r->combine), r->combine.n, io, w, r->off_parts);
  }
  return CTGB_OK;
}

static int ragged_run(const ctgb_ragged* r, int op, const void* const* in, void* const* out, void* ws,
                      size_t wsb, void* stream) {
  if (!r) return fail(CTGB_ERR_INVALID, "null ragged batch");
  if (!in || !out) return fail(CTGB_ERR_INVALID, "null pointer arrays");
  if (op < 0 || op > 4) return fail(CTGB_ERR_INVALID, "unknown operator");
  const size_t need = (op == CTGB_OP_PROJECTION || op == CTGB_OP_BACKPROJECTION_T) ? r->ws_img : r->ws_sino;
  if (!ws || wsb < need) return fail(CTGB_ERR_WORKSPACE, "workspace too small: need " + std::to_string(need));
  if ((reinterpret_cast<uintptr_t>(ws) & 255) != 0) return fail(CTGB_ERR_INVALID, "workspace must be 256-byte aligned");
  int cur = -1;
  CTGB_CUDA(cudaGetDevice(&cur));
  if (cur != r->device) CTGB_CUDA(cudaSetDevice(r->device));
  int rc = r->dtype == 0 ? ragged_run_t<float>(r, op, in, out, ws, stream)
                         : ragged_run_t<double>(r, op, in, out, ws, stream);
  const cudaError_t e = cudaGetLastError();
  if (cur != r->device && cur >= 0) cudaSetDevice(cur);
  if (rc != CTGB_OK) return rc;
  if (e != cudaSuccess) return fail(CTGB_ERR_CUDA, std::string("ragged launch: ") + cudaGetErrorString(e));
  return CTGB_OK;
}

}  // namespace ctgb

// ----------------------------------------------------------------------------
// C ABI
// ----------------------------------------------------------------------------
extern "C" {

int ctgb_version(void) { return 1; }

const char* ctgb_last_error(void) { return ctgb::g_err.c_str(); }

int ctgb_wait_timeouts(int device, unsigned long long* count, int reset) {
  using namespace ctgb;
  if (!count) return fail(CTGB_ERR_INVALID, "null count");
  int cur = -1;
  CTGB_CUDA(cudaGetDevice(&cur));
  if (cur != device) CTGB_CUDA(cudaSetDevice(device));
  cudaError_t e = cudaMemcpyFromSymbol(count, g_wait_timeouts, sizeof(unsigned long long));
  if (e == cudaSuccess && reset) {
    const unsigned long long zero = 0;
    e = cudaMemcpyToSymbol(g_wait_timeouts, &zero, sizeof(zero));
  }
  if (cur != device && cur >= 0) cudaSetDevice(cur);
  if (e != cudaSuccess) return fail(CTGB_ERR_CUDA, std::string("wait counter: ") + cudaGetErrorString(e));
  return CTGB_OK;
}

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

int ctgb_plan_set_schedule(ctgb_plan* plan, int op, int slices_per_thread, int warps_per_cta) {
  if (!plan) return ctgb::fail(CTGB_ERR_INVALID, "null plan");
  if (op < 0 || op > 5) return ctgb::fail(CTGB_ERR_INVALID, "unknown operator");
  if (!(slices_per_thread == 0 || slices_per_thread == 1 || slices_per_thread == 2 || slices_per_thread == 4 ||
        slices_per_thread == 8 || slices_per_thread == 16))
    return ctgb::fail(CTGB_ERR_INVALID, "slices_per_thread must be 0 (default), 1, 2, 4, 8 or 16");
  if (!(warps_per_cta == 0 || warps_per_cta == 4 || warps_per_cta == 8))
    return ctgb::fail(CTGB_ERR_INVALID, "warps_per_cta must be 0 (default), 4 or 8");
  plan->sb_cap[op] = slices_per_thread;
  plan->warps[op] = warps_per_cta == 0 ? 8 : warps_per_cta;
  return CTGB_OK;
}

int ctgb_plan_set_kernel_events(ctgb_plan* plan, void* start_event, void* stop_event) {
  if (!plan) return ctgb::fail(CTGB_ERR_INVALID, "null plan");
  if ((start_event == nullptr) != (stop_event == nullptr))
    return ctgb::fail(CTGB_ERR_INVALID, "give both events or neither");
  plan->ev_start = static_cast<cudaEvent_t>(start_event);
  plan->ev_stop = static_cast<cudaEvent_t>(stop_event);
  return CTGB_OK;
}

int ctgb_plan_set_filter(ctgb_plan* plan, int window, int ea_exact) {
  using namespace ctgb;
  if (!plan) return fail(CTGB_ERR_INVALID, "null plan");
  HostGeom g2 = plan->geom;
  std::string err;
  if (!filter_taps(g2, window, ea_exact != 0, err)) return fail(CTGB_ERR_INVALID, err);
  int cur = -1;
  CTGB_CUDA(cudaGetDevice(&cur));
  if (cur != plan->device) CTGB_CUDA(cudaSetDevice(plan->device));
  // kernels of this plan still in flight may be reading the taps
  cudaError_t e = cudaDeviceSynchronize();
  const size_t n = g2.taps.size();
  if (e == cudaSuccess) {
    if (plan->dtype == 0) {
      std::vector<float> hi(n), lo(n);
      for (size_t i = 0; i < n; ++i) { hi[i] = (float)g2.taps[i]; lo[i] = (float)g2.taps_lo[i]; }
      e = cudaMemcpy(const_cast<float*>(plan->pf.taps), hi.data(), n * sizeof(float), cudaMemcpyHostToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(const_cast<float*>(plan->pf.tapl), lo.data(), n * sizeof(float), cudaMemcpyHostToDevice);
    } else {
      e = cudaMemcpy(const_cast<double*>(plan->pd.taps), g2.taps.data(), n * sizeof(double), cudaMemcpyHostToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(const_cast<double*>(plan->pd.tapl), g2.taps_lo.data(), n * sizeof(double),
                       cudaMemcpyHostToDevice);
    }
  }
  if (cur != plan->device && cur >= 0) cudaSetDevice(cur);
  if (e != cudaSuccess) return fail(CTGB_ERR_CUDA, std::string("filter taps: ") + cudaGetErrorString(e));
  plan->geom.taps = g2.taps;
  plan->geom.taps_lo = g2.taps_lo;
  plan->pf.even_taps = plan->pd.even_taps = window != kRamLak;
  return CTGB_OK;
}

int ctgb_plan_set_wait_limit(ctgb_plan* plan, unsigned long long limit_ns) {
  if (!plan) return ctgb::fail(CTGB_ERR_INVALID, "null plan");
  if (limit_ns > 10 * ctgb::kWaitLimitNs)
    return ctgb::fail(CTGB_ERR_INVALID, "wait limit above 10 s; the default is 1 s");
  plan->pf.wait_ns = plan->pd.wait_ns = limit_ns;
  return CTGB_OK;
}

int ctgb_plan_set_summation(ctgb_plan* plan, int compensated) {
  if (!plan) return ctgb::fail(CTGB_ERR_INVALID, "null plan");
  if (compensated != 0 && compensated != 1) return ctgb::fail(CTGB_ERR_INVALID, "compensated must be 0 or 1");
  if (!compensated && plan->dtype != CTGB_FLOAT32)
    return ctgb::fail(CTGB_ERR_INVALID, "plain summation is offered for float32 plans only");
  plan->plain = !compensated;
  return CTGB_OK;
}

int ctgb_plan_set_unroll(ctgb_plan* plan, int op, int steps) {
  if (!plan) return ctgb::fail(CTGB_ERR_INVALID, "null plan");
  if (op < 0 || op > 5) return ctgb::fail(CTGB_ERR_INVALID, "unknown operator");
  if (!(steps == 0 || steps == 2 || steps == 3)) return ctgb::fail(CTGB_ERR_INVALID, "steps must be 0 (default), 2 or 3");
  plan->unroll[op] = steps == 0 ? 3 : steps;
  return CTGB_OK;
}

size_t ctgb_workspace_size(const ctgb_plan* plan, int op, int batch) {
  if (!plan || batch <= 0 || op < 0 || op > 6) return 0;
  if (op == CTGB_OP_DATA_GRADIENT) return ctgb::gradient_workspace_bytes(plan, batch);
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
int ctgb_backprojection_sv(const ctgb_plan* p, const void* sino, void* images, int batch, void* ws, size_t wsb,
                           void* stream) {
  return ctgb::dispatch(p, CTGB_OP_BACKPROJECTION_SV, sino, images, batch, ws, wsb, stream);
}
int ctgb_data_gradient(const ctgb_plan* p, const void* image, const void* sino, void* residual, void* grad, int batch,
                       void* ws, size_t wsb, void* stream) {
  return ctgb::dispatch_gradient(p, image, sino, residual, grad, batch, ws, wsb, stream);
}

int ctgb_projection_noalloc(const ctgb_plan* p, const void* image, void* sino, int batch, void* stream) {
  return ctgb::projection_noalloc(p, image, sino, batch, stream);
}

size_t ctgb_projection_noalloc_max_bytes(void) { return ctgb::kNoAllocScratchBytes; }

int ctgb_ragged_create(ctgb_ragged** ragged, const ctgb_plan* const* plans, int n_slices, int device) {
  if (!ragged || !plans) return ctgb::fail(CTGB_ERR_INVALID, "null pointer");
  *ragged = nullptr;
  if (n_slices < 1 || n_slices > ctgb::kMaxRagged)
    return ctgb::fail(CTGB_ERR_INVALID, "ragged batches hold 1 to " + std::to_string(ctgb::kMaxRagged) + " slices");
  for (int i = 0; i < n_slices; ++i) {
    if (!plans[i]) return ctgb::fail(CTGB_ERR_INVALID, "null plan in ragged batch");
    if (plans[i]->dtype != plans[0]->dtype)
      return ctgb::fail(CTGB_ERR_INVALID, "the plans of a ragged batch share one dtype");
    if (plans[i]->device != device) return ctgb::fail(CTGB_ERR_INVALID, "plan on another device");
  }
  auto* r = new ctgb_ragged();
  r->n = n_slices;
  r->device = device;
  r->dtype = plans[0]->dtype;
  int cur = -1;
  cudaGetDevice(&cur);
  cudaSetDevice(device);
  int rc = r->dtype == 0 ? ctgb::ragged_build<float>(r, plans, n_slices) : ctgb::ragged_build<double>(r, plans, n_slices);
  if (cur >= 0) cudaSetDevice(cur);
  if (rc != CTGB_OK) {
    if (r->dev) cudaFree(r->dev);
    ctgb::free_host_plans(r);
    delete r;
    return rc;
  }
  *ragged = r;
  return CTGB_OK;
}

int ctgb_ragged_destroy(ctgb_ragged* ragged) {
  if (!ragged) return CTGB_OK;
  if (ragged->dev) cudaFree(ragged->dev);
  ctgb::free_host_plans(ragged);
  delete ragged;
  return CTGB_OK;
}

size_t ctgb_ragged_workspace_size(const ctgb_ragged* ragged, int op) {
  if (!ragged || op < 0 || op > 4) return 0;
  return (op == CTGB_OP_PROJECTION || op == CTGB_OP_BACKPROJECTION_T) ? ragged->ws_img : ragged->ws_sino;
}

int ctgb_ragged_run(const ctgb_ragged* ragged, int op, const void* const* in, void* const* out, void* workspace,
                    size_t workspace_bytes, void* stream) {
  return ctgb::ragged_run(ragged, op, in, out, workspace, workspace_bytes, stream);
}

long ctgb_geometry_query(const double* options, int n_options, int dtype, int what, double* out, size_t n_out) {
  ctgb::HostGeom g;
  std::string err;
  if (!ctgb::build_geometry(options, n_options, dtype, g, err)) {
    ctgb::fail(CTGB_ERR_INVALID, err);
    return -1;
  }
  std::vector<double> flags(g.flags.begin(), g.flags.end());
  std::vector<double> split;
  if (what == 7) {  // the image gather's line maps as the device stores them
    const int L = g.L;
    split.assign((size_t)g.V * L * 4, 0.0);
    for (size_t i = 0; i < (size_t)g.V * L; ++i) {
      const double alpha = g.lp[2 * i], sigma = g.lp[2 * i + 1];
      if (!(sigma > 0)) continue;
      double* o = &split[4 * i];
      ctgb::split_line_map(alpha, sigma, (g.flags[i / L] & 1) ? g.W : g.H, dtype == 0 ? 24 : 53, o);
      if (dtype == 0)
        for (int j = 0; j < 4; ++j) o[j] = (double)(float)o[j];
    }
  }
  const std::vector<double>* src = nullptr;
  switch (what) {
    case 0: src = &flags; break;
    case 1: src = &g.db; break;
    case 2: src = &g.fq; break;
    case 3: src = &g.lp; break;
    case 4: src = &g.inv; break;
    case 5: src = &g.wpre; break;
    case 6: src = &g.taps; break;
    case 7: src = &split; break;
    default: ctgb::fail(CTGB_ERR_INVALID, "unknown geometry table"); return -1;
  }
  if (out) {
    const size_t n = std::min(n_out, src->size());
    std::memcpy(out, src->data(), n * sizeof(double));
  }
  return (long)src->size();
}

}  // extern "C"
