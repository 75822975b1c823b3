// kNN graph adjacency of CTLIB's `laplacian` (src/laplacian_cuda_kernel.cu:46-128,
// src/ctlib.cpp:101-104) for GB300 (sm_103a), behind ctgb_laplacian in ctgb.h.
//
// For n points x_i of dimension dim the reference builds the full n x n matrix
// dist[i][j] = |x_i|^2 + |x_j|^2 - 2 <x_i, x_j> (a norm kernel, a norm-sum
// kernel and a GEMM), takes the k smallest entries of every row with
// torch::topk, divides them by the median of all n*k selected distances,
// applies exp(-.), normalises each row to sum 1 and returns a sparse COO
// matrix with float32 values.
//
// Here the n x n matrix never exists. One kernel computes 64 x 128 tiles of
// distances from shared-memory chunks of the points (register-blocked FP32 or
// FP64 FMAs, each warp 8 rows x 128 columns) and folds them from registers
// straight into per-row sorted lists of the k best (distance, column) pairs;
// column ranges are split over CTAs to fill the GPU and the partial lists
// merged. The lists are ordered by
// distance, then by column index, so the selected set and its order do not
// depend on the tile schedule or the split (ties go to the smaller index). The
// median is a radix select over the n*k selected distances (the lower median,
// as torch::median) and a last kernel writes the COO indices and weights.
//
// Traffic: the points are read once per 128-column tile from L2; HBM sees the
// points, the n*k lists and the output, instead of 2 n^2 distances.

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <string>

#include "ctgb.h"
#include "ctgb_internal.h"

namespace ctgb {
namespace lap {

constexpr int TM = 64;    // rows (points i) per CTA
constexpr int TN = 128;   // columns (points j) per tile
constexpr int DC = 32;    // dimension chunk staged in shared memory
constexpr int NT = 256;   // threads per CTA: 16 x 16, 4 rows x 8 columns each
constexpr int SA = TM + 4, SBW = TN + 4;  // padded row strides (16-byte multiples)
constexpr int kMaxSplit = 8;
constexpr int kMaxK = 256;

template <class T>
__device__ __forceinline__ bool lexless(T av, int ai, T bv, int bi) {
  return av < bv || (av == bv && ai < bi);
}

template <class T>
__device__ __forceinline__ void ld4s(const T* p, T* v) {
  if constexpr (sizeof(T) == 4) {
    const float4 a = *reinterpret_cast<const float4*>(p);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  } else {
    const double2 a = reinterpret_cast<const double2*>(p)[0];
    const double2 b = reinterpret_cast<const double2*>(p)[1];
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
}

// |x_i|^2 in the reference's order: sum += v * v over the dimension, one FMA
// per term (src/laplacian_cuda_kernel.cu:10-22)
template <class T>
__global__ void k_sqnorm(const T* __restrict__ x, int n, int dim, T* __restrict__ norm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T* r = x + (size_t)i * dim;
  T s = T(0);
  for (int d = 0; d < dim; ++d) s = fma(r[d], r[d], s);
  norm[i] = s;
}

// Insert (cv, cj) into the sorted list (Lv, Li) of K entries, dropping the
// last one; the whole warp takes part. The caller guarantees that (cv, cj)
// precedes the last entry. Lists of up to 32 entries are shifted through
// registers (lane e holds entry e), longer ones chunk by chunk in shared memory.
template <class T>
__device__ __forceinline__ void list_insert(T* Lv, int* Li, int K, T cv, int cj, int lane) {
  if (K <= 32) {
    const bool in = lane < K;
    T v = in ? Lv[lane] : T(0);
    int ix = in ? Li[lane] : INT_MAX;
    const int p = __popc(__ballot_sync(0xffffffffu, in && lexless(v, ix, cv, cj)));
    const T uv = __shfl_up_sync(0xffffffffu, v, 1);
    const int ui = __shfl_up_sync(0xffffffffu, ix, 1);
    if (lane == p) { v = cv; ix = cj; }
    else if (lane > p) { v = uv; ix = ui; }
    __syncwarp();
    if (in) { Lv[lane] = v; Li[lane] = ix; }
    __syncwarp();
    return;
  }
  int p = 0;
  for (int e0 = 0; e0 < K; e0 += 32) {
    const int e = e0 + lane;
    const bool less = e < K && lexless(Lv[e], Li[e], cv, cj);
    p += __popc(__ballot_sync(0xffffffffu, less));
  }
  // shift [p, K-2] up by one, highest chunk first so no entry is overwritten
  // before it is read
  const int nmove = K - 1 - p;
  for (int m = nmove > 0 ? (nmove - 1) / 32 : -1; m >= 0; --m) {
    const int e = p + 1 + lane + 32 * m;
    const bool act = e <= K - 1;
    T v = T(0);
    int ix = 0;
    if (act) { v = Lv[e - 1]; ix = Li[e - 1]; }
    __syncwarp();
    if (act) { Lv[e] = v; Li[e] = ix; }
    __syncwarp();
  }
  if (lane == 0) { Lv[p] = cv; Li[p] = cj; }
  __syncwarp();
}

// lists of up to kStageK entries leave room for a per-warp staging area of the
// tile's distances at three CTAs per SM
constexpr int kStageK = 32;

template <class T>
size_t knn_smem_bytes(int K) {
  const size_t stage = K <= kStageK ? (size_t)TM * TN : 0;
  return ((size_t)DC * SA + (size_t)DC * SBW + stage + (size_t)TM * K) * sizeof(T) + (size_t)TM * K * 4;
}

// ordered unsigned keys of floating-point values (sign-magnitude flipped)
template <class T>
struct Key;
template <>
struct Key<float> {
  using U = unsigned int;
  static constexpr int kPasses = 4;
  __device__ static U enc(float v) {
    const U u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
  }
  __device__ static float dec(U k) { return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k); }
};
template <>
struct Key<double> {
  using U = unsigned long long;
  static constexpr int kPasses = 8;
  __device__ static U enc(double v) {
    const U u = (U)__double_as_longlong(v);
    return (u >> 63) ? ~u : (u | (1ull << 63));
  }
  __device__ static double dec(U k) { return __longlong_as_double((long long)((k >> 63) ? (k & ~(1ull << 63)) : ~k)); }
};

// lowers a row's shared bound to v (an fp32 K-th distance; NaN or +inf leave it)
template <class T>
__device__ __forceinline__ void publish_bound(unsigned* b, T v) {
  const float f = (float)v;
  if (f < INFINITY) atomicMin(b, Key<float>::enc(f));
}

// Stage one DC-wide chunk of the points [base, base + rows) (rows < lim are
// real, the rest zero) into s[kk][row] (row stride S). With `vec` the rows are
// read as 16-byte vectors along the dimension (dim a multiple of the vector
// width, 16-byte aligned rows), else element by element.
template <class T, int ROWS, int S>
__device__ __forceinline__ void stage_chunk(T* __restrict__ s, const T* __restrict__ x, int base, int lim, int dim,
                                            int k0, int kc, bool vec) {
  constexpr int VW = 16 / (int)sizeof(T);
  if (vec) {
    constexpr int NV = DC / VW;
    for (int e = threadIdx.x; e < ROWS * NV; e += NT) {
      const int r = e / NV, kv = e % NV;
      const int g = base + r;
      T v[VW];
      if (g < lim && kv * VW < kc) {
        const T* src = x + (size_t)g * dim + k0 + kv * VW;
        if constexpr (sizeof(T) == 4) {
          const float4 a = *reinterpret_cast<const float4*>(src);
          v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        } else {
          const double2 a = *reinterpret_cast<const double2*>(src);
          v[0] = a.x; v[1] = a.y;
        }
      } else {
#pragma unroll
        for (int t = 0; t < VW; ++t) v[t] = T(0);
      }
#pragma unroll
      for (int t = 0; t < VW; ++t) s[(kv * VW + t) * S + r] = v[t];
    }
  } else {
    for (int e = threadIdx.x; e < ROWS * DC; e += NT) {
      const int r = e / DC, kk = e % DC;
      const int g = base + r;
      s[kk * S + r] = (g < lim && kk < kc) ? x[(size_t)g * dim + k0 + kk] : T(0);
    }
  }
}

// Warp-wide bitonic sort of 128 (value, column) pairs, 4 per lane (element
// 4 * lane + q), ascending in (value, column) order.
template <class T>
__device__ __forceinline__ void warp_sort128(T (&v)[4], int (&ix)[4], int lane) {
#pragma unroll
  for (int s = 2; s <= 128; s <<= 1) {
#pragma unroll
    for (int jj = s >> 1; jj > 0; jj >>= 1) {
      if (jj >= 4) {
        const int lm = jj >> 2;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const T pv = __shfl_xor_sync(0xffffffffu, v[q], lm);
          const int pi = __shfl_xor_sync(0xffffffffu, ix[q], lm);
          const int e = 4 * lane + q;
          const bool keep_min = ((e & jj) == 0) == ((e & s) == 0);
          const bool take = keep_min ? lexless(pv, pi, v[q], ix[q]) : lexless(v[q], ix[q], pv, pi);
          if (take) { v[q] = pv; ix[q] = pi; }
        }
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (q & jj) continue;
          const int q2 = q | jj;
          const bool asc = ((4 * lane + q) & s) == 0;
          const bool sw = asc ? lexless(v[q2], ix[q2], v[q], ix[q]) : lexless(v[q], ix[q], v[q2], ix[q2]);
          if (sw) {
            const T tv = v[q]; v[q] = v[q2]; v[q2] = tv;
            const int ti = ix[q]; ix[q] = ix[q2]; ix[q2] = ti;
          }
        }
      }
    }
  }
}

// Rows [i0, i0 + TM) against columns [c_begin, c_end): the K smallest
// (distance, column) pairs of each row, sorted, into out_v / out_i at
// [(row * nsplit + split) * K]. dist = fma(-2, <x_i, x_j>, |x_j|^2 + |x_i|^2),
// the reference's norm sum with the GEMM's -2 x^T x added
// (src/laplacian_cuda_kernel.cu:25-43, 88-106).
//
// Warp w owns rows 8w .. 8w+7 of the block: per 128-column tile each lane
// accumulates 8 rows x 4 columns (lane l: columns 4l .. 4l+3) from the shared
// chunks and then folds its distances straight into the warp's lists (kept in
// shared memory): the first tile of a split is sorted whole (when K <= 128),
// later tiles insert only candidates that beat the current K-th entry. Three
// CTAs per SM for fp32 (80 registers); fp64 needs more registers and runs one.
template <class T>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? 3 : 1)
    k_knn(const T* __restrict__ x, const T* __restrict__ norm, int n, int dim, int K, int cols_per_split, int nsplit,
          bool vec, T* __restrict__ out_v, int* __restrict__ out_i, unsigned* __restrict__ gbound) {
  extern __shared__ __align__(16) unsigned char lap_smem[];
  T* sA = reinterpret_cast<T*>(lap_smem);  // [DC][SA]: x_i chunk, transposed
  T* sB = sA + DC * SA;                     // [DC][SBW]: x_j chunk, transposed
  const bool staged = K <= kStageK;
  T* sD = sB + DC * SBW;                    // [TM][TN] if staged: the tile's distances, for per-row work
  T* lv = sD + (staged ? TM * TN : 0);      // [TM][K]: list values
  int* li = reinterpret_cast<int*>(lv + TM * K);  // [TM][K]: list columns
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i0 = blockIdx.x * TM;
  const int split = blockIdx.y;
  const int c_begin = split * cols_per_split;
  const int c_end = min(n, c_begin + cols_per_split);
  const int rw = warp * 8;  // first row of this warp within the block
  const T inf = T(INFINITY);
  for (int e = lane; e < 8 * K; e += 32) { lv[rw * K + e] = inf; li[rw * K + e] = INT_MAX; }
  T ni[8];
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const int r = i0 + rw + a;
    ni[a] = r < n ? norm[r] : T(0);
  }
  for (int j0 = c_begin; j0 < c_end; j0 += TN) {
    T acc[8][4];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[a][q] = T(0);
    for (int k0 = 0; k0 < dim; k0 += DC) {
      const int kc = min(DC, dim - k0);
      __syncthreads();  // every warp is done with the previous chunk
      stage_chunk<T, TM, SA>(sA, x, i0, n, dim, k0, kc, vec);
      stage_chunk<T, TN, SBW>(sB, x, j0, c_end, dim, k0, kc, vec);
      __syncthreads();
#pragma unroll 4
      for (int kk = 0; kk < kc; ++kk) {
        T av[8], bv[4];
        ld4s<T>(sA + kk * SA + rw, av);
        ld4s<T>(sA + kk * SA + rw + 4, av + 4);
        ld4s<T>(sB + kk * SBW + 4 * lane, bv);
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[a][q] = fma(av[a], bv[q], acc[a][q]);
      }
    }
    // distances; columns past the range are NaN (never selected)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int gj = j0 + 4 * lane + q;
      const T nj = gj < c_end ? norm[gj] : T(0);
#pragma unroll
      for (int a = 0; a < 8; ++a) acc[a][q] = gj < c_end ? fma(T(-2), acc[a][q], nj + ni[a]) : T(NAN);
    }
    const bool first = j0 == c_begin && K <= TN;
    // rows that may take a candidate: one at or below both the row's current
    // K-th distance and the other column ranges' bound for the row (a candidate
    // farther than some range's K-th distance cannot be among the row's K
    // nearest; fp32 with several ranges, otherwise no bound). The exact tests
    // follow for these rows only. A split's first tile is sorted whole.
    unsigned todo = 0;
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const int r = i0 + rw + a;
      T thr = lv[(rw + a) * K + K - 1];
      if (gbound != nullptr && r < n) thr = fmin(thr, (T)Key<float>::dec(gbound[r]));
      bool any = first;
#pragma unroll
      for (int q = 0; q < 4; ++q) any = any || acc[a][q] <= thr;
      if (__ballot_sync(0xffffffffu, any) && r < n) todo |= 1u << a;
    }
    // those rows one at a time (a rolled loop keeps the sort and insert code
    // single), reading their distances back from the warp's staging area
    T* wD = sD + rw * TN;
    if (todo && staged) {
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        if constexpr (sizeof(T) == 4) {
          *reinterpret_cast<float4*>(wD + a * TN + 4 * lane) = make_float4(acc[a][0], acc[a][1], acc[a][2], acc[a][3]);
        } else {
          reinterpret_cast<double2*>(wD + a * TN + 4 * lane)[0] = make_double2(acc[a][0], acc[a][1]);
          reinterpret_cast<double2*>(wD + a * TN + 4 * lane)[1] = make_double2(acc[a][2], acc[a][3]);
        }
      }
      __syncwarp();
    }
    while (todo) {
      const int a = __ffs(todo) - 1;
      todo &= todo - 1;
      T d4[4];
      if (staged) {
        ld4s<T>(wD + a * TN + 4 * lane, d4);
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          T r = acc[0][q];
#pragma unroll
          for (int b = 1; b < 8; ++b) r = a == b ? acc[b][q] : r;
          d4[q] = r;
        }
      }
      T* Lv = lv + (rw + a) * K;
      int* Li = li + (rw + a) * K;
      if (first) {
        int ix[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const bool ok = d4[q] == d4[q];  // NaN (past the range) sorts last
          ix[q] = ok ? j0 + 4 * lane + q : INT_MAX;
          if (!ok) d4[q] = inf;
        }
        warp_sort128<T>(d4, ix, lane);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (4 * lane + q < K) { Lv[4 * lane + q] = d4[q]; Li[4 * lane + q] = ix[q]; }
        __syncwarp();
        if (gbound != nullptr && lane == 0) publish_bound(gbound + i0 + rw + a, Lv[K - 1]);
        continue;
      }
      if (gbound != nullptr) {
        const T bound = (T)Key<float>::dec(gbound[i0 + rw + a]);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (d4[q] > bound) d4[q] = T(NAN);  // never selected
      }
      T tv = Lv[K - 1];
      int ti = Li[K - 1];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const T dv = d4[q];
        const int j = j0 + 4 * lane + q;
        bool pass = lexless(dv, j, tv, ti);
        unsigned m = __ballot_sync(0xffffffffu, pass);
        while (m) {
          const int src = __ffs(m) - 1;
          const T cv = __shfl_sync(0xffffffffu, dv, src);
          const int cj = __shfl_sync(0xffffffffu, j, src);
          list_insert<T>(Lv, Li, K, cv, cj, lane);
          tv = Lv[K - 1];
          ti = Li[K - 1];
          if (lane == src) pass = false;
          pass = pass && lexless(dv, j, tv, ti);
          m = __ballot_sync(0xffffffffu, pass);
        }
      }
      if (gbound != nullptr && lane == 0) publish_bound(gbound + i0 + rw + a, tv);
    }
  }
  __syncwarp();
#pragma unroll 1
  for (int a = 0; a < 8; ++a) {
    const int gi = i0 + rw + a;
    if (gi >= n) break;
    const size_t o = ((size_t)gi * nsplit + split) * K;
    for (int e = lane; e < K; e += 32) {
      out_v[o + e] = lv[(rw + a) * K + e];
      out_i[o + e] = li[(rw + a) * K + e];
    }
  }
}

// merge the nsplit sorted partial lists of each row into its K best
template <class T>
__global__ void k_knn_merge(const T* __restrict__ pv, const int* __restrict__ pi, int n, int nsplit, int K,
                            T* __restrict__ fv, int* __restrict__ fi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int pos[kMaxSplit];
#pragma unroll
  for (int s = 0; s < kMaxSplit; ++s) pos[s] = 0;
  for (int e = 0; e < K; ++e) {
    int best = 0;
    T bv = T(0);
    int bi = INT_MAX;
    bool have = false;
#pragma unroll
    for (int s = 0; s < kMaxSplit; ++s) {
      if (s < nsplit && pos[s] < K) {
        const size_t o = ((size_t)i * nsplit + s) * K + pos[s];
        const T v = pv[o];
        const int ix = pi[o];
        if (!have || lexless(v, ix, bv, bi)) { best = s; bv = v; bi = ix; have = true; }
      }
    }
#pragma unroll
    for (int s = 0; s < kMaxSplit; ++s) pos[s] += s == best;
    fv[(size_t)i * K + e] = bv;
    fi[(size_t)i * K + e] = bi;
  }
}

struct SelectState {
  unsigned long long prefix, mask, rank;
  unsigned int hist[256];
  unsigned int ticket;
};

__global__ void k_select_init(SelectState* st, unsigned long long rank) {
  for (int b = threadIdx.x; b < 256; b += blockDim.x) st->hist[b] = 0;
  if (threadIdx.x == 0) { st->prefix = 0; st->mask = 0; st->rank = rank; st->ticket = 0; }
}

// One 8-bit digit (most significant first) of the radix select of the value of
// rank st->rank among v[0, m). Every CTA histograms the digit of the values
// that match the digits found so far; the last CTA to finish (ticket) reads
// and clears the histogram, picks the digit, and after the last digit writes
// the value.
template <class T>
__global__ void __launch_bounds__(256) k_select_pass(const T* __restrict__ v, size_t m, int shift, SelectState* st,
                                                     T* __restrict__ out) {
  using U = typename Key<T>::U;
  __shared__ unsigned int h[256];
  __shared__ bool last;
  for (int b = threadIdx.x; b < 256; b += blockDim.x) h[b] = 0;
  __syncthreads();
  const U prefix = (U)st->prefix, mask = (U)st->mask;
  // the values share most leading digits, so the lanes of a warp that hit the
  // same bin add once, through their leader
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t m_round = (m + 31) / 32 * 32;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < m_round; e += stride) {
    unsigned bin = 256u;  // no bin
    if (e < m) {
      const U key = Key<T>::enc(v[e]);
      if ((key & mask) == prefix) bin = (unsigned)(key >> shift) & 255u;
    }
    const unsigned same = __match_any_sync(0xffffffffu, bin);
    if (bin < 256u && (threadIdx.x & 31) == (unsigned)(__ffs(same) - 1)) atomicAdd(&h[bin], (unsigned)__popc(same));
  }
  __syncthreads();
  for (int b = threadIdx.x; b < 256; b += blockDim.x)
    if (h[b]) atomicAdd(&st->hist[b], h[b]);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&st->ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  // the last CTA: read (and clear) the global histogram together, then one
  // thread picks the digit
  __threadfence();
  for (int b = threadIdx.x; b < 256; b += blockDim.x) h[b] = atomicExch(&st->hist[b], 0u);
  __syncthreads();
  if (threadIdx.x != 0) return;
  unsigned long long rank = st->rank;
  int b = 0;
  for (; b < 255; ++b) {
    if (rank < h[b]) break;
    rank -= h[b];
  }
  const U np = prefix | ((U)b << shift);
  st->prefix = np;
  st->mask = mask | ((U)255 << shift);
  st->rank = rank;
  st->ticket = 0;
  if (shift == 0) *out = Key<T>::dec(np);
}

__device__ __forceinline__ float exp_t(float v) { return expf(v); }
__device__ __forceinline__ double exp_t(double v) { return exp(v); }

// weights of row i: exp(-(d / median)), normalised to sum 1, as float32 with
// COO indices (i, j) (src/laplacian_cuda_kernel.cu:112-126)
template <class T>
__global__ void k_lap_weights(const T* __restrict__ fv, const int* __restrict__ fi, int n, int K,
                              const T* __restrict__ med, long long* __restrict__ ind, float* __restrict__ val) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T md = *med;
  const T* d = fv + (size_t)i * K;
  T s = T(0);
  for (int e = 0; e < K; ++e) s += exp_t(-(d[e] / md));
  const size_t nk = (size_t)n * K;
  for (int e = 0; e < K; ++e) {
    const size_t o = (size_t)i * K + e;
    val[o] = (float)(exp_t(-(d[e] / md)) / s);
    ind[o] = i;
    ind[nk + o] = fi[o];
  }
}

struct Layout {
  int max_split;  // column splits the partial-list buffers hold
  size_t off_norm, off_pv, off_pi, off_fv, off_fi, off_state, off_med, off_bound, total;
};

inline size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

// Workspace: norms, partial lists of up to max_split column splits (bounded to
// 256 MiB), the merged lists, the select state and the median.
inline Layout layout(int n, int k, size_t es) {
  Layout L{};
  const size_t nk = (size_t)n * k;
  const size_t per_split = nk * (es + 4);
  L.max_split = (int)std::max<size_t>(1, std::min<size_t>(kMaxSplit, ((size_t)256 << 20) / per_split));
  size_t off = 0;
  L.off_norm = off; off = al256(off + (size_t)n * es);
  if (L.max_split > 1) {
    L.off_pv = off; off = al256(off + nk * L.max_split * es);
    L.off_pi = off; off = al256(off + nk * L.max_split * 4);
  }
  L.off_fv = off; off = al256(off + nk * es);
  L.off_fi = off; off = al256(off + nk * 4);
  L.off_state = off; off = al256(off + sizeof(SelectState));
  L.off_med = off; off = al256(off + es);
  L.off_bound = off; off = al256(off + (size_t)n * 4);
  L.total = off;
  return L;
}

// Column splits: at least one full wave of CTAs where max_split allows (the
// kernel needs every resident slot to hide its latencies), then the count that
// minimises waves x CTA length, a CTA costing its tiles plus about two tiles of
// list set-up. The result does not depend on the choice.
inline int choose_split(int n, int max_split, int slots) {
  const int rows = (n + TM - 1) / TM;
  slots = std::max(1, slots);
  int best = 0;
  double best_cost = 0;
  for (int pass = 0; pass < 2 && best == 0; ++pass) {
    for (int ns = 1; ns <= max_split; ++ns) {
      const int cps = ((n + ns - 1) / ns + TN - 1) / TN * TN;
      if ((n + cps - 1) / cps != ns) continue;
      if (pass == 0 && rows * ns < slots) continue;
      const double waves = std::ceil((double)rows * ns / slots);
      const double cost = waves * (cps / TN + 2);
      if (best == 0 || cost < best_cost * 0.97) { best = ns; best_cost = cost; }
    }
  }
  if (best == 0) {  // no split reaches a full wave: the most splits there are
    for (int ns = max_split; ns >= 1 && best == 0; --ns) {
      const int cps = ((n + ns - 1) / ns + TN - 1) / TN * TN;
      if ((n + cps - 1) / cps == ns) best = ns;
    }
  }
  return std::max(1, best);
}

template <class T>
int run(const T* x, int n, int dim, int k, long long* ind, float* val, unsigned char* ws, cudaStream_t st) {
  const Layout L = layout(n, k, sizeof(T));
  T* norm = reinterpret_cast<T*>(ws + L.off_norm);
  T* fv = reinterpret_cast<T*>(ws + L.off_fv);
  int* fi = reinterpret_cast<int*>(ws + L.off_fi);
  SelectState* sel = reinterpret_cast<SelectState*>(ws + L.off_state);
  T* med = reinterpret_cast<T*>(ws + L.off_med);
  const size_t smem = knn_smem_bytes<T>(k);
  int dev = 0, optin = 0, sms = 0, occ = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return fail(CTGB_ERR_CUDA, std::string("laplacian: ") + cudaGetErrorString(e));
  if (smem > (size_t)optin)
    return fail(CTGB_ERR_INVALID, "laplacian: k too large for this dtype (" + std::to_string(smem) +
                                      " bytes of shared memory per CTA needed)");
  e = cudaFuncSetAttribute(k_knn<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_knn<T>, NT, smem);
  if (e != cudaSuccess) return fail(CTGB_ERR_CUDA, std::string("laplacian smem: ") + cudaGetErrorString(e));
  const int ns = choose_split(n, L.max_split, sms * std::max(1, occ));
  const int cps = ((n + ns - 1) / ns + TN - 1) / TN * TN;
  T* pv = ns > 1 ? reinterpret_cast<T*>(ws + L.off_pv) : fv;
  int* pi = ns > 1 ? reinterpret_cast<int*>(ws + L.off_pi) : fi;
  constexpr int VW = 16 / (int)sizeof(T);
  const bool vec = dim % VW == 0 && (reinterpret_cast<uintptr_t>(x) & 15) == 0;
  k_sqnorm<T><<<(n + 255) / 256, 256, 0, st>>>(x, n, dim, norm);
  dim3 grid((n + TM - 1) / TM, ns);
  // shared per-row bounds between the column ranges (fp32): start at "none"
  unsigned* gbound = nullptr;
  if (sizeof(T) == 4 && ns > 1) {
    gbound = reinterpret_cast<unsigned*>(ws + L.off_bound);
    e = cudaMemsetAsync(gbound, 0xFF, (size_t)n * 4, st);
    if (e != cudaSuccess) return fail(CTGB_ERR_CUDA, std::string("laplacian bounds: ") + cudaGetErrorString(e));
  }
  k_knn<T><<<grid, NT, smem, st>>>(x, norm, n, dim, k, cps, ns, vec, pv, pi, gbound);
  if (ns > 1) k_knn_merge<T><<<(n + 127) / 128, 128, 0, st>>>(pv, pi, n, ns, k, fv, fi);
  const size_t m = (size_t)n * k;
  k_select_init<<<1, 256, 0, st>>>(sel, (m - 1) / 2);
  const int sb = (int)std::max<size_t>(1, std::min<size_t>((m + 2047) / 2048, (size_t)sms * 4));
  for (int p = Key<T>::kPasses - 1; p >= 0; --p) k_select_pass<T><<<sb, 256, 0, st>>>(fv, m, 8 * p, sel, med);
  k_lap_weights<T><<<(n + 127) / 128, 128, 0, st>>>(fv, fi, n, k, med, ind, val);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(CTGB_ERR_CUDA, std::string("laplacian launch: ") + cudaGetErrorString(e));
  return CTGB_OK;
}

}  // namespace lap
}  // namespace ctgb

extern "C" {

size_t ctgb_laplacian_workspace_size(int n, int dim, int k, int dtype) {
  if (n < 1 || dim < 1 || k < 1 || k > n || (dtype != CTGB_FLOAT32 && dtype != CTGB_FLOAT64)) return 0;
  return ctgb::lap::layout(n, k, dtype == CTGB_FLOAT32 ? 4 : 8).total;
}

int ctgb_laplacian(const void* points, int n, int dim, int k, int dtype, long long* indices, float* values,
                   void* workspace, size_t workspace_bytes, void* stream) {
  using namespace ctgb;
  if (dtype != CTGB_FLOAT32 && dtype != CTGB_FLOAT64) return fail(CTGB_ERR_INVALID, "laplacian: bad dtype");
  if (n < 1 || dim < 1) return fail(CTGB_ERR_INVALID, "laplacian: need at least one point of dimension >= 1");
  if (k < 1 || k > n) return fail(CTGB_ERR_INVALID, "laplacian: k must be in [1, n]");
  if (k > lap::kMaxK) return fail(CTGB_ERR_INVALID, "laplacian: k > 256 is not supported");
  if ((size_t)n * (size_t)k > (size_t)INT_MAX) return fail(CTGB_ERR_INVALID, "laplacian: n * k too large");
  if (!points || !indices || !values || !workspace) return fail(CTGB_ERR_INVALID, "laplacian: null pointer");
  if ((reinterpret_cast<uintptr_t>(workspace) & 255) != 0)
    return fail(CTGB_ERR_INVALID, "workspace must be 256-byte aligned");
  const size_t es = dtype == CTGB_FLOAT32 ? 4 : 8;
  if ((reinterpret_cast<uintptr_t>(points) & (es - 1)) != 0)
    return fail(CTGB_ERR_INVALID, "laplacian: points not aligned to their element size");
  if (workspace_bytes < lap::layout(n, k, es).total) return fail(CTGB_ERR_WORKSPACE, "laplacian: workspace too small");
  auto* ws = static_cast<unsigned char*>(workspace);
  auto st = static_cast<cudaStream_t>(stream);
  if (dtype == CTGB_FLOAT32)
    return lap::run<float>(static_cast<const float*>(points), n, dim, k, indices, values, ws, st);
  return lap::run<double>(static_cast<const double*>(points), n, dim, k, indices, values, ws, st);
}

}  // extern "C"
