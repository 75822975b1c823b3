// CPU execution of CUDA C++ kernel source, used ONLY to run the reference's own
// kernels (read from the reference checkout at build time) on the host so that
// the oracle can be pinned against the reference's outputs. Test infrastructure.
//
// Model: one CTA at a time; its threads are ucontext coroutines that run until
// __syncthreads() or return, so every thread of the block reaches barrier k
// before any passes it. Threads that returned count as arrived (the Volta+
// rule the reference relies on for its barrier inside `if (dIndex < dets)`).
// `__shared__` variables become function-local statics, i.e. one copy per
// kernel instantiation shared by the coroutines of the running block.
// atomicAdd is a plain read-modify-write (coroutines never preempt each other).
// Accessor indices are bounds-checked; violations are counted, not faulted.
#pragma once

#include <ucontext.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <functional>
#include <vector>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ static
#define __restrict__ __restrict

struct emu_dim3 {
  unsigned x = 1, y = 1, z = 1;
};

namespace emu {

inline emu_dim3 g_thread, g_block, g_blockdim, g_griddim;
inline long g_oob = 0;  // out-of-range accessor indices seen

struct Coro {
  ucontext_t ctx;
  bool done = true;
  std::vector<char> stack;
};

inline ucontext_t g_sched;
inline std::vector<Coro> g_threads;
inline int g_cur = -1;
inline const std::function<void()>* g_body = nullptr;

inline void sync() { swapcontext(&g_threads[g_cur].ctx, &g_sched); }

inline void coro_entry() {
  (*g_body)();
  g_threads[g_cur].done = true;
}

inline void launch(emu_dim3 grid, emu_dim3 block, const std::function<void()>& body) {
  const int nt = (int)(block.x * block.y * block.z);
  if ((int)g_threads.size() < nt) g_threads.resize(nt);
  for (auto& t : g_threads)
    if (t.stack.empty()) t.stack.resize(1 << 16);
  g_griddim = grid;
  g_blockdim = block;
  g_body = &body;
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        g_block = emu_dim3{bx, by, bz};
        for (int t = 0; t < nt; ++t) {
          Coro& c = g_threads[t];
          getcontext(&c.ctx);
          c.ctx.uc_stack.ss_sp = c.stack.data();
          c.ctx.uc_stack.ss_size = c.stack.size();
          c.ctx.uc_link = &g_sched;
          makecontext(&c.ctx, coro_entry, 0);
          c.done = false;
        }
        int live = nt;
        while (live > 0) {
          for (int t = 0; t < nt; ++t) {
            if (g_threads[t].done) continue;
            g_cur = t;
            g_thread = emu_dim3{t % block.x, (t / block.x) % block.y, t / (block.x * block.y)};
            swapcontext(&g_sched, &g_threads[t].ctx);
            if (g_threads[t].done) --live;
          }
        }
      }
  g_cur = -1;
}

}  // namespace emu

#define threadIdx emu::g_thread
#define blockIdx emu::g_block
#define blockDim emu::g_blockdim
#define gridDim emu::g_griddim
#define __syncthreads() emu::sync()

template <class T>
inline T atomicAdd(T* p, T v) {
  T old = *p;
  *p = old + v;
  return old;
}

using std::abs;
using std::acos;
using std::ceil;
using std::cos;
using std::floor;
using std::max;
using std::min;
using std::round;
using std::sin;
using std::sqrt;

namespace torch {

struct RestrictPtrTraits {};

template <class T, size_t N>
struct EmuAccessor {
  T* data;
  const size_t* sizes;
  const size_t* strides;
  EmuAccessor<T, N - 1> operator[](size_t i) const {
    if (i >= sizes[0]) { ++emu::g_oob; i = 0; }
    return EmuAccessor<T, N - 1>{data + i * strides[0], sizes + 1, strides + 1};
  }
};

template <class T>
struct EmuAccessor<T, 1> {
  T* data;
  const size_t* sizes;
  const size_t* strides;
  T& operator[](size_t i) const {
    if (i >= sizes[0]) { ++emu::g_oob; i = 0; }
    return data[i * strides[0]];
  }
};

template <class T, size_t N, class PtrTraits, class index_t>
struct PackedTensorAccessor {
  T* data;
  size_t sizes_[N];
  size_t strides_[N];
  EmuAccessor<T, N - 1> operator[](size_t i) const {
    if (i >= sizes_[0]) { ++emu::g_oob; i = 0; }
    return EmuAccessor<T, N - 1>{data + i * strides_[0], sizes_ + 1, strides_ + 1};
  }
};

}  // namespace torch
