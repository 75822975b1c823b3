// FP32 FMA throughput probe (benchmark support only; not part of the operator
// ABI). Every thread runs 8 independent register-resident FMA chains, so the
// FP32 pipes, not latency or memory, bound the kernel. One FMA = one lane-op.
#include <cuda_runtime.h>

__global__ void __launch_bounds__(256) k_ffma(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f;
  float x4 = x0 + 4.f, x5 = x0 + 5.f, x6 = x0 + 6.f, x7 = x0 + 7.f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
      x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
    }
  }
  const float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 1234.5678f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

extern "C" int ctgb_peak_ffma(int blocks, int iters, float* out, void* stream) {
  k_ffma<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(out, iters, 0.9999f, 1e-4f);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// FMAs issued per thread per loop iteration
extern "C" int ctgb_peak_ffma_per_iter(void) { return 32; }
