// FP32 FMA throughput probe: the denominator of the pair kernel's roofline
// (the pair laws run on the FP32 pipe, not on tensor cores).  Eight
// independent FMA chains per thread, two waves of 8 blocks x 256 threads per
// SM, timed with CUDA events on the caller's stream.
//
// Also the accuracy check of the float-float functions (ffmath.cuh): each
// input is rounded to float-float, the function applied, the result widened
// back to FP64 for the caller to compare with an FP64 reference.
#include <algorithm>

#include <cuda_runtime.h>

#include "../../include/bromoc_gpu.h"
#include "ffmath.cuh"
#include "gridsync.cuh"

namespace {

__global__ void k_ff_check(int fn, int n, const double *x, double *out) {
  using namespace bgpu;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const f2 a = f2_of(x[i]), b = f2_of(x[i + 1 < n ? i + 1 : 0]);
  f2 r = a;
  switch (fn) {
    case BROMOC_FF_EXP: r = f2_exp(a); break;
    case BROMOC_FF_COS: r = f2_cos(a); break;
    case BROMOC_FF_SQRT: r = f2_sqrt(a); break;
    case BROMOC_FF_RCP: r = f2_rcp(a); break;
    case BROMOC_FF_MUL: r = f2_mul(a, b); break;
    case BROMOC_FF_DIV: r = f2_div(a, b); break;
    case BROMOC_FF_ADD: r = f2_add(a, b); break;
    case BROMOC_FF_RSQRT: r = f2_rsqrt(a); break;
    default: break;
  }
  out[i] = f2_dbl(r);
}

__global__ void __launch_bounds__(256) k_fma_peak(float *out, int iters,
                                                  float b, float c) {
  float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1.0f, a2 = a0 + 2.0f, a3 = a0 + 3.0f;
  float a4 = a0 + 4.0f, a5 = a0 + 5.0f, a6 = a0 + 6.0f, a7 = a0 + 7.0f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      a0 = fmaf(a0, b, c);
      a1 = fmaf(a1, b, c);
      a2 = fmaf(a2, b, c);
      a3 = fmaf(a3, b, c);
      a4 = fmaf(a4, b, c);
      a5 = fmaf(a5, b, c);
      a6 = fmaf(a6, b, c);
      a7 = fmaf(a7, b, c);
    }
  }
  const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 1234.5f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Bounded-wait self-test: block 0 waits (the grid barrier's own wait, at
// most `spins` polls) for an arrival on *ctr; block 1 makes it only when
// `arrive` is set.  Without it the wait runs out, records kErrBarrier in
// st->err and the kernel returns.  An ordinary launch of two blocks: block 1
// needs nothing from block 0, so both end either way.
__global__ void k_wait_selftest(unsigned *ctr, bgpu::DevState *st, int spins, int arrive) {
  using namespace bgpu;
  if (threadIdx.x != 0) return;
  if (blockIdx.x == 1) {
    if (arrive) release_add(ctr, 1u);
    return;
  }
  wait_at_least(ctr, 1u, st, true, spins);
}

}  // namespace

extern "C" int bromoc_gpu_wait_selftest(int32_t spins, int32_t arrive, int32_t *err_word) {
  if (!err_word || spins < 1) return BROMOC_E_ARG;
  struct Buf {
    unsigned ctr;
    bgpu::DevState st;
  } *d = nullptr;
  if (cudaMalloc(&d, sizeof(Buf)) != cudaSuccess) return BROMOC_E_NOMEM;
  int rc = BROMOC_OK;
  if (cudaMemset(d, 0, sizeof(Buf)) != cudaSuccess) rc = BROMOC_E_CUDA;
  if (!rc) {
    k_wait_selftest<<<2, 32>>>(&d->ctr, &d->st, spins, arrive ? 1 : 0);
    int err = 0;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpy(&err, &d->st.err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = BROMOC_E_CUDA;
    *err_word = err;
  }
  cudaFree(d);
  return rc;
}

extern "C" int bromoc_gpu_fp32_peak(void *stream, double *tflops) {
  if (!tflops) return BROMOC_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return BROMOC_E_CUDA;
  const int blocks = sms * 16, threads = 256, iters = 4096;
  float *out = nullptr;
  cudaEvent_t e0, e1;
  if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(float)) != cudaSuccess)
    return BROMOC_E_NOMEM;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0.0;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0, s);
    k_fma_peak<<<blocks, threads, 0, s>>>(out, iters, 1.0000001f, 1e-7f);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = 2.0 * 64.0 * iters * (double)blocks * threads;
    if (rep > 0 && ms > 0.f) best = std::max(best, flops / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return BROMOC_E_CUDA;
  *tflops = best;
  return BROMOC_OK;
}

extern "C" int bromoc_gpu_ff_check(int32_t fn, int32_t n, const double *x, double *out) {
  if (!x || !out || n < 1 || fn < BROMOC_FF_EXP || fn > BROMOC_FF_RSQRT) return BROMOC_E_ARG;
  double *d = nullptr;
  if (cudaMalloc(&d, 2 * (size_t)n * sizeof(double)) != cudaSuccess) return BROMOC_E_NOMEM;
  int rc = BROMOC_OK;
  if (cudaMemcpy(d, x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
    rc = BROMOC_E_CUDA;
  if (!rc) {
    k_ff_check<<<(n + 127) / 128, 128>>>(fn, n, d, d + n);
    if (cudaMemcpy(out, d + n, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost) !=
        cudaSuccess)
      rc = BROMOC_E_CUDA;
  }
  cudaFree(d);
  return rc;
}
