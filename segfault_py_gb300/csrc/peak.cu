// peak.cu -- FMA-throughput microkernel: the FP64 / FP32 CUDA-core peak that
// the roofline fractions of the quartet kernels are quoted against.  Eight
// independent dependent-FMA chains per thread, 8 CTAs of 256 threads per SM.
#include <cstdint>

#include "segfock.h"
#include "sf_internal.h"

namespace {

template <typename R>
__global__ void __launch_bounds__(256) fma_chain_kernel(R *sink, int iters, R a, R b) {
  R x0 = (R)threadIdx.x * (R)1e-3, x1 = x0 + (R)1, x2 = x0 + (R)2, x3 = x0 + (R)3;
  R x4 = x0 + (R)4, x5 = x0 + (R)5, x6 = x0 + (R)6, x7 = x0 + (R)7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  const R s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (R)-12345.0) sink[threadIdx.x] = s;   // never true; keeps the chains alive
}

template <typename R>
int run(int iters, double *flops, float *ms, cudaStream_t st) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SF_ECUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return SF_ECUDA;
  R *sink = nullptr;
  if (cudaMalloc(&sink, 256 * sizeof(R)) != cudaSuccess) return SF_ECUDA;
  const int blocks = sms * 8;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chain_kernel<R><<<blocks, 256, 0, st>>>(sink, iters / 8, (R)0.999999, (R)1e-7);   // warm-up
  cudaEventRecord(e0, st);
  fma_chain_kernel<R><<<blocks, 256, 0, st>>>(sink, iters, (R)0.999999, (R)1e-7);
  cudaEventRecord(e1, st);
  cudaError_t e = cudaEventSynchronize(e1);
  float t = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (e != cudaSuccess) return SF_ECUDA;
  *ms = t;
  *flops = 2.0 * 32.0 * (double)iters * blocks * 256.0;
  return SF_OK;
}

}  // namespace

extern "C" int sf_fma_peak(int32_t precision, double *flops, float *ms, void *stream) {
  if (!flops || !ms) return SF_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == SF_PREC_FP64) return run<double>(512, flops, ms, st);
  if (precision == SF_PREC_FP32) return run<float>(32768, flops, ms, st);
  return SF_EINVAL;
}
