// Throughput probes used as roofline denominators by bench.py: FP64 FMA,
// CUDA's double-precision exp, FP32 FMA, the SFU exp2 and the FP64
// kernels' own table exponential, each measured with CUDA events on a
// private stream.  A measurement helper (include/crs_probe.h), not part of
// the evaluation API.
#include <cuda_runtime.h>
#include <math.h>

#include <cmath>

#include "../../include/crs.h"
#include "../../include/crs_probe.h"
#include "crs_exp.cuh"

namespace {
constexpr int CH = 8;

__global__ void p_dfma(double *out, double a, double b, int iters) {
  double x[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) x[c] = threadIdx.x * 1e-3 + c;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < CH; ++c) x[c] = fma(x[c], a, b);
  double s = 0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void p_dexp(double *out, double a, double b, int iters) {
  double x[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) x[c] = threadIdx.x * 1e-6 + c * 1e-3;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < CH; ++c) x[c] = exp(x[c]) * a - b;
  double s = 0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void p_ffma(double *out, float a, float b, int iters) {
  float x[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) x[c] = threadIdx.x * 1e-3f + c;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < CH; ++c) x[c] = fmaf(x[c], a, b);
  float s = 0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void p_ex2(double *out, float a, float b, int iters) {
  float x[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) x[c] = threadIdx.x * 1e-6f + c * 1e-3f;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      float y;
      asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x[c]));
      x[c] = y * a;
    }
  float s = 0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
// The table exponential of the FP64 kernels (crs_exp.cuh), table staged in
// shared memory as the kernels stage it.  x <- exp(-x) stays in
// [exp(-1), 1] and adds no FP64 instruction to exp_t's own (the negation
// is an operand modifier), so the rate is the exponential's alone.
__global__ void p_texp(double *out, const double *gtab, int iters) {
  __shared__ double tab[256];
  for (int j = threadIdx.x; j < 256; j += blockDim.x) tab[j] = gtab[j];
  __syncthreads();
  double x[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) x[c] = threadIdx.x * 1e-6 + c * 1e-3;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < CH; ++c) x[c] = crs::texp::exp_t(-x[c], tab);
  double s = 0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" int crs_probe_peaks(double out[5]) {
  if (!out) return CRS_ERR_ARG;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 4, threads = 256;
  double *buf = nullptr, *gtab = nullptr;
  cudaStream_t s;
  cudaEvent_t e0, e1;
  if (cudaMalloc(&buf, sizeof(double) * (blocks * threads + 256)) != cudaSuccess)
    return CRS_ERR_CUDA;
  gtab = buf + blocks * threads;
  double htab[256];
  for (int j = 0; j < 256; ++j) htab[j] = (double)std::exp2((long double)j / 256.0L);
  if (cudaMemcpy(gtab, htab, sizeof htab, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(buf);
    return CRS_ERR_CUDA;
  }
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int iters[5] = {4096, 256, 16384, 4096, 512};
  for (int k = 0; k < 5; ++k) {
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, s);
      switch (k) {
        case 0: p_dfma<<<blocks, threads, 0, s>>>(buf, 1.0000001, 1e-9, iters[k]); break;
        case 1: p_dexp<<<blocks, threads, 0, s>>>(buf, 1.0000001, 1e-9, iters[k]); break;
        case 2: p_ffma<<<blocks, threads, 0, s>>>(buf, 1.0000001f, 1e-9f, iters[k]); break;
        case 3: p_ex2<<<blocks, threads, 0, s>>>(buf, 1.0000001f, 1e-9f, iters[k]); break;
        default: p_texp<<<blocks, threads, 0, s>>>(buf, gtab, iters[k]); break;
      }
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep && ms < best) best = ms;
    }
    out[k] = (double)blocks * threads * iters[k] * CH / (best * 1e-3);
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  cudaFree(buf);
  return err == cudaSuccess ? CRS_OK : CRS_ERR_CUDA;
}
