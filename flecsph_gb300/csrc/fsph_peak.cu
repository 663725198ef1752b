// fsph_peak.cu -- arithmetic-throughput probe used as the roofline
// denominator for the FP64 / FP32 pair kernels (the measured peaks file of
// the host carries only HBM and tensor-core figures).  Each thread runs
// eight independent FMA chains held in registers; no memory traffic.
#include <cuda_runtime.h>

#include "fsph_internal.cuh"

namespace {

template<class T>
__global__ void k_fma_chain(T * out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  T x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for(int i = 0; i < iters; ++i) {
#pragma unroll
    for(int k = 0; k < 16; ++k) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if(s == (T)-1.2345)
    out[blockIdx.x] = s;
}

// FP32 on Blackwell's packed FP32x2 instructions (two FMAs per lane per
// instruction)
__global__ void k_fma2_chain(float * out, int iters, float a, float b) {
  const float t = threadIdx.x;
  float2 x[8];
  for(int k = 0; k < 8; ++k)
    x[k] = make_float2(t + k, t - k);
  const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
  for(int i = 0; i < iters; ++i) {
#pragma unroll
    for(int k = 0; k < 16; ++k) {
#pragma unroll
      for(int j = 0; j < 8; ++j)
        x[j] = __ffma2_rn(x[j], a2, b2);
    }
  }
  float s = 0.f;
  for(int k = 0; k < 8; ++k)
    s += x[k].x + x[k].y;
  if(s == -1.2345f)
    out[blockIdx.x] = s;
}

double run_probe_fma2(int nsm, int iters) {
  float * out = nullptr;
  if(cudaMalloc(&out, sizeof(float) * nsm * 64) != cudaSuccess)
    return -1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = nsm * 8, threads = 256;
  k_fma2_chain<<<blocks, threads>>>(out, 16, 0.999999f, 1e-7f);
  cudaEventRecord(e0);
  k_fma2_chain<<<blocks, threads>>>(out, iters, 0.999999f, 1e-7f);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if(cudaGetLastError() != cudaSuccess || ms <= 0)
    return -1;
  double flops = 2.0 * 2 * 8 * 16 * (double)iters * blocks * threads;
  return flops / (ms * 1e-3) / 1e12;
}

template<class T>
double run_probe(int nsm, int iters) {
  T * out = nullptr;
  if(cudaMalloc(&out, sizeof(T) * nsm * 64) != cudaSuccess)
    return -1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = nsm * 8, threads = 256;
  k_fma_chain<T><<<blocks, threads>>>(out, 16, (T)0.999999, (T)1e-7);
  cudaEventRecord(e0);
  k_fma_chain<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if(cudaGetLastError() != cudaSuccess || ms <= 0)
    return -1;
  double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
  return flops / (ms * 1e-3) / 1e12;
}

}  // namespace

extern "C" fsph_status fsph_measure_peak(int32_t device, int32_t kind,
  double * tflops) {
  if(!tflops || kind < 0 || kind > 2)
    return FSPH_ERR_ARG;
  if(cudaSetDevice(device) != cudaSuccess)
    return FSPH_ERR_NO_DEVICE;
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  double best = 0;
  for(int rep = 0; rep < 3; ++rep) {
    double v = kind == 0 ? run_probe<double>(nsm, 4096)
             : kind == 1 ? run_probe<float>(nsm, 16384)
                         : run_probe_fma2(nsm, 16384);
    if(v < 0)
      return FSPH_ERR_CUDA;
    best = v > best ? v : best;
  }
  *tflops = best;
  return FSPH_OK;
}
