// Device throughput probes used to pick the arithmetic of the leaf kernel and
// to state its compute roof: FP64 FMA, FP64 add, FP32 FMA and 64-bit integer
// add rates, each from independent dependency chains timed with CUDA events.
#include "dkt_internal.cuh"
#include "../../include/dkt_gb300.h"

namespace dkt {

constexpr int PROBE_CHAINS = 8;

template <typename T, int KIND>
__global__ void k_probe(T *out, int iters, T a, T b)
{
  T x[PROBE_CHAINS];
#pragma unroll
  for (int c = 0; c < PROBE_CHAINS; c++) x[c] = (T) (threadIdx.x + c);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; c++) {
      if (KIND == 0) x[c] = x[c] * a + b;     // fused multiply-add
      else x[c] = x[c] + b;                   // add
    }
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < PROBE_CHAINS; c++) s += x[c];
  if (s == (T) 12345) out[0] = s;   // keeps the chains live
}

template <typename T, int KIND>
static double run_probe(T a, T b)
{
  int dev = 0, sms = 0;
  DKT_CUDA(cudaGetDevice(&dev));
  DKT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256, iters = 2048;
  DBuf<T> out(1);
  k_probe<T, KIND><<<blocks, threads>>>(out.p, 64, a, b);
  check_launch("probe");
  cudaEvent_t e0, e1;
  DKT_CUDA(cudaEventCreate(&e0));
  DKT_CUDA(cudaEventCreate(&e1));
  DKT_CUDA(cudaEventRecord(e0));
  k_probe<T, KIND><<<blocks, threads>>>(out.p, iters, a, b);
  DKT_CUDA(cudaEventRecord(e1));
  DKT_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  DKT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double ops = (double) blocks * threads * iters * PROBE_CHAINS;
  return ops / (ms * 1e-3);   // operations per second
}

}  // namespace dkt

extern "C" int dkt_probe_device(double *out4)
{
  if (!out4) return DKT_E_ARG;
  try {
    out4[0] = 2.0 * dkt::run_probe<double, 0>(1.0000001, 1e-9) / 1e12;   // FP64 FMA, TFLOP/s
    out4[1] = dkt::run_probe<double, 1>(1.0, 1e-9) / 1e12;               // FP64 add, Tops/s
    out4[2] = 2.0 * dkt::run_probe<float, 0>(1.0000001f, 1e-9f) / 1e12;  // FP32 FMA, TFLOP/s
    out4[3] = dkt::run_probe<long long, 1>(1, 3) / 1e12;                 // int64 add, Tops/s
  } catch (...) {
    return DKT_E_CUDA;
  }
  return DKT_OK;
}
