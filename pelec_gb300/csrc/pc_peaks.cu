// pc_peaks.cu — arithmetic peak rates of the current GPU, measured by
// bench.py for the FP64 roofline of the MOL kernels (HBM bandwidth comes from
// the measured copy rate).  Throughput kernels: every thread runs 8
// independent dependency chains so that issue, not latency, bounds them.
#include <cuda_runtime.h>

namespace {

template <typename T, int NCH>
__global__ void fma_chains(T* out, int iters, T a, T b) {
  T acc[NCH];
#pragma unroll
  for (int c = 0; c < NCH; ++c) acc[c] = (T)(threadIdx.x + c);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < NCH; ++c) acc[c] = fma(acc[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < NCH; ++c) s += acc[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
float time_rate(int blocks, int threads, int iters, T* buf) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chains<T, 8><<<blocks, threads>>>(buf, iters / 10, (T)0.999999, (T)1e-7);  // warm-up
  cudaEventRecord(e0);
  fma_chains<T, 8><<<blocks, threads>>>(buf, iters, (T)0.999999, (T)1e-7);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

}  // namespace

// out[0] = FP64 FMA TFLOP/s, out[1] = FP32 FMA TFLOP/s (2 flops per FMA).
// Returns 0 on success, a CUDA error code otherwise.
extern "C" int pc_measure_fp_rates(double* out) {
  int dev = 0;
  cudaDeviceProp p;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess) return 1;
  const int blocks = p.multiProcessorCount * 8, threads = 256;
  void* buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * blocks * threads) != cudaSuccess) return 2;
  const int it64 = 2000, it32 = 20000;
  const float ms64 = time_rate<double>(blocks, threads, it64, static_cast<double*>(buf));
  const float ms32 = time_rate<float>(blocks, threads, it32, static_cast<float*>(buf));
  cudaFree(buf);
  if (cudaGetLastError() != cudaSuccess) return 3;
  const double n = 2.0 * 8.0 * blocks * (double)threads;
  out[0] = n * it64 / (ms64 * 1e-3) / 1e12;
  out[1] = n * it32 / (ms32 * 1e-3) / 1e12;
  return 0;
}
