// FP64 FMA throughput of the GPU: eight independent DFMA chains per thread,
// 8 blocks of 256 threads per SM, best of five launches (CUDA events).
// Prints DFMA/s and DFMA per SM per clock at the device's maximum clock; the
// FP64 force path's fraction of the FP64 pipe is quoted against this rate.
#include <cuda_runtime.h>
#include <cstdio>
__global__ void k(double* out, int iters) {
  double a[8];
  for (int i = 0; i < 8; ++i) a[i] = threadIdx.x * 1e-3 + i;
  const double b = 1.0000001, c = 1e-9;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = fma(a[i], b, c);
  double s = 0; for (int i = 0; i < 8; ++i) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
int main() {
  int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  double* out; cudaMalloc(&out, sizeof(double) * blocks * threads);
  k<<<blocks, threads>>>(out, 16); cudaDeviceSynchronize();
  cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(a); k<<<blocks, threads>>>(out, iters); cudaEventRecord(b); cudaEventSynchronize(b);
    float ms; cudaEventElapsedTime(&ms, a, b); if (ms < best) best = ms;
  }
  const double dfma = (double)blocks * threads * iters * 8;
  int clk; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, 0);
  printf("DFMA/s %.4e  per SM per clk at %d MHz: %.3f  (%.3f ms) err=%s\n", dfma / (best * 1e-3), clk / 1000,
         dfma / (best * 1e-3) / sms / (clk * 1e3), best, cudaGetErrorString(cudaGetLastError()));
  return 0;
}
