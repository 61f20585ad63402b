// Throughput probes for the arithmetic paths the library can use on GB300:
// FP64 FMA (DFMA), FP64 mma.sync (DMMA m8n8k4) and the legacy bf16 mma.sync
// (m16n8k16, FP32 accumulate).  Prints one JSON object.  Every kernel runs a
// fixed number of independent dependency chains per thread; the grid is a
// multiple of the SM count.  No waits, no shared memory, bounded loops.
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdint>

#define CK(x) do { cudaError_t e = (x); if (e != cudaSuccess) { \
  fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e)); return 1; } } while (0)

__global__ void k_dfma(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_dmma(double* out, int iters) {
  double a = 1.0 + threadIdx.x * 1e-6, b = 1.0 - threadIdx.x * 1e-6;
  double c[4][2];
#pragma unroll
  for (int k = 0; k < 4; ++k) { c[k][0] = 0; c[k][1] = 0; }
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                   : "+d"(c[k][0]), "+d"(c[k][1]) : "d"(a), "d"(b));
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) s += c[k][0] + c[k][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_hmma_bf16(float* out, int iters) {
  uint32_t a0 = 0x3f803f80u + threadIdx.x, a1 = a0, a2 = a0, a3 = a0;
  uint32_t b0 = 0x3f803f80u, b1 = b0;
  float c[4][4];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int j = 0; j < 4; ++j) c[k][j] = 0.f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
      asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                   : "+f"(c[k][0]), "+f"(c[k][1]), "+f"(c[k][2]), "+f"(c[k][3])
                   : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
  float s = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int j = 0; j < 4; ++j) s += c[k][j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename F>
static float time_ms(F f) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  f();  // warm-up
  cudaDeviceSynchronize();
  cudaEventRecord(a);
  f();
  cudaEventRecord(b);
  cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms;
}

int main() {
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
  int clk = 0;
  cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, 0);
  const int threads = 256, blocks = sms * 8;
  const size_t nthr = (size_t)threads * blocks;
  double* dout;
  CK(cudaMalloc(&dout, nthr * sizeof(double)));
  const int it_dfma = 4096, it_dmma = 2048, it_hmma = 8192;
  float ms_dfma = time_ms([&] { k_dfma<<<blocks, threads>>>(dout, it_dfma, 1.0000001, 1e-7); });
  CK(cudaGetLastError());
  float ms_dmma = time_ms([&] { k_dmma<<<blocks, threads>>>(dout, it_dmma); });
  CK(cudaGetLastError());
  float ms_hmma = time_ms([&] { k_hmma_bf16<<<blocks, threads>>>((float*)dout, it_hmma); });
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  double fl_dfma = 2.0 * 8 * it_dfma * (double)nthr;
  double fl_dmma = 512.0 * 4 * it_dmma * (double)(nthr / 32);
  double fl_hmma = 4096.0 * 4 * it_hmma * (double)(nthr / 32);
  printf("{\"sms\": %d, \"clock_khz_attr\": %d, \"fp64_dfma_tflops\": %.4f, \"fp64_dmma_tflops\": %.4f, "
         "\"bf16_mma_sync_tflops\": %.2f, \"ms\": [%.3f, %.3f, %.3f]}\n",
         sms, clk, fl_dfma / ms_dfma / 1e9, fl_dmma / ms_dmma / 1e9, fl_hmma / ms_hmma / 1e9, ms_dfma,
         ms_dmma, ms_hmma);
  cudaFree(dout);
  return 0;
}
