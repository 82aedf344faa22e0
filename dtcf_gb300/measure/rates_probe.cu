// Arithmetic-rate probe of the GPU: FP64 FMA, FP64 tensor (DMMA m8n8k4 and
// m16n8k4), FP32 FMA, legacy bf16 mma.sync, IMMA s8 and F2I throughput.
// Every thread writes one output element; no waits, no shared state.
// Built and run by `python bench.py --rates`.
#include <cstdio>
#include <cuda_runtime.h>
#define ITERS 4096
__global__ void k_ffma64(double* out, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < ITERS; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void k_ffma32(float* out, float a, float b) {
  float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < ITERS; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void k_dmma(double* out) {
  double a = threadIdx.x * 1e-3, b = 1.0 - threadIdx.x * 1e-4;
  double c[4][2] = {};
  for (int i = 0; i < ITERS / 4; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(c[j][0]), "+d"(c[j][1]) : "d"(a), "d"(b));
  }
  double s = 0; for (int j = 0; j < 4; ++j) s += c[j][0] + c[j][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_dmma16(double* out) {
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, b = 1.0 - threadIdx.x * 1e-4;
  double c[4][4] = {};
  for (int i = 0; i < ITERS / 4; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      asm volatile("mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
                   : "+d"(c[j][0]), "+d"(c[j][1]), "+d"(c[j][2]), "+d"(c[j][3]) : "d"(a0), "d"(a1), "d"(b));
  }
  double s = 0; for (int j = 0; j < 4; ++j) s += c[j][0] + c[j][1] + c[j][2] + c[j][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_hmma(float* out) {
  unsigned a0 = 0x3f803f80u ^ threadIdx.x, a1 = a0, a2 = a0, a3 = a0, b0 = 0x3f803f80u, b1 = b0;
  float c[4][4] = {};
  for (int i = 0; i < ITERS / 4; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
                   : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3]) : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
  float s = 0; for (int j = 0; j < 4; ++j) s += c[j][0] + c[j][1] + c[j][2] + c[j][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_imma(int* out) {
  unsigned a0 = 0x01020304u ^ threadIdx.x, a1 = a0, a2 = a0, a3 = a0, b0 = 0x01010101u, b1 = b0;
  int c[4][4] = {};
  for (int i = 0; i < ITERS / 4; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      asm volatile("mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
                   : "+r"(c[j][0]), "+r"(c[j][1]), "+r"(c[j][2]), "+r"(c[j][3]) : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
  int s = 0; for (int j = 0; j < 4; ++j) s += c[j][0] + c[j][1] + c[j][2] + c[j][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_f2i(int* out, float a) {
  float x = threadIdx.x * 1.5f; int acc0 = 0, acc1 = 0, acc2 = 0, acc3 = 0;
  for (int i = 0; i < ITERS; ++i) {
    acc0 += __float2int_rn(x); acc1 += __float2int_rn(x + 1.f); acc2 += __float2int_rn(x + 2.f); acc3 += __float2int_rn(x + 3.f);
    x += a;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc0 + acc1 + acc2 + acc3;
}
int main() {
  int nsm; cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0);
  int clk; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, 0);
  printf("SMs %d clock %d kHz\n", nsm, clk);
  const int blocks = nsm * 8, threads = 256; size_t n = (size_t)blocks * threads;
  void* buf; cudaMalloc(&buf, n * 8);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  float ms;
  auto run = [&](const char* name, double flops_per_thread, auto launch) {
    launch(); cudaDeviceSynchronize();
    cudaEventRecord(e0); for (int r = 0; r < 5; ++r) launch(); cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    double tot = flops_per_thread * n * 5;
    printf("%-10s %.3f ms  %.2f TFLOP/s (or Tops)  err=%s\n", name, ms / 5, tot / (ms * 1e-3) / 1e12, cudaGetErrorString(cudaGetLastError()));
  };
  run("ffma64", 2.0 * 8 * ITERS, [&] { k_ffma64<<<blocks, threads>>>((double*)buf, 0.999, 1e-3); });
  run("ffma32", 2.0 * 8 * ITERS, [&] { k_ffma32<<<blocks, threads>>>((float*)buf, 0.999f, 1e-3f); });
  // per warp: ITERS mma m8n8k4 => 2*8*8*4 flops each; per thread /32
  run("dmma8", (double)ITERS * 2 * 8 * 8 * 4 / 32, [&] { k_dmma<<<blocks, threads>>>((double*)buf); });
  run("dmma16", (double)ITERS * 2 * 16 * 8 * 4 / 32, [&] { k_dmma16<<<blocks, threads>>>((double*)buf); });
  run("hmma_bf16", (double)ITERS * 2 * 16 * 8 * 16 / 32, [&] { k_hmma<<<blocks, threads>>>((float*)buf); });
  run("imma_s8", (double)ITERS * 2 * 16 * 8 * 32 / 32, [&] { k_imma<<<blocks, threads>>>((int*)buf); });
  run("f2i", 4.0 * ITERS, [&] { k_f2i<<<blocks, threads>>>((int*)buf, 0.25f); });
  cudaFree(buf);
  return 0;
}
