// peaks_probe.cu -- arithmetic peak rates of the GPU the library runs on:
// FP64 DFMA, FP32 FFMA and FP64 DMMA (mma.sync m8n8k4), register-resident
// FMA chains, 8 CTAs of 256 threads per SM, CUDA events, three repetitions.
// These are the FP64 and FP32 denominators of the benchmark's roofline (the
// HBM and BF16 ones are measured separately).  Not part of libqbg.so; built
// and run by python -m qball_gb300.peaks.
#include <cstdio>
#include <cuda_runtime.h>

template <int ITERS>
__global__ void k_dfma(double* out, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
#pragma unroll 4
  for (int i = 0; i < ITERS; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <int ITERS>
__global__ void k_ffma(float* out, float a, float b) {
  float x[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) x[j] = threadIdx.x + j;
#pragma unroll 4
  for (int i = 0; i < ITERS; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) x[j] = fmaf(x[j], a, b);
  }
  float s = 0;
#pragma unroll
  for (int j = 0; j < 16; ++j) s += x[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <int ITERS>
__global__ void k_dmma(double* out) {
  double a = threadIdx.x * 1e-3, b = 1.0 - threadIdx.x * 1e-4;
  double c[4][2] = {};
#pragma unroll 2
  for (int i = 0; i < ITERS; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                   : "+d"(c[j][0]), "+d"(c[j][1]) : "d"(a), "d"(b));
  }
  double s = 0;
  for (int j = 0; j < 4; ++j) s += c[j][0] + c[j][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int main() {
  cudaDeviceProp p; cudaGetDeviceProperties(&p, 0);
  printf("%s SMs=%d cc=%d.%d\n", p.name, p.multiProcessorCount, p.major, p.minor);
  double* dd; float* df; cudaMalloc(&dd, 1 << 26); cudaMalloc(&df, 1 << 26);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  const int blocks = p.multiProcessorCount * 8, threads = 256;
  const int IT = 4096;
  for (int rep = 0; rep < 3; ++rep) {
    float ms;
    cudaEventRecord(e0); k_dfma<IT><<<blocks, threads>>>(dd, 0.999, 1e-3); cudaEventRecord(e1);
    cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    double fl = 2.0 * 8 * IT * (double)blocks * threads;
    printf("DFMA  %.3f TFLOP/s (%.3f ms)\n", fl / ms / 1e9, ms);
    cudaEventRecord(e0); k_ffma<IT><<<blocks, threads>>>(df, 0.999f, 1e-3f); cudaEventRecord(e1);
    cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    fl = 2.0 * 16 * IT * (double)blocks * threads;
    printf("FFMA  %.3f TFLOP/s (%.3f ms)\n", fl / ms / 1e9, ms);
    cudaEventRecord(e0); k_dmma<IT / 4><<<blocks, threads>>>(dd); cudaEventRecord(e1);
    cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    fl = 2.0 * 8 * 8 * 4 * 4 * (IT / 4) * (double)blocks * threads / 32;
    printf("DMMA  %.3f TFLOP/s (%.3f ms)\n", fl / ms / 1e9, ms);
  }
  cudaError_t err = cudaGetLastError();
  printf("err=%s\n", cudaGetErrorString(err));
  return err != cudaSuccess;
}
