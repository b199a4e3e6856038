// dg_probe.cu -- FP64 FMA throughput of the current GPU (the binding roof of
// the DG kernels on GB300), measured with CUDA events.
#include <cuda_runtime.h>

#include <string>

#include "dg_device.cuh"
#include "dg_internal.h"
#include "../../include/dg_test.h"

namespace {
__global__ void k_fma64(double *out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = threadIdx.x * 1e-3 + k;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, b);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_reciprocal(const double *x, double *r, double *q, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    r[i] = dg::rcp(x[i]);
    q[i] = 1.0 / x[i];
  }
}
__global__ void k_sqrt(const double *x, double *r, double *q, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    r[i] = dg::sqrt_pos(x[i]);
    q[i] = __dsqrt_rn(x[i]);
  }
}
__global__ void k_physical(const double *U, int *fast, int *exact, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double *u = U + 4 * (size_t)i;
    fast[i] = dg::physical_f32(u) ? 1 : 0;
    exact[i] = dg::Euler::physical_fp64(u) ? 1 : 0;
  }
}
}  // namespace

// the Euler positivity test's single-precision filter and its FP64 test on
// the device for n host states U[4 i .. 4 i + 3] = (rho, m_x, m_y, E):
// fast[i] = 1 where the filter settles the state as physical, exact[i] = 1
// where the FP64 test finds it physical
extern "C" dg_status dg_probe_physical(int device, int n, const double *U, int *fast, int *exact) {
  if (n < 0 || (n && (!U || !fast || !exact))) return dg::fail(DG_BAD_ARG, "bad arguments");
  if (!n) return DG_OK;
  if (cudaSetDevice(device) != cudaSuccess) return dg::fail(DG_CUDA_ERROR, "cudaSetDevice");
  double *d = nullptr;
  int *f = nullptr;
  const size_t b = sizeof(double) * 4 * (size_t)n;
  if (cudaMalloc(&d, b) != cudaSuccess) return dg::fail(DG_CUDA_ERROR, "cudaMalloc");
  if (cudaMalloc(&f, 2 * sizeof(int) * (size_t)n) != cudaSuccess) {
    cudaFree(d);
    return dg::fail(DG_CUDA_ERROR, "cudaMalloc");
  }
  cudaError_t e = cudaMemcpy(d, U, b, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_physical<<<(n + 255) / 256, 256>>>(d, f, f + n, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(fast, f, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(exact, f + n, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost);
  cudaFree(d);
  cudaFree(f);
  return e == cudaSuccess ? DG_OK : dg::fail(DG_CUDA_ERROR, cudaGetErrorString(e));
}

// the sound speed's square root (dg::sqrt_pos) and IEEE sqrt on the device
// for n host values: r[i] = sqrt_pos(x[i]), q[i] = sqrt(x[i])
extern "C" dg_status dg_probe_sqrt(int device, int n, const double *x, double *r, double *q) {
  if (n < 0 || (n && (!x || !r || !q))) return dg::fail(DG_BAD_ARG, "bad arguments");
  if (!n) return DG_OK;
  if (cudaSetDevice(device) != cudaSuccess) return dg::fail(DG_CUDA_ERROR, "cudaSetDevice");
  double *d = nullptr;
  const size_t b = sizeof(double) * (size_t)n;
  if (cudaMalloc(&d, 3 * b) != cudaSuccess) return dg::fail(DG_CUDA_ERROR, "cudaMalloc");
  cudaError_t e = cudaMemcpy(d, x, b, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_sqrt<<<(n + 255) / 256, 256>>>(d, d + n, d + 2 * (size_t)n, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(r, d + n, b, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(q, d + 2 * (size_t)n, b, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? DG_OK : dg::fail(DG_CUDA_ERROR, cudaGetErrorString(e));
}

// the flux kernels' reciprocal (dg::rcp) and IEEE division on the device for
// n host values: r[i] = rcp(x[i]), q[i] = 1 / x[i]
extern "C" dg_status dg_probe_reciprocal(int device, int n, const double *x, double *r,
                                         double *q) {
  if (n < 0 || (n && (!x || !r || !q))) return dg::fail(DG_BAD_ARG, "bad arguments");
  if (!n) return DG_OK;
  if (cudaSetDevice(device) != cudaSuccess) return dg::fail(DG_CUDA_ERROR, "cudaSetDevice");
  double *d = nullptr;
  const size_t b = sizeof(double) * (size_t)n;
  if (cudaMalloc(&d, 3 * b) != cudaSuccess) return dg::fail(DG_CUDA_ERROR, "cudaMalloc");
  cudaError_t e = cudaMemcpy(d, x, b, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_reciprocal<<<(n + 255) / 256, 256>>>(d, d + n, d + 2 * (size_t)n, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(r, d + n, b, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(q, d + 2 * (size_t)n, b, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? DG_OK : dg::fail(DG_CUDA_ERROR, cudaGetErrorString(e));
}

extern "C" dg_status dg_measure_fp64_peak(int device, double *tflops) {
  if (!tflops) return dg::fail(DG_BAD_ARG, "null argument");
  if (cudaSetDevice(device) != cudaSuccess) return dg::fail(DG_CUDA_ERROR, "cudaSetDevice");
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 8, threads = 256, iters = 2000;
  double *d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * blocks * threads) != cudaSuccess)
    return dg::fail(DG_CUDA_ERROR, "cudaMalloc");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; rep++) {
    cudaEventRecord(e0);
    k_fma64<<<blocks, threads>>>(d, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (err != cudaSuccess) return dg::fail(DG_CUDA_ERROR, cudaGetErrorString(err));
  *tflops = 2.0 * 8 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return DG_OK;
}
