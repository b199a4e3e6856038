/* shim.h -- lets the reference's CUDA kernel sources compile as host C++.
 *
 * Test infrastructure only (part of the oracle): nothing in the product
 * includes this.  The reference files are compiled where they lie; this
 * header only supplies what nvcc would have supplied:
 *   - the CUDA qualifiers become nothing, so __global__ kernels are plain
 *     functions and __constant__/__device__ globals are plain globals;
 *   - blockIdx/threadIdx/blockDim are host globals that the driver sets
 *     before calling a kernel body once per index (blockDim.x = 1,
 *     threadIdx.x = idx), i.e. the grid becomes a sequential loop;
 *   - cudaMemcpyToSymbol("name", ...) (the string-name form the reference
 *     uses, src/2d/conservation/conserv_kernels.cu:78-125) is routed to a
 *     lookup the driver defines after the kernels are in scope;
 *   - sqrtf is mapped to sqrt so the geometry is FP64 throughout.
 */
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

using std::abs;
/* <algorithm> cannot be used under -I- (libstdc++ quote-includes its own
 * headers), so the two helpers the kernels call are defined here */
static inline double min(double a, double b) { return a < b ? a : b; }
static inline double max(double a, double b) { return a > b ? a : b; }
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }

#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__
#define __syncthreads() ((void)0)
/* FP64 geometry: the reference's preval_* kernels call sqrtf on doubles */
#define sqrtf(x) sqrt(x)

struct shim_dim3 {
  unsigned x, y, z;
};
extern shim_dim3 threadIdx, blockIdx, blockDim;

typedef int cudaError_t;
#define cudaSuccess 0

/* string-name symbol copy, resolved by the driver */
int cudaMemcpyToSymbol(const char *name, void *src, size_t bytes);

/* the reference defines a CAS-based double atomicAdd it never calls
 * (conserv_kernels.cu:182-194); these make it compile */
static inline unsigned long long atomicCAS(unsigned long long *a, unsigned long long cmp,
                                           unsigned long long val) {
  unsigned long long old = *a;
  if (old == cmp) *a = val;
  return old;
}
static inline long long __double_as_longlong(double d) {
  long long r;
  memcpy(&r, &d, sizeof r);
  return r;
}
static inline double __longlong_as_double(long long l) {
  double r;
  memcpy(&r, &l, sizeof r);
  return r;
}
static inline double sinpi(double x) { return sin(M_PI * x); }
static inline double cospi(double x) { return cos(M_PI * x); }
