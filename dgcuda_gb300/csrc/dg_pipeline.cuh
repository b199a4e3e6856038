// dg_pipeline.cuh -- one SSP-RK3 stage of the tensor-core Euler path as a
// single persistent launch.
//
// A stage is three kinds of work: the Riemann flux of every side (k_face,
// FP64-bound), the cell means of the stage output (k_means, with the
// limiter) and the element stage (k_element_oz, latency-bound: its FP64,
// integer and tensor phases leave the FP64 pipe idle about half the time).
// As three launches they run one after another.  Here every block of one
// persistent launch takes work items off one list -- face tiles of 128
// sides, means tiles and element tiles of 64 elements -- so that blocks on
// the same SM run face tiles while others run element tiles, and the FP64
// pipe does the faces in the element stage's idle cycles.
//
// Dependencies: the means of an element need the fluxes of its three sides;
// the element stage needs them too and, with the limiter, the means of the
// element's three neighbours.  The host builds the list (dg_solver.cpp,
// pipe_build) so that every item comes after all the items it needs; a
// block waits for those (a flag per item, set with release semantics after
// the item's writes) before it starts.  Items are handed out in list order,
// and an item only ever waits for items earlier in the list, which running
// blocks hold (face items wait for nothing), so the waits end.  Each wait
// has a deadline all the same (about a second): a block that reaches it sets
// the error word, and every block stops at its next item; the host reports
// DG_TIMEOUT.  The results are bit for bit those of the three launches:
// the same bodies run on the same inputs.
#pragma once
#include "dg_ozaki.cuh"

namespace dg {
namespace oz {

enum { kItemFace = 0, kItemMeans = 1, kItemElem = 2 };
constexpr int kFaceTile = kOzThreads;  // sides per face item (one per thread)
constexpr int kElemTile = kOzElems;    // elements per means / element item
constexpr long long kWaitCycles = 2000000000ll;  // about a second at 2 GHz

__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// thread 0 waits until every flag flags[list[i]] is set (or the error word
// is, or the deadline passes: then it sets the error word); the block gets
// whether it may go on
__device__ __forceinline__ bool wait_all(const int *flags, const int *list, int n, int *err,
                                         int *ok_s) {
  if (threadIdx.x == 0) {
    int good = 1;
    const long long t0 = clock64();
    for (int i = 0; i < n && good; i++) {
      while (!ld_acquire(flags + list[i])) {
        if (ld_acquire(err)) {
          good = 0;
          break;
        }
        if (clock64() - t0 > kWaitCycles) {
          atomicExch(err, 1);
          good = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    *ok_s = good;
  }
  __syncthreads();
  const int r = *ok_s;
  __syncthreads();
  return r != 0;
}

// after the block's writes of an item: every thread fences its own, then
// thread 0 sets the item's flag
__device__ __forceinline__ void publish(int *flag) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) st_release(flag, 1);
}

template <class Eq, int P, bool LIM>
__global__ void __launch_bounds__(kOzThreads, P <= 3 ? 4 : 3)
    k_stage_oz(const __grid_constant__ Tab<P> tab, const __grid_constant__ EqP q,
               const __grid_constant__ ElemArgs a, const __grid_constant__ FaceArgs fa,
               const __grid_constant__ PipeArgs pa, double *__restrict__ M,
               const Tabs *__restrict__ ozt) {
  extern __shared__ __align__(16) double smem_d[];
  __shared__ int item_s, ok_s;
  int *err = pa.work + 1;
  int *flags = pa.work + 2;
  for (;;) {
    if (threadIdx.x == 0) item_s = ld_acquire(err) ? pa.nitems : atomicAdd(pa.work, 1);
    __syncthreads();
    const int it = item_s;
    __syncthreads();
    if (it >= pa.nitems) break;
    const int code = pa.items[it], type = code >> 29, tile = code & 0x1FFFFFFF;
    if (type == kItemFace) {
      const int s = tile * kFaceTile + (int)threadIdx.x;
      if (s < fa.S) face_body<Eq, P, LIM>(tab, q, fa, s);
      publish(flags + tile);
    } else if (LIM && type == kItemMeans) {
      const int b = pa.fdep_ptr[tile];
      if (!wait_all(flags, pa.fdep + b, pa.fdep_ptr[tile + 1] - b, err, &ok_s)) break;
      const int e = tile * kElemTile + (int)threadIdx.x;
      if (threadIdx.x < kElemTile && e < a.K) means_body<Eq, P>(tab, a, fa.Fs, M, e);
      publish(flags + pa.nface + tile);
    } else {
      bool ok;
      if (LIM) {
        const int b = pa.mdep_ptr[tile];
        ok = wait_all(flags + pa.nface, pa.mdep + b, pa.mdep_ptr[tile + 1] - b, err, &ok_s);
      } else {
        const int b = pa.fdep_ptr[tile];
        ok = wait_all(flags, pa.fdep + b, pa.fdep_ptr[tile + 1] - b, err, &ok_s);
      }
      if (!ok) break;
      element_oz_tile<Eq, P, LIM>(tab, q, a, ozt, tile, smem_d);
    }
  }
}

}  // namespace oz
}  // namespace dg
