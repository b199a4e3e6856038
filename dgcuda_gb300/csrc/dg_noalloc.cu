// dg_noalloc.cu -- the right-hand side without any device allocation.
//
// dg_rhs_device_noalloc evaluates du/dt like dg_rhs, but takes device
// pointers and keeps all of its working memory -- the state in internal
// element order, the edge traces, the side fluxes, the internal result and
// two scalars -- in one statically sized __device__ array defined below.
// It calls no cudaMalloc, cudaFree or other allocating routine.
//
// Who needs this: code that may not allocate device memory at the moment it
// evaluates the operator -- a host application that hands this library a
// fixed memory budget up front and forbids allocation afterwards (device
// memory owned by its own pool), or a latency-critical loop where a
// cudaMalloc would synchronise the device and stall every stream.
//
// The call runs on the solver's stream (dg_solver_stream) and returns once
// that stream has finished its work: the caller's input must be ready with
// respect to that stream when the call is made.
//
// Limits: the array holds DG_NOALLOC_SCRATCH_BYTES (32 MiB) on every GPU that
// loads the library, for the life of the process; problems whose working set
// exceeds it are rejected with DG_UNSUPPORTED.  All calls share the one
// array, so calls whose work overlaps on the GPU (different streams or
// threads without ordering) race on it.  Every call overwrites all of the
// scratch it reads, so nothing carries over from the previous call.  The
// first call on a device looks up the array's device address and keeps it
// for the life of the process (make that first call before any stream
// capture); after cudaDeviceReset, or any teardown of the device's primary
// context, the kept address is stale and the entry point must not be called
// again in that process.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "dg_internal.h"
#include "dg_launch.h"

#define DG_NOALLOC_SCRATCH_BYTES (32u << 20)

static __device__ __align__(256) unsigned char g_noalloc_scratch[DG_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_addr[kMaxDevices] = {nullptr};

// Device address of the array on `device` (which must be current).  Host
// code cannot use g_noalloc_scratch itself: on the host that name is a
// stand-in object, not device memory.  Looked up once per device.
dg_status scratch_for(int device, unsigned char **out) {
  if (device < 0 || device >= kMaxDevices) return dg::fail(DG_BAD_ARG, "device ordinal too large");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return dg::fail(DG_CUDA_ERROR, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_addr[device] = p;
  }
  *out = static_cast<unsigned char *>(g_addr[device]);
  return DG_OK;
}

__global__ void k_noalloc_scalars(dg::DevScalars *ds, double t) {
  ds->t = t;
  ds->dt = 0.0;
  ds->one = 1.0;
  ds->zero = 0.0;
}

size_t round256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace

extern "C" dg_status dg_rhs_device_noalloc(dg_solver *s, double t, const double *C_device,
                                           double *dCdt_device) {
  if (!s || !C_device || !dCdt_device) return dg::fail(DG_BAD_ARG, "null argument");
  dg::SolverView v = dg::solver_view(s);
  cudaError_t e = cudaSetDevice(v.device);
  if (e != cudaSuccess) return dg::fail(DG_CUDA_ERROR, cudaGetErrorString(e));
  const size_t Kp = (size_t)v.ctx.m.Kp, n1 = (size_t)v.p + 1;
  const size_t b_state = round256(sizeof(double) * v.N * v.np * Kp);
  const size_t b_T = round256(sizeof(double) * (size_t)v.K * 3 * n1 * v.N);
  const size_t b_F = round256(sizeof(double) * (size_t)v.S * n1 * v.N);
  const size_t b_ds = round256(sizeof(dg::DevScalars));
  const size_t need = 2 * b_state + b_T + b_F + b_ds;
  if (need > DG_NOALLOC_SCRATCH_BYTES)
    return dg::fail(DG_UNSUPPORTED,
                    "dg_rhs_device_noalloc: this problem needs " + std::to_string(need) +
                        " bytes of scratch, more than the static " +
                        std::to_string((size_t)DG_NOALLOC_SCRATCH_BYTES) + " bytes");
  unsigned char *base = nullptr;
  dg_status st = scratch_for(v.device, &base);
  if (st != DG_OK) return st;
  double *in = reinterpret_cast<double *>(base);
  double *out = reinterpret_cast<double *>(base + b_state);
  double *T = reinterpret_cast<double *>(base + 2 * b_state);
  double *Fh = reinterpret_cast<double *>(base + 2 * b_state + b_T);
  dg::DevScalars *ds = reinterpret_cast<dg::DevScalars *>(base + 2 * b_state + b_T + b_F);

  dg::Ctx c = v.ctx;  // same mesh, tables and stream; scratch from the static array
  c.T = T;
  c.Fh = Fh;
  c.ds = ds;
  k_noalloc_scalars<<<1, 1, 0, v.st>>>(ds, t);
  dg::launch_permute_in(v.st, C_device, in, c.m.perm, v.N * v.np, v.K, c.m.Kp);
  v.ops->trace(c, in);
  v.ops->face(c, &ds->t, 0.0);
  v.ops->element(c, in, nullptr, out, 0.0, 0.0, 1.0, &ds->one);
  dg::launch_permute_out(v.st, out, dCdt_device, c.m.perm, v.N * v.np, v.K, c.m.Kp);
  e = cudaStreamSynchronize(v.st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return dg::fail(DG_CUDA_ERROR, cudaGetErrorString(e));
  return DG_OK;
}
