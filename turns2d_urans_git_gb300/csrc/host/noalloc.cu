// noalloc.cu -- residual norms of step.f:58-93 without any device allocation.
//
// For callers that must not allocate device memory during their iteration
// loop: a driver that has handed the whole device arena to its own pool, a
// real-time loop where cudaMalloc's implicit device synchronisation is not
// acceptable, or a process that runs under a hard memory cap.  The per-block
// partial sums live in a file-scope __device__ array of fixed size instead
// of a buffer obtained from cudaMalloc, so the call allocates nothing (no
// cudaMalloc / cudaFree, no allocating library routine).
//
// Limits and contract:
//  * jd*kd <= OT2D_NOALLOC_MAX_CELLS (1,048,576 array cells, e.g. a
//    1025 x 1023 mesh); larger meshes are rejected with OT2D_ERR_ARG before
//    anything is launched.
//  * The first call on a device looks up the device address of the static
//    scratch (cudaGetSymbolAddress, with that device current) and keeps it
//    for the life of the process.  cudaDeviceReset unloads the module, so
//    the kept address is stale afterwards: a process that resets the device
//    must not call this routine again.
//  * Every call ends with cudaStreamSynchronize and a copy into the caller's
//    host buffer, so no call may be made while its stream is being captured.
//  * The scratch is shared by every call on the device: two calls that
//    overlap in time (different host threads, or different streams without
//    an ordering between them) race on it.  Serialise them.
//  * The scratch needs no initial value: every partial the final pass reads
//    is written by the first pass of the same call.
#include <cuda_runtime.h>

#include <mutex>

#include "runtime.h"

namespace ot2d {
namespace {

constexpr int NA_BS = 256;
constexpr int NA_MAX_BLOCKS = OT2D_NOALLOC_MAX_CELLS / NA_BS;
constexpr int NA_NOUT = 6;

__device__ __align__(256) NormPart g_na_part[NA_MAX_BLOCKS];
__device__ __align__(256) double g_na_out[NA_NOUT];

// per-cell partial of step.f:67-88 (the same expressions as the residual
// kernels' norm epilogue), block tree reduction in a fixed order
__global__ void __launch_bounds__(NA_BS) k_na_partials(const double* __restrict__ s,
                                                       const int32_t* __restrict__ iblank, int jd, int kd, int js,
                                                       int je, int ks, int ke, int nmv, NormPart* __restrict__ part) {
  __shared__ NormPart sh[NA_BS];
  const int cid = blockIdx.x * NA_BS + threadIdx.x;
  const int64_t n2 = (int64_t)jd * kd;
  NormPart np{0.0, 0.0, 0.0, 0x7fffffffffffffffLL};
  if (cid < n2) {
    const int j = cid % jd + 1, k = cid / jd + 1;
    if (j >= js && j <= je && k >= ks && k <= ke) {
      const int64_t o = cid;
      const int ibi = iblank[o];
      const double m = (double)(ibi > 0 ? ibi : 0);
      for (int n = 1; n <= nmv; ++n) {
        const double smrs = fabs(s[(int64_t)(n - 1) * n2 + o]) * m;
        const long long key = ((long long)(k - 1) * (nmv + 1) + n) * (long long)jd + (j - 1);
        if (smrs > np.resmax || (smrs == np.resmax && key < np.key)) { np.resmax = smrs; np.key = key; }
      }
      const double s0 = s[o], s1 = s0 * m, s2 = s[n2 + o] * m, s3 = s[2 * n2 + o] * m, s4 = s[3 * n2 + o] * m;
      np.resrho = s0 * s0;
      np.rsum = s1 * s1 + s2 * s2 + s3 * s3 + s4 * s4;
    }
  }
  sh[threadIdx.x] = np;
  __syncthreads();
  for (int st = NA_BS / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) sh[threadIdx.x] = norm_combine(sh[threadIdx.x], sh[threadIdx.x + st]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// one warp: lane l combines partials l, l+32, ... in order, then a fixed
// shuffle tree; out = rsum, resrho, resmax, j, k, n of the maximum
__global__ void k_na_final(const NormPart* __restrict__ part, int nblk, int jd, int kd, int nmv,
                           double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  NormPart acc{0.0, 0.0, 0.0, 0x7fffffffffffffffLL};
  for (int b = lane; b < nblk; b += 32) acc = norm_combine(acc, part[b]);
  acc = warp_norm_reduce(acc);
  if (lane != 0) return;
  const double volum = (double)jd * (double)kd;
  out[0] = sqrt(acc.rsum / volum);
  out[1] = sqrt(acc.resrho / volum);
  out[2] = acc.resmax;
  if (acc.key == 0x7fffffffffffffffLL) { out[3] = out[4] = out[5] = 0.0; return; }
  const long long jk = acc.key / jd;
  out[3] = (double)(acc.key % jd + 1);
  out[4] = (double)(jk / (nmv + 1) + 1);
  out[5] = (double)(jk % (nmv + 1));
}

// device addresses of the static scratch, looked up once per device
struct NaDev { bool ready = false; NormPart* part = nullptr; double* out = nullptr; };
constexpr int NA_MAX_DEV = 64;
NaDev g_na_dev[NA_MAX_DEV];
std::mutex g_na_mu;

int na_setup(NaDev*& d) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEV) return OT2D_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_na_mu);
  NaDev& e = g_na_dev[dev];
  if (!e.ready) {
    if (cudaGetSymbolAddress((void**)&e.part, g_na_part) != cudaSuccess) return OT2D_ERR_CUDA;
    if (cudaGetSymbolAddress((void**)&e.out, g_na_out) != cudaSuccess) return OT2D_ERR_CUDA;
    e.ready = true;
  }
  d = &e;
  return OT2D_OK;
}

}  // namespace
}  // namespace ot2d

using namespace ot2d;

extern "C" int ot2d_norms_noalloc(const double* s, const int32_t* iblank, int32_t jd, int32_t kd, int32_t js,
                                  int32_t je, int32_t ks, int32_t ke, int32_t nmv, double* out, void* stream) {
  if (!s || !iblank || !out || jd < 1 || kd < 1 || nmv < 4 || js < 1 || je > jd || ks < 1 || ke > kd)
    return OT2D_ERR_ARG;
  if ((int64_t)jd * kd > OT2D_NOALLOC_MAX_CELLS) return OT2D_ERR_ARG;
  NaDev* d = nullptr;
  if (int e = na_setup(d)) return e;
  cudaStream_t st = (cudaStream_t)stream;
  const int nblk = (int)(((int64_t)jd * kd + NA_BS - 1) / NA_BS);
  k_na_partials<<<nblk, NA_BS, 0, st>>>(s, iblank, jd, kd, js, je, ks, ke, nmv, d->part);
  k_na_final<<<1, 32, 0, st>>>(d->part, nblk, jd, kd, nmv, d->out);
  if (cudaGetLastError() != cudaSuccess) return OT2D_ERR_CUDA;
  if (cudaMemcpyAsync(out, d->out, NA_NOUT * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return OT2D_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return OT2D_ERR_CUDA;
  return OT2D_OK;
}
