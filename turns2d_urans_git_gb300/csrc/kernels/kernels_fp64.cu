// kernels_fp64.cu -- the plain FP64 path.  Compiled with -fmad=false so that
// a*b+c rounds twice, as the reference Fortran and the oracle evaluate it.
#include "launchers.cuh"
namespace ot2d {
OT2D_INSTANTIATE(double)

namespace {
__global__ void k_stqol(const double* __restrict__ q, double* __restrict__ qtn, double* __restrict__ qtnm1,
                        double* __restrict__ qnewt, int64_t qs, int nv, int ntac, int istep) {
  const int64_t n = qs * nv;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    mv_stqol_elem(q, qtn, qtnm1, qnewt, i, ntac, istep);
}
}  // namespace

cudaError_t launch_stqol(const double* q, double* qtn, double* qtnm1, double* qnewt, int64_t qs, int nv, int ntac,
                         int istep, cudaStream_t st) {
  const int64_t n = qs * nv;
  if (n <= 0) return cudaSuccess;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_stqol<<<(int)blocks, 256, 0, st>>>(q, qtn, qtnm1, qnewt, qs, nv, ntac, istep);
  return cudaGetLastError();
}

cudaError_t branch_of_device(Branch*& out) {
  static thread_local Branch br[16];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 16) return cudaErrorInvalidDevice;
  Branch& b = br[dev];
  if (!b.st) {
    if ((e = cudaStreamCreateWithFlags(&b.st, cudaStreamNonBlocking)) != cudaSuccess) return e;
    if ((e = cudaEventCreateWithFlags(&b.fork, cudaEventDisableTiming)) != cudaSuccess) return e;
    if ((e = cudaEventCreateWithFlags(&b.join, cudaEventDisableTiming)) != cudaSuccess) return e;
    if ((e = cudaEventCreateWithFlags(&b.join_end, cudaEventDisableTiming)) != cudaSuccess) return e;
    for (cudaEvent_t* ev : {&b.resid, &b.rbc, &b.edges})
      if ((e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming)) != cudaSuccess) return e;
  }
  out = &b;
  return cudaSuccess;
}
}
