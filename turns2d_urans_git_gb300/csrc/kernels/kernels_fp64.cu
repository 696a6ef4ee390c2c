// kernels_fp64.cu -- the plain FP64 path.  Compiled with -fmad=false so that
// a*b+c rounds twice, as the reference Fortran and the oracle evaluate it.
#include "launchers.cuh"
namespace ot2d {
OT2D_INSTANTIATE(double)

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
  }
  out = &b;
  return cudaSuccess;
}
}
