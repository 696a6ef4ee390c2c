// kernels_fp64.cu -- the plain FP64 path.  Compiled with -fmad=false so that
// a*b+c rounds twice, as the reference Fortran and the oracle evaluate it.
#include "launchers.cuh"
namespace ot2d {
OT2D_INSTANTIATE(double)
}
