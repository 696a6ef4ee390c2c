// resid_f64_8x32.cu -- the fused residual of the plain FP64 path on 8x32 tiles.
#include "k_resid_launch.cuh"
namespace ot2d {
template cudaError_t launch_resid_shape<double, 8, 32>(const Slice<double>*, const Batch&, int, cudaStream_t);
}
