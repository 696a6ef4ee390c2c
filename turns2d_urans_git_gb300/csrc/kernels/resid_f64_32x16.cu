// resid_f64_32x16.cu -- the fused residual of the plain FP64 path on 32x16 tiles.
#include "k_resid_launch.cuh"
namespace ot2d {
template cudaError_t launch_resid_shape<double, 32, 16>(const Slice<double>*, const Batch&, int, cudaStream_t);
}
