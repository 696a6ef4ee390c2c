// resid_f64_32x8.cu -- the fused residual of the plain FP64 path on 32x8 tiles.
#include "k_resid_launch.cuh"
namespace ot2d {
template cudaError_t launch_resid_shape<double, 32, 8>(const Slice<double>*, const Batch&, int, cudaStream_t);
}
