// resid_f64_16x16.cu -- the fused residual of the plain FP64 path on 16x16 tiles.
#include "k_resid_launch.cuh"
namespace ot2d {
template cudaError_t launch_resid_shape<double, 16, 16>(const Slice<double>*, const Batch&, int, cudaStream_t);
}
