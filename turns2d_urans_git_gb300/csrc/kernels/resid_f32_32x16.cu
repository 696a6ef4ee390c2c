// resid_f32_32x16.cu -- the fused residual of the FP32-mixed path on 32x16 tiles.
#include "k_resid_launch.cuh"
namespace ot2d {
template cudaError_t launch_resid_shape<float, 32, 16>(const Slice<float>*, const Batch&, int, cudaStream_t);
}
