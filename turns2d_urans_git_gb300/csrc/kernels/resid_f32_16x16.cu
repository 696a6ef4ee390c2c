// resid_f32_16x16.cu -- the fused residual of the FP32-mixed path on 16x16 tiles.
#include "k_resid_launch.cuh"
namespace ot2d {
template cudaError_t launch_resid_shape<float, 16, 16>(const Slice<float>*, const Batch&, int, cudaStream_t);
}
