// resid_f32_8x32.cu -- the fused residual of the FP32-mixed path on 8x32 tiles.
#include "k_resid_launch.cuh"
namespace ot2d {
template cudaError_t launch_resid_shape<float, 8, 32>(const Slice<float>*, const Batch&, int, cudaStream_t);
}
