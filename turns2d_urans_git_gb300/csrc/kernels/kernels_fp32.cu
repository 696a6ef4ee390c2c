// kernels_fp32.cu -- the FP32-mixed path (FP32 residual, Jacobian and sweeps;
// FP64 state update, norms and forces).  Fused multiply-add is allowed here.
#include "launchers.cuh"
namespace ot2d {
OT2D_INSTANTIATE(float)
}
