// k_resid_launch.cuh -- launcher of the fused residual for one tile shape.
// Included only by the resid_*.cu units, one per (precision, tile shape), so
// that the residual's twelve kernel variants of a shape compile in parallel
// with the rest of the library.
#pragma once
#include "kernels.cuh"

namespace ot2d {

template <class R, int TJ, int TK>
cudaError_t launch_resid_shape(const Slice<R>* d_sl, const Batch& b, int flags, cudaStream_t st) {
  constexpr size_t smem = rt_smem_bytes<R, TJ, TK>();
  static DeviceOnce once;
  cudaError_t ae = once.run([&](int&) {
    const void* ks[] = {(const void*)k_resid<R, false, 0, TJ, TK>, (const void*)k_resid<R, false, 1, TJ, TK>,
                        (const void*)k_resid<R, false, 2, TJ, TK>, (const void*)k_resid<R, false, 4, TJ, TK>,
                        (const void*)k_resid<R, true, 0, TJ, TK>, (const void*)k_resid<R, true, 1, TJ, TK>,
                        (const void*)k_resid<R, true, 2, TJ, TK>, (const void*)k_resid<R, true, 4, TJ, TK>};
    for (const void* k : ks) {
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  });
  if (ae != cudaSuccess) return ae;
  // one launch per (preconditioning, reconstruction family) in the batch
  const int m = b.lim_mask ? b.lim_mask : 15;
  const dim3 g(b.tile_blocks), t(TJ * TK);
  for (int pre = 0; pre <= (b.precon ? 1 : 0); ++pre) {
    if (m & 1) {
      if (pre) k_resid<R, true, 0, TJ, TK><<<g, t, smem, st>>>(d_sl, b.d_tfirst, b.nslice, flags, b.d_part);
      else k_resid<R, false, 0, TJ, TK><<<g, t, smem, st>>>(d_sl, b.d_tfirst, b.nslice, flags, b.d_part);
    }
    if (m & 2) {
      if (pre) k_resid<R, true, 1, TJ, TK><<<g, t, smem, st>>>(d_sl, b.d_tfirst, b.nslice, flags, b.d_part);
      else k_resid<R, false, 1, TJ, TK><<<g, t, smem, st>>>(d_sl, b.d_tfirst, b.nslice, flags, b.d_part);
    }
    if (m & 4) {
      if (pre) k_resid<R, true, 4, TJ, TK><<<g, t, smem, st>>>(d_sl, b.d_tfirst, b.nslice, flags, b.d_part);
      else k_resid<R, false, 4, TJ, TK><<<g, t, smem, st>>>(d_sl, b.d_tfirst, b.nslice, flags, b.d_part);
    }
    if (m & 8) {
      if (pre) k_resid<R, true, 2, TJ, TK><<<g, t, smem, st>>>(d_sl, b.d_tfirst, b.nslice, flags, b.d_part);
      else k_resid<R, false, 2, TJ, TK><<<g, t, smem, st>>>(d_sl, b.d_tfirst, b.nslice, flags, b.d_part);
    }
  }
  return cudaGetLastError();
}

}  // namespace ot2d
