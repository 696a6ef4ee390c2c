// runtime.h -- device residency of solves and batch construction shared by
// the batched solver (solver.cu) and the drop-in layer (dropin.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>
#include "ot2d.h"
#include "../kernels/dev_common.cuh"
#include "../kernels/k_misc.cuh"
#include "../kernels/k_lusgs.cuh"
#include "../kernels/launch.h"

namespace ot2d {

// reduction / status record of one slice (red: 9 doubles, ist: 6 ints)
//  red: rsum, resrho, resmax, resmax key, rsum at it 1, rsum now, peak rsum, 10^-orders,
//       1/(oat*h) of the physical-time term (time.f:195-200)
//  ist: istep0, istep (physical steps), status bits (1 norm, 2 monitor, 4 sweep
//       timeout, 8 no motion entry, 16 folded cell), iteration of convergence,
//       Newton iteration within the physical step (1..itnmax), spare
constexpr int RED_N = 9, IST_N = 6;

// All device arrays of one solve (every time instance), carved from one
// allocation.  FP64 arrays always exist; the compute-type arrays alias the
// FP64 ones on the plain path.
struct DevSolve {
  ot2d_params P{};
  int precision = OT2D_FP64;
  int nspec = 1;
  size_t n2 = 0, nvert = 0, wstride = 0;
  void* mem = nullptr;
  size_t bytes = 0;
  ot2d_params* dP = nullptr;
  double *q64 = nullptr, *xx64 = nullptr, *xy64 = nullptr, *yx64 = nullptr, *yy64 = nullptr;
  double *ug64 = nullptr, *vg64 = nullptr, *xv = nullptr, *yv = nullptr, *Ds = nullptr;
  int32_t* iblank = nullptr;
  // compute type (double* or float*)
  void *q = nullptr, *s = nullptr, *xx = nullptr, *xy = nullptr, *yx = nullptr, *yy = nullptr;
  void *fxa = nullptr, *fya = nullptr, *gxa = nullptr, *gya = nullptr, *ftj = nullptr, *gtj = nullptr;
  void *ug = nullptr, *vg = nullptr, *tscale = nullptr, *bt = nullptr, *turmu = nullptr, *sn = nullptr, *w = nullptr;
  void* lurec = nullptr;
  void* quad = nullptr;     // ilim +-2: quad's face states and line work (k_quad.cuh), per time instance
  double* wd2 = nullptr;   // SST wall term (k-omega SST instances only)
  // time-accurate moving grid (iunst = 1): centres, previous vertex levels,
  // stqol levels (itnmax > 1) and the per-step pitch table (own allocation)
  double *xc = nullptr, *yc = nullptr, *xold = nullptr, *yold = nullptr, *xole = nullptr, *yole = nullptr;
  double *qtn = nullptr, *qtnm1 = nullptr, *qnewt = nullptr;
  double* motion = nullptr;
  int nmotion = 0;
  void* sinf = nullptr;    // f32 freestream residual (mixed path only)
  int nscratch = 0;        // scratch arrays per time instance
};

// bytes one solve needs on the device
size_t solve_bytes(const ot2d_params& p, int precision);
// Launch limits of a batch whose tallest mesh has kd_max array rows and
// whose widest has jd_max columns: the LU-SGS sweep runs one warp per 32
// interior rows in one CTA (at most 1024 threads, kd - 2 <= 1024) with its
// record ring, cross-band rings and first-row halo terms in shared memory
// (at most 227 KB), and the force kernel stages 3 doubles per wall cell.
// precon: the batch holds a preconditioned (preilu2d) mesh.
bool batch_fits(int precision, bool precon, int kd_max, int jd_max);
// allocate + fill the geometry and the freestream state of a solve from the
// vertex grid of time instance 1 (xv1, yv1: jmax*kmax).  Returns OT2D_OK,
// OT2D_ERR_ARG (bad grid / params) or OT2D_ERR_NOMEM / OT2D_ERR_CUDA.
int solve_create(DevSolve& d, const ot2d_params& p, int precision, const double* xv1, const double* yv1,
                 cudaStream_t st);
void solve_destroy(DevSolve& d);
// Per physical step 1..nsteps of a pitching solve: sin and cos of the pitch
// increment and of its negative (motion.f:576-583), uploaded to d.motion.
int solve_motion_table(DevSolve& d, int nsteps, cudaStream_t st);

// Slice view of time instance nsp (1-based) of a solve; red/ist point into
// the caller's status table.
template <class R>
Slice<R> make_slice(const DevSolve& d, int nsp, double* red, int32_t* ist);

// Device-side batch: slice array + prefix tables, rebuilt when membership
// changes.
template <class R>
struct DevBatch {
  Batch b;
  Slice<R>* d_sl = nullptr;
  int32_t* d_idx = nullptr;   // first / jfirst / kfirst, 3*(n+1)
  NormPart* d_part = nullptr;
  size_t cap_sl = 0, cap_part = 0;
  int rt_shape = 0;   // residual tile shape the next build lays out (rt_shape_dims)
  int build(const std::vector<Slice<R>>& sl, cudaStream_t st);  // returns OT2D status
  void release();
};

const char* cuda_err_name(cudaError_t e);

}  // namespace ot2d
