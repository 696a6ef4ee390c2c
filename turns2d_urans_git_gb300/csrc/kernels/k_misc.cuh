// k_misc.cuh -- time-spectral coupling (src/sources.f:2-27), residual
// norms (src/step.f:58-93), state update (src/step.f:203-213), the
// speed-of-sound monitor (src/step.f:332-392) and the FP64 wall-force
// integration (src/forces.f:130-398).
#pragma once
#include "dev_common.cuh"

namespace ot2d {

// timespectralrhs for one interior cell of slice nsp: s(n) -= rotf*Ds(nsp,m)*q(m)
// over m = 1..nspec (sources.f:16-24).  q of instance m lives at
// q + (m-nsp)*jd*kd in the reference layout.
template <class R>
__device__ __forceinline__ void ts_cell(const Slice<R>& S, const ot2d_params& p, const double* Ds, int j, int k,
                                        R* s, int nv) {
  const int64_t o = at(S.jd, j, k), n2 = (int64_t)S.jd * S.kd;
  const R rotf = (R)p.rotf;
  for (int n = 1; n <= nv; ++n) {
    R acc = s[n - 1];
    for (int m = 1; m <= S.nspec; ++m) {
      R dsn = (R)Ds[(int64_t)(m - 1) * S.nspec + (S.nsp - 1)];
      R qm = S.q[(int64_t)(n - 1) * S.qs + (int64_t)(m - S.nsp) * n2 + o];
      acc = acc - rotf * dsn * qm;
    }
    s[n - 1] = acc;
  }
}

// norm partial of one cell (step.f:67-88): rsum (masked), resrho, resmax
struct NormPart {
  double rsum, resrho, resmax;
  long long key;  // loop-order key of the resmax location (k, n, j)
};
__device__ __forceinline__ NormPart norm_combine(NormPart a, NormPart b) {
  NormPart r;
  r.rsum = a.rsum + b.rsum;
  r.resrho = a.resrho + b.resrho;
  if (b.resmax > a.resmax || (b.resmax == a.resmax && b.key < a.key)) { r.resmax = b.resmax; r.key = b.key; }
  else { r.resmax = a.resmax; r.key = a.key; }
  return r;
}

// fixed shuffle tree over the 32 lanes of a warp; lane 0 gets the result
__device__ __forceinline__ NormPart warp_norm_reduce(NormPart a) {
  for (int off = 16; off > 0; off >>= 1) {
    NormPart o;
    o.rsum = __shfl_down_sync(0xffffffffu, a.rsum, off);
    o.resrho = __shfl_down_sync(0xffffffffu, a.resrho, off);
    o.resmax = __shfl_down_sync(0xffffffffu, a.resmax, off);
    o.key = __shfl_down_sync(0xffffffffu, a.key, off);
    if ((threadIdx.x & 31) < off) a = norm_combine(a, o);
  }
  return a;
}

// The same partial inside the residual kernel's warps: the maximum stays in
// the compute type R (the maximum of floats, and its ties, are the same
// taken in float or in double), so the float path's shuffle tree spends
// the FP64 pipe on the two sums only.
template <class R>
struct NormPartR {
  double rsum, resrho;
  R resmax;
  long long key;
};
template <class R>
__device__ __forceinline__ NormPartR<R> warp_norm_reduce_r(NormPartR<R> a) {
  for (int off = 16; off > 0; off >>= 1) {
    NormPartR<R> o;
    o.rsum = __shfl_down_sync(0xffffffffu, a.rsum, off);
    o.resrho = __shfl_down_sync(0xffffffffu, a.resrho, off);
    o.resmax = __shfl_down_sync(0xffffffffu, a.resmax, off);
    o.key = __shfl_down_sync(0xffffffffu, a.key, off);
    if ((threadIdx.x & 31) < off) {
      a.rsum = a.rsum + o.rsum;
      a.resrho = a.resrho + o.resrho;
      if (o.resmax > a.resmax || (o.resmax == a.resmax && o.key < a.key)) { a.resmax = o.resmax; a.key = o.key; }
    }
  }
  return a;
}

// Wall force integrands of one wall cell (forces.f:168-205, :269-379)
struct ForceCell { double zz, sxx, syy; };

}  // namespace ot2d
