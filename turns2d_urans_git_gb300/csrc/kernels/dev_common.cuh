// dev_common.cuh -- shared device-side definitions for the sm_103a kernels.
//
// Layout in HBM is the reference's: column-major q(jd,kd,nspec,nq) with j
// fastest, 1-based Fortran indices in all index arithmetic below
// (src/modules.f, src/step.f:17-30).  One "slice" is one time instance of one
// solve; a launch covers a ragged batch of slices of different sizes.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "ot2d_params.h"

namespace ot2d {

// Device view of one time instance of one solve.  R is the arithmetic type
// of the residual / Jacobian / sweeps (double for the plain path, float for
// the mixed path); the conservative state is always kept in FP64 (q64).
template <class R>
struct Slice {
  const ot2d_params* P;  // device copy of the instance's params_global
  int32_t jd, kd, nsp, nspec;
  int64_t qs;            // distance between variables of q and s (jd*kd*nspec)
  R* q;                  // compute copy of q (== q64 for R = double)
  double* q64;           // FP64 master state
  R* s;                  // residual / correction (nv variables)
  const R *xx, *xy, *yx, *yy;        // J-scaled cell metrics (setup.f:523-531)
  const R *fxa, *fya, *gxa, *gya;    // face normals from the vertex grid (eulerrhs.f:109-115, :218-222)
  const R *ftj, *gtj;                // face grid speeds (time-spectral), null if steady
  const R *ug, *vg;                  // cell grid velocities, null if steady
  R *tscale, *bt, *turmu;
  const int32_t* iblank;
  const R* sn;                       // SA / SST wall distance (static geometry)
  const double* wd2;                 // SST wall term dely2 on the wall halo cells (null unless SST)
  const R* sinf;                     // mixed path: f32 residual of the uniform freestream (4 vars), or null
  // constants of the residual derived from the double parameters once, on
  // the host (slice_consts): reconstruction (eulerrhs.f:40-53), Sutherland
  // and Prandtl factors (visrhs.f:36-44)
  R k_th, k_qt, k_epsl_x, k_epsl_y, k_c2b, k_c2bp, k_prtr, k_gkpr, k_dre, k_gm1, k_ggm1;
  // Turkel low-Mach preconditioning (iprecon): Mp**2, or -1 without it.
  // A face has bt = 1 (eulerrhs.f:78, :185), so its bSq is Mp**2 itself.
  R k_mp2;
  // parameters the compute kernels read per cell, converted once (GB300's
  // FP64 pipe is narrow: a double -> float conversion per cell and use
  // costs more issue slots than the float arithmetic around it)
  R k_gamma, k_rmue, k_rey, k_eps2, k_epsv, k_h, k_timeac, k_dualtime, k_cfltur;
  R k_mp, k_rinf, k_uinf, k_vinf, k_einf, k_pinf;     // the q boundary conditions
  R* w;                              // scratch of this slice (phase dependent)
  R* lurec;                          // LU-SGS sweep records (skewed bands)
  R* quad;                           // ilim +-2: face states and line work of quad (k_quad.cuh), or null
  int64_t wstride;                   // distance between scratch arrays (>= jd*kd)
  double* red;                       // per-slice reduction output
  int32_t* ist;                      // per-slice counters: istep0, istep, status bits, convergence
                                     // iteration, Newton iteration of the physical step
  const double* Ds;                  // time-spectral operator Ds(nspec,nspec)
  // FP64 geometry kept for FP64-only work (forces, BC metrics in mixed mode)
  const double *xx64, *xy64, *yx64, *yy64, *ug64, *vg64;
  // time-accurate moving grid (iunst = 1, motiontype = 1); null otherwise
  double *xc, *yc;                        // cell centres, rotated every physical step
  double *xv, *yv, *xold, *yold, *xole, *yole;   // vertices now and at the two previous levels
  double *qtn, *qtnm1, *qnewt;            // stqol levels (itnmax > 1), (jd,kd,nspec,nv)
  const double* motion;                   // per physical step: sin, cos of the pitch increment and of its negative
  int32_t nmotion;                        // physical steps in the table
  int32_t nbc;                            // &bcinp entries (params nbc)
  int32_t lim;                            // reconstruction family: 0 central, 1 MUSCL, 2 quad, 4 WENO (rt_lim_class)
};

// The limiter switches rhsup dispatches (eulerrhs.f:84-97): |ilim| 0
// central, 1 MUSCL, 2 PPM quadratic, ilim 4 WENO5; any other value
// reconstructs nothing in the reference, and is refused here.
__host__ __device__ __forceinline__ bool rt_lim_known(int ilim) {
  return ilim == 0 || ilim == 1 || ilim == -1 || ilim == 2 || ilim == -2 || ilim == 4;
}
// Reconstruction family of a limiter switch: ilim 4 -> weno, |ilim| 1 ->
// muscld_new, |ilim| 2 -> quad, otherwise the unlimited central slope of
// iflux.
__host__ __device__ __forceinline__ int rt_lim_class(int ilim) {
  const int a = ilim < 0 ? -ilim : ilim;
  return ilim == 4 ? 4 : (a == 1 ? 1 : (a == 2 ? 2 : 0));
}
// elements of R of a slice's quad block (k_quad.cuh): 40 arrays of jd*kd
__host__ __device__ __forceinline__ int64_t quad_elems(int jd, int kd) { return (int64_t)40 * jd * kd; }

// Fill the residual constants of a slice from its parameters (host side;
// the same double expressions the kernels would evaluate).
template <class R>
inline void slice_consts(Slice<R>& S, const ot2d_params& p) {
  const int irhs = p.irhsy < 0 ? -p.irhsy : p.irhsy;
  S.k_th = (R)((double)(irhs - 2) / (double)irhs);
  S.k_qt = (irhs == 1) ? (R)0.0 : (R)0.25;
  const double ex = 10. / (double)p.jmax, ey = 10. / (double)p.kmax;
  S.k_epsl_x = (R)((ex * ex) * ex);
  S.k_epsl_y = (R)((ey * ey) * ey);
  S.k_c2b = (R)(198.6 / p.tinf);
  S.k_c2bp = S.k_c2b + (R)1.;
  S.k_prtr = (R)(p.pr / 0.9);
  S.k_gkpr = (R)(p.gamma / p.pr);
  S.k_dre = (R)(.5 / p.rey);
  S.k_gm1 = (R)p.gm1;
  S.k_ggm1 = (R)p.ggm1;
  S.k_mp2 = p.iprecon ? (R)(p.Mp * p.Mp) : (R)-1;
  S.nbc = p.nbc;
  S.lim = rt_lim_class(p.ilim);
  S.k_gamma = (R)p.gamma; S.k_rmue = (R)p.rmue; S.k_rey = (R)p.rey;
  S.k_eps2 = (R)(p.epse * 2.); S.k_epsv = (R)1. + S.k_eps2;
  S.k_mp = (R)p.Mp; S.k_rinf = (R)p.rinf; S.k_uinf = (R)p.uinf; S.k_vinf = (R)p.vinf;
  S.k_einf = (R)p.einf; S.k_pinf = (R)p.pinf;
  S.k_h = (R)p.h; S.k_timeac = (R)p.timeac; S.k_dualtime = (R)p.dualtime; S.k_cfltur = (R)p.cfltur;
}

// Fortran SIGN(a,b): |a| with the IEEE sign of b (gfortran semantics).
template <class R> __device__ __forceinline__ R fsign(R a, R b) { return copysign(fabs(a), b); }

// f32 -> f64 from the bits (sign; exponent rebiased by 1023 - 127; mantissa
// moved up 29 places): exact for every normal float, zero and inf, NaN
// stays NaN, subnormal inputs become a zero of their sign as in the mixed
// path's flush-to-zero arithmetic.  Integer operations only, so the FP64
// state update keeps GB300's narrow FP64 pipe for its additions.
__device__ __forceinline__ double f2d_bits_ftz(float x) {
  const uint32_t u = __float_as_uint(x);
  const uint64_t s = (uint64_t)(u >> 31) << 63;
  const uint32_t e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  uint64_t r;
  if (e == 0) r = s;
  else if (e == 0xffu) r = s | (0x7ffull << 52) | ((uint64_t)m << 29);
  else r = s | ((uint64_t)(e + 896u) << 52) | ((uint64_t)m << 29);
  return __longlong_as_double((long long)r);
}

// f64 -> f32 from the bits, rounded to nearest, ties to even, with the
// mixed path's flush to zero: the 29 dropped mantissa bits decide the
// rounding (the carry of a round-up moves into the exponent, and past the
// largest finite float into inf); a result below the smallest normal float
// becomes a zero of its sign unless it rounds up to that float; inf stays
// inf, NaN stays NaN.  Integer operations only (see f2d_bits_ftz).
__device__ __forceinline__ float d2f_bits_rn_ftz(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const uint32_t s = (uint32_t)(b >> 63) << 31;
  const int e = (int)((b >> 52) & 0x7ff);
  const uint64_t m = b & 0xfffffffffffffull;
  uint32_t r;
  if (e == 0x7ff) {
    r = s | 0x7f800000u | (m ? (0x400000u | (uint32_t)(m >> 29)) : 0u);
  } else {
    const int E = e - 896;   // float exponent field before rounding
    if (E >= 255) {
      r = s | 0x7f800000u;
    } else if (E <= 0) {
      // [2^-127, 2^-126) rounds to 2^-126 from 2^-126 - 2^-150 up
      r = (E == 0 && m >= 0xfffffe0000000ull) ? (s | 0x800000u) : s;
    } else {
      const uint32_t mant = (uint32_t)(m >> 29), rem = (uint32_t)(m & 0x1fffffffu);
      const uint32_t up = (rem > 0x10000000u || (rem == 0x10000000u && (mant & 1u))) ? 1u : 0u;
      r = s | (((uint32_t)E << 23) + mant + up);
    }
  }
  return __uint_as_float(r);
}
// MAX / MIN as the oracle evaluates them (first argument on ties).
template <class R> __device__ __forceinline__ R fmax2(R a, R b) { return (b > a) ? b : a; }
template <class R> __device__ __forceinline__ R fmin2(R a, R b) { return (b < a) ? b : a; }
template <class R> __device__ __forceinline__ R sq(R x) { return x * x; }
template <class R> __device__ __forceinline__ R cube(R x) { return (x * x) * x; }
template <class R> __device__ __forceinline__ R pow6(R x) { R t = (x * x) * x; return t * t; }
__device__ __forceinline__ double rsqrt_(double x) { return sqrt(x); }

// exact widening to double
__device__ __forceinline__ double to_d(float x) { return (double)x; }
__device__ __forceinline__ double to_d(double x) { return x; }

// 1-based (j,k) -> linear offset inside one slice
__device__ __forceinline__ int64_t at(int jd, int j, int k) { return (int64_t)(k - 1) * jd + (j - 1); }

// Batched launch: slices are mapped onto a 1-D grid through a prefix table
// (first block of each slice).  Returns the slice index of this block.
__device__ __forceinline__ int find_slice(const int32_t* __restrict__ first, int nslice, int b) {
  int lo = 0, hi = nslice - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(first + mid) <= b) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// bc.f:20-33: convert one &bcinp entry to halo-cell indices
__device__ __forceinline__ void bc_range(const ot2d_params& p, int ib, int& js, int& je, int& ks, int& ke) {
  js = p.jbcs[ib]; je = p.jbce[ib]; ks = p.kbcs[ib]; ke = p.kbce[ib];
  if (js < 0) js = p.jmax + js + 1;
  if (ks < 0) ks = p.kmax + ks + 1;
  if (je < 0) je = p.jmax + je + 1;
  if (ke < 0) ke = p.kmax + ke + 1;
  if (js > 1) js = js + p.nhalo;
  if (ks > 1) ks = ks + p.nhalo;
  if (je < p.jmax) je = je + p.nhalo - 1;
  if (ke < p.kmax) ke = ke + p.nhalo - 1;
  if (je == p.jmax) je = p.jd;
  if (ke == p.kmax) ke = p.kd;
}

__device__ __forceinline__ int isign1(int idir) { return idir >= 0 ? 1 : -1; }

}  // namespace ot2d
