// k_sst.cuh -- Menter k-omega SST solve komegasst (src/komegasst.f:2-1520,
// constants src/komega.h:1-8), without the transition model.
//
// Same structure as the SA solve: cell-parallel preparation of the fields,
// the BCs on one CTA per slice, a gather-form assembly of both equations'
// right-hand sides and Jacobian bands in which every interior cell adds its
// own contributions in the reference's order, the j-direction tridiagonal
// solves one warp per 32 lines, and the k-direction solves one thread per
// line fused with the update and the eddy viscosity.
//
// Arrays the reference fills only on the interior (strain, F1, F2) are read
// on the halo by findturm and komegadiffus; they are 0 there (what the
// reference reads from a freshly mapped allocation), and k_sst_prep
// re-zeroes them every iteration.
#pragma once
#include "dev_common.cuh"
#include "k_bc.cuh"
#include "launch.h"

namespace ot2d {

// komega.h:1-8 (decimal literals are doubles under -r8)
struct SSTc {
  static constexpr double sigmak1 = 0.85, sigmaw1 = 0.5, beta1 = 0.075, sigmak2 = 1.0, sigmaw2 = 0.856;
  static constexpr double beta2 = 0.0828, betastar = 0.09;
  static constexpr double gamma1 = 5. / 9, gamma2 = 0.44;
};

// scratch arrays of one slice; band b of equation n (0: k, 1: omega) is at
// slot K_BAND + 2*b + n with b: 0 aj, 1 cj, 2 ak, 3 ck, 4 bjmat, 5 sjmat
enum SSTw { K_VMUL = 0, K_RHO, K_U, K_V, K_STRAIN, K_F1, K_F2, K_CDKW, K_UX, K_UY, K_VX, K_VY, K_TXX, K_TXY, K_TYY,
            K_BAND };
enum { KB_AJ = 0, KB_CJ, KB_AK, KB_CK, KB_BJ, KB_SJ };
static_assert(K_BAND + 12 == SST_NSCRATCH, "SST scratch layout");
__host__ __device__ constexpr int kband(int b, int n) { return K_BAND + 2 * b + n; }

__device__ __forceinline__ bool sst_slice(const ot2d_params& p) { return !p.lamin && p.iturb == 2; }

// lamvis (samodel2d.f:200-240) and rho, u, v of komegasst.f:55-62, all
// cells; strain, F1, F2 zeroed on the halo ring
template <class R>
__device__ __forceinline__ void sst_prep_cell(const Slice<R>& S, const ot2d_params& p, int j, int k) {
  const int64_t o = at(S.jd, j, k), qs = S.qs, ws = S.wstride;
  const R c2b = S.k_c2b, c2bp = S.k_c2bp;
  const R q1 = S.q[o], q2 = S.q[qs + o], q3 = S.q[2 * qs + o], q4 = S.q[3 * qs + o], J = S.q[(p.nq - 1) * qs + o];
  const R ra = (R)1. / q1;
  const R uvel = q2 * ra, vvel = q3 * ra;
  const R ei = q4 * ra - (R)0.5 * (sq(uvel) + sq(vvel));
  const R tt = S.k_ggm1 * ei;
  S.w[K_VMUL * ws + o] = c2bp * tt * sqrt(tt) / (c2b + tt);
  S.w[K_RHO * ws + o] = q1 * J;
  S.w[K_U * ws + o] = q2 / q1;
  S.w[K_V * ws + o] = q3 / q1;
  if (j < p.jbeg || j > p.jend || k < p.kbeg || k > p.kend) {
    S.w[K_STRAIN * ws + o] = (R)0;
    S.w[K_F1 * ws + o] = (R)0;
    S.w[K_F2 * ws + o] = (R)0;
  }
}

// kwvortic (strain, komegasst.f:270-318), turbstress (:321-371, with the
// eddy viscosity of the previous step), crossdiff (:374-414) and blend
// (:417-461) at one interior cell
template <class R>
__device__ void sst_fields_cell(const Slice<R>& S, const ot2d_params& p, int j, int k) {
  const int jd = S.jd; const int64_t qs = S.qs, ws = S.wstride;
  const int nmv = p.nmv;
  auto W = [&](int a, int jj, int kk) { return S.w[a * ws + at(jd, jj, kk)]; };
  auto Q = [&](int jj, int kk, int n) { return S.q[(int64_t)(n - 1) * qs + at(jd, jj, kk)]; };
  const int64_t o = at(jd, j, k);
  const R xx = S.xx[o], xy = S.xy[o], yx = S.yx[o], yy = S.yy[o];
  const R rei = (R)1. / S.k_rey;
  // kwvortic / turbstress share the velocity gradients
  const R usi = (R)0.5 * (W(K_U, j + 1, k) - W(K_U, j - 1, k)), vsi = (R)0.5 * (W(K_V, j + 1, k) - W(K_V, j - 1, k));
  const R ueta = (R)0.5 * (W(K_U, j, k + 1) - W(K_U, j, k - 1)), veta = (R)0.5 * (W(K_V, j, k + 1) - W(K_V, j, k - 1));
  const R ux = xx * usi + yx * ueta, uy = xy * usi + yy * ueta;
  const R vx = xx * vsi + yx * veta, vy = xy * vsi + yy * veta;
  {
    const R sxx = ux, sxy = (R)0.5 * (uy + vx), syy = vy;
    S.w[K_STRAIN * ws + o] = sqrt((R)2. * (sxx * sxx + (R)2. * sxy * sxy + syy * syy));
  }
  S.w[K_UX * ws + o] = ux; S.w[K_UY * ws + o] = uy; S.w[K_VX * ws + o] = vx; S.w[K_VY * ws + o] = vy;
  const R sfdiv = (R)(2. / 3) * (ux + vy);
  const R tm = S.turmu[o], q5 = Q(j, k, nmv + 1), q6 = Q(j, k, nmv + 2);
  S.w[K_TXX * ws + o] = tm * rei * ((R)2.0 * ux - sfdiv) - (R)(2. / 3) * q5;
  S.w[K_TYY * ws + o] = tm * rei * ((R)2.0 * vy - sfdiv) - (R)(2. / 3) * q5;
  S.w[K_TXY * ws + o] = tm * rei * (uy + vx);
  // crossdiff
  const R rho = W(K_RHO, j, k);
  const R ksi = (R)0.5 * (Q(j + 1, k, nmv + 1) / W(K_RHO, j + 1, k) - Q(j - 1, k, nmv + 1) / W(K_RHO, j - 1, k));
  const R keta = (R)0.5 * (Q(j, k + 1, nmv + 1) / W(K_RHO, j, k + 1) - Q(j, k - 1, nmv + 1) / W(K_RHO, j, k - 1));
  const R omegasi = (R)0.5 * (Q(j + 1, k, nmv + 2) / W(K_RHO, j + 1, k) - Q(j - 1, k, nmv + 2) / W(K_RHO, j - 1, k));
  const R omegaeta = (R)0.5 * (Q(j, k + 1, nmv + 2) / W(K_RHO, j, k + 1) - Q(j, k - 1, nmv + 2) / W(K_RHO, j, k - 1));
  const R kx = ksi * xx + keta * yx, ky = ksi * xy + keta * yy;
  const R omegax = omegasi * xx + omegaeta * yx, omegay = omegasi * xy + omegaeta * yy;
  R cdkw = kx * omegax + ky * omegay;
  cdkw = cdkw * (R)2 * (R)SSTc::sigmaw2 * rho * rho / q6;
  S.w[K_CDKW * ws + o] = cdkw;
  // blend
  const R sn = S.sn[o];
  const R a1 = rei * sqrt(q5 * rho) / ((R)0.09 * q6 * sn);
  const R a2 = (R)500 * rei * rei * W(K_VMUL, j, k) / (q6 * sq(sn));
  const R cd = fmax2(cdkw, (R)1e-10);
  const R a3 = (R)4 * q5 * (R)SSTc::sigmaw2 / (cd * sq(sn));
  const R arg1 = fmin2(fmax2(a1, a2), a3);
  const R arg2 = fmax2((R)2 * a1, a2);
  S.w[K_F1 * ws + o] = tanh(sq(sq(arg1)));
  S.w[K_F2 * ws + o] = tanh(sq(arg2));
}

// findturm, komegasst.f:190-215, at one cell (rho, strain, F2 of this step)
template <class R>
__device__ __forceinline__ R sst_turm(const ot2d_params& p, R rho, R q5, R q6, R strain, R F2) {
  const R a1 = (R)0.31, rei = (R)1. / (R)p.rey;
  R t = a1 * rho * q5 / fmax2(a1 * q6, F2 * rho * strain * rei);
  return fmax2(t, (R)1e-20);
}
template <class R>
__device__ __forceinline__ void sst_turm_cell(const Slice<R>& S, const ot2d_params& p, int j, int k) {
  const int64_t o = at(S.jd, j, k), qs = S.qs, ws = S.wstride;
  S.turmu[o] = sst_turm(p, S.w[K_RHO * ws + o], S.q[(int64_t)p.nmv * qs + o], S.q[(int64_t)(p.nmv + 1) * qs + o],
                        S.w[K_STRAIN * ws + o], S.w[K_F2 * ws + o]);
}

// komegabc (komegasst.f:906-974 and the per-type routines :977-1432) on
// variables nmv+1, nmv+2 of q64, one CTA per slice.  rho, u, v, vmul are
// the fields of the start of the step (scratch); wd2 holds, on each wall
// halo cell, the squared distance from the first interior cell centre to
// the wall face midpoint (dely2, :1006-1007 / :1048-1049).
template <class R>
__device__ void sst_bc_slice(const Slice<R>& S, const double* wd2) {
  const ot2d_params& p = *S.P;
  const int jd = p.jd, kd = p.kd, n5 = p.nmv + 1, n6 = p.nmv + 2;
  const int64_t ws = S.wstride;
  QV q{S.q64, jd, S.qs};
  const double *xx = S.xx64, *xy = S.xy64, *yx = S.yx64, *yy = S.yy64, *ug = S.ug64, *vg = S.vg64;
  auto W = [&](int a, int j, int k) { return (double)S.w[a * ws + at(jd, j, k)]; };
  auto G = [&](const double* a, int j, int k) { return a ? a[at(jd, j, k)] : 0.0; };
  const double foso = 1.0;
  for (int ib = 0; ib < p.nbc; ++ib) {
    int js, je, ks, ke; bc_range(p, ib, js, je, ks, ke);
    const int idir = p.ibdir[ib], t = p.ibtyp[ib], iadd = isign1(idir), iadir = idir < 0 ? -idir : idir;
    if (t == 3 || t == 4) {
      if (iadir == 1) {
        for (int k = ks + threadIdx.x; k <= ke; k += blockDim.x)
          for (int jc = 1; jc <= je - js + 1; ++jc) {
            int j = (idir == 1) ? je - jc + 1 : js + jc - 1, j1 = j + iadd, j2 = j1 + iadd;
            q(j, k, n5) = (1. + foso) * q(j1, k, n5) - foso * q(j2, k, n5);
            q(j, k, n6) = (1. + foso) * q(j1, k, n6) - foso * q(j2, k, n6);
          }
      } else if (iadir == 2) {
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x)
          for (int kc = 1; kc <= ke - ks + 1; ++kc) {
            int k = (idir == 2) ? ke - kc + 1 : ks + kc - 1, k1 = k + iadd, k2 = k1 + iadd;
            q(j, k, n5) = (1. + foso) * q(j, k1, n5) - foso * q(j, k2, n5);
            q(j, k, n6) = (1. + foso) * q(j, k1, n6) - foso * q(j, k2, n6);
          }
      }
    } else if (t == 5) {
      const double rei = 1. / p.rey;
      const int istep0 = S.ist ? S.ist[0] : p.istep0;
      double tt = ((double)istep0 - 1.) / 30.;
      if (tt > 1. || p.iread > 0) tt = 1.;
      const double scal = (10. - 15. * tt + 6. * tt * tt) * ((tt * tt) * tt);
      if (iadir == 1) {
        // one halo cell deep (nhalo = 1): komegasst.f:1000-1021
        const int j = (idir == 1) ? je : js, j1 = j + iadd;
        for (int k = ks + threadIdx.x; k <= ke; k += blockDim.x) {
          const double dely2 = wd2[at(jd, j, k)];
          const double vmulwall = 0.5 * (W(K_VMUL, j1, k) + W(K_VMUL, j, k));
          const double omegawall = 60. * vmulwall * rei * rei / (SSTc::beta1 * dely2);
          const double qwall5 = -q(j1, k, n5);
          const double qwall6 = 2 * omegawall - 6. * W(K_VMUL, j1, k) * rei * rei / (SSTc::beta1 * dely2);
          q(j, k, n5) = scal * qwall5 + (1. - scal) * q(j, k, n5);
          q(j, k, n6) = scal * qwall6 + (1. - scal) * q(j, k, n6);
        }
      } else if (iadir == 2) {
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x) {
          const int k = (idir == 2) ? ke : ks, k1 = k + iadd;
          const double dely2 = wd2[at(jd, j, k)];
          const double vmulwall = 0.5 * (W(K_VMUL, j, k1) + W(K_VMUL, j, k1));
          const double omegawall = 60. * vmulwall * rei * rei / (SSTc::beta1 * dely2);
          const double qwall5 = -q(j, k1, n5);
          const double qwall6 = 2 * omegawall - 6. * W(K_VMUL, j, k1) * rei * rei / (SSTc::beta1 * dely2);
          q(j, k, n5) = scal * qwall5 + (1. - scal) * q(j, k, n5);
          q(j, k, n6) = scal * qwall6 + (1. - scal) * q(j, k, n6);
          for (int kc = 1; kc <= ke - ks; ++kc) {
            int kk = (idir == 2) ? ke - kc : ks + kc, kk1 = kk + iadd, kk2 = kk1 + iadd;
            q(j, kk, n5) = (1. + foso) * q(j, kk1, n5) - foso * q(j, kk2, n5);
            q(j, kk, n6) = (1. + foso) * q(j, kk1, n6) - foso * q(j, kk2, n6);
          }
        }
      }
    } else if (t == 10 || t == 11) {
      if (iadir == 1) {
        for (int k = ks + threadIdx.x; k <= ke; k += blockDim.x)
          for (int jc = 1; jc <= je - js + 1; ++jc) {
            int j, j1;
            if (idir == 1) { j = je - jc + 1; j1 = je + jc; } else { j = js + jc - 1; j1 = js - jc; }
            q(j, k, n5) = q(j1, k, n5); q(j, k, n6) = q(j1, k, n6);
          }
      } else if (iadir == 2) {
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x)
          for (int kc = 1; kc <= ke - ks + 1; ++kc) {
            int k, k1;
            if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
            q(j, k, n5) = q(j, k1, n5); q(j, k, n6) = q(j, k1, n6);
          }
      }
    } else if (t == 22) {
      if (iadir == 1) {
        const int jj = je - js + 1;
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x) {
          const int jc = (idir == 1) ? jd - 2 * jj + (j - js + 1) : 1 + 2 * jj - (je - j + 1);
          for (int k = ks; k <= ke; ++k) { q(j, k, n5) = q(jc, k, n5); q(j, k, n6) = q(jc, k, n6); }
        }
      } else {
        const int kk = ke - ks + 1;
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x)
          for (int k = ks; k <= ke; ++k) {
            const int kc = (idir == 2) ? kd - 2 * kk + (k - ks + 1) : 1 + 2 * kk - (ke - k + 1);
            q(j, k, n5) = q(j, kc, n5); q(j, k, n6) = q(j, kc, n6);
          }
      }
    } else if (t == 51) {
      if (iadir == 2)
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x)
          for (int kc = 1; kc <= ke - ks + 1; ++kc) {
            int k, k1;
            if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
            const int jj = jd - j + 1;
            q(j, k, n5) = q(jj, k1, n5); q(j, k, n6) = q(jj, k1, n6);
            q(jj, k, n5) = q(j, k1, n5); q(jj, k, n6) = q(j, k1, n6);
          }
    } else if (t == 46) {
      const int nj = je - js + 1, nk = ke - ks + 1;
      for (int idx = threadIdx.x; idx < nj * nk; idx += blockDim.x) {
        const int j = js + idx % nj, k = ks + idx / nj;
        q(j, k, n5) = p.tkeinf * W(K_RHO, j, k);
        q(j, k, n6) = p.tomegainf * W(K_RHO, j, k);
      }
    } else if (t == 47) {
      if (iadir == 1) {
        for (int k = ks + threadIdx.x; k <= ke; k += blockDim.x) {
          const int j = (idir == 1) ? je : js, j1 = j + iadd;
          q(j, k, n5) = p.tkeinf * W(K_RHO, j, k);
          q(j, k, n6) = p.tomegainf * W(K_RHO, j, k);
          double uu = (W(K_U, j, k) - G(ug, j, k) + W(K_U, j1, k) - G(ug, j1, k)) * xx[at(jd, j, k)];
          uu = uu + (W(K_V, j, k) - G(vg, j, k) + W(K_V, j1, k) - G(vg, j1, k)) * xy[at(jd, j, k)];
          uu = uu * iadd;
          if (uu < 0.) { q(j, k, n5) = q(j1, k, n5); q(j, k, n6) = q(j1, k, n6); }
          for (int jc = 1; jc <= je - js; ++jc) {
            const int jx = (idir == 1) ? je - jc : js + jc;
            q(jx, k, n5) = q(jx + iadd, k, n5); q(jx, k, n6) = q(jx + iadd, k, n6);
          }
        }
      } else if (iadir == 2) {
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x) {
          const int k = (idir == 2) ? ke : ks, k1 = k + iadd;
          q(j, k, n5) = p.tkeinf * W(K_RHO, j, k);
          q(j, k, n6) = p.tomegainf * W(K_RHO, j, k);
          double uu = (W(K_U, j, k) - G(ug, j, k) + W(K_U, j, k1) - G(ug, j, k1)) * yx[at(jd, j, k)];
          uu = uu + (W(K_V, j, k) - G(vg, j, k) + W(K_V, j, k1) - G(vg, j, k1)) * yy[at(jd, j, k)];
          uu = uu * iadd;
          if (uu < 0.) { q(j, k, n5) = q(j, k1, n5); q(j, k, n6) = q(j, k1, n6); }
          for (int kc = 1; kc <= ke - ks; ++kc) {
            const int kx = (idir == 2) ? ke - kc : ks + kc;
            q(j, kx, n5) = q(j, kx + iadd, n5); q(j, kx, n6) = q(j, kx + iadd, n6);
          }
        }
      }
    }
    __syncthreads();
  }
}

// Right-hand sides and bands of both equations at one interior cell:
// komegarhslhs (komegasst.f:464-590) -- convection (:507-580), source
// (komegasource, :847-903), diffusion (komegadiffus, :593-844) -- in the
// reference's accumulation order, then the time scaling of :100-131.
template <class R>
__device__ void sst_rhs_cell(const Slice<R>& S, const ot2d_params& p, int j, int k) {
  const int jd = S.jd; const int64_t qs = S.qs, ws = S.wstride;
  const int nmv = p.nmv, nq = p.nq;
  auto W = [&](int a, int jj, int kk) { return S.w[a * ws + at(jd, jj, kk)]; };
  auto Q = [&](int jj, int kk, int n) { return S.q[(int64_t)(n - 1) * qs + at(jd, jj, kk)]; };
  auto X = [&](const R* a, int jj, int kk) { return a[at(jd, jj, kk)]; };
  const int64_t o = at(jd, j, k);
  const R rey = S.k_rey, rei = (R)1. / S.k_rey;
  // ---- convection: upwind split of this cell (:508-511, :546-549)
  const R ugc = S.ug ? S.ug[o] : (R)0, vgc = S.vg ? S.vg[o] : (R)0;
  const R u0 = W(K_U, j, k), v0 = W(K_V, j, k);
  const R uu = S.xx[o] * (u0 - ugc) + S.xy[o] * (v0 - vgc);
  const R up = (R)0.5 * (uu + fabs(uu)), um = (R)0.5 * (uu - fabs(uu));
  const R vv = S.yx[o] * (u0 - ugc) + S.yy[o] * (v0 - vgc);
  const R vp = (R)0.5 * (vv + fabs(vv)), vm = (R)0.5 * (vv - fabs(vv));
  R sj[2], aj[2], cj[2], ak[2], ck[2], bj[2];
  for (int n = 0; n < 2; ++n) {
    const int nn = nmv + 1 + n;
    const R qc = Q(j, k, nn);
    R t = S.s[(int64_t)(nn - 1) * qs + o];
    t = t - up * (qc - Q(j - 1, k, nn)) - um * (Q(j + 1, k, nn) - qc);
    t = t - vp * (qc - Q(j, k - 1, nn)) - vm * (Q(j, k + 1, nn) - qc);
    sj[n] = t;
    aj[n] = (R)0.0 - up; cj[n] = (R)0.0 + um;
    bj[n] = (R)0.0 + up - um;
    ak[n] = (R)0.0 - vp; ck[n] = (R)0.0 + vm;
    bj[n] = bj[n] + vp - vm;
  }
  // ---- source
  const R rho = W(K_RHO, j, k), q5 = Q(j, k, nmv + 1), q6 = Q(j, k, nmv + 2);
  const R F1 = W(K_F1, j, k);
  {
    R prod = W(K_TXX, j, k) * W(K_UX, j, k) + W(K_TXY, j, k) * (W(K_UY, j, k) + W(K_VX, j, k)) +
             W(K_TYY, j, k) * W(K_VY, j, k);
    const R kdes = (R)SSTc::betastar * rey * q6 * q5 / rho;
    const R ksust = (R)SSTc::betastar * rey * (R)p.tkeinf * (R)p.tomegainf * rho;
    const R prodlim = (R)10. * kdes;
    prod = fmin2(prod, prodlim);
    const R kprod = prod;
    const R beta = F1 * (R)SSTc::beta1 + ((R)1 - F1) * (R)SSTc::beta2;
    const R omegades = beta * rey * q6 * q6 / rho;
    const R omegasust = beta * rey * sq((R)p.tomegainf) * rho;
    const R omegacrossdiff = ((R)1 - F1) * W(K_CDKW, j, k) * rei;
    sj[0] = sj[0] + kprod - kdes + ksust;
    const R gammap = F1 * (R)SSTc::gamma1 + ((R)1 - F1) * (R)SSTc::gamma2;
    sj[1] = sj[1] + gammap * rho / S.turmu[o] * prod - omegades + omegacrossdiff + omegasust;
    bj[0] = bj[0] + kdes / q5;
    bj[1] = bj[1] + ((R)2 * omegades + fabs(omegacrossdiff)) / q6;
  }
  // ---- diffusion, j direction: faces j-1/2 (chp(j-1)) and j+1/2 (chp(j))
  {
    const R xxc = S.xx[o], xyc = S.xy[o];
    const R dmxp = (R)0.5 * (xxc + X(S.xx, j + 1, k)), dmyp = (R)0.5 * (xyc + X(S.xy, j + 1, k));
    const R dmxm = (R)0.5 * (X(S.xx, j - 1, k) + xxc), dmym = (R)0.5 * (X(S.xy, j - 1, k) + xyc);
    const R dxp = dmxp * xxc + dmyp * xyc;
    const R dxm = dmxm * xxc + dmym * xyc;
    const R vnulp = (R)0.5 * (W(K_VMUL, j, k) + W(K_VMUL, j + 1, k)), vnup = (R)0.5 * (S.turmu[o] + X(S.turmu, j + 1, k));
    const R vnulm = (R)0.5 * (W(K_VMUL, j - 1, k) + W(K_VMUL, j, k)), vnum = (R)0.5 * (X(S.turmu, j - 1, k) + S.turmu[o]);
    const R F1m = W(K_F1, j - 1, k);
    const R rm = W(K_RHO, j - 1, k), rp = W(K_RHO, j + 1, k);
    for (int n = 0; n < 2; ++n) {
      const int nn = nmv + 1 + n;
      const R sg1 = (R)(n == 0 ? SSTc::sigmak1 : SSTc::sigmaw1), sg2 = (R)(n == 0 ? SSTc::sigmak2 : SSTc::sigmaw2);
      const R chpp = rei * (vnulp + (F1 * sg1 + ((R)1. - F1) * sg2) * vnup);
      const R chpm = rei * (vnulm + (F1m * sg1 + ((R)1. - F1m) * sg2) * vnum);
      const R dnp = Q(j + 1, k, nn) / rp - Q(j, k, nn) / rho;
      const R dnm = Q(j, k, nn) / rho - Q(j - 1, k, nn) / rm;
      const R dcp = dxp * (chpp), dcm = dxm * (chpm);
      const R ax = fmax2(dcm, (R)0.0), cx = fmax2(dcp, (R)0.0);
      sj[n] = sj[n] - ax * dnm + cx * dnp;
      aj[n] = aj[n] - ax / rm;
      cj[n] = cj[n] - cx / rp;
      bj[n] = bj[n] + (ax + cx) / rho;
    }
  }
  // ---- diffusion, k direction
  {
    const R yxc = S.yx[o], yyc = S.yy[o];
    const R dmxp = (R)0.5 * (yxc + X(S.yx, j, k + 1)), dmyp = (R)0.5 * (yyc + X(S.yy, j, k + 1));
    const R dmxm = (R)0.5 * (X(S.yx, j, k - 1) + yxc), dmym = (R)0.5 * (X(S.yy, j, k - 1) + yyc);
    const R dyp = dmxp * yxc + dmyp * yyc;
    const R dym = dmxm * yxc + dmym * yyc;
    const R vnulp = (R)0.5 * (W(K_VMUL, j, k) + W(K_VMUL, j, k + 1)), vnup = (R)0.5 * (S.turmu[o] + X(S.turmu, j, k + 1));
    const R vnulm = (R)0.5 * (W(K_VMUL, j, k - 1) + W(K_VMUL, j, k)), vnum = (R)0.5 * (X(S.turmu, j, k - 1) + S.turmu[o]);
    const R F1m = W(K_F1, j, k - 1);
    const R rm = W(K_RHO, j, k - 1), rp = W(K_RHO, j, k + 1);
    for (int n = 0; n < 2; ++n) {
      const int nn = nmv + 1 + n;
      const R sg1 = (R)(n == 0 ? SSTc::sigmak1 : SSTc::sigmaw1), sg2 = (R)(n == 0 ? SSTc::sigmak2 : SSTc::sigmaw2);
      const R chpp = rei * (vnulp + (F1 * sg1 + ((R)1. - F1) * sg2) * vnup);
      const R chpm = rei * (vnulm + (F1m * sg1 + ((R)1. - F1m) * sg2) * vnum);
      const R dnp = Q(j, k + 1, nn) / rp - Q(j, k, nn) / rho;
      const R dnm = Q(j, k, nn) / rho - Q(j, k - 1, nn) / rm;
      const R dcp = dyp * (chpp), dcm = dym * (chpm);
      const R ay = fmax2(dcm, (R)0.0), cy = fmax2(dcp, (R)0.0);
      sj[n] = sj[n] - ay * dnm + cy * dnp;
      ak[n] = ak[n] - ay / rm;
      ck[n] = ck[n] - cy / rp;
      bj[n] = bj[n] + (ay + cy) / rho;
    }
  }
  // ---- time scaling (:100-131)
  R oat = (R)1.0;
  const int istep = S.ist ? S.ist[1] : p.istep;
  if (p.ntac == -2) oat = (R)0.5;
  if (p.ntac >= 2 && istep > 1) oat = (R)(2. / 3.);
  if (p.ntac == 3 && istep > 2) oat = (R)(6. / 11.);
  R tscal = S.tscale[o];
  if (p.timeac == 1) {
    const R dtpseudo_turb = (R)10.0;
    const int ibi = S.iblank[o];
    const R ib = (R)(ibi > 0 ? ibi : 0);
    const R Jc = S.q[(int64_t)(nq - 1) * qs + o];
    tscal = ib * ((R)1.0 + (R)0.002 * sqrt(Jc)) / ((R)1. + sqrt(Jc));
    tscal = tscal * dtpseudo_turb;
    tscal = tscal / ((R)1. + tscal / S.k_h / oat);
  }
  for (int n = 0; n < 2; ++n) {
    S.w[kband(KB_AJ, n) * ws + o] = aj[n] * tscal;
    S.w[kband(KB_CJ, n) * ws + o] = cj[n] * tscal;
    S.w[kband(KB_AK, n) * ws + o] = ak[n] * tscal;
    S.w[kband(KB_CK, n) * ws + o] = ck[n] * tscal;
    S.w[kband(KB_BJ, n) * ws + o] = (R)1. + bj[n] * tscal;
    S.w[kband(KB_SJ, n) * ws + o] = sj[n] * tscal;
  }
}

// lsolvek2 (komegasst.f:1478-1518) of both equations on one j-line, then
// the update of :135-152 (s = sjmat, q += s*max(iblank,0), clipped at
// 1e-20*rho, in FP64) and findturm of the updated cell (:185; the second
// komegabc changes only halo cells).
template <class R>
__device__ void sst_lsolvek_line(const Slice<R>& S, const ot2d_params& p, int j) {
  const int jd = S.jd; const int64_t ws = S.wstride, qs = S.qs;
  const int ks = p.kbeg, ke = p.kend, nmv = p.nmv;
  for (int n = 0; n < 2; ++n) {
    const R* a = S.w + kband(KB_AK, n) * ws; R* c = S.w + kband(KB_CK, n) * ws;
    const R* b = S.w + kband(KB_BJ, n) * ws; R* sv = S.w + kband(KB_SJ, n) * ws;
    int64_t o = at(jd, j, ks);
    R bb = (R)1. / b[o];
    R sp = sv[o] * bb, cp = c[o] * bb;
    sv[o] = sp; c[o] = cp;
    for (int k = ks + 1; k <= ke; ++k) {
      o = at(jd, j, k);
      bb = (R)1. / (b[o] - a[o] * cp);
      sp = (sv[o] - a[o] * sp) * bb;
      cp = c[o] * bb;
      sv[o] = sp; c[o] = cp;
    }
    R snext = sp;
    for (int k = ke - 1; k >= ks; --k) {
      o = at(jd, j, k);
      const R x = sv[o] - c[o] * snext;
      sv[o] = x;
      snext = x;
    }
  }
  const R* s0 = S.w + kband(KB_SJ, 0) * ws; const R* s1 = S.w + kband(KB_SJ, 1) * ws;
  double* q5 = S.q64 + (int64_t)nmv * qs; double* q6 = S.q64 + (int64_t)(nmv + 1) * qs;
  const double tkelim = 1e-20, tomegalim = 1e-20, relfac = 1.;
  for (int k = ks; k <= ke; ++k) {
    const int64_t o = at(jd, j, k);
    const R r5 = (R)relfac * s0[o], r6 = (R)relfac * s1[o];
    S.s[(int64_t)nmv * qs + o] = r5;
    S.s[(int64_t)(nmv + 1) * qs + o] = r6;
    const int ibi = S.iblank[o];
    const double ib = (double)(ibi > 0 ? ibi : 0);
    const double rho = (double)S.w[K_RHO * ws + o];
    double v5 = q5[o] + (double)r5 * ib, v6 = q6[o] + (double)r6 * ib;
    v5 = fmax2(v5, tkelim * rho);
    v6 = fmax2(v6, tomegalim * rho);
    q5[o] = v5; q6[o] = v6;
    if constexpr (sizeof(R) != sizeof(double)) {
      S.q[(int64_t)nmv * qs + o] = (R)v5;
      S.q[(int64_t)(nmv + 1) * qs + o] = (R)v6;
    }
    S.turmu[o] = sst_turm(p, (R)rho, (R)v5, (R)v6, S.w[K_STRAIN * ws + o], S.w[K_F2 * ws + o]);
  }
}

}  // namespace ot2d
