// k_bc.cuh -- boundary conditions on the halo cells of q (bc), on the
// residual (rbc) and on the SA variable (turbc).  The &bcinp table is
// applied in order (later entries see the halo values of earlier ones, as
// in src/bc.f:19-83): one launch per entry for q, one CTA per slice walking
// the table for the residual and SA.  The q BCs compute in the path's
// compute type: FP64 on the FP64 state for the plain path, float on the
// compute copy for the mixed path (whose FP64 halo ring is widened from it
// at the end).
#pragma once
#include "dev_common.cuh"

namespace ot2d {

struct QV {  // FP64 view of one slice of q
  double* p; int jd; int64_t qs;
  __device__ __forceinline__ double& operator()(int j, int k, int n) const {
    return p[(int64_t)(n - 1) * qs + (int64_t)(k - 1) * jd + (j - 1)];
  }
};

// View of one slice of q in the compute type T of the boundary conditions:
// the FP64 state for the plain path, the float compute copy for the mixed
// path (its BCs run in float, like its residual; the FP64 halo is widened
// from them afterwards, k_bc).
template <class T>
struct QVT {
  T* p; int jd; int64_t qs;
  __device__ __forceinline__ T& operator()(int j, int k, int n) const {
    return p[(int64_t)(n - 1) * qs + (int64_t)(k - 1) * jd + (j - 1)];
  }
};
// gas and freestream constants of the BCs in the compute type
template <class T>
struct BcK { T gm1, ggm1, gamma, mp, rinf, uinf, vinf, einf, pinf; int nq, jd, iread; };
template <class R>
__device__ __forceinline__ BcK<R> bc_consts(const Slice<R>& S) {
  return BcK<R>{S.k_gm1, S.k_ggm1, S.k_gamma, S.k_mp, S.k_rinf, S.k_uinf, S.k_vinf, S.k_einf, S.k_pinf,
                S.P->nq, S.jd, S.P->iread};
}

// bc.f:1757-1776 style (rho,u,v,p) extrapolation into halo cell (j,k)
template <class T>
static __device__ __forceinline__ void extrap_prim(const BcK<T>& K, QVT<T> q, int j, int k, int j1, int k1, int j2, int k2,
                                            T foso) {
  const int nq = K.nq; const T gm1 = K.gm1;
  T rho1 = q(j1, k1, 1) * q(j1, k1, nq);
  T rho2 = q(j2, k2, 1) * q(j2, k2, nq);
  T u1 = q(j1, k1, 2) / q(j1, k1, 1);
  T u2 = q(j2, k2, 2) / q(j2, k2, 1);
  T v1 = q(j1, k1, 3) / q(j1, k1, 1);
  T v2 = q(j2, k2, 3) / q(j2, k2, 1);
  T p1 = gm1 * (q(j1, k1, 4) - (T)0.5 * (sq(q(j1, k1, 2)) + sq(q(j1, k1, 3))) / q(j1, k1, 1)) * q(j1, k1, nq);
  T pp2 = gm1 * (q(j2, k2, 4) - (T)0.5 * (sq(q(j2, k2, 2)) + sq(q(j2, k2, 3))) / q(j2, k2, 1)) * q(j2, k2, nq);
  T r = (((T)1. + foso) * rho1 - foso * rho2) / q(j, k, nq);
  q(j, k, 1) = r;
  T a = (((T)1. + foso) * u1 - foso * u2) * r;
  T b = (((T)1. + foso) * v1 - foso * v2) * r;
  q(j, k, 2) = a; q(j, k, 3) = b;
  T press = ((T)1. + foso) * p1 - foso * pp2;
  q(j, k, 4) = press / (gm1 * q(j, k, nq)) + (T)0.5 * (sq(a) + sq(b)) / r;
}

// bcwall (bc.f:1669-1801) with bctany + uv (bc.f:1328-1415, :2224-2264),
// one wall column j, wall along k (idir = +-2)
template <class T>
static __device__ void bcwall_col(const BcK<T>& K, QVT<T> q, const T* xx, const T* xy, const T* yx,
                           const T* yy, const T* ug, const T* vg, int j, int ks, int ke, int idir,
                           int invsc, int istep0) {
  const int jd = K.jd, nq = K.nq; const T gm1 = K.gm1;
  int iadd = isign1(idir);
  int k = (idir == 2) ? ke : ks;
  int k1 = k + iadd, k2 = k1 + iadd;
  T foso = invsc ? (T)1.0 : (T)0.0;
  auto M = [&](const T* a, int jj, int kk) { return a[at(jd, jj, kk)]; };
  auto G = [&](const T* a, int jj, int kk) { return a ? a[at(jd, jj, kk)] : (T)0.0; };
  T u, v;
  {
    T ft = (T)1.0;
    T u1 = (q(j, k1, 2) * M(xx, j, k) + q(j, k1, 3) * M(xy, j, k)) / q(j, k1, 1);
    T v1 = (q(j, k1, 2) * M(yx, j, k) + q(j, k1, 3) * M(yy, j, k)) / q(j, k1, 1);
    if (invsc) {
      T u2 = (q(j, k2, 2) * M(xx, j, k) + q(j, k2, 3) * M(xy, j, k)) / q(j, k2, 1);
      u = ((T)1. + ft) * u1 - ft * u2;
    } else {
      u = G(ug, j, k) * M(xx, j, k) + G(vg, j, k) * M(xy, j, k) + G(ug, j, k1) * M(xx, j, k1) +
          G(vg, j, k1) * M(xy, j, k1) - u1;
    }
    v = G(ug, j, k) * M(yx, j, k) + G(vg, j, k) * M(yy, j, k) + G(ug, j, k1) * M(yx, j, k1) +
        G(vg, j, k1) * M(yy, j, k1) - v1;
  }
  T t11 = (M(yy, j, k)), t12 = -(M(xy, j, k)), t21 = -(M(yx, j, k)), t22 = (M(xx, j, k));
  T vol = (T)1. / (t22 * t11 - t12 * t21);
  T uwall = (t11 * u + t12 * v) * vol;
  T vwall = (t21 * u + t22 * v) * vol;
  {
    T rho1 = q(j, k1, 1) * q(j, k1, nq);
    T rho2 = q(j, k2, 1) * q(j, k2, nq);
    T p1 = gm1 * (q(j, k1, 4) - (T)0.5 * (sq(q(j, k1, 2)) + sq(q(j, k1, 3))) / q(j, k1, 1)) * q(j, k1, nq);
    T pp2 = gm1 * (q(j, k2, 4) - (T)0.5 * (sq(q(j, k2, 2)) + sq(q(j, k2, 3))) / q(j, k2, 1)) * q(j, k2, nq);
    T r = (((T)1. + foso) * rho1 - foso * rho2) / q(j, k, nq);
    q(j, k, 1) = r;
    T a = uwall * r, b = vwall * r;
    q(j, k, 2) = a; q(j, k, 3) = b;
    T press = ((T)1. + foso) * p1 - foso * pp2;
    q(j, k, 4) = press / (gm1 * q(j, k, nq)) + (T)0.5 * (sq(a) + sq(b)) / r;
  }
  for (int kc = 1; kc <= ke - ks; ++kc) {
    int kk = (idir == 2) ? ke - kc : ks + kc;
    int kk1 = kk + iadd, kk2 = kk1 + iadd;
    extrap_prim(K, q, j, kk, j, kk1, j, kk2, (T)1.0);
  }
  T t = (T)istep0 / (T)30.;
  if (t > (T)1. || K.iread > 0) t = (T)1.;
  T scal = ((T)10. - (T)15. * t + (T)6. * t * t) * cube(t);
  T rscal = (T)1. - scal;
  for (int kk = ks; kk <= ke; ++kk) {
    T ajacinv = (T)1. / q(j, kk, nq);
    q(j, kk, 1) = q(j, kk, 1) * scal + rscal * K.rinf * ajacinv;
    q(j, kk, 2) = q(j, kk, 2) * scal + rscal * K.rinf * K.uinf * ajacinv;
    q(j, kk, 3) = q(j, kk, 3) * scal + rscal * K.rinf * K.vinf * ajacinv;
    q(j, kk, 4) = q(j, kk, 4) * scal + rscal * K.einf * ajacinv;
  }
}

// bcout_trkl first-row cell (bc.f:712-835), Turkel form with bt, Mp
template <class T>
static __device__ void trkl_cell(const BcK<T>& K, QVT<T> q, int j, int k, int j1, int k1, int j2, int k2, T mx, T my,
                          T ugc, T vgc, T btc, int iadd) {
  const int nq = K.nq; const T gm1 = K.gm1, ggm1 = K.ggm1, gamma = K.gamma, Mp = K.mp;
  const T foso = (T)1.0;
  T snorm = -(T)1. * iadd / sqrt(sq(mx) + sq(my));
  T xxn = mx * snorm, xyn = my * snorm;
  T qext[4], qbar[4], delq[4], delw[4];
  for (int n = 1; n <= 4; ++n) qext[n - 1] = ((T)1. + foso) * q(j1, k1, n) * q(j1, k1, nq) - foso * q(j2, k2, n) * q(j2, k2, nq);
  qbar[0] = (T)0.5 * (qext[0] + K.rinf);
  qbar[1] = (T)0.5 * (qext[1] + K.rinf * K.uinf);
  qbar[2] = (T)0.5 * (qext[2] + K.rinf * K.vinf);
  qbar[3] = (T)0.5 * (qext[3] + K.einf);
  delq[0] = (T)0.5 * (K.rinf - qext[0]);
  delq[1] = (T)0.5 * (K.rinf * K.uinf - qext[1]);
  delq[2] = (T)0.5 * (K.rinf * K.vinf - qext[2]);
  delq[3] = (T)0.5 * (K.einf - qext[3]);
  T rho = qbar[0], rrho = (T)1. / rho;
  T uu = qbar[1] * rrho, vv = qbar[2] * rrho, e = qbar[3] * rrho;
  T uv2 = (T)0.5 * (uu * uu + vv * vv);
  T cjkl = sqrt(ggm1 * (e - uv2));
  T c2i = (T)1. / (cjkl * cjkl);
  T ge = gamma * e - gm1 * uv2;
  T qq = (uu - ugc) * xxn + (vv - vgc) * xyn;
  T bSq = sq(Mp) / (btc - sq(Mp) * (btc - 1));
  T Z = sqrt(((T)1. - bSq) * qq * ((T)1. - bSq) * qq + (T)4. * bSq * cjkl * cjkl);
  T Zi = (T)1. / Z;
  T R = (T)0.5 * (((T)1. - bSq) * qq + Z);
  T S = (T)0.5 * (((T)1. - bSq) * qq - Z);
  T sqs = fsign((T)1., qq), sR = fsign((T)1., R + bSq * qq), sR2 = fsign((T)1., R + qq * bSq);
  T sS = fsign((T)1., S + bSq * qq), sS2 = fsign((T)1., S + qq * bSq);
  delw[0] = ((T)1. - uv2 * gm1 * c2i) * sqs * delq[0];
  delw[0] = delw[0] + uu * c2i * gm1 * sqs * delq[1];
  delw[0] = delw[0] + vv * c2i * gm1 * sqs * delq[2];
  delw[0] = delw[0] - gm1 * c2i * sqs * delq[3];
  delw[1] = (vv * xxn - uu * xyn) * sqs * delq[0];
  delw[1] = delw[1] + xyn * sqs * delq[1];
  delw[1] = delw[1] - xxn * sqs * delq[2];
  delw[2] = -Zi * (uv2 * gm1 * c2i * S + bSq * qq) * sR * delq[0];
  delw[2] = delw[2] + (xxn * bSq + S * uu * gm1 * c2i) * Zi * sR * delq[1];
  delw[2] = delw[2] + (xyn * bSq + S * vv * gm1 * c2i) * Zi * sR2 * delq[2];
  delw[2] = delw[2] - S * gm1 * c2i * Zi * sR2 * delq[3];
  delw[3] = Zi * (uv2 * gm1 * c2i * R + qq * bSq) * sS * delq[0];
  delw[3] = delw[3] - (xxn * bSq + R * uu * gm1 * c2i) * Zi * sS * delq[1];
  delw[3] = delw[3] - (xyn * bSq + R * vv * gm1 * c2i) * Zi * sS2 * delq[2];
  delw[3] = delw[3] + R * gm1 * c2i * Zi * sS2 * delq[3];
  delq[0] = delw[0] + delw[2] + delw[3];
  delq[1] = uu * delw[0] + xyn * delw[1] + (uu + xxn * R / bSq) * delw[2];
  delq[1] = delq[1] + (uu + xxn * S / bSq) * delw[3];
  delq[2] = vv * delw[0] - xxn * delw[1] + (vv + xyn * R / bSq) * delw[2];
  delq[2] = delq[2] + (vv + xyn * S / bSq) * delw[3];
  delq[3] = uv2 * delw[0] + (uu * xyn - vv * xxn) * delw[1];
  delq[3] = delq[3] + (ge + R * qq / bSq) * delw[2];
  delq[3] = delq[3] + (ge + S * qq / bSq) * delw[3];
  T J = q(j, k, nq);
  for (int n = 1; n <= 4; ++n) q(j, k, n) = (qbar[n - 1] - delq[n - 1]) / J;
}

// bc.f:2-86 for BC entry ib of one slice (the &bcinp table's order is kept
// by the caller: one launch per entry).  The cells of an entry are
// independent; thread tid of nthr takes every nthr-th of them, so an entry
// can be spread over several CTAs (the far-field and wall BCs are FP64
// arithmetic, and one SM's FP64 pipe per slice made them a long serial
// stretch of the iteration).  bt (time.f) enters the Turkel-form far field
// through bSq = Mp**2/(bt - Mp**2*(bt-1)): the slice's bt array, else 1.
template <class R>
__device__ void bc_entry(const Slice<R>& S, int istep0, int ib, int tid, int nthr) {
  using T = R;
  const ot2d_params& p = *S.P;
  const int jd = p.jd;
  const BcK<T> K = bc_consts(S);
  QVT<T> q{S.q, jd, S.qs};
  const T *xx = S.xx, *xy = S.xy, *yx = S.yx, *yy = S.yy, *ug = S.ug, *vg = S.vg;
  auto btv = [&](int j, int k) -> T {
    const int64_t o = at(jd, j, k);
    return S.bt ? S.bt[o] : (T)1.0;
  };
  {
    int js, je, ks, ke; bc_range(p, ib, js, je, ks, ke);
    const int idir = p.ibdir[ib], t = p.ibtyp[ib], iadd = isign1(idir), iadir = idir < 0 ? -idir : idir;
    if (t == 3 || t == 4 || t == 5) {
      int invsc = (t == 3) ? 1 : (t == 4) ? 0 : p.invisc;
      if (iadir == 2)
        for (int j = js + tid; j <= je; j += nthr) bcwall_col(K, q, xx, xy, yx, yy, ug, vg, j, ks, ke, idir, invsc, istep0);
    } else if (t == 51) {
      if (iadir == 2)
        for (int j = js + tid; j <= je; j += nthr)
          for (int kc = 1; kc <= ke - ks + 1; ++kc) {
            int k, k1;
            if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
            int jj = jd - j + 1;
            T scale1 = q(jj, k1, p.nq) / q(j, k, p.nq);
            T scale2 = q(j, k1, p.nq) / q(jj, k, p.nq);
            for (int n = 1; n <= 4; ++n) q(j, k, n) = q(jj, k1, n) * scale1;
            for (int n = 1; n <= 4; ++n) q(jj, k, n) = q(j, k1, n) * scale2;
          }
    } else if (t == 47) {
      if (iadir == 1) {
        for (int k = ks + tid; k <= ke; k += nthr) {
          int j = (idir == 1) ? je : js, j1 = j + iadd, j2 = j1 + iadd;
          trkl_cell(K, q, j, k, j1, k, j2, k, xx[at(jd, j, k)], xy[at(jd, j, k)], ug ? ug[at(jd, j, k)] : (T)0.0,
                    vg ? vg[at(jd, j, k)] : (T)0.0, btv(j, k), iadd);
          for (int jc = 1; jc <= je - js; ++jc) {
            int jx = (idir == 1) ? je - jc : js + jc;
            extrap_prim(K, q, jx, k, jx + iadd, k, jx + 2 * iadd, k, (T)0.0);
          }
        }
      } else if (iadir == 2) {
        for (int j = js + tid; j <= je; j += nthr) {
          int k = (idir == 2) ? ke : ks, k1 = k + iadd, k2 = k1 + iadd;
          trkl_cell(K, q, j, k, j, k1, j, k2, yx[at(jd, j, k)], yy[at(jd, j, k)], ug ? ug[at(jd, j, k)] : (T)0.0,
                    vg ? vg[at(jd, j, k)] : (T)0.0, btv(j, k), iadd);
          for (int kc = 1; kc <= ke - ks; ++kc) {
            int kx = (idir == 2) ? ke - kc : ks + kc;
            extrap_prim(K, q, j, kx, j, kx + iadd, j, kx + 2 * iadd, (T)0.0);
          }
        }
      }
    } else if (t == 46) {
      for (int idx = tid; idx < (je - js + 1) * (ke - ks + 1); idx += nthr) {
        int j = js + idx % (je - js + 1), k = ks + idx / (je - js + 1);
        T rj = (T)1. / q(j, k, p.nq);
        T r = K.rinf * rj, a = K.rinf * K.uinf * rj, b = K.rinf * K.vinf * rj;
        q(j, k, 1) = r; q(j, k, 2) = a; q(j, k, 3) = b;
        q(j, k, 4) = K.pinf / K.gm1 * rj + (T)0.5 * (sq(a) + sq(b)) / r;
      }
    } else if (t == 10 || t == 11) {
      const int nq = p.nq;
      if (iadir == 1) {
        for (int k = ks + tid; k <= ke; k += nthr)
          for (int jc = 1; jc <= je - js + 1; ++jc) {
            if (t == 10) {
              int j = (idir == 1) ? je - jc + 1 : js + jc - 1, j1 = j + iadd;
              T s1 = q(j1, k, nq) / q(j, k, nq);
              for (int n = 1; n <= 4; ++n) q(j, k, n) = ((T)1. + (T)0.0) * q(j1, k, n) * s1 - (T)0.0 * q(j1 + iadd, k, n) * (q(j1 + iadd, k, nq) / q(j, k, nq));
            } else {
              int j, j1;
              if (idir == 1) { j = je - jc + 1; j1 = je + jc; } else { j = js + jc - 1; j1 = js - jc; }
              T sc = q(j1, k, nq) / q(j, k, nq);
              q(j, k, 1) = q(j1, k, 1) * sc; q(j, k, 2) = -q(j1, k, 2) * sc;
              q(j, k, 3) = q(j1, k, 3) * sc; q(j, k, 4) = q(j1, k, 4) * sc;
            }
          }
      } else if (iadir == 2) {
        for (int j = js + tid; j <= je; j += nthr)
          for (int kc = 1; kc <= ke - ks + 1; ++kc) {
            if (t == 10) {
              int k = (idir == 2) ? ke - kc + 1 : ks + kc - 1, k1 = k + iadd;
              T s1 = q(j, k1, nq) / q(j, k, nq);
              for (int n = 1; n <= 4; ++n) q(j, k, n) = ((T)1. + (T)0.0) * q(j, k1, n) * s1 - (T)0.0 * q(j, k1 + iadd, n) * (q(j, k1 + iadd, nq) / q(j, k, nq));
            } else {
              int k, k1;
              if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
              T sc = q(j, k1, nq) / q(j, k, nq);
              q(j, k, 1) = q(j, k1, 1) * sc; q(j, k, 2) = q(j, k1, 2) * sc;
              q(j, k, 3) = -q(j, k1, 3) * sc; q(j, k, 4) = q(j, k1, 4) * sc;
            }
          }
      }
    } else if (t == 22) {
      const int nq = p.nq;
      if (iadir == 1) {
        int jj = je - js + 1;
        for (int j = js + tid; j <= je; j += nthr) {
          int jc = (idir == 1) ? jd - 2 * jj + (j - js + 1) : 1 + 2 * jj - (je - j + 1);
          for (int k = ks; k <= ke; ++k) {
            T sc = q(jc, k, nq) / q(j, k, nq);
            for (int n = 1; n <= 4; ++n) q(j, k, n) = q(jc, k, n) * sc;
          }
        }
      } else {
        int kk = ke - ks + 1;
        for (int j = js + tid; j <= je; j += nthr)
          for (int k = ks; k <= ke; ++k) {
            int kc = (idir == 2) ? p.kd - 2 * kk + (k - ks + 1) : 1 + 2 * kk - (ke - k + 1);
            T sc = q(j, kc, nq) / q(j, k, nq);
            for (int n = 1; n <= 4; ++n) q(j, k, n) = q(j, kc, n) * sc;
          }
      }
    }
  }
}

// Refresh the compute copy of the halo ring (variables n0..n1) from q64.
template <class R>
__device__ void shadow_ring(const Slice<R>& S, int n0, int n1) {
  if constexpr (sizeof(R) == sizeof(double)) {
    return;
  } else {
    const int jd = S.jd, kd = S.kd;
    const int nring = 2 * jd + 2 * (kd - 2);
    for (int n = n0; n <= n1; ++n)
      for (int i = threadIdx.x; i < nring; i += blockDim.x) {
        int j, k;
        if (i < jd) { j = i + 1; k = 1; }
        else if (i < 2 * jd) { j = i - jd + 1; k = kd; }
        else if (i < 2 * jd + kd - 2) { j = 1; k = i - 2 * jd + 2; }
        else { j = jd; k = i - (2 * jd + kd - 2) + 2; }
        int64_t o = (int64_t)(n - 1) * S.qs + at(jd, j, k);
        S.q[o] = (R)S.q64[o];
      }
  }
}

// Mixed path: widen the float halo ring (variables n0..n1) that the BCs
// wrote into the FP64 state (the forces, the stored files and the
// time-accurate levels read q64 there); nothing for the plain path.
template <class R>
__device__ void widen_ring(const Slice<R>& S, int n0, int n1) {
  if constexpr (sizeof(R) == sizeof(double)) {
    return;
  } else {
    const int jd = S.jd, kd = S.kd;
    const int nring = 2 * jd + 2 * (kd - 2);
    for (int n = n0; n <= n1; ++n)
      for (int i = threadIdx.x; i < nring; i += blockDim.x) {
        int j, k;
        if (i < jd) { j = i + 1; k = 1; }
        else if (i < 2 * jd) { j = i - jd + 1; k = kd; }
        else if (i < 2 * jd + kd - 2) { j = 1; k = i - 2 * jd + 2; }
        else { j = jd; k = i - (2 * jd + kd - 2) + 2; }
        int64_t o = (int64_t)(n - 1) * S.qs + at(jd, j, k);
        S.q64[o] = (double)S.q[o];
      }
  }
}

// rbc, bc.f:88-177: zero wall / far-field halo residuals, mirror the wake
template <class R>
__device__ void rbc_slice(const Slice<R>& S) {
  const ot2d_params& p = *S.P;
  const int jd = p.jd, nq = p.nq;
  QV q{S.q64, jd, S.qs};
  auto s = [&](int j, int k, int n) -> R& { return S.s[(int64_t)(n - 1) * S.qs + at(jd, j, k)]; };
  for (int ib = 0; ib < p.nbc; ++ib) {
    int js, je, ks, ke; bc_range(p, ib, js, je, ks, ke);
    const int idir = p.ibdir[ib], t = p.ibtyp[ib], iadd = isign1(idir), iadir = idir < 0 ? -idir : idir;
    if (t == 3 || t == 4 || t == 5 || t == 46 || t == 47) {
      int nj = je - js + 1, nk = ke - ks + 1;
      for (int idx = threadIdx.x; idx < nj * nk; idx += blockDim.x) {
        int j = js + idx % nj, k = ks + idx / nj;
        for (int n = 1; n <= 4; ++n) s(j, k, n) = (R)0;
      }
    } else if (t == 51 && iadir == 2) {
      for (int j = js + threadIdx.x; j <= je; j += blockDim.x)
        for (int kc = 1; kc <= ke - ks + 1; ++kc) {
          int k, k1;
          if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
          int jj = jd - j + 1;
          R scale1 = (R)(q(jj, k1, nq) / q(j, k, nq));
          R scale2 = (R)(q(j, k1, nq) / q(jj, k, nq));
          for (int n = 1; n <= 4; ++n) s(j, k, n) = s(jj, k1, n) * scale1;
          for (int n = 1; n <= 4; ++n) s(jj, k, n) = s(j, k1, n) * scale2;
        }
    } else if (t == 10 || t == 11) {
      if (iadir == 1) {
        for (int k = ks + threadIdx.x; k <= ke; k += blockDim.x)
          for (int jc = 1; jc <= je - js + 1; ++jc) {
            int j, j1;
            if (t == 10) { j = (idir == 1) ? je - jc + 1 : js + jc - 1; j1 = j + iadd; }
            else if (idir == 1) { j = je - jc + 1; j1 = je + jc; } else { j = js + jc - 1; j1 = js - jc; }
            R sc = (R)(q(j1, k, nq) / q(j, k, nq));
            for (int n = 1; n <= 4; ++n) s(j, k, n) = (t == 11 && n == 2) ? -s(j1, k, n) * sc : (t == 10 ? (R)(1. + 0.0) * s(j1, k, n) * sc - (R)0 : s(j1, k, n) * sc);
          }
      } else if (iadir == 2) {
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x)
          for (int kc = 1; kc <= ke - ks + 1; ++kc) {
            int k, k1;
            if (t == 10) { k = (idir == 2) ? ke - kc + 1 : ks + kc - 1; k1 = k + iadd; }
            else if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
            R sc = (R)(q(j, k1, nq) / q(j, k, nq));
            for (int n = 1; n <= 4; ++n) s(j, k, n) = (t == 11 && n == 3) ? -s(j, k1, n) * sc : (t == 10 ? (R)(1. + 0.0) * s(j, k1, n) * sc - (R)0 : s(j, k1, n) * sc);
          }
      }
    } else if (t == 22) {
      if (iadir == 1) {
        int jj = je - js + 1;
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x) {
          int jc = (idir == 1) ? jd - 2 * jj + (j - js + 1) : 1 + 2 * jj - (je - j + 1);
          for (int k = ks; k <= ke; ++k) {
            R sc = (R)(q(jc, k, nq) / q(j, k, nq));
            for (int n = 1; n <= 4; ++n) s(j, k, n) = s(jc, k, n) * sc;
          }
        }
      } else {
        int kk = ke - ks + 1;
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x)
          for (int k = ks; k <= ke; ++k) {
            int kc = (idir == 2) ? p.kd - 2 * kk + (k - ks + 1) : 1 + 2 * kk - (ke - k + 1);
            R sc = (R)(q(j, kc, nq) / q(j, k, nq));
            for (int n = 1; n <= 4; ++n) s(j, k, n) = s(j, kc, n) * sc;
          }
      }
    }
    __syncthreads();
  }
}

// turbc, samodel2d.f:827-1303, on variable n5 = nmv+1 of q64.  u, v are the
// cell velocities the SA step computed at its start (samodel2d.f:74-76);
// null: formed here from q as k_sa_prep forms them (q2/q1, q3/q1 in the
// compute precision), so that turbc can run beside k_sa_prep.
template <class R>
__device__ void turbc_slice(const Slice<R>& S, const R* u, const R* v) {
  const ot2d_params& p = *S.P;
  const int jd = p.jd, kd = p.kd, n5 = p.nmv + 1;
  QV q{S.q64, jd, S.qs};
  const double *xx = S.xx64, *xy = S.xy64, *yx = S.yx64, *yy = S.yy64, *ug = S.ug64, *vg = S.vg64;
  // velocity component n (1: u, 2: v) of cell (j, k)
  auto U = [&](const R* a, int n, int j, int k) {
    const int64_t o = at(jd, j, k);
    if (a) return (double)a[o];
    return (double)(S.q[n * S.qs + o] / S.q[o]);
  };
  auto G = [&](const double* a, int j, int k) { return a ? a[at(jd, j, k)] : 0.0; };
  for (int ib = 0; ib < p.nbc; ++ib) {
    int js, je, ks, ke; bc_range(p, ib, js, je, ks, ke);
    const int idir = p.ibdir[ib], t = p.ibtyp[ib], iadd = isign1(idir), iadir = idir < 0 ? -idir : idir;
    if (t == 3 || t == 4) {
      if (iadir == 1) {
        for (int k = ks + threadIdx.x; k <= ke; k += blockDim.x)
          for (int jc = 1; jc <= je - js + 1; ++jc) {
            int j = (idir == 1) ? je - jc + 1 : js + jc - 1, j1 = j + iadd, j2 = j1 + iadd;
            q(j, k, n5) = (1. + 1.0) * q(j1, k, n5) - 1.0 * q(j2, k, n5);
          }
      } else if (iadir == 2) {
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x)
          for (int kc = 1; kc <= ke - ks + 1; ++kc) {
            int k = (idir == 2) ? ke - kc + 1 : ks + kc - 1, k1 = k + iadd, k2 = k1 + iadd;
            q(j, k, n5) = (1. + 1.0) * q(j, k1, n5) - 1.0 * q(j, k2, n5);
          }
      }
    } else if (t == 5) {
      if (iadir == 2)
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x) {
          int k = (idir == 2) ? ke : ks, k1 = k + iadd;
          q(j, k, n5) = -q(j, k1, n5);
          for (int kc = 1; kc <= ke - ks; ++kc) {
            int kk = (idir == 2) ? ke - kc : ks + kc, kk1 = kk + iadd, kk2 = kk1 + iadd;
            q(j, kk, n5) = (1. + 1.0) * q(j, kk1, n5) - 1.0 * q(j, kk2, n5);
          }
        }
    } else if (t == 10 || t == 11) {
      if (iadir == 1) {
        for (int k = ks + threadIdx.x; k <= ke; k += blockDim.x)
          for (int jc = 1; jc <= je - js + 1; ++jc) {
            int j, j1;
            if (idir == 1) { j = je - jc + 1; j1 = je + jc; } else { j = js + jc - 1; j1 = js - jc; }
            q(j, k, n5) = q(j1, k, n5);
          }
      } else if (iadir == 2) {
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x)
          for (int kc = 1; kc <= ke - ks + 1; ++kc) {
            int k, k1;
            if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
            q(j, k, n5) = q(j, k1, n5);
          }
      }
    } else if (t == 22) {
      if (iadir == 1) {
        int jj = je - js + 1;
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x) {
          int jc = (idir == 1) ? jd - 2 * jj + (j - js + 1) : 1 + 2 * jj - (je - j + 1);
          for (int k = ks; k <= ke; ++k) q(j, k, n5) = q(jc, k, n5);
        }
      } else {
        int kk = ke - ks + 1;
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x)
          for (int k = ks; k <= ke; ++k) {
            int kc = (idir == 2) ? kd - 2 * kk + (k - ks + 1) : 1 + 2 * kk - (ke - k + 1);
            q(j, k, n5) = q(j, kc, n5);
          }
      }
    } else if (t == 51) {
      if (iadir == 2)
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x)
          for (int kc = 1; kc <= ke - ks + 1; ++kc) {
            int k, k1;
            if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
            int jj = jd - j + 1;
            q(j, k, n5) = q(jj, k1, n5);
            q(jj, k, n5) = q(j, k1, n5);
          }
    } else if (t == 46) {
      int nj = je - js + 1, nk = ke - ks + 1;
      for (int idx = threadIdx.x; idx < nj * nk; idx += blockDim.x) q(js + idx % nj, ks + idx / nj, n5) = p.vnuinf;
    } else if (t == 47) {
      if (iadir == 1) {
        for (int k = ks + threadIdx.x; k <= ke; k += blockDim.x) {
          int j = (idir == 1) ? je : js, j1 = j + iadd;
          q(j, k, n5) = p.vnuinf;
          double uu = (U(u, 1, j, k) - G(ug, j, k) + U(u, 1, j1, k) - G(ug, j1, k)) * xx[at(jd, j, k)];
          uu = uu + (U(v, 2, j, k) - G(vg, j, k) + U(v, 2, j1, k) - G(vg, j1, k)) * xy[at(jd, j, k)];
          uu = uu * iadd;
          if (uu < 0.) q(j, k, n5) = q(j1, k, n5);
          for (int jc = 1; jc <= je - js; ++jc) {
            int jx = (idir == 1) ? je - jc : js + jc;
            q(jx, k, n5) = q(jx + iadd, k, n5);
          }
        }
      } else if (iadir == 2) {
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x) {
          int k = (idir == 2) ? ke : ks, k1 = k + iadd;
          q(j, k, n5) = p.vnuinf;
          double uu = (U(u, 1, j, k) - G(ug, j, k) + U(u, 1, j, k1) - G(ug, j, k1)) * yx[at(jd, j, k)];
          uu = uu + (U(v, 2, j, k) - G(vg, j, k) + U(v, 2, j, k1) - G(vg, j, k1)) * yy[at(jd, j, k)];
          uu = uu * iadd;
          if (uu < 0.) q(j, k, n5) = q(j, k1, n5);
          for (int kc = 1; kc <= ke - ks; ++kc) {
            int kx = (idir == 2) ? ke - kc : ks + kc;
            q(j, kx, n5) = q(j, kx + iadd, n5);
          }
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace ot2d
