// k_bc.cuh -- boundary conditions on the halo cells of q (bc), on the
// residual (rbc) and on the SA variable (turbc).  One CTA per slice walks the
// &bcinp table in order (later entries see the halo values of earlier ones,
// as in src/bc.f:19-83); threads split the cells of one boundary line.
// q is updated in FP64 (q64); the compute copy's halo ring is refreshed at
// the end when the compute type is float.
#pragma once
#include "dev_common.cuh"

namespace ot2d {

struct QV {  // FP64 view of one slice of q
  double* p; int jd; int64_t qs;
  __device__ __forceinline__ double& operator()(int j, int k, int n) const {
    return p[(int64_t)(n - 1) * qs + (int64_t)(k - 1) * jd + (j - 1)];
  }
};

// bc.f:1757-1776 style (rho,u,v,p) extrapolation into halo cell (j,k)
static __device__ __forceinline__ void extrap_prim(const ot2d_params& p, QV q, int j, int k, int j1, int k1, int j2, int k2,
                                            double foso) {
  const int nq = p.nq; const double gm1 = p.gm1;
  double rho1 = q(j1, k1, 1) * q(j1, k1, nq);
  double rho2 = q(j2, k2, 1) * q(j2, k2, nq);
  double u1 = q(j1, k1, 2) / q(j1, k1, 1);
  double u2 = q(j2, k2, 2) / q(j2, k2, 1);
  double v1 = q(j1, k1, 3) / q(j1, k1, 1);
  double v2 = q(j2, k2, 3) / q(j2, k2, 1);
  double p1 = gm1 * (q(j1, k1, 4) - 0.5 * (sq(q(j1, k1, 2)) + sq(q(j1, k1, 3))) / q(j1, k1, 1)) * q(j1, k1, nq);
  double pp2 = gm1 * (q(j2, k2, 4) - 0.5 * (sq(q(j2, k2, 2)) + sq(q(j2, k2, 3))) / q(j2, k2, 1)) * q(j2, k2, nq);
  double r = ((1. + foso) * rho1 - foso * rho2) / q(j, k, nq);
  q(j, k, 1) = r;
  double a = ((1. + foso) * u1 - foso * u2) * r;
  double b = ((1. + foso) * v1 - foso * v2) * r;
  q(j, k, 2) = a; q(j, k, 3) = b;
  double press = (1. + foso) * p1 - foso * pp2;
  q(j, k, 4) = press / (gm1 * q(j, k, nq)) + 0.5 * (sq(a) + sq(b)) / r;
}

// bcwall (bc.f:1669-1801) with bctany + uv (bc.f:1328-1415, :2224-2264),
// one wall column j, wall along k (idir = +-2)
static __device__ void bcwall_col(const ot2d_params& p, QV q, const double* xx, const double* xy, const double* yx,
                           const double* yy, const double* ug, const double* vg, int j, int ks, int ke, int idir,
                           int invsc, int istep0) {
  const int jd = p.jd, nq = p.nq; const double gm1 = p.gm1;
  int iadd = isign1(idir);
  int k = (idir == 2) ? ke : ks;
  int k1 = k + iadd, k2 = k1 + iadd;
  double foso = invsc ? 1.0 : 0.0;
  auto M = [&](const double* a, int jj, int kk) { return a[at(jd, jj, kk)]; };
  auto G = [&](const double* a, int jj, int kk) { return a ? a[at(jd, jj, kk)] : 0.0; };
  double u, v;
  {
    double ft = 1.0;
    double u1 = (q(j, k1, 2) * M(xx, j, k) + q(j, k1, 3) * M(xy, j, k)) / q(j, k1, 1);
    double v1 = (q(j, k1, 2) * M(yx, j, k) + q(j, k1, 3) * M(yy, j, k)) / q(j, k1, 1);
    if (invsc) {
      double u2 = (q(j, k2, 2) * M(xx, j, k) + q(j, k2, 3) * M(xy, j, k)) / q(j, k2, 1);
      u = (1. + ft) * u1 - ft * u2;
    } else {
      u = G(ug, j, k) * M(xx, j, k) + G(vg, j, k) * M(xy, j, k) + G(ug, j, k1) * M(xx, j, k1) +
          G(vg, j, k1) * M(xy, j, k1) - u1;
    }
    v = G(ug, j, k) * M(yx, j, k) + G(vg, j, k) * M(yy, j, k) + G(ug, j, k1) * M(yx, j, k1) +
        G(vg, j, k1) * M(yy, j, k1) - v1;
  }
  double t11 = (M(yy, j, k)), t12 = -(M(xy, j, k)), t21 = -(M(yx, j, k)), t22 = (M(xx, j, k));
  double vol = 1. / (t22 * t11 - t12 * t21);
  double uwall = (t11 * u + t12 * v) * vol;
  double vwall = (t21 * u + t22 * v) * vol;
  {
    double rho1 = q(j, k1, 1) * q(j, k1, nq);
    double rho2 = q(j, k2, 1) * q(j, k2, nq);
    double p1 = gm1 * (q(j, k1, 4) - 0.5 * (sq(q(j, k1, 2)) + sq(q(j, k1, 3))) / q(j, k1, 1)) * q(j, k1, nq);
    double pp2 = gm1 * (q(j, k2, 4) - 0.5 * (sq(q(j, k2, 2)) + sq(q(j, k2, 3))) / q(j, k2, 1)) * q(j, k2, nq);
    double r = ((1. + foso) * rho1 - foso * rho2) / q(j, k, nq);
    q(j, k, 1) = r;
    double a = uwall * r, b = vwall * r;
    q(j, k, 2) = a; q(j, k, 3) = b;
    double press = (1. + foso) * p1 - foso * pp2;
    q(j, k, 4) = press / (gm1 * q(j, k, nq)) + 0.5 * (sq(a) + sq(b)) / r;
  }
  for (int kc = 1; kc <= ke - ks; ++kc) {
    int kk = (idir == 2) ? ke - kc : ks + kc;
    int kk1 = kk + iadd, kk2 = kk1 + iadd;
    extrap_prim(p, q, j, kk, j, kk1, j, kk2, 1.0);
  }
  double t = (double)istep0 / 30.;
  if (t > 1. || p.iread > 0) t = 1.;
  double scal = (10. - 15. * t + 6. * t * t) * cube(t);
  double rscal = 1. - scal;
  for (int kk = ks; kk <= ke; ++kk) {
    double ajacinv = 1. / q(j, kk, nq);
    q(j, kk, 1) = q(j, kk, 1) * scal + rscal * p.rinf * ajacinv;
    q(j, kk, 2) = q(j, kk, 2) * scal + rscal * p.rinf * p.uinf * ajacinv;
    q(j, kk, 3) = q(j, kk, 3) * scal + rscal * p.rinf * p.vinf * ajacinv;
    q(j, kk, 4) = q(j, kk, 4) * scal + rscal * p.einf * ajacinv;
  }
}

// bcout_trkl first-row cell (bc.f:712-835), Turkel form with bt, Mp
static __device__ void trkl_cell(const ot2d_params& p, QV q, int j, int k, int j1, int k1, int j2, int k2, double mx, double my,
                          double ugc, double vgc, double btc, int iadd) {
  const int nq = p.nq; const double gm1 = p.gm1, ggm1 = p.ggm1, gamma = p.gamma, Mp = p.Mp;
  const double foso = 1.0;
  double snorm = -1. * iadd / sqrt(sq(mx) + sq(my));
  double xxn = mx * snorm, xyn = my * snorm;
  double qext[4], qbar[4], delq[4], delw[4];
  for (int n = 1; n <= 4; ++n) qext[n - 1] = (1. + foso) * q(j1, k1, n) * q(j1, k1, nq) - foso * q(j2, k2, n) * q(j2, k2, nq);
  qbar[0] = 0.5 * (qext[0] + p.rinf);
  qbar[1] = 0.5 * (qext[1] + p.rinf * p.uinf);
  qbar[2] = 0.5 * (qext[2] + p.rinf * p.vinf);
  qbar[3] = 0.5 * (qext[3] + p.einf);
  delq[0] = 0.5 * (p.rinf - qext[0]);
  delq[1] = 0.5 * (p.rinf * p.uinf - qext[1]);
  delq[2] = 0.5 * (p.rinf * p.vinf - qext[2]);
  delq[3] = 0.5 * (p.einf - qext[3]);
  double rho = qbar[0], rrho = 1. / rho;
  double uu = qbar[1] * rrho, vv = qbar[2] * rrho, e = qbar[3] * rrho;
  double uv2 = 0.5 * (uu * uu + vv * vv);
  double cjkl = sqrt(ggm1 * (e - uv2));
  double c2i = 1. / (cjkl * cjkl);
  double ge = gamma * e - gm1 * uv2;
  double qq = (uu - ugc) * xxn + (vv - vgc) * xyn;
  double bSq = sq(Mp) / (btc - sq(Mp) * (btc - 1));
  double Z = sqrt((1. - bSq) * qq * (1. - bSq) * qq + 4. * bSq * cjkl * cjkl);
  double Zi = 1. / Z;
  double R = 0.5 * ((1. - bSq) * qq + Z);
  double S = 0.5 * ((1. - bSq) * qq - Z);
  double sqs = fsign(1., qq), sR = fsign(1., R + bSq * qq), sR2 = fsign(1., R + qq * bSq);
  double sS = fsign(1., S + bSq * qq), sS2 = fsign(1., S + qq * bSq);
  delw[0] = (1. - uv2 * gm1 * c2i) * sqs * delq[0];
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
  double J = q(j, k, nq);
  for (int n = 1; n <= 4; ++n) q(j, k, n) = (qbar[n - 1] - delq[n - 1]) / J;
}

// Apply the q boundary conditions of one slice.  Called by all threads of
// one CTA; bt64: the time-step factor bt of time.f (FP64) given by the
// caller, else the slice's own bt array, else 1 (bt enters the Turkel-form
// far field through bSq = Mp**2/(bt - Mp**2*(bt-1)))
template <class R>
__device__ void bc_slice(const Slice<R>& S, const double* bt64, int istep0) {
  const ot2d_params& p = *S.P;
  const int jd = p.jd;
  QV q{S.q64, jd, S.qs};
  const double *xx = S.xx64, *xy = S.xy64, *yx = S.yx64, *yy = S.yy64, *ug = S.ug64, *vg = S.vg64;
  auto btv = [&](int j, int k) -> double {
    const int64_t o = at(jd, j, k);
    return bt64 ? bt64[o] : (S.bt ? (double)S.bt[o] : 1.0);
  };
  for (int ib = 0; ib < p.nbc; ++ib) {
    int js, je, ks, ke; bc_range(p, ib, js, je, ks, ke);
    const int idir = p.ibdir[ib], t = p.ibtyp[ib], iadd = isign1(idir), iadir = idir < 0 ? -idir : idir;
    if (t == 3 || t == 4 || t == 5) {
      int invsc = (t == 3) ? 1 : (t == 4) ? 0 : p.invisc;
      if (iadir == 2)
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x) bcwall_col(p, q, xx, xy, yx, yy, ug, vg, j, ks, ke, idir, invsc, istep0);
    } else if (t == 51) {
      if (iadir == 2)
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x)
          for (int kc = 1; kc <= ke - ks + 1; ++kc) {
            int k, k1;
            if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
            int jj = jd - j + 1;
            double scale1 = q(jj, k1, p.nq) / q(j, k, p.nq);
            double scale2 = q(j, k1, p.nq) / q(jj, k, p.nq);
            for (int n = 1; n <= 4; ++n) q(j, k, n) = q(jj, k1, n) * scale1;
            for (int n = 1; n <= 4; ++n) q(jj, k, n) = q(j, k1, n) * scale2;
          }
    } else if (t == 47) {
      if (iadir == 1) {
        for (int k = ks + threadIdx.x; k <= ke; k += blockDim.x) {
          int j = (idir == 1) ? je : js, j1 = j + iadd, j2 = j1 + iadd;
          trkl_cell(p, q, j, k, j1, k, j2, k, xx[at(jd, j, k)], xy[at(jd, j, k)], ug ? ug[at(jd, j, k)] : 0.0,
                    vg ? vg[at(jd, j, k)] : 0.0, btv(j, k), iadd);
          for (int jc = 1; jc <= je - js; ++jc) {
            int jx = (idir == 1) ? je - jc : js + jc;
            extrap_prim(p, q, jx, k, jx + iadd, k, jx + 2 * iadd, k, 0.0);
          }
        }
      } else if (iadir == 2) {
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x) {
          int k = (idir == 2) ? ke : ks, k1 = k + iadd, k2 = k1 + iadd;
          trkl_cell(p, q, j, k, j, k1, j, k2, yx[at(jd, j, k)], yy[at(jd, j, k)], ug ? ug[at(jd, j, k)] : 0.0,
                    vg ? vg[at(jd, j, k)] : 0.0, btv(j, k), iadd);
          for (int kc = 1; kc <= ke - ks; ++kc) {
            int kx = (idir == 2) ? ke - kc : ks + kc;
            extrap_prim(p, q, j, kx, j, kx + iadd, j, kx + 2 * iadd, 0.0);
          }
        }
      }
    } else if (t == 46) {
      for (int idx = threadIdx.x; idx < (je - js + 1) * (ke - ks + 1); idx += blockDim.x) {
        int j = js + idx % (je - js + 1), k = ks + idx / (je - js + 1);
        double rj = 1. / q(j, k, p.nq);
        double r = p.rinf * rj, a = p.rinf * p.uinf * rj, b = p.rinf * p.vinf * rj;
        q(j, k, 1) = r; q(j, k, 2) = a; q(j, k, 3) = b;
        q(j, k, 4) = p.pinf / p.gm1 * rj + 0.5 * (sq(a) + sq(b)) / r;
      }
    } else if (t == 10 || t == 11) {
      const int nq = p.nq;
      if (iadir == 1) {
        for (int k = ks + threadIdx.x; k <= ke; k += blockDim.x)
          for (int jc = 1; jc <= je - js + 1; ++jc) {
            if (t == 10) {
              int j = (idir == 1) ? je - jc + 1 : js + jc - 1, j1 = j + iadd;
              double s1 = q(j1, k, nq) / q(j, k, nq);
              for (int n = 1; n <= 4; ++n) q(j, k, n) = (1. + 0.0) * q(j1, k, n) * s1 - 0.0 * q(j1 + iadd, k, n) * (q(j1 + iadd, k, nq) / q(j, k, nq));
            } else {
              int j, j1;
              if (idir == 1) { j = je - jc + 1; j1 = je + jc; } else { j = js + jc - 1; j1 = js - jc; }
              double sc = q(j1, k, nq) / q(j, k, nq);
              q(j, k, 1) = q(j1, k, 1) * sc; q(j, k, 2) = -q(j1, k, 2) * sc;
              q(j, k, 3) = q(j1, k, 3) * sc; q(j, k, 4) = q(j1, k, 4) * sc;
            }
          }
      } else if (iadir == 2) {
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x)
          for (int kc = 1; kc <= ke - ks + 1; ++kc) {
            if (t == 10) {
              int k = (idir == 2) ? ke - kc + 1 : ks + kc - 1, k1 = k + iadd;
              double s1 = q(j, k1, nq) / q(j, k, nq);
              for (int n = 1; n <= 4; ++n) q(j, k, n) = (1. + 0.0) * q(j, k1, n) * s1 - 0.0 * q(j, k1 + iadd, n) * (q(j, k1 + iadd, nq) / q(j, k, nq));
            } else {
              int k, k1;
              if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
              double sc = q(j, k1, nq) / q(j, k, nq);
              q(j, k, 1) = q(j, k1, 1) * sc; q(j, k, 2) = q(j, k1, 2) * sc;
              q(j, k, 3) = -q(j, k1, 3) * sc; q(j, k, 4) = q(j, k1, 4) * sc;
            }
          }
      }
    } else if (t == 22) {
      const int nq = p.nq;
      if (iadir == 1) {
        int jj = je - js + 1;
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x) {
          int jc = (idir == 1) ? jd - 2 * jj + (j - js + 1) : 1 + 2 * jj - (je - j + 1);
          for (int k = ks; k <= ke; ++k) {
            double sc = q(jc, k, nq) / q(j, k, nq);
            for (int n = 1; n <= 4; ++n) q(j, k, n) = q(jc, k, n) * sc;
          }
        }
      } else {
        int kk = ke - ks + 1;
        for (int j = js + threadIdx.x; j <= je; j += blockDim.x)
          for (int k = ks; k <= ke; ++k) {
            int kc = (idir == 2) ? p.kd - 2 * kk + (k - ks + 1) : 1 + 2 * kk - (ke - k + 1);
            double sc = q(j, kc, nq) / q(j, k, nq);
            for (int n = 1; n <= 4; ++n) q(j, k, n) = q(j, kc, n) * sc;
          }
      }
    }
    __syncthreads();
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
// cell velocities the SA step computed at its start (samodel2d.f:74-76).
template <class R>
__device__ void turbc_slice(const Slice<R>& S, const R* u, const R* v) {
  const ot2d_params& p = *S.P;
  const int jd = p.jd, kd = p.kd, n5 = p.nmv + 1;
  QV q{S.q64, jd, S.qs};
  const double *xx = S.xx64, *xy = S.xy64, *yx = S.yx64, *yy = S.yy64, *ug = S.ug64, *vg = S.vg64;
  auto U = [&](const R* a, int j, int k) { return (double)a[at(jd, j, k)]; };
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
          double uu = (U(u, j, k) - G(ug, j, k) + U(u, j1, k) - G(ug, j1, k)) * xx[at(jd, j, k)];
          uu = uu + (U(v, j, k) - G(vg, j, k) + U(v, j1, k) - G(vg, j1, k)) * xy[at(jd, j, k)];
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
          double uu = (U(u, j, k) - G(ug, j, k) + U(u, j, k1) - G(ug, j, k1)) * yx[at(jd, j, k)];
          uu = uu + (U(v, j, k) - G(vg, j, k) + U(v, j, k1) - G(vg, j, k1)) * yy[at(jd, j, k)];
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
