/*
 * oracle_bc.cpp -- TEST INFRASTRUCTURE ONLY (see oracle_common.h).
 * FP64 restatement of the reference's boundary conditions on q (bc) and on
 * the residual (rbc), src/bc.f.
 */
#include <cstdio>
#include <cstdlib>
#include "oracle.h"

namespace oro {

/* bc.f:2224-2264 */
static void uv(int js, int je, int k, A2 xx, A2 xy, A2 yx, A2 yy, const double* u, const double* v,
               double* uwall, double* vwall) {
  for (int j = js; j <= je; ++j) {
    double t11 = (yy(j, k)), t12 = -(xy(j, k)), t21 = -(yx(j, k)), t22 = (xx(j, k));
    double vol = 1. / (t22 * t11 - t12 * t21);
    uwall[j] = (t11 * u[j] + t12 * v[j]) * vol;
    vwall[j] = (t21 * u[j] + t22 * v[j]) * vol;
  }
}

/* bc.f:1328-1415 (idir = +-2 only; the reference prints and skips idir=+-1) */
static void bctany(const P& p, A3 q, double* uwall, double* vwall, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg,
                   int js, int je, int ks, int ke, int idir, int invsc) {
  int iadd = isign(1, idir), iadir = std::abs(idir);
  if (iadir != 2) return;
  int k = (idir == 2) ? ke : ks;
  int k1 = k + iadd, k2 = k1 + iadd;
  double foso = 1.0;
  std::vector<double> u(p.jd + 2), v(p.jd + 2);
  if (invsc) {
    for (int j = js; j <= je; ++j) {
      double u1 = (q(j, k1, 2) * xx(j, k) + q(j, k1, 3) * xy(j, k)) / q(j, k1, 1);
      double u2 = (q(j, k2, 2) * xx(j, k) + q(j, k2, 3) * xy(j, k)) / q(j, k2, 1);
      u[j] = (1. + foso) * u1 - foso * u2;
      double v1 = (q(j, k1, 2) * yx(j, k) + q(j, k1, 3) * yy(j, k)) / q(j, k1, 1);
      v[j] = ug(j, k) * yx(j, k) + vg(j, k) * yy(j, k) + ug(j, k1) * yx(j, k1) + vg(j, k1) * yy(j, k1) - v1;
    }
  } else {
    for (int j = js; j <= je; ++j) {
      double u1 = (q(j, k1, 2) * xx(j, k) + q(j, k1, 3) * xy(j, k)) / q(j, k1, 1);
      double v1 = (q(j, k1, 2) * yx(j, k) + q(j, k1, 3) * yy(j, k)) / q(j, k1, 1);
      u[j] = ug(j, k) * xx(j, k) + vg(j, k) * xy(j, k) + ug(j, k1) * xx(j, k1) + vg(j, k1) * xy(j, k1) - u1;
      v[j] = ug(j, k) * yx(j, k) + vg(j, k) * yy(j, k) + ug(j, k1) * yx(j, k1) + vg(j, k1) * yy(j, k1) - v1;
    }
  }
  uv(js, je, k, xx, xy, yx, yy, u.data(), v.data(), uwall, vwall);
}

/* extrapolation of (rho, u, v, p) used by several wall/outflow routines,
 * e.g. bc.f:1757-1776 */
static inline void extrap_prim(const P& p, A3 q, int nq, int j, int k, int j1, int k1, int j2, int k2, double foso) {
  const double gm1 = p.gm1;
  double rho1 = q(j1, k1, 1) * q(j1, k1, nq);
  double rho2 = q(j2, k2, 1) * q(j2, k2, nq);
  double u1 = q(j1, k1, 2) / q(j1, k1, 1);
  double u2 = q(j2, k2, 2) / q(j2, k2, 1);
  double v1 = q(j1, k1, 3) / q(j1, k1, 1);
  double v2 = q(j2, k2, 3) / q(j2, k2, 1);
  double p1 = gm1 * (q(j1, k1, 4) - 0.5 * (p2(q(j1, k1, 2)) + p2(q(j1, k1, 3))) / q(j1, k1, 1)) * q(j1, k1, nq);
  double pp2 = gm1 * (q(j2, k2, 4) - 0.5 * (p2(q(j2, k2, 2)) + p2(q(j2, k2, 3))) / q(j2, k2, 1)) * q(j2, k2, nq);
  q(j, k, 1) = ((1. + foso) * rho1 - foso * rho2) / q(j, k, nq);
  q(j, k, 2) = ((1. + foso) * u1 - foso * u2) * q(j, k, 1);
  q(j, k, 3) = ((1. + foso) * v1 - foso * v2) * q(j, k, 1);
  double press = (1. + foso) * p1 - foso * pp2;
  q(j, k, 4) = press / (gm1 * q(j, k, nq)) + 0.5 * (p2(q(j, k, 2)) + p2(q(j, k, 3))) / q(j, k, 1);
}

/* bc.f:1669-1801 */
static void bcwall(const P& p, A3 q, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg,
                   int js, int je, int ks, int ke, int idir, int invsc) {
  const int nq = p.nq; const double gm1 = p.gm1;
  int iadd = isign(1, idir), iadir = std::abs(idir);
  if (iadir != 2) return;
  int k = (idir == 2) ? ke : ks;
  int k1 = k + iadd, k2 = k1 + iadd;
  double foso = invsc ? 1.0 : 0.0;
  std::vector<double> uwall(p.jd + 2), vwall(p.jd + 2);
  bctany(p, q, uwall.data(), vwall.data(), xx, xy, yx, yy, ug, vg, js, je, ks, ke, idir, invsc);
  for (int j = js; j <= je; ++j) {
    double rho1 = q(j, k1, 1) * q(j, k1, nq);
    double rho2 = q(j, k2, 1) * q(j, k2, nq);
    double p1 = gm1 * (q(j, k1, 4) - 0.5 * (p2(q(j, k1, 2)) + p2(q(j, k1, 3))) / q(j, k1, 1)) * q(j, k1, nq);
    double pp2 = gm1 * (q(j, k2, 4) - 0.5 * (p2(q(j, k2, 2)) + p2(q(j, k2, 3))) / q(j, k2, 1)) * q(j, k2, nq);
    q(j, k, 1) = ((1. + foso) * rho1 - foso * rho2) / q(j, k, nq);
    q(j, k, 2) = uwall[j] * q(j, k, 1);
    q(j, k, 3) = vwall[j] * q(j, k, 1);
    double press = (1. + foso) * p1 - foso * pp2;
    q(j, k, 4) = press / (gm1 * q(j, k, nq)) + 0.5 * (p2(q(j, k, 2)) + p2(q(j, k, 3))) / q(j, k, 1);
  }
  for (int kc = 1; kc <= ke - ks; ++kc) {
    k = (idir == 2) ? ke - kc : ks + kc;
    k1 = k + iadd; k2 = k1 + iadd;
    for (int j = js; j <= je; ++j) extrap_prim(p, q, nq, j, k, j, k1, j, k2, 1.0);
  }
  double t = (double)p.istep0 / 30.;
  if (t > 1. || p.iread > 0) t = 1.;
  double scal = (10. - 15. * t + 6. * t * t) * p3(t);
  double rscal = 1. - scal;
  for (k = ks; k <= ke; ++k)
    for (int j = js; j <= je; ++j) {
      double ajacinv = 1. / q(j, k, nq);
      q(j, k, 1) = q(j, k, 1) * scal + rscal * p.rinf * ajacinv;
      q(j, k, 2) = q(j, k, 2) * scal + rscal * p.rinf * p.uinf * ajacinv;
      q(j, k, 3) = q(j, k, 3) * scal + rscal * p.rinf * p.vinf * ajacinv;
      q(j, k, 4) = q(j, k, 4) * scal + rscal * p.einf * ajacinv;
    }
}

/* bc.f:1962-2026 */
static void bcextp(const P& p, A3 q, int js, int je, int ks, int ke, int idir) {
  const int nq = p.nq; const double foso = 0.0;
  int iadd = isign(1, idir), iadir = std::abs(idir);
  if (iadir == 1) {
    for (int jc = 1; jc <= je - js + 1; ++jc) {
      int j = (idir == 1) ? je - jc + 1 : js + jc - 1;
      int j1 = j + iadd, j2 = j1 + iadd;
      for (int k = ks; k <= ke; ++k) {
        double s1 = q(j1, k, nq) / q(j, k, nq), s2 = q(j2, k, nq) / q(j, k, nq);
        for (int n = 1; n <= 4; ++n) q(j, k, n) = (1. + foso) * q(j1, k, n) * s1 - foso * q(j2, k, n) * s2;
      }
    }
  } else if (iadir == 2) {
    for (int kc = 1; kc <= ke - ks + 1; ++kc) {
      int k = (idir == 2) ? ke - kc + 1 : ks + kc - 1;
      int k1 = k + iadd, k2 = k1 + iadd;
      for (int j = js; j <= je; ++j) {
        double s1 = q(j, k1, nq) / q(j, k, nq), s2 = q(j, k2, nq) / q(j, k, nq);
        for (int n = 1; n <= 4; ++n) q(j, k, n) = (1. + foso) * q(j, k1, n) * s1 - foso * q(j, k2, n) * s2;
      }
    }
  }
}

/* bc.f:2096-2157 */
static void bcsym(const P& p, A3 q, int js, int je, int ks, int ke, int idir) {
  const int nq = p.nq; int iadir = std::abs(idir);
  if (iadir == 1) {
    for (int jc = 1; jc <= je - js + 1; ++jc) {
      int j, j1;
      if (idir == 1) { j = je - jc + 1; j1 = je + jc; } else { j = js + jc - 1; j1 = js - jc; }
      for (int k = ks; k <= ke; ++k) {
        double sc = q(j1, k, nq) / q(j, k, nq);
        q(j, k, 1) = q(j1, k, 1) * sc; q(j, k, 2) = -q(j1, k, 2) * sc;
        q(j, k, 3) = q(j1, k, 3) * sc; q(j, k, 4) = q(j1, k, 4) * sc;
      }
    }
  } else if (iadir == 2) {
    for (int kc = 1; kc <= ke - ks + 1; ++kc) {
      int k, k1;
      if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
      for (int j = js; j <= je; ++j) {
        double sc = q(j, k1, nq) / q(j, k, nq);
        q(j, k, 1) = q(j, k1, 1) * sc; q(j, k, 2) = q(j, k1, 2) * sc;
        q(j, k, 3) = -q(j, k1, 3) * sc; q(j, k, 4) = q(j, k1, 4) * sc;
      }
    }
  }
}

/* bc.f:180-262 (q) / bc.f:265-357 (s): periodic copy from the overlap */
static void periodic_copy(const P& p, A3 q, A3 dst, int js, int je, int ks, int ke, int idir) {
  const int jd = p.jd, kd = p.kd, nq = p.nq;
  if (idir == 1 || idir == -1) {
    int jj = je - js + 1;
    for (int j = js; j <= je; ++j) {
      int jc = (idir == 1) ? jd - 2 * jj + (j - js + 1) : 1 + 2 * jj - (je - j + 1);
      for (int k = ks; k <= ke; ++k) {
        double sc = q(jc, k, nq) / q(j, k, nq);
        for (int n = 1; n <= 4; ++n) dst(j, k, n) = dst(jc, k, n) * sc;
      }
    }
  } else if (idir == 2 || idir == -2) {
    int kk = ke - ks + 1;
    for (int k = ks; k <= ke; ++k) {
      int kc = (idir == 2) ? kd - 2 * kk + (k - ks + 1) : 1 + 2 * kk - (ke - k + 1);
      for (int j = js; j <= je; ++j) {
        double sc = q(j, kc, nq) / q(j, k, nq);
        for (int n = 1; n <= 4; ++n) dst(j, k, n) = dst(j, kc, n) * sc;
      }
    }
  }
}

/* bc.f:1516-1573 (q) / bc.f:1576-1633 (s): wake-cut averaging */
static void wake_copy(const P& p, A3 q, A3 dst, int js, int je, int ks, int ke, int idir) {
  const int jd = p.jd, nq = p.nq;
  if (std::abs(idir) != 2) return;
  for (int kc = 1; kc <= ke - ks + 1; ++kc) {
    int k, k1;
    if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
    for (int j = js; j <= je; ++j) {
      int jj = jd - j + 1;
      double scale1 = q(jj, k1, nq) / q(j, k, nq);
      double scale2 = q(j, k1, nq) / q(jj, k, nq);
      for (int n = 1; n <= 4; ++n) dst(j, k, n) = dst(jj, k1, n) * scale1;
      for (int n = 1; n <= 4; ++n) dst(jj, k, n) = dst(j, k1, n) * scale2;
    }
  }
}

/* bc.f:360-407 */
static void bcout_inf(const P& p, A3 q, int js, int je, int ks, int ke, int idir) {
  const int nq = p.nq; int iadir = std::abs(idir);
  if (iadir != 1 && iadir != 2) return;
  for (int k = ks; k <= ke; ++k)
    for (int j = js; j <= je; ++j) {
      double rj = 1. / q(j, k, nq);
      q(j, k, 1) = p.rinf * rj;
      q(j, k, 2) = p.rinf * p.uinf * rj;
      q(j, k, 3) = p.rinf * p.vinf * rj;
      q(j, k, 4) = p.pinf / p.gm1 * rj + 0.5 * (p2(q(j, k, 2)) + p2(q(j, k, 3))) / q(j, k, 1);
    }
}

/* bc.f:694-983: characteristic far field in Turkel form (bt = 1, Mp = 1) */
static void bcout_trkl(const P& p, A3 q, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 bt,
                       int js, int je, int ks, int ke, int idir) {
  const int nq = p.nq; const double gm1 = p.gm1, ggm1 = p.ggm1, gamma = p.gamma, Mp = p.Mp;
  int iadd = isign(1, idir), iadir = std::abs(idir);
  /* one boundary cell (jb,kb) with interior neighbours at offset (dj,dk)*1, *2 */
  auto cell = [&](int j, int k, int j1, int k1, int j2, int k2, double mx, double my, double ugc, double vgc, double btc) {
    double foso = 1.0;
    double snorm = -1. * iadd / std::sqrt(p2(mx) + p2(my));
    double xxn = mx * snorm, xyn = my * snorm;
    double qext[4], qbar[4], delq[4], delw[4];
    for (int n = 1; n <= 4; ++n)
      qext[n - 1] = (1. + foso) * q(j1, k1, n) * q(j1, k1, nq) - foso * q(j2, k2, n) * q(j2, k2, nq);
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
    double cjkl = std::sqrt(ggm1 * (e - uv2));
    double c2i = 1. / (cjkl * cjkl);
    double ge = gamma * e - gm1 * uv2;
    double qq = (uu - ugc) * xxn + (vv - vgc) * xyn;
    double bSq = p2(Mp) / (btc - p2(Mp) * (btc - 1));
    double Z = std::sqrt((1. - bSq) * qq * (1. - bSq) * qq + 4. * bSq * cjkl * cjkl);
    double Zi = 1. / Z;
    double R = 0.5 * ((1. - bSq) * qq + Z);
    double S = 0.5 * ((1. - bSq) * qq - Z);
    double sq = fsign(1., qq), sR = fsign(1., R + bSq * qq), sR2 = fsign(1., R + qq * bSq);
    double sS = fsign(1., S + bSq * qq), sS2 = fsign(1., S + qq * bSq);
    delw[0] = (1. - uv2 * gm1 * c2i) * sq * delq[0];
    delw[0] = delw[0] + uu * c2i * gm1 * sq * delq[1];
    delw[0] = delw[0] + vv * c2i * gm1 * sq * delq[2];
    delw[0] = delw[0] - gm1 * c2i * sq * delq[3];
    delw[1] = (vv * xxn - uu * xyn) * sq * delq[0];
    delw[1] = delw[1] + xyn * sq * delq[1];
    delw[1] = delw[1] - xxn * sq * delq[2];
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
    for (int n = 1; n <= 4; ++n) q(j, k, n) = (qbar[n - 1] - delq[n - 1]) / q(j, k, nq);
  };
  if (iadir == 1) {
    int j = (idir == 1) ? je : js;
    int j1 = j + iadd, j2 = j1 + iadd;
    for (int k = ks; k <= ke; ++k) cell(j, k, j1, k, j2, k, xx(j, k), xy(j, k), ug(j, k), vg(j, k), bt(j, k));
    for (int jc = 1; jc <= je - js; ++jc) {
      j = (idir == 1) ? je - jc : js + jc;
      j1 = j + iadd; j2 = j1 + iadd;
      for (int k = ks; k <= ke; ++k) extrap_prim(p, q, nq, j, k, j1, k, j2, k, 0.0);
    }
  } else if (iadir == 2) {
    int k = (idir == 2) ? ke : ks;
    int k1 = k + iadd, k2 = k1 + iadd;
    for (int j = js; j <= je; ++j) cell(j, k, j, k1, j, k2, yx(j, k), yy(j, k), ug(j, k), vg(j, k), bt(j, k));
    for (int kc = 1; kc <= ke - ks; ++kc) {
      k = (idir == 2) ? ke - kc : ks + kc;
      k1 = k + iadd; k2 = k1 + iadd;
      for (int j = js; j <= je; ++j) extrap_prim(p, q, nq, j, k, j, k1, j, k2, 0.0);
    }
  }
}

/* bc.f:2-85 */
void bc(const P& p, A3 q, A2 x, A2 y, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 bt) {
  (void)x; (void)y;
  for (int ib = 0; ib < p.nbc; ++ib) {
    int js, je, ks, ke; bc_range(p, ib, js, je, ks, ke);
    int idir = p.ibdir[ib], t = p.ibtyp[ib];
    if (t == 3) bcwall(p, q, xx, xy, yx, yy, ug, vg, js, je, ks, ke, idir, 1);
    else if (t == 4) bcwall(p, q, xx, xy, yx, yy, ug, vg, js, je, ks, ke, idir, 0);
    else if (t == 5) bcwall(p, q, xx, xy, yx, yy, ug, vg, js, je, ks, ke, idir, p.invisc);
    else if (t == 10) bcextp(p, q, js, je, ks, ke, idir);
    else if (t == 11) bcsym(p, q, js, je, ks, ke, idir);
    else if (t == 22) periodic_copy(p, q, q, js, je, ks, ke, idir);
    else if (t == 51) wake_copy(p, q, q, js, je, ks, ke, idir);
    else if (t == 46) bcout_inf(p, q, js, je, ks, ke, idir);
    else if (t == 47) bcout_trkl(p, q, xx, xy, yx, yy, ug, vg, bt, js, je, ks, ke, idir);
  }
}

/* bc.f:2029-2093 */
static void rbcextp(const P& p, A3 q, A3 s, int js, int je, int ks, int ke, int idir) {
  const int nq = p.nq; const double foso = 0.0;
  int iadd = isign(1, idir), iadir = std::abs(idir);
  if (iadir == 1) {
    for (int jc = 1; jc <= je - js + 1; ++jc) {
      int j = (idir == 1) ? je - jc + 1 : js + jc - 1;
      int j1 = j + iadd, j2 = j1 + iadd;
      for (int k = ks; k <= ke; ++k) {
        double s1 = q(j1, k, nq) / q(j, k, nq), s2 = q(j2, k, nq) / q(j, k, nq);
        for (int n = 1; n <= 4; ++n) s(j, k, n) = (1. + foso) * s(j1, k, n) * s1 - foso * s(j2, k, n) * s2;
      }
    }
  } else if (iadir == 2) {
    for (int kc = 1; kc <= ke - ks + 1; ++kc) {
      int k = (idir == 2) ? ke - kc + 1 : ks + kc - 1;
      int k1 = k + iadd, k2 = k1 + iadd;
      for (int j = js; j <= je; ++j) {
        double s1 = q(j, k1, nq) / q(j, k, nq), s2 = q(j, k2, nq) / q(j, k, nq);
        for (int n = 1; n <= 4; ++n) s(j, k, n) = (1. + foso) * s(j, k1, n) * s1 - foso * s(j, k2, n) * s2;
      }
    }
  }
}

/* bc.f:2160-2221 */
static void rbcsym(const P& p, A3 q, A3 s, int js, int je, int ks, int ke, int idir) {
  const int nq = p.nq; int iadir = std::abs(idir);
  if (iadir == 1) {
    for (int jc = 1; jc <= je - js + 1; ++jc) {
      int j, j1;
      if (idir == 1) { j = je - jc + 1; j1 = je + jc; } else { j = js + jc - 1; j1 = js - jc; }
      for (int k = ks; k <= ke; ++k) {
        double sc = q(j1, k, nq) / q(j, k, nq);
        s(j, k, 1) = s(j1, k, 1) * sc; s(j, k, 2) = -s(j1, k, 2) * sc;
        s(j, k, 3) = s(j1, k, 3) * sc; s(j, k, 4) = s(j1, k, 4) * sc;
      }
    }
  } else if (iadir == 2) {
    for (int kc = 1; kc <= ke - ks + 1; ++kc) {
      int k, k1;
      if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
      for (int j = js; j <= je; ++j) {
        double sc = q(j, k1, nq) / q(j, k, nq);
        s(j, k, 1) = s(j, k1, 1) * sc; s(j, k, 2) = s(j, k1, 2) * sc;
        s(j, k, 3) = -s(j, k1, 3) * sc; s(j, k, 4) = s(j, k1, 4) * sc;
      }
    }
  }
}

/* bc.f:88-177.  Types 3/4/5/46/47 hit zero_residuals first (bc.f:125-130),
 * so the rbcwall / rbcout_trkl branches below it are unreachable and are not
 * restated. */
void rbc(const P& p, A3 q, A3 s) {
  for (int ib = 0; ib < p.nbc; ++ib) {
    int js, je, ks, ke; bc_range(p, ib, js, je, ks, ke);
    int idir = p.ibdir[ib], t = p.ibtyp[ib];
    if (t == 3 || t == 4 || t == 5 || t == 46 || t == 47) {
      for (int j = js; j <= je; ++j) for (int k = ks; k <= ke; ++k) for (int n = 1; n <= 4; ++n) s(j, k, n) = 0.0;
    } else if (t == 10) rbcextp(p, q, s, js, je, ks, ke, idir);
    else if (t == 11) rbcsym(p, q, s, js, je, ks, ke, idir);
    else if (t == 22) periodic_copy(p, q, s, js, je, ks, ke, idir);
    else if (t == 51) wake_copy(p, q, s, js, je, ks, ke, idir);
  }
}

}  // namespace oro
