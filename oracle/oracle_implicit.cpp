/*
 * oracle_implicit.cpp -- TEST INFRASTRUCTURE ONLY (see oracle_common.h).
 * FP64 restatement of the local time step (src/time.f), the LU-SGS
 * hyperplane operator ilu2d (src/lhs.f:470-814) and the diagonalised ADI
 * operator arc2d with its pentadiagonal line inversions (src/lhs.f:817-1057,
 * lhsinv :1536-1816, pentadag :1819-1873; ilhs = 2).
 */
#include <cstdio>
#include <cstdlib>
#include "oracle.h"

namespace oro {

/* time.f:2-108, one time instance (the reference loops nsp outside) */
void time_step(const P& pin, A3 q, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 tscale, A2 bt, I2 iblank) {
  // time.f:30-35: time-accurate preconditioning switches to dual time
  P p = pin;
  if (p.iprecon && (p.timeac == 1 && !p.timespectral)) { p.idual = 1; p.idual_turb = 1; }
  const int jd = p.jd, kd = p.kd, nq = p.nq;
  double oat = 1.0;
  if (p.ntac >= 2 && p.istep > 1) oat = 2. / 3.;
  if (p.ntac == 3 && p.istep > 2) oat = 6. / 11.;
  double jac_factor = p.invisc ? 0.01 : 0.002;
  const double h = p.h, timeac = p.timeac;
  if (p.iconstant_cfl == 0) {
    if (p.idual == 0) {
      for (int k = 1; k <= kd; ++k) for (int j = 1; j <= jd; ++j) {
        double ib = (double)(iblank(j, k) > 0 ? iblank(j, k) : 0);
        tscale(j, k) = oat * h * ib * (1.0 + jac_factor * (1. - timeac) * std::sqrt(q(j, k, nq))) /
                       (1.0 + (1. - timeac) * std::sqrt(q(j, k, nq)));
        bt(j, k) = 1.;
      }
    } else {
      for (int k = 1; k <= kd; ++k) for (int j = 1; j <= jd; ++j) {
        double ib = (double)(iblank(j, k) > 0 ? iblank(j, k) : 0);
        tscale(j, k) = ib * (1.0 + jac_factor * std::sqrt(q(j, k, nq))) / (1.0 + std::sqrt(q(j, k, nq)));
        if (p.iprecon)   // time.f:62-66
          tscale(j, k) = 100. * ib * (1.0 + 0.005 * std::sqrt(q(j, k, nq))) / (1.0 + std::sqrt(q(j, k, nq)));
        tscale(j, k) = tscale(j, k) * p.dualtime;
        bt(j, k) = 1. / (1. + tscale(j, k) / h / oat);
        tscale(j, k) = tscale(j, k) / (1. + tscale(j, k) / h / oat);
      }
    }
  } else {
    for (int k = 1; k <= kd; ++k) for (int j = 1; j <= jd; ++j) {
      double u = q(j, k, 2) / q(j, k, 1), v = q(j, k, 3) / q(j, k, 1), e = q(j, k, 4) / q(j, k, 1);
      double uu = (u - ug(j, k)) * xx(j, k) + (v - vg(j, k)) * xy(j, k);
      double vv = (u - ug(j, k)) * yx(j, k) + (v - vg(j, k)) * yy(j, k);
      double dxdx = p2(xx(j, k)) + p2(xy(j, k));
      double dydy = p2(yx(j, k)) + p2(yy(j, k));
      double asq = p.ggm1 * (e - 0.5 * (p2(u) + p2(v)));
      double lam_j = std::fabs(uu) + std::sqrt(asq * dxdx);
      double lam_k = std::fabs(vv) + std::sqrt(asq * dydy);
      double ib = (double)(iblank(j, k) > 0 ? iblank(j, k) : 0);
      if (p.idual == 0) {
        tscale(j, k) = h / (lam_j + lam_k);
        tscale(j, k) = tscale(j, k) * ib;
        bt(j, k) = 1.;
      } else {
        double hnew = p.dualtime / (lam_j + lam_k);
        tscale(j, k) = hnew * ib;
        tscale(j, k) = tscale(j, k) / (1. + tscale(j, k) / h / oat);
        bt(j, k) = 1. / (1. + tscale(j, k) / h / oat);
      }
    }
  }
}

/* lhs.f:470-814 */
void ilu2d(const P& p, A3 q, A3 s, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 turmu, A2 tscale) {
  const int jd = p.jd, kd = p.kd, nq = p.nq;
  const int js = p.jbeg, je = p.jend, ks = p.kbeg, ke = p.kend;
  const double gamma = p.gamma, gm1 = p.gm1, ggm1 = p.ggm1;
  size_t n2 = (size_t)jd * kd;
  std::vector<double> d_(n2), uv_(n2), vn_(n2), ge_(n2), qx_(n2), qy_(n2), cx_(n2), cy_(n2), st_(n2 * 4);
  A2 d{d_.data(), jd}, uv{uv_.data(), jd}, vn{vn_.data(), jd}, ge{ge_.data(), jd};
  A2 qx{qx_.data(), jd}, qy{qy_.data(), jd}, cx{cx_.data(), jd}, cy{cy_.data(), jd};
  A3 st{st_.data(), jd, n2};
  int mdim = (jd > kd ? jd : kd) + 2;
  std::vector<double> a_[5], b_[5];
  for (int n = 1; n <= 4; ++n) { a_[n].assign(mdim, 0.); b_[n].assign(mdim, 0.); }
  std::vector<int> ms(js + ks + je + ke + 2), me(js + ks + je + ke + 2);
  double eps2 = p.epse * 2., epsv = 1. + eps2;
  for (int m = js + ks; m <= je + ke; ++m) {
    ms[m] = (js > m - ke) ? js : m - ke;
    me[m] = (je < m - js) ? je : m - js;
  }
  for (int k = ks - 1; k <= ke + 1; ++k)
    for (int j = js - 1; j <= je + 1; ++j) {
      double dj = 1.0 / q(j, k, 1);
      q(j, k, 2) = q(j, k, 2) * dj;
      q(j, k, 3) = q(j, k, 3) * dj;
      q(j, k, 4) = q(j, k, 4) * dj;
      q(j, k, 1) = q(j, k, 1) * q(j, k, nq);
    }
  for (int k = ks - 1; k <= ke + 1; ++k)
    for (int j = js - 1; j <= je + 1; ++j) {
      double uu = q(j, k, 2), vv = q(j, k, 3);
      double uv2 = 0.5 * (uu * uu + vv * vv);
      double cjkl = std::sqrt(ggm1 * (q(j, k, 4) - uv2));
      double rj1 = xx(j, k), rj2 = xy(j, k);
      double qq1 = rj1 * uu + rj2 * vv;
      double qqx = std::fabs(-rj1 * ug(j, k) - rj2 * vg(j, k) + qq1);
      double rr1 = std::sqrt(p2(rj1) + p2(rj2));
      double rk1 = yx(j, k), rk2 = yy(j, k);
      double qq2 = rk1 * uu + rk2 * vv;
      double qqy = std::fabs(-rk1 * ug(j, k) - rk2 * vg(j, k) + qq2);
      double rr2 = std::sqrt(p2(rk1) + p2(rk2));
      double vnu = 2.0 * rr2 * rr2 * (p.rmue + turmu(j, k)) / (p.rey * q(j, k, 1));
      double svt = tscale(j, k);
      d(j, k) = 1.0 / (1.0 + svt * ((qqx + qqy + cjkl * (rr1 + rr2)) * epsv + vnu));
      uv(j, k) = uv2; qx(j, k) = qq1; cx(j, k) = cjkl * rr1;
      qy(j, k) = qq2; cy(j, k) = cjkl * rr2; vn(j, k) = vnu;
      ge(j, k) = gamma * q(j, k, 4) - gm1 * uv2;
    }
  for (int k = ks; k <= ke; ++k) for (int n = 1; n <= 4; ++n) s(js - 1, k, n) = s(js - 1, k, n) * d(js - 1, k);
  for (int k = ks; k <= ke; ++k) for (int n = 1; n <= 4; ++n) s(je + 1, k, n) = s(je + 1, k, n) * d(je + 1, k);
  for (int j = js; j <= je; ++j) for (int n = 1; n <= 4; ++n) s(j, ks - 1, n) = s(j, ks - 1, n) * d(j, ks - 1);
  for (int j = js; j <= je; ++j) for (int n = 1; n <= 4; ++n) s(j, ke + 1, n) = s(j, ke + 1, n) * d(j, ke + 1);
  for (int k = ks - 1; k <= ke + 1; ++k)
    for (int j = js - 1; j <= je + 1; ++j)
      for (int n = 1; n <= 4; ++n) st(j, k, n) = s(j, k, n);
  if (p.iunst == 2) { std::fprintf(stderr, "oracle: ilu2d iunst=2 not restated\n"); std::abort(); }
  /* forward sweep */
  for (int m = js + ks; m <= je + ke; ++m) {
    for (int j = ms[m]; j <= me[m]; ++j) {
      int k = m - j, j1 = j - 1;
      double uu = q(j1, k, 2), vv = q(j1, k, 3), uv2 = uv(j1, k);
      double ri1 = xx(j1, k), ri2 = xy(j1, k), qq = qx(j1, k), cc = cx(j1, k);
      double qqx = -ri1 * ug(j1, k) - ri2 * vg(j1, k) + qq;
      double sp1 = std::fabs(qqx) + cc, sm2 = eps2 * sp1;
      double chkx = 0.5 + fsign(0.5, qqx + cc);
      double spec = chkx * (qqx + sp1) + sm2;
      double s1 = s(j1, k, 1), s2 = s(j1, k, 2), s3 = s(j1, k, 3), s4 = s(j1, k, 4);
      double a4 = chkx * (ri1 * s2 + ri2 * s3 - qq * s1);
      double a2 = chkx * gm1 * (uv2 * s1 - (uu * s2 + vv * s3) + s4);
      a_[1][j] = a4 + spec * s1;
      a_[2][j] = ri1 * a2 + uu * a4 + spec * s2;
      a_[3][j] = ri2 * a2 + vv * a4 + spec * s3;
      a_[4][j] = qq * a2 + ge(j1, k) * a4 + spec * s4;
    }
    for (int j = ms[m]; j <= me[m]; ++j) {
      int k = m - j, k1 = k - 1;
      double uu = q(j, k1, 2), vv = q(j, k1, 3), uv2 = uv(j, k1);
      double ri1 = yx(j, k1), ri2 = yy(j, k1), qq = qy(j, k1), cc = cy(j, k1), vnu = vn(j, k1);
      double qqy = -ri1 * ug(j, k1) - ri2 * vg(j, k1) + qq;
      double sp1 = std::fabs(qqy) + cc, sm2 = eps2 * sp1;
      double chky = 0.5 + fsign(0.5, qqy + cc);
      double spec = chky * (qqy + sp1) + vnu + sm2;
      double s1 = s(j, k1, 1), s2 = s(j, k1, 2), s3 = s(j, k1, 3), s4 = s(j, k1, 4);
      double a4 = chky * (ri1 * s2 + ri2 * s3 - qq * s1);
      double a2 = chky * gm1 * (uv2 * s1 - (uu * s2 + vv * s3) + s4);
      b_[1][j] = a4 + spec * s1;
      b_[2][j] = ri1 * a2 + uu * a4 + spec * s2;
      b_[3][j] = ri2 * a2 + vv * a4 + spec * s3;
      b_[4][j] = qq * a2 + ge(j, k1) * a4 + spec * s4;
    }
    for (int j = ms[m]; j <= me[m]; ++j) {
      int k = m - j;
      double svt = tscale(j, k), sv = svt * 0.5, di = d(j, k);
      for (int n = 1; n <= 4; ++n) s(j, k, n) = (st(j, k, n) + sv * (a_[n][j] + b_[n][j])) * di;
    }
  }
  /* backward sweep */
  for (int m = je + ke; m >= js + ks; --m) {
    for (int j = ms[m]; j <= me[m]; ++j) {
      int k = m - j, j1 = j + 1;
      double uu = q(j1, k, 2), vv = q(j1, k, 3), uv2 = uv(j1, k);
      double ri1 = xx(j1, k), ri2 = xy(j1, k), qq = qx(j1, k), cc = cx(j1, k);
      double qqx = -ri1 * ug(j1, k) - ri2 * vg(j1, k) + qq;
      double sp1 = std::fabs(qqx) + cc, sm2 = eps2 * sp1;
      double chkx = 0.5 - fsign(0.5, qqx - cc);
      double spec = chkx * (qqx - sp1) - sm2;
      double s1 = s(j1, k, 1), s2 = s(j1, k, 2), s3 = s(j1, k, 3), s4 = s(j1, k, 4);
      double a4 = chkx * (ri1 * s2 + ri2 * s3 - qq * s1);
      double a2 = chkx * gm1 * (uv2 * s1 - (uu * s2 + vv * s3) + s4);
      a_[1][j] = a4 + spec * s1;
      a_[2][j] = ri1 * a2 + uu * a4 + spec * s2;
      a_[3][j] = ri2 * a2 + vv * a4 + spec * s3;
      a_[4][j] = qq * a2 + ge(j1, k) * a4 + spec * s4;
    }
    for (int j = ms[m]; j <= me[m]; ++j) {
      int k = m - j, k1 = k + 1;
      double uu = q(j, k1, 2), vv = q(j, k1, 3), uv2 = uv(j, k1);
      double ri1 = yx(j, k1), ri2 = yy(j, k1), qq = qy(j, k1), cc = cy(j, k1), vnu = vn(j, k1);
      double qqy = -ri1 * ug(j, k1) - ri2 * vg(j, k1) + qq;
      double sp1 = std::fabs(qqy) + cc, sm2 = eps2 * sp1;
      double chky = 0.5 - fsign(0.5, qqy - cc);
      double spec = chky * (qqy - sp1) - vnu - sm2;
      double s1 = s(j, k1, 1), s2 = s(j, k1, 2), s3 = s(j, k1, 3), s4 = s(j, k1, 4);
      double a4 = chky * (ri1 * s2 + ri2 * s3 - qq * s1);
      double a2 = chky * gm1 * (uv2 * s1 - (uu * s2 + vv * s3) + s4);
      b_[1][j] = a4 + spec * s1;
      b_[2][j] = ri1 * a2 + uu * a4 + spec * s2;
      b_[3][j] = ri2 * a2 + vv * a4 + spec * s3;
      b_[4][j] = qq * a2 + ge(j, k1) * a4 + spec * s4;
    }
    for (int j = ms[m]; j <= me[m]; ++j) {
      int k = m - j;
      double svt = tscale(j, k), sv = svt * 0.5, di = d(j, k);
      for (int n = 1; n <= 4; ++n) s(j, k, n) = s(j, k, n) - sv * (a_[n][j] + b_[n][j]) * di;
    }
  }
  for (int k = ks - 1; k <= ke + 1; ++k)
    for (int j = js - 1; j <= je + 1; ++j) {
      q(j, k, 1) = q(j, k, 1) / q(j, k, nq);
      q(j, k, 2) = q(j, k, 2) * q(j, k, 1);
      q(j, k, 3) = q(j, k, 3) * q(j, k, 1);
      q(j, k, 4) = q(j, k, 4) * q(j, k, 1);
    }
}

/* lhs.f:2-467 (preilu2d): ilu2d with Turkel's low-Mach preconditioner --
 * the preconditioned spectral radii in the diagonal and in the chk / spec
 * split, and every neighbour contribution multiplied by the preconditioner
 * (the same transform as rhslom) before its spec term */
void preilu2d(const P& p, A3 q, A3 s, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 turmu, A2 tscale, A2 bt) {
  const int jd = p.jd, kd = p.kd, nq = p.nq;
  const int js = p.jbeg, je = p.jend, ks = p.kbeg, ke = p.kend;
  const double gamma = p.gamma, gm1 = p.gm1, ggm1 = p.ggm1, Mp2 = p.Mp * p.Mp;
  size_t n2 = (size_t)jd * kd;
  std::vector<double> d_(n2), uv_(n2), vn_(n2), ge_(n2), qx_(n2), qy_(n2), cx_(n2), cy_(n2), st_(n2 * 4);
  A2 d{d_.data(), jd}, uv{uv_.data(), jd}, vn{vn_.data(), jd}, ge{ge_.data(), jd};
  A2 qx{qx_.data(), jd}, qy{qy_.data(), jd}, cx{cx_.data(), jd}, cy{cy_.data(), jd};
  A3 st{st_.data(), jd, n2};
  int mdim = (jd > kd ? jd : kd) + 2;
  std::vector<double> a_[5], b_[5];
  for (int n = 1; n <= 4; ++n) { a_[n].assign(mdim, 0.); b_[n].assign(mdim, 0.); }
  std::vector<int> ms(js + ks + je + ke + 2), me(js + ks + je + ke + 2);
  double eps2 = p.epse * 2., epsv = 1. + eps2;
  for (int m = js + ks; m <= je + ke; ++m) {
    ms[m] = (js > m - ke) ? js : m - ke;
    me[m] = (je < m - js) ? je : m - js;
  }
  auto bsq = [&](int j, int k) { return Mp2 / (bt(j, k) - Mp2 * (bt(j, k) - 1)); };
  for (int k = ks - 1; k <= ke + 1; ++k)
    for (int j = js - 1; j <= je + 1; ++j) {
      double dj = 1.0 / q(j, k, 1);
      q(j, k, 2) = q(j, k, 2) * dj;
      q(j, k, 3) = q(j, k, 3) * dj;
      q(j, k, 4) = q(j, k, 4) * dj;
      q(j, k, 1) = q(j, k, 1) * q(j, k, nq);
    }
  for (int k = ks - 1; k <= ke + 1; ++k)
    for (int j = js - 1; j <= je + 1; ++j) {
      double uu = q(j, k, 2), vv = q(j, k, 3);
      double uv2 = 0.5 * (uu * uu + vv * vv);
      double cjkl = std::sqrt(ggm1 * (q(j, k, 4) - uv2));
      double rj1 = xx(j, k), rj2 = xy(j, k);
      double qq1 = rj1 * uu + rj2 * vv;
      double qqx = std::fabs(-rj1 * ug(j, k) - rj2 * vg(j, k) + qq1);
      double rr1 = std::sqrt(p2(rj1) + p2(rj2));
      double rk1 = yx(j, k), rk2 = yy(j, k);
      double qq2 = rk1 * uu + rk2 * vv;
      double qqy = std::fabs(-rk1 * ug(j, k) - rk2 * vg(j, k) + qq2);
      double rr2 = std::sqrt(p2(rk1) + p2(rk2));
      double vnu = 2.0 * rr2 * rr2 * (p.rmue + turmu(j, k)) / (p.rey * q(j, k, 1));
      double svt = tscale(j, k);
      ge(j, k) = gamma * q(j, k, 4) - gm1 * uv2;
      uv(j, k) = uv2; qx(j, k) = qq1; cx(j, k) = cjkl * rr1;
      qy(j, k) = qq2; cy(j, k) = cjkl * rr2; vn(j, k) = vnu;
      double bSq = bsq(j, k);
      double X = std::sqrt(((1. - bSq) * qqx) * ((1. - bSq) * qqx) + ((4. * bSq) * cx(j, k)) * cx(j, k));
      double term = 0.5 * ((bSq + 1.) * qqx + X);
      double Y = std::sqrt(((1. - bSq) * qqy) * ((1. - bSq) * qqy) + ((4. * bSq) * cy(j, k)) * cy(j, k));
      term = term + 0.5 * ((bSq + 1.) * qqy + Y);
      d(j, k) = 1.0 / (1.0 + svt * (term * epsv + vnu));
    }
  for (int k = ks; k <= ke; ++k) for (int n = 1; n <= 4; ++n) s(js - 1, k, n) = s(js - 1, k, n) * d(js - 1, k);
  for (int k = ks; k <= ke; ++k) for (int n = 1; n <= 4; ++n) s(je + 1, k, n) = s(je + 1, k, n) * d(je + 1, k);
  for (int j = js; j <= je; ++j) for (int n = 1; n <= 4; ++n) s(j, ks - 1, n) = s(j, ks - 1, n) * d(j, ks - 1);
  for (int j = js; j <= je; ++j) for (int n = 1; n <= 4; ++n) s(j, ke + 1, n) = s(j, ke + 1, n) * d(j, ke + 1);
  for (int k = ks - 1; k <= ke + 1; ++k)
    for (int j = js - 1; j <= je + 1; ++j)
      for (int n = 1; n <= 4; ++n) st(j, k, n) = s(j, k, n);
  if (p.iunst == 2) { std::fprintf(stderr, "oracle: preilu2d iunst=2 not restated\n"); std::abort(); }
  // one neighbour's contribution (lhs.f:178-208): convective split, the
  // preconditioner, then +/- spec * s
  auto contrib = [&](int jn, int kn, double ri1, double ri2, double qq, double cc, const double* vnu, bool fwd,
                     double* out) {
    double uu = q(jn, kn, 2), vv = q(jn, kn, 3), uv2 = uv(jn, kn);
    double qqn = -ri1 * ug(jn, kn) - ri2 * vg(jn, kn) + qq;
    double bSq = bsq(jn, kn);
    double X = std::sqrt(((1. - bSq) * qqn) * ((1. - bSq) * qqn) + ((4. * bSq) * cc) * cc);
    double chk = fwd ? 0.5 + fsign(0.5, (bSq + 1.) * qqn + X) : 0.5 - fsign(0.5, (bSq + 1.) * qqn - X);
    double sp1 = 0.5 * ((bSq + 1.) * std::fabs(qqn) + X);
    double sm2 = eps2 * sp1;
    double spec = vnu ? chk * sp1 + *vnu + sm2 : chk * sp1 + sm2;
    double s1 = s(jn, kn, 1), s2 = s(jn, kn, 2), s3 = s(jn, kn, 3), s4 = s(jn, kn, 4);
    double a4 = chk * (ri1 * s2 + ri2 * s3 - qq * s1);
    double a2 = chk * gm1 * (uv2 * s1 - (uu * s2 + vv * s3) + s4);
    double t[5];
    t[1] = a4 + chk * qqn * s1;
    t[2] = ri1 * a2 + uu * a4 + chk * qqn * s2;
    t[3] = ri2 * a2 + vv * a4 + chk * qqn * s3;
    t[4] = qq * a2 + ge(jn, kn) * a4 + chk * qqn * s4;
    double r[5];
    r[1] = uv(jn, kn) * t[1] - uu * t[2] - vv * t[3] + t[4];
    r[2] = uu * r[1];
    r[3] = vv * r[1];
    r[4] = ge(jn, kn) * r[1];
    double cjkl = std::sqrt(ggm1 * (q(jn, kn, 4) - uv(jn, kn)));
    double term = gm1 * (bSq - 1.) / (cjkl * cjkl);
    for (int n = 1; n <= 4; ++n) {
      r[n] = r[n] * term;
      r[n] = r[n] + t[n];
    }
    double sv4[5] = {0, s1, s2, s3, s4};
    for (int n = 1; n <= 4; ++n) out[n] = fwd ? r[n] + spec * sv4[n] : r[n] - spec * sv4[n];
  };
  double c[5];
  /* forward sweep */
  for (int m = js + ks; m <= je + ke; ++m) {
    for (int j = ms[m]; j <= me[m]; ++j) {
      int k = m - j, j1 = j - 1;
      contrib(j1, k, xx(j1, k), xy(j1, k), qx(j1, k), cx(j1, k), nullptr, true, c);
      for (int n = 1; n <= 4; ++n) a_[n][j] = c[n];
    }
    for (int j = ms[m]; j <= me[m]; ++j) {
      int k = m - j, k1 = k - 1;
      contrib(j, k1, yx(j, k1), yy(j, k1), qy(j, k1), cy(j, k1), &vn(j, k1), true, c);
      for (int n = 1; n <= 4; ++n) b_[n][j] = c[n];
    }
    for (int j = ms[m]; j <= me[m]; ++j) {
      int k = m - j;
      double svt = tscale(j, k), sv = svt * 0.5, di = d(j, k);
      for (int n = 1; n <= 4; ++n) s(j, k, n) = (st(j, k, n) + sv * (a_[n][j] + b_[n][j])) * di;
    }
  }
  /* backward sweep */
  for (int m = je + ke; m >= js + ks; --m) {
    for (int j = ms[m]; j <= me[m]; ++j) {
      int k = m - j, j1 = j + 1;
      contrib(j1, k, xx(j1, k), xy(j1, k), qx(j1, k), cx(j1, k), nullptr, false, c);
      for (int n = 1; n <= 4; ++n) a_[n][j] = c[n];
    }
    for (int j = ms[m]; j <= me[m]; ++j) {
      int k = m - j, k1 = k + 1;
      contrib(j, k1, yx(j, k1), yy(j, k1), qy(j, k1), cy(j, k1), &vn(j, k1), false, c);
      for (int n = 1; n <= 4; ++n) b_[n][j] = c[n];
    }
    for (int j = ms[m]; j <= me[m]; ++j) {
      int k = m - j;
      double svt = tscale(j, k), sv = svt * 0.5, di = d(j, k);
      for (int n = 1; n <= 4; ++n) s(j, k, n) = s(j, k, n) - sv * (a_[n][j] + b_[n][j]) * di;
    }
  }
  for (int k = ks - 1; k <= ke + 1; ++k)
    for (int j = js - 1; j <= je + 1; ++j) {
      q(j, k, 1) = q(j, k, 1) / q(j, k, nq);
      q(j, k, 2) = q(j, k, 2) * q(j, k, 1);
      q(j, k, 3) = q(j, k, 3) * q(j, k, 1);
      q(j, k, 4) = q(j, k, 4) * q(j, k, 1);
    }
}

/* sources.f:97-148 (rhslom): the residual multiplied by the low-Mach
 * preconditioner on the interior */
void rhslom(const P& p, A3 q, A3 s, A2 bt) {
  const double gamma = p.gamma, gm1 = p.gm1, Mp2 = p.Mp * p.Mp;
  for (int j = p.jbeg; j <= p.jend; ++j)
    for (int k = p.kbeg; k <= p.kend; ++k) {
      double u = q(j, k, 2) / q(j, k, 1);
      double v = q(j, k, 3) / q(j, k, 1);
      double phiSq = 0.5 * (u * u + v * v);
      double ge = q(j, k, 4) / q(j, k, 1) * gamma - phiSq * gm1;
      double aSq = (q(j, k, 4) / q(j, k, 1) - phiSq) * gm1 * gamma;
      double tmp[5] = {0, s(j, k, 1), s(j, k, 2), s(j, k, 3), s(j, k, 4)};
      s(j, k, 1) = phiSq * tmp[1] - u * tmp[2] - v * tmp[3] + tmp[4];
      s(j, k, 2) = u * s(j, k, 1);
      s(j, k, 3) = v * s(j, k, 1);
      s(j, k, 4) = ge * s(j, k, 1);
      double bSq = Mp2 / (bt(j, k) - Mp2 * (bt(j, k) - 1));
      for (int n = 1; n <= 4; ++n) {
        s(j, k, n) = s(j, k, n) * (gm1 * (bSq - 1.) / aSq);
        s(j, k, n) = s(j, k, n) + tmp[n];
      }
    }
}

/* lhs.f:1819-1873 (1-based a..f of length N) */
static void pentadag(double* a, double* b, double* c, double* d, double* e, double* f, int N) {
  auto A = [&](int i) -> double& { return a[i - 1]; };
  auto B = [&](int i) -> double& { return b[i - 1]; };
  auto Cc = [&](int i) -> double& { return c[i - 1]; };
  auto D = [&](int i) -> double& { return d[i - 1]; };
  auto E = [&](int i) -> double& { return e[i - 1]; };
  auto F = [&](int i) -> double& { return f[i - 1]; };
  int i = 1;
  double d0 = 1.0 / Cc(i);
  D(i + 1) = D(i + 1) * d0;
  E(i + 2) = E(i + 2) * d0;
  F(i) = F(i) * d0;
  i = 2;
  double d1 = B(i - 1);
  d0 = 1.0 / (Cc(i) - d1 * D(i));
  F(i) = (F(i) - d1 * F(i - 1)) * d0;
  D(i + 1) = (D(i + 1) - d1 * E(i + 1)) * d0;
  E(i + 2) = E(i + 2) * d0;
  for (i = 3; i <= N; ++i) {
    d1 = A(i - 2);
    double d2 = (B(i - 1) - A(i - 2) * D(i - 1));
    d0 = 1. / (Cc(i) - d2 * D(i) - d1 * E(i));
    F(i) = (F(i) - d2 * F(i - 1) - d1 * F(i - 2)) * d0;
    if (i <= N - 1) {
      D(i + 1) = (D(i + 1) - d2 * E(i + 1)) * d0;
      if (i <= N - 2) E(i + 2) = (E(i + 2)) * d0;
    }
  }
  i = N - 1;
  d1 = D(i + 1);
  F(i) = F(i) - d1 * F(i + 1);
  for (i = N - 2; i >= 1; --i) {
    d1 = D(i + 1);
    double d2 = E(i + 2);
    F(i) = F(i) - d1 * F(i + 1) - d2 * F(i + 2);
  }
}

/* lhs.f:1536-1816: pentadiagonal inversion along direction idir (1: j
 * lines, m = j, n = k; 2: k lines, m = k, n = j) over m = ms..me, n = ns..ne */
static void lhsinv(const P& p, A3 q, A3 s, A2 qn, A2 cn, A2 d2p, int ms, int me, int ns, int ne, int idir, A2 xn,
                   A2 yn, A2 vnu, I2 iblank, A2 tscale, A2 bt) {
  const int nq = p.nq, nmv = p.nmv;
  const size_t L = (size_t)me + 3;
  std::vector<double> jcbn(L), tscal(L), v1(L), v2(L), v3(L), g(L), atmp(L), btmp(L), ctmp(L), dtmp(L), etmp(L);
  std::vector<double> a(L), b(L), c(L), d(L), e(L), f(L), a1(L), b1(L), c1(L), d1(L), e1(L), f1(L);
  std::vector<double> diag(L * (nq + 1));
  auto DG = [&](int m, int i) -> double& { return diag[(size_t)m * (nq + 1) + i]; };
  const double dis2 = 10.0, dis4 = 0.1, Mp = p.Mp;
  auto Q = [&](int m, int n, int v) -> double& { return idir == 1 ? q(m, n, v) : q(n, m, v); };
  auto S = [&](int m, int n, int v) -> double& { return idir == 1 ? s(m, n, v) : s(n, m, v); };
  auto X2 = [&](A2 a2, int m, int n) -> double& { return idir == 1 ? a2(m, n) : a2(n, m); };
  auto IB = [&](int m, int n) { return idir == 1 ? iblank(m, n) : iblank(n, m); };
  for (int n = ns; n <= ne; ++n) {
    for (int m = ms; m <= me; ++m) {
      jcbn[m] = Q(m, n, nq);
      tscal[m] = X2(tscale, m, n);
      g[m] = X2(d2p, m, n);
      (void)IB(m, n);
      const double btv = X2(bt, m, n);
      const double bSq = (Mp * Mp) / (btv - (Mp * Mp) * (btv - 1));
      const double qv = X2(qn, m, n), cv = X2(cn, m, n);
      const double X = std::sqrt(((1. - bSq) * qv) * ((1. - bSq) * qv) + 4. * bSq * cv * cv);
      DG(m, 1) = qv;
      DG(m, 2) = qv;
      DG(m, 3) = 0.5 * ((bSq + 1.) * qv + X);
      DG(m, 4) = 0.5 * ((bSq + 1.) * qv - X);
      DG(m, nq) = 0.5 * ((bSq + 1.) * std::fabs(qv) + X) / Q(m, n, nq);
    }
    for (int m = ms + 1; m <= me - 1; ++m) {
      v1[m] = (X2(xn, m, n) * X2(xn, m, n) + X2(yn, m, n) * X2(yn, m, n)) / Q(m, n, nq);
      v1[m] = v1[m] + (X2(xn, m + 1, n) * X2(xn, m + 1, n) + X2(yn, m + 1, n) * X2(yn, m + 1, n)) / Q(m + 1, n, nq);
      v1[m] = v1[m] * Q(m, n, nq) * X2(vnu, m, n);
      v3[m] = (X2(xn, m, n) * X2(xn, m, n) + X2(yn, m, n) * X2(yn, m, n)) / Q(m, n, nq);
      v3[m] = v3[m] + (X2(xn, m - 1, n) * X2(xn, m - 1, n) + X2(yn, m - 1, n) * X2(yn, m - 1, n)) / Q(m - 1, n, nq);
      v3[m] = v3[m] * Q(m, n, nq) * X2(vnu, m, n);
      v2[m] = 0.5 * (v1[m] + v3[m]);
    }
    v1[ms] = v2[ms] = v3[ms] = 0;
    v1[me] = v2[me] = v3[me] = 0;
    auto dn = [&](int m) { return DG(m, nq); };
    for (int m = ms + 3; m <= me - 3; ++m) {
      const double c2 = 0.5 * ((g[m] + g[m + 1])) * dis2, c2m = 0.5 * ((g[m] + g[m - 1])) * dis2;
      const double c4p = (dis4 - fmin2(dis4, .5 * dis2 * (g[m + 2] + g[m + 1])));
      const double c4 = (dis4 - fmin2(dis4, 1. * c2)), c4m = (dis4 - fmin2(dis4, 1. * c2m));
      const double c4m2 = (dis4 - fmin2(dis4, .5 * dis2 * (g[m - 2] + g[m - 1])));
      atmp[m] = (dn(m + 1) + dn(m + 2)) * c4p;
      btmp[m] = -((dn(m + 2) + dn(m + 1)) * c4p + (dn(m + 1) + dn(m)) * (3. * c4 + c2));
      ctmp[m] = +((dn(m - 1) + dn(m)) * (3. * c4m + c2m) + (dn(m + 1) + dn(m)) * (3. * c4 + c2));
      dtmp[m] = -((dn(m - 2) + dn(m - 1)) * c4m2 + (dn(m) + dn(m - 1)) * (3. * c4m + c2m));
      etmp[m] = (dn(m - 1) + dn(m - 2)) * c4m2;
    }
    {
      const int m = ms + 2;
      const double c2 = 0.5 * ((g[m] + g[m + 1])) * dis2, c2m = 0.5 * ((g[m] + g[m - 1])) * dis2;
      const double c4p = (dis4 - fmin2(dis4, .5 * dis2 * (g[m + 2] + g[m + 1])));
      const double c4 = (dis4 - 1. * fmin2(dis4, c2)), c4m = (dis4 - fmin2(dis4, 1. * c2m));
      const double c4m2 = (dis4 - fmin2(dis4, 1. * dis2 * (g[m - 1])));
      atmp[m] = (dn(m + 1) + dn(m + 2)) * c4p;
      btmp[m] = -((dn(m + 2) + dn(m + 1)) * c4p + (dn(m + 1) + dn(m)) * (3. * c4 + c2));
      ctmp[m] = ((dn(m - 1) + dn(m)) * (3. * c4m + c2m) + (dn(m + 1) + dn(m)) * (3. * c4 + c2));
      dtmp[m] = -((2. * dn(m - 1)) * c4m2 + (dn(m) + dn(m - 1)) * (3. * c4m + c2m));
    }
    {
      const int m = ms + 1;
      const double c2 = 0.5 * ((g[m] + g[m + 1])) * dis2, c2m = ((g[m])) * dis2;
      const double c4p = (dis4 - fmin2(dis4, .5 * dis2 * (g[m + 2] + g[m + 1])));
      const double c4 = (dis4 - fmin2(dis4, 1. * c2)), c4m = (dis4 - fmin2(dis4, 1. * c2m));
      atmp[m] = (dn(m + 1) + dn(m + 2)) * c4p;
      btmp[m] = -((dn(m + 2) + dn(m + 1)) * c4p + (dn(m + 1) + dn(m)) * (3. * c4 + c2));
      ctmp[m] = (2. * (dn(m)) * (2. * c4m + c2m) + (dn(m + 1) + dn(m)) * (3. * c4 + c2));
    }
    {
      const int m = me - 2;
      const double c2 = 0.5 * ((g[m] + g[m + 1])) * dis2, c2m = 0.5 * ((g[m] + g[m - 1])) * dis2;
      const double c4p = (dis4 - fmin2(dis4, 1. * dis2 * (g[m + 1])));
      const double c4 = (dis4 - fmin2(dis4, 1. * c2)), c4m = (dis4 - fmin2(dis4, 1. * c2m));
      const double c4m2 = (dis4 - fmin2(dis4, .5 * dis2 * (g[m - 2] + g[m - 1])));
      btmp[m] = -(2. * (dn(m + 1)) * c4p + (dn(m + 1) + dn(m)) * (3. * c4 + c2));
      ctmp[m] = ((dn(m - 1) + dn(m)) * (3. * c4m + c2m) + (dn(m + 1) + dn(m)) * (2. * c4 + c2));
      dtmp[m] = -((dn(m - 2) + dn(m - 1)) * c4m2 + (dn(m) + dn(m - 1)) * (3. * c4m + c2m));
      etmp[m] = (dn(m - 1) + dn(m - 2)) * c4m2;
    }
    {
      const int m = me - 1;
      const double c2 = ((g[m])) * dis2, c2m = 0.5 * ((g[m] + g[m - 1])) * dis2;
      const double c4 = (dis4 - fmin2(dis4, 1. * c2)), c4m = (dis4 - fmin2(dis4, 1. * c2m));
      const double c4m2 = (dis4 - fmin2(dis4, .5 * dis2 * (g[m - 2] + g[m - 1])));
      ctmp[m] = +((dn(m - 1) + dn(m)) * (3. * c4m + c2m) + 2. * (dn(m)) * (2. * c4 + c2));
      dtmp[m] = -((dn(m - 2) + dn(m - 1)) * c4m2 + (dn(m) + dn(m - 1)) * (3. * c4m + c2m));
      etmp[m] = (dn(m - 1) + dn(m - 2)) * c4m2;
    }
    for (int m = ms; m <= me; ++m) {
      atmp[m] = atmp[m] * jcbn[m]; btmp[m] = btmp[m] * jcbn[m]; ctmp[m] = ctmp[m] * jcbn[m];
      dtmp[m] = dtmp[m] * jcbn[m]; etmp[m] = etmp[m] * jcbn[m];
    }
    for (int i = 1; i <= nmv; ++i) {
      for (int m = ms; m <= me; ++m) {
        a1[m] = atmp[m]; b1[m] = btmp[m]; c1[m] = ctmp[m]; d1[m] = dtmp[m]; e1[m] = etmp[m];
        f1[m] = S(m, n, i);
        b1[m] = b1[m] - DG(m, i) * 0.5;
        d1[m] = d1[m] + DG(m, i) * 0.5;
        b1[m] = b1[m] - 0.5 * v1[m];
        c1[m] = c1[m] + v2[m];
        d1[m] = d1[m] - 0.5 * v3[m];
        a1[m] = (m <= me - 2) ? a1[m] * tscal[m + 2] : a1[m] * tscal[m];
        b1[m] = (m <= me - 1) ? b1[m] * tscal[m + 1] : b1[m] * tscal[m];
        d1[m] = (m >= ms + 1) ? d1[m] * tscal[m - 1] : d1[m] * tscal[m];
        e1[m] = (m >= ms + 2) ? e1[m] * tscal[m - 2] : e1[m] * tscal[m];
        c1[m] = c1[m] * tscal[m] + 1.0;
      }
      for (int m = ms + 1; m <= me - 1; ++m) {
        a[m - ms] = a1[m]; b[m - ms] = b1[m]; c[m - ms] = c1[m];
        d[m - ms] = d1[m]; e[m - ms] = e1[m]; f[m - ms] = f1[m];
      }
      const int N = me - ms - 1;
      f[1] = f[1] - b1[ms] * f1[ms] / c1[ms];
      f[N] = f[N] - d1[me] * f1[me] / c1[me];
      d[1] = 0; e[1] = 0; e[2] = 0;
      b[N] = 0; a[N] = 0; a[N - 1] = 0;
      pentadag(&a[1], &b[1], &c[1], &d[1], &e[1], &f[1], N);
      for (int m = ms + 1; m <= me - 1; ++m) S(m, n, i) = f[m - ms];
    }
  }
}

/* lhs.f:1333-1533: the upwind-split line inversion of ilhs = 3 (a
 * tridiagonal system solved with pentadag) */
static void lhsinv_up(const P& p, A3 q, A3 s, A2 qn, A2 cn, int ms, int me, int ns, int ne, int idir, A2 xn, A2 yn,
                      A2 vnu, A2 tscale, A2 bt) {
  const int nq = p.nq, nmv = p.nmv;
  const size_t L = (size_t)me + 3;
  std::vector<double> tscal(L), v1(L), v2(L), v3(L);
  std::vector<double> a(L), b(L), c(L), d(L), e(L), f(L), a1(L), b1(L), c1(L), d1(L), e1(L), f1(L);
  std::vector<double> dp(L * 5), dm(L * 5);
  const double epsval = 0.05, fac = 1.05, Mp = p.Mp;
  auto Q = [&](int m, int n, int v) -> double& { return idir == 1 ? q(m, n, v) : q(n, m, v); };
  auto S = [&](int m, int n, int v) -> double& { return idir == 1 ? s(m, n, v) : s(n, m, v); };
  auto X2 = [&](A2 a2, int m, int n) -> double& { return idir == 1 ? a2(m, n) : a2(n, m); };
  for (int n = ns; n <= ne; ++n) {
    for (int m = ms; m <= me; ++m) {
      tscal[m] = X2(tscale, m, n);
      const double btv = X2(bt, m, n);
      const double bSq = (Mp * Mp) / (btv - (Mp * Mp) * (btv - 1));
      const double qv = X2(qn, m, n), cv = X2(cn, m, n);
      const double X = std::sqrt(((1. - bSq) * qv) * ((1. - bSq) * qv) + 4. * bSq * cv * cv);
      const double eig1 = qv, eig2 = 0.5 * ((bSq + 1.) * qv + X), eig3 = 0.5 * ((bSq + 1.) * qv - X);
      const double eps = epsval * std::sqrt(p2(X2(xn, m, n)) + p2(X2(yn, m, n)));
      const double eg[5] = {0, eig1, eig1, eig2, eig3};
      for (int i = 1; i <= 4; ++i) {
        dp[(size_t)m * 5 + i] = 0.5 * (eg[i] + fac * std::sqrt(p2(eg[i]) + p2(eps)));
        dm[(size_t)m * 5 + i] = 0.5 * (eg[i] - fac * std::sqrt(p2(eg[i]) + p2(eps)));
      }
    }
    for (int m = ms + 1; m <= me - 1; ++m) {
      v1[m] = (X2(xn, m, n) * X2(xn, m, n) + X2(yn, m, n) * X2(yn, m, n)) / Q(m, n, nq);
      v1[m] = v1[m] + (X2(xn, m + 1, n) * X2(xn, m + 1, n) + X2(yn, m + 1, n) * X2(yn, m + 1, n)) / Q(m + 1, n, nq);
      v1[m] = v1[m] * Q(m, n, nq) * X2(vnu, m, n);
      v3[m] = (X2(xn, m, n) * X2(xn, m, n) + X2(yn, m, n) * X2(yn, m, n)) / Q(m, n, nq);
      v3[m] = v3[m] + (X2(xn, m - 1, n) * X2(xn, m - 1, n) + X2(yn, m - 1, n) * X2(yn, m - 1, n)) / Q(m - 1, n, nq);
      v3[m] = v3[m] * Q(m, n, nq) * X2(vnu, m, n);
      v2[m] = 0.5 * (v1[m] + v3[m]);
    }
    v1[ms] = v2[ms] = v3[ms] = 0;
    v1[me] = v2[me] = v3[me] = 0;
    for (int i = 1; i <= nmv; ++i) {
      for (int m = ms; m <= me; ++m) {
        a1[m] = 0.; b1[m] = 0.; c1[m] = 0.; d1[m] = 0.; e1[m] = 0.;
        f1[m] = S(m, n, i);
        b1[m] = b1[m] - dp[(size_t)m * 5 + i];
        d1[m] = d1[m] + dm[(size_t)m * 5 + i];
        c1[m] = c1[m] + dp[(size_t)m * 5 + i] - dm[(size_t)m * 5 + i];
        b1[m] = b1[m] - 0.5 * v1[m];
        c1[m] = c1[m] + v2[m];
        d1[m] = d1[m] - 0.5 * v3[m];
        b1[m] = (m <= me - 1) ? b1[m] * tscal[m + 1] : b1[m] * tscal[m];
        d1[m] = (m >= ms + 1) ? d1[m] * tscal[m - 1] : d1[m] * tscal[m];
        c1[m] = c1[m] * tscal[m] + 1.0;
      }
      for (int m = ms + 1; m <= me - 1; ++m) {
        a[m - ms] = a1[m]; b[m - ms] = b1[m]; c[m - ms] = c1[m];
        d[m - ms] = d1[m]; e[m - ms] = e1[m]; f[m - ms] = f1[m];
      }
      const int N = me - ms - 1;
      f[1] = f[1] - b1[ms] * f1[ms] / c1[ms];
      f[N] = f[N] - d1[me] * f1[me] / c1[me];
      d[1] = 0; e[1] = 0; e[2] = 0;
      b[N] = 0; a[N] = 0; a[N - 1] = 0;
      pentadag(&a[1], &b[1], &c[1], &d[1], &e[1], &f[1], N);
      for (int m = ms + 1; m <= me - 1; ++m) S(m, n, i) = f[m - ms];
    }
  }
}

/* lhs.f:817-1057 (ilhs = 2, or 3 with lhsinv_up).  The tmp coefficient arrays of lhsinv at m = ms
 * and m = me are never assigned by the reference and are read as 0 here
 * (what a fresh allocation holds). */
/* lhs.f:817-1057 (arc2d); pre: lhs.f:1060-1330 (arc2d_precon), the same
 * ADI with Turkel's preconditioned eigenvectors in T_xi^-1, N^-1 and T_eta
 * (bSq = Mp**2/(bt - Mp**2 (bt-1)) per cell) and the contravariant
 * velocities taken relative to the grid before they are stored */
void arc2d(const P& p, A3 q, A3 s, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 turmu, I2 iblank, A2 tscale, A2 bt,
           bool pre) {
  const int jd = p.jd, kd = p.kd, nq = p.nq;
  const int js = p.jbeg, je = p.jend, ks = p.kbeg, ke = p.kend;
  const size_t n2 = (size_t)jd * kd;
  std::vector<double> buf(n2 * 11, 0.0);
  int slot = 0;
  auto mk = [&]() { return A2{buf.data() + n2 * (slot++), jd}; };
  A2 pr = mk(), d2px = mk(), d2py = mk(), uv = mk(), vn = mk(), ge = mk(), qx = mk(), qy = mk(), cx = mk(), cy = mk();
  const double gm1 = p.gm1, ggm1 = p.ggm1;
  /* :853-860 conservative -> primitive (rho, u, v, e) */
  for (int k = ks - 1; k <= ke + 1; ++k) for (int j = js - 1; j <= je + 1; ++j) {
    double dj = 1.0 / q(j, k, 1);
    q(j, k, 2) = q(j, k, 2) * dj;
    q(j, k, 3) = q(j, k, 3) * dj;
    q(j, k, 4) = q(j, k, 4) * dj;
    q(j, k, 1) = q(j, k, 1) * q(j, k, nq);
  }
  /* :863-917 multiply by T_xi inverse */
  for (int k = ks - 1; k <= ke + 1; ++k) for (int j = js - 1; j <= je + 1; ++j) {
    double uu = q(j, k, 2), vv = q(j, k, 3);
    double uv2 = 0.5 * (uu * uu + vv * vv);
    double cjkl = std::sqrt(ggm1 * (q(j, k, 4) - uv2));
    double c2i = 1.0 / (cjkl * cjkl);
    pr(j, k) = (q(j, k, 4) - uv2) * gm1 * q(j, k, 1);
    double rj1 = xx(j, k), rj2 = xy(j, k);
    double qq1;
    if (pre) {  /* :1116, :1134 */
      qq1 = rj1 * (uu - ug(j, k)) + rj2 * (vv - vg(j, k));
      qx(j, k) = qq1;
    } else {
      qq1 = rj1 * uu + rj2 * vv;
      qx(j, k) = qq1 - (rj1 * ug(j, k) + rj2 * vg(j, k));
    }
    double rr1 = std::sqrt(p2(rj1) + p2(rj2));
    rj1 = rj1 / rr1; rj2 = rj2 / rr1;
    double rk1 = yx(j, k), rk2 = yy(j, k);
    if (pre) {
      qy(j, k) = rk1 * (uu - ug(j, k)) + rk2 * (vv - vg(j, k));
    } else {
      double qq2 = rk1 * uu + rk2 * vv;
      qy(j, k) = qq2 - (rk1 * ug(j, k) + rk2 * vg(j, k));
    }
    double rr2 = std::sqrt(p2(rk1) + p2(rk2));
    rk1 = rk1 / rr2; rk2 = rk2 / rr2;
    double vnu = (p.rmue + turmu(j, k)) / (p.rey * q(j, k, 1));
    uv(j, k) = uv2;
    cx(j, k) = cjkl * rr1;
    cy(j, k) = cjkl * rr2;
    vn(j, k) = vnu;
    ge(j, k) = p.gamma * q(j, k, 4) - gm1 * uv2;
    double a1 = s(j, k, 2) * uu + s(j, k, 3) * vv - s(j, k, 4);
    a1 = a1 * gm1 * c2i;
    a1 = a1 + s(j, k, 1) * (1.0 - uv2 * gm1 * c2i);
    double a2 = (rj1 * vv - rj2 * uu) * s(j, k, 1) + rj2 * s(j, k, 2) - rj1 * s(j, k, 3);
    double a3 = uv2 * s(j, k, 1) - s(j, k, 2) * uu - s(j, k, 3) * vv + s(j, k, 4);
    a3 = a3 * gm1 * c2i;
    if (pre) {  /* :1141-1164 */
      double bSq = p.Mp * p.Mp / (bt(j, k) - p.Mp * p.Mp * (bt(j, k) - 1));
      double X = std::sqrt(((1. - bSq) * qq1) * ((1. - bSq) * qq1) + 4. * bSq * cx(j, k) * cx(j, k)) / rr1;
      double Y = 0.5 * ((1.0 - bSq) * qq1 / rr1 + X);
      double Z = 0.5 * ((1.0 - bSq) * qq1 / rr1 - X);
      double qqmxt = qq1 + ug(j, k) * rj1 * rr1 + vg(j, k) * rj2 * rr1;
      double a4 = qqmxt * s(j, k, 1) / rr1 - rj1 * s(j, k, 2) - rj2 * s(j, k, 3);
      a4 = a4 * bSq;
      s(j, k, 1) = a1;
      s(j, k, 2) = a2;
      s(j, k, 3) = -(Z * a3 + a4) / X;
      s(j, k, 4) = (Y * a3 + a4) / X;
      continue;
    }
    double a4 = qq1 * s(j, k, 1) / rr1 - rj1 * s(j, k, 2) - rj2 * s(j, k, 3);
    s(j, k, 1) = a1;
    s(j, k, 2) = a2;
    s(j, k, 3) = 0.5 * (a3 - a4 / cjkl);
    s(j, k, 4) = 0.5 * (a3 + a4 / cjkl);
  }
  /* :919-935 */
  for (int k = ks - 1; k <= ke + 1; ++k) for (int j = js; j <= je; ++j) {
    d2px(j, k) = std::fabs(pr(j + 1, k) - 2. * pr(j, k) + pr(j - 1, k));
    d2px(j, k) = d2px(j, k) / std::fabs(pr(j + 1, k) + 2. * pr(j, k) + pr(j - 1, k));
  }
  for (int k = ks - 1; k <= ke + 1; ++k) { d2px(js - 1, k) = 0; d2px(je + 1, k) = 0; }
  if (p.ilhs == 3) lhsinv_up(p, q, s, qx, cx, js - 1, je + 1, ks - 1, ke + 1, 1, xx, xy, vn, tscale, bt);
  else lhsinv(p, q, s, qx, cx, d2px, js - 1, je + 1, ks - 1, ke + 1, 1, xx, xy, vn, iblank, tscale, bt);
  /* :948-975 multiply by N inverse */
  for (int k = ks - 1; k <= ke + 1; ++k) for (int j = js - 1; j <= je + 1; ++j) {
    double cjkl = std::sqrt(ggm1 * (q(j, k, 4) - uv(j, k)));
    double rj1 = xx(j, k), rj2 = xy(j, k), rr1 = std::sqrt(rj1 * rj1 + rj2 * rj2);
    double rk1 = yx(j, k), rk2 = yy(j, k), rr2 = std::sqrt(rk1 * rk1 + rk2 * rk2);
    double a1 = (rj1 * rk1 + rj2 * rk2) / rr1 / rr2;
    double a2 = (rj1 * rk2 - rj2 * rk1) / rr1 / rr2;
    if (pre) {  /* :1207-1231 */
      double bSq = p.Mp * p.Mp / (bt(j, k) - p.Mp * p.Mp * (bt(j, k) - 1));
      double X = std::sqrt(((1.0 - bSq) * qx(j, k)) * ((1.0 - bSq) * qx(j, k)) + 4. * bSq * cx(j, k) * cx(j, k)) / rr1;
      double Y = 0.5 * ((1.0 - bSq) * qx(j, k) / rr1 + X);
      double Z = 0.5 * ((1.0 - bSq) * qx(j, k) / rr1 - X);
      double X1 = std::sqrt(((1.0 - bSq) * qy(j, k)) * ((1.0 - bSq) * qy(j, k)) + 4. * bSq * cy(j, k) * cy(j, k)) / rr2;
      double Y1 = 0.5 * ((1.0 - bSq) * qy(j, k) / rr2 + X1);
      double Z1 = 0.5 * ((1.0 - bSq) * qy(j, k) / rr2 - X1);
      double a4 = a1 * s(j, k, 2) + (Y * s(j, k, 3) + Z * s(j, k, 4)) * a2 / bSq;
      double a5 = -(a2 * bSq * s(j, k, 2) - (Y * a1 - Z1) * s(j, k, 3) - (Z * a1 - Z1) * s(j, k, 4)) / X1;
      double a6 = (a2 * bSq * s(j, k, 2) - (Y * a1 - Y1) * s(j, k, 3) - (Z * a1 - Y1) * s(j, k, 4)) / X1;
      (void)cjkl;
      s(j, k, 2) = a4;
      s(j, k, 3) = a5;
      s(j, k, 4) = a6;
      continue;
    }
    double a4 = a1 * s(j, k, 2) + (cjkl * s(j, k, 3) - cjkl * s(j, k, 4)) * a2;
    double a5 = -0.5 * (a2 * s(j, k, 2) / cjkl - (a1 + 1) * s(j, k, 3) + (a1 - 1) * s(j, k, 4));
    double a6 = 0.5 * (a2 * s(j, k, 2) / cjkl - (a1 - 1) * s(j, k, 3) + (a1 + 1) * s(j, k, 4));
    s(j, k, 2) = a4;
    s(j, k, 3) = a5;
    s(j, k, 4) = a6;
  }
  /* :977-993 */
  for (int k = ks; k <= ke; ++k) for (int j = js - 1; j <= je + 1; ++j) {
    d2py(j, k) = std::fabs(pr(j, k + 1) - 2. * pr(j, k) + pr(j, k - 1));
    d2py(j, k) = d2py(j, k) / std::fabs(pr(j, k + 1) + 2. * pr(j, k) + pr(j, k - 1));
  }
  for (int j = js - 1; j <= je + 1; ++j) { d2py(j, ks - 1) = 0; d2py(j, ke + 1) = 0; }
  if (p.ilhs == 3) lhsinv_up(p, q, s, qy, cy, ks - 1, ke + 1, js - 1, je + 1, 2, yx, yy, vn, tscale, bt);
  else lhsinv(p, q, s, qy, cy, d2py, ks - 1, ke + 1, js - 1, je + 1, 2, yx, yy, vn, iblank, tscale, bt);
  /* :1005-1034 multiply by T_eta */
  for (int k = ks - 1; k <= ke + 1; ++k) for (int j = js - 1; j <= je + 1; ++j) {
    double uu = q(j, k, 2), vv = q(j, k, 3);
    double cjkl = std::sqrt(ggm1 * (q(j, k, 4) - uv(j, k)));
    double rk1 = yx(j, k), rk2 = yy(j, k);
    if (pre) {  /* :1264-1298 */
      double qq2 = qy(j, k);
      double rr2 = std::sqrt(rk1 * rk1 + rk2 * rk2);
      rk1 = rk1 / rr2; rk2 = rk2 / rr2;
      double bSq = p.Mp * p.Mp / (bt(j, k) - p.Mp * p.Mp * (bt(j, k) - 1));
      double X = std::sqrt(((1. - bSq) * qq2) * ((1. - bSq) * qq2) + 4. * bSq * cy(j, k) * cy(j, k)) / rr2;
      double Y = 0.5 * ((1. - bSq) * qq2 / rr2 + X);
      double Z = 0.5 * ((1. - bSq) * qq2 / rr2 - X);
      double qqmxt = qq2 + ug(j, k) * rk1 * rr2 + vg(j, k) * rk2 * rr2;
      double a1 = s(j, k, 1) + s(j, k, 3) + s(j, k, 4);
      double a2 = uu * s(j, k, 1) + rk2 * s(j, k, 2) + (uu + rk1 * Y / bSq) * s(j, k, 3);
      a2 = a2 + (uu + rk1 * Z / bSq) * s(j, k, 4);
      double a3 = vv * s(j, k, 1) - rk1 * s(j, k, 2) + (vv + rk2 * Y / bSq) * s(j, k, 3);
      a3 = a3 + (vv + rk2 * Z / bSq) * s(j, k, 4);
      double a4 = uv(j, k) * s(j, k, 1) + (rk2 * uu - rk1 * vv) * s(j, k, 2);
      a4 = a4 + (ge(j, k) + Y * qqmxt / rr2 / bSq) * s(j, k, 3);
      a4 = a4 + (ge(j, k) + Z * qqmxt / rr2 / bSq) * s(j, k, 4);
      (void)cjkl;
      s(j, k, 1) = a1; s(j, k, 2) = a2; s(j, k, 3) = a3; s(j, k, 4) = a4;
      continue;
    }
    double qq2 = qy(j, k) + (rk1 * ug(j, k) + rk2 * vg(j, k));
    double rr2 = std::sqrt(rk1 * rk1 + rk2 * rk2);
    rk1 = rk1 / rr2; rk2 = rk2 / rr2;
    double a1 = s(j, k, 1) + s(j, k, 3) + s(j, k, 4);
    double a2 = uu * s(j, k, 1) + rk2 * s(j, k, 2) + (uu + rk1 * cjkl) * s(j, k, 3);
    a2 = a2 + (uu - rk1 * cjkl) * s(j, k, 4);
    double a3 = vv * s(j, k, 1) - rk1 * s(j, k, 2) + (vv + rk2 * cjkl) * s(j, k, 3);
    a3 = a3 + (vv - rk2 * cjkl) * s(j, k, 4);
    double a4 = uv(j, k) * s(j, k, 1) + (rk2 * uu - rk1 * vv) * s(j, k, 2);
    a4 = a4 + (ge(j, k) + cjkl * qq2 / rr2) * s(j, k, 3);
    a4 = a4 + (ge(j, k) - cjkl * qq2 / rr2) * s(j, k, 4);
    s(j, k, 1) = a1; s(j, k, 2) = a2; s(j, k, 3) = a3; s(j, k, 4) = a4;
  }
  if (p.iunst == 2) {
    for (int k = ks - 1; k <= ke + 1; ++k) for (int j = js - 1; j <= je + 1; ++j) {
      double a2 = s(j, k, 2), a3 = s(j, k, 3);
      double a4 = 1.0 + p2(tscale(j, k) * p.rotf);
      s(j, k, 2) = (a2 + tscale(j, k) * p.rotf * a3) / a4;
      s(j, k, 3) = (a3 - tscale(j, k) * p.rotf * a2) / a4;
    }
  }
  /* :1047-1054 primitive -> conservative */
  for (int k = ks - 1; k <= ke + 1; ++k) for (int j = js - 1; j <= je + 1; ++j) {
    q(j, k, 1) = q(j, k, 1) / q(j, k, nq);
    q(j, k, 2) = q(j, k, 2) * q(j, k, 1);
    q(j, k, 3) = q(j, k, 3) * q(j, k, 1);
    q(j, k, 4) = q(j, k, 4) * q(j, k, 1);
  }
}

}  // namespace oro
