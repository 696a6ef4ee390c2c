/*
 * oracle_implicit.cpp -- TEST INFRASTRUCTURE ONLY (see oracle_common.h).
 * FP64 restatement of the local time step (src/time.f) and the LU-SGS
 * hyperplane operator ilu2d (src/lhs.f:470-814).
 */
#include <cstdio>
#include <cstdlib>
#include "oracle.h"

namespace oro {

/* time.f:2-108, one time instance (the reference loops nsp outside) */
void time_step(const P& p, A3 q, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 tscale, A2 bt, I2 iblank) {
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

}  // namespace oro
