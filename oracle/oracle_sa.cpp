/*
 * oracle_sa.cpp -- TEST INFRASTRUCTURE ONLY (see oracle_common.h).
 * FP64 restatement of the Spalart-Allmaras solve vmu_sa and its helpers
 * (src/samodel2d.f:2-1385, constants src/sadata.h:2-4).
 */
#include <cstdio>
#include <cstdlib>
#include "oracle.h"

namespace oro {

/* sadata.h:2-4 (decimal literals are doubles under -r8) */
static const double cb1 = 0.1355, sigma = 0.6666667, cb2 = 0.622, akt = 0.41, cw1 = 3.2390678;
static const double cw2 = 0.3, cw3 = 2., cv1 = 7.1, ct3 = 1.2, ct4 = 0.5;

/* samodel2d.f:200-240 (also called by komegasst, komegasst.f:49) */
void lamvis(const P& p, A3 q, A2 vmul) {
  double c2b = 198.6 / p.tinf, c2bp = c2b + 1.;
  for (int k = 1; k <= p.kd; ++k) for (int j = 1; j <= p.jd; ++j) {
    double ra = 1. / q(j, k, 1);
    double uvel = q(j, k, 2) * ra, vvel = q(j, k, 3) * ra;
    double ei = q(j, k, 4) * ra - 0.5 * (p2(uvel) + p2(vvel));
    double tt = p.ggm1 * ei;
    vmul(j, k) = c2bp * tt * std::sqrt(tt) / (c2b + tt);
  }
}

/* samodel2d.f:243-293 (kwdist, komegasst.f:218-268, is the same computation) */
void dist(const P& p, A2 sn, A2 x, A2 y, const double* xv_, const double* yv_) {
  const int jd = p.jd, kd = p.kd, jmax = p.jmax, nhalo = p.nhalo;
  auto xv = [&](int j, int k) { return xv_[(size_t)(k - 1) * jmax + (j - 1)]; };
  auto yv = [&](int j, int k) { return yv_[(size_t)(k - 1) * jmax + (j - 1)]; };
  for (int j = p.jtail1; j <= p.jtail2; ++j) sn(j, 1) = 0.0;
  for (int j = p.jtail1; j <= p.jtail2; ++j)
    for (int k = 2; k <= kd; ++k) {
      int jv = j - nhalo;
      sn(j, k) = std::sqrt(p2(x(j, k) - 0.5 * (xv(jv, 1) + xv(jv + 1, 1))) + p2(y(j, k) - 0.5 * (yv(jv, 1) + yv(jv + 1, 1))));
    }
  for (int j = 1; j <= p.jtail1 - 1; ++j)
    for (int k = 1; k <= kd; ++k) {
      int jv = p.jtail1 - nhalo;
      sn(j, k) = std::sqrt(p2(x(j, k) - xv(jv, 1)) + p2(y(j, k) - yv(jv, 1)));
    }
  for (int j = p.jtail2 + 1; j <= jd; ++j)
    for (int k = 1; k <= kd; ++k) {
      int jv = p.jtail1 - nhalo;
      sn(j, k) = std::sqrt(p2(x(j, k) - xv(jv, 1)) + p2(y(j, k) - yv(jv, 1)));
    }
}

/* samodel2d.f:296-333 */
static void vortic(A2 vort, A2 u, A2 v, A2 xx, A2 xy, A2 yx, A2 yy, int js, int je, int ks, int ke) {
  double dx2 = 0.5, dy2 = 0.5;
  for (int k = ks; k <= ke; ++k) for (int j = js; j <= je; ++j) {
    double ux = (u(j + 1, k) - u(j - 1, k)) * dx2, vx = (v(j + 1, k) - v(j - 1, k)) * dx2;
    double uy = (u(j, k + 1) - u(j, k - 1)) * dy2, vy = (v(j, k + 1) - v(j, k - 1)) * dy2;
    double tx = xy(j, k) * ux - xx(j, k) * vx + yy(j, k) * uy - yx(j, k) * vy;
    vort(j, k) = std::fabs(tx);
  }
}

/* samodel2d.f:372-399 */
static void c_turm(const P& p, A3 q, A2 turmu, A2 vmul) {
  const int nq = p.nq, nmv = p.nmv;
  for (int k = 1; k <= p.kd; ++k) for (int j = 1; j <= p.jd; ++j) {
    double vnul = vmul(j, k) / (q(j, k, 1) * q(j, k, nq));
    double chi = q(j, k, nmv + 1) / vnul;
    double fv1 = p3(chi) / (p3(chi) + p3(cv1));
    turmu(j, k) = q(j, k, 1) * q(j, k, nq) * q(j, k, nmv + 1) * fv1;
  }
}

/* samodel2d.f:453-542 */
static void convec(const P& p, A3 q, A2 u, A2 v, A2 sjmat, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg,
                   A2 aj, A2 bj, A2 cj, A2 ak, A2 bk, A2 ck, int js, int je, int ks, int ke) {
  const int jd = p.jd, nmv = p.nmv; size_t n2 = (size_t)jd * p.kd;
  std::vector<double> um_(n2), up_(n2), vm_(n2), vp_(n2);
  A2 um{um_.data(), jd}, up{up_.data(), jd}, vm{vm_.data(), jd}, vp{vp_.data(), jd};
  for (int k = ks - 1; k <= ke + 1; ++k) for (int j = js - 1; j <= je + 1; ++j) {
    double uu = xx(j, k) * (u(j, k) - ug(j, k)) + xy(j, k) * (v(j, k) - vg(j, k));
    double vv = yx(j, k) * (u(j, k) - ug(j, k)) + yy(j, k) * (v(j, k) - vg(j, k));
    up(j, k) = 0.5 * (uu + std::fabs(uu)); um(j, k) = 0.5 * (uu - std::fabs(uu));
    vp(j, k) = 0.5 * (vv + std::fabs(vv)); vm(j, k) = 0.5 * (vv - std::fabs(vv));
  }
  const int n5 = nmv + 1;
  for (int k = ks; k <= ke; ++k) for (int j = js; j <= je; ++j) {
    sjmat(j, k) = sjmat(j, k) - up(j, k) * (q(j, k, n5) - q(j - 1, k, n5)) - um(j, k) * (q(j + 1, k, n5) - q(j, k, n5));
    sjmat(j, k) = sjmat(j, k) - vp(j, k) * (q(j, k, n5) - q(j, k - 1, n5)) - vm(j, k) * (q(j, k + 1, n5) - q(j, k, n5));
  }
  for (int k = ks - 1; k <= ke + 1; ++k) for (int j = js; j <= je; ++j) {
    double fwd = (up(j + 1, k) > 1.0e-12) ? 1.0 : 0.0;
    double bck = (um(j - 1, k) < -1.0e-12) ? 1.0 : 0.0;
    aj(j + 1, k) = aj(j + 1, k) - fwd * (up(j, k) + um(j, k));
    bj(j, k) = bj(j, k) + up(j, k) - um(j, k);
    cj(j - 1, k) = cj(j - 1, k) + bck * (up(j, k) + um(j, k));
  }
  for (int k = ks; k <= ke; ++k) for (int j = js - 1; j <= je + 1; ++j) {
    double fwd = (vp(j, k + 1) > 1.0e-12) ? 1.0 : 0.0;
    double bck = (vm(j, k - 1) < -1.0e-12) ? 1.0 : 0.0;
    ak(j, k + 1) = ak(j, k + 1) - fwd * (vp(j, k) + vm(j, k));
    bk(j, k) = bk(j, k) + vp(j, k) - vm(j, k);
    ck(j, k - 1) = ck(j, k - 1) + bck * (vp(j, k) + vm(j, k));
  }
}

/* samodel2d.f:545-688 */
static void diffus(const P& p, A3 q, A2 sjmat, A2 vmul, A2 xx, A2 xy, A2 yx, A2 yy,
                   A2 aj, A2 bj, A2 cj, A2 ak, A2 bk, A2 ck, int js, int je, int ks, int ke) {
  const int jd = p.jd, kd = p.kd, nq = p.nq, n5 = p.nmv + 1; const double rey = p.rey;
  size_t n2 = (size_t)jd * kd;
  std::vector<double> chp_(n2), dnuhp_(n2), dmxh_(n2), dmyh_(n2);
  A2 chp{chp_.data(), jd}, dnuhp{dnuhp_.data(), jd}, dmxh{dmxh_.data(), jd}, dmyh{dmyh_.data(), jd};
  for (int k = ks - 1; k <= ke + 1; ++k) for (int j = js - 1; j <= je; ++j) {
    dmxh(j, k) = 0.5 * (xx(j, k) + xx(j + 1, k));
    dmyh(j, k) = 0.5 * (xy(j, k) + xy(j + 1, k));
    double vnulh = 0.5 * (vmul(j, k) / q(j, k, 1) / q(j, k, nq) + vmul(j + 1, k) / q(j + 1, k, 1) / q(j + 1, k, nq));
    double vnuh = 0.5 * (q(j, k, n5) + q(j + 1, k, n5));
    chp(j, k) = (1. + cb2) / sigma / rey * (vnulh + vnuh);
    dnuhp(j, k) = q(j + 1, k, n5) - q(j, k, n5);
  }
  for (int j = js; j <= je; ++j) for (int k = ks - 1; k <= ke + 1; ++k) {
    double dxp = dmxh(j, k) * xx(j, k) + dmyh(j, k) * xy(j, k);
    double dxm = dmxh(j - 1, k) * xx(j, k) + dmyh(j - 1, k) * xy(j, k);
    double c2 = cb2 / sigma / rey;
    c2 = c2 * (vmul(j, k) / q(j, k, 1) / q(j, k, nq) + q(j, k, n5));
    double dcp = dxp * (chp(j, k) - c2), dcm = dxm * (chp(j - 1, k) - c2);
    double ax = 0.0, cx = 0.0;
    if (k != ke + 1 && k != ks - 1) { ax = fmax2(dcm, 0.0); cx = fmax2(dcp, 0.0); }
    sjmat(j, k) = sjmat(j, k) - ax * dnuhp(j - 1, k) + cx * dnuhp(j, k);
    aj(j, k) = aj(j, k) - ax; cj(j, k) = cj(j, k) - cx; bj(j, k) = bj(j, k) + ax + cx;
  }
  for (int k = 1; k <= kd; ++k) { aj(je + 1, k) = 0.0; cj(js - 1, k) = 0.0; }
  for (int k = ks - 1; k <= ke; ++k) for (int j = js - 1; j <= je + 1; ++j) {
    dmxh(j, k) = 0.5 * (yx(j, k) + yx(j, k + 1));
    dmyh(j, k) = 0.5 * (yy(j, k) + yy(j, k + 1));
    double vnulh = 0.5 * (vmul(j, k) / q(j, k, 1) / q(j, k, nq) + vmul(j, k + 1) / q(j, k + 1, 1) / q(j, k + 1, nq));
    double vnuh = 0.5 * (q(j, k, n5) + q(j, k + 1, n5));
    chp(j, k) = (1. + cb2) / sigma / rey * (vnulh + vnuh);
    dnuhp(j, k) = q(j, k + 1, n5) - q(j, k, n5);
  }
  for (int k = ks; k <= ke; ++k) for (int j = js - 1; j <= je + 1; ++j) {
    double dyp = dmxh(j, k) * yx(j, k) + dmyh(j, k) * yy(j, k);
    double dym = dmxh(j, k - 1) * yx(j, k) + dmyh(j, k - 1) * yy(j, k);
    double c2 = cb2 / sigma / rey;
    c2 = c2 * (vmul(j, k) / q(j, k, 1) / q(j, k, nq) + q(j, k, n5));
    double dcp = dyp * (chp(j, k) - c2), dcm = dym * (chp(j, k - 1) - c2);
    double ay = 0.0, cy = 0.0;
    if (j != js - 1 && j != je + 1) { ay = fmax2(dcm, 0.0); cy = fmax2(dcp, 0.0); }
    sjmat(j, k) = sjmat(j, k) - ay * dnuhp(j, k - 1) + cy * dnuhp(j, k);
    ak(j, k) = ak(j, k) - ay; ck(j, k) = ck(j, k) - cy; bk(j, k) = bk(j, k) + ay + cy;
  }
  for (int j = 1; j <= jd; ++j) { ak(j, ke + 1) = 0.0; ck(j, ks - 1) = 0.0; }
}

/* samodel2d.f:691-824 (isour = 0, fturf = 0, no transition, no objective) */
static void source(const P& p, A3 q, A2 sn, A2 sjmat, A2 vmul, A2 vort, A2 bk, int js, int je, int ks, int ke) {
  const int nq = p.nq, n5 = p.nmv + 1; const double rey = p.rey;
  const double d2min = 1.e-12, rmax = 10.0, stilim = 1.e-12, fturf = 0.0;
  for (int k = ks; k <= ke; ++k) for (int j = js; j <= je; ++j) {
    double vnul = vmul(j, k) / q(j, k, 1) / q(j, k, nq);
    double chi = q(j, k, n5) / vnul;
    double d = sn(j, k);
    chi = fmax2(chi, 1.e-12);
    double fv1 = (p3(chi)) / (p3(chi) + p3(cv1));
    double fv2 = 1. - chi / (1. + chi * fv1);
    double fv3 = 1.0;
    double ft2 = fturf * ct3 * std::exp(-1. * ct4 * chi * chi);
    double dchi = 1. / vnul;
    double dfv1 = (3. * p3(cv1)) * (p2(chi)) * dchi * p2(1. / (p3(chi) + p3(cv1)));
    double dfv2 = (fv2 - 1.) / chi / vnul + (1. - fv2) * (1 - fv2) * (dfv1 + fv1 / chi / vnul);
    double dfv3 = 0.0;
    double dft2 = (-2. * ct4) * chi * dchi * ft2;
    double d2 = fmax2(p2(d), d2min);
    double stilda = vort(j, k) * fv3 + vnul / (d2 * akt * akt * rey) * chi * fv2;
    stilda = fmax2(stilda, stilim);
    double r = q(j, k, n5) / (d2 * akt * akt * rey) / stilda;
    r = fmin2(r, rmax);
    double g = r + cw2 * (p6(r) - r);
    double fw = (1. + p6(cw3)) / (p6(g) + p6(cw3));
    fw = g * (std::pow(fw, 1. / 6.));
    double dstild = vort(j, k) * dfv3 + vnul * (dchi * fv2 + chi * dfv2) / (d2 * akt * akt * rey);
    double dr = vnul * (dchi - chi * dstild / stilda) / stilda / (d2 * akt * akt * rey);
    double dg = dr * (1. + cw2 * (6. * std::pow(r, 5.) - 1.));
    double dfw = std::pow((1. + p6(cw3)) / (p6(g) + p6(cw3)), 1. / 6.);
    dfw = dfw * dg * (1. - p6(g) / (p6(g) + p6(cw3)));
    double pro = cb1 * stilda * (1. - ft2);
    double des = (cw1 * fw - cb1 / (akt * akt) * ft2) / d2 / rey;
    double prod = cb1 * stilda * (1. - ft2) * q(j, k, n5);
    double dest = (cw1 * fw - cb1 / (akt * akt) * ft2) * q(j, k, n5) * q(j, k, n5) / d2 / rey;
    double dpro = pro * dstild / stilda - cb1 * stilda * dft2;
    double ddes = (cw1 * dfw - cb1 / (akt * akt) * dft2) / d2 / rey * vnul * chi;
    ddes = ddes + des;
    ddes = ddes * q(j, k, n5);
    dpro = dpro * q(j, k, n5);
    sjmat(j, k) = sjmat(j, k) + prod - dest;
    double tk1 = fmax2(des * q(j, k, n5) - pro, 0.0);
    double tk2 = fmax2(ddes - dpro, 0.0);
    bk(j, k) = bk(j, k) + tk1 + tk2;
  }
}

/* samodel2d.f:827-1303 (turbc and the per-type routines it dispatches) */
static void turbc(const P& p, A3 q, A2 u, A2 v, A2 ug, A2 vg, A2 xx, A2 xy, A2 yx, A2 yy) {
  const int jd = p.jd, kd = p.kd, n5 = p.nmv + 1;
  for (int ib = 0; ib < p.nbc; ++ib) {
    int js, je, ks, ke; bc_range(p, ib, js, je, ks, ke);
    int idir = p.ibdir[ib], t = p.ibtyp[ib];
    int iadd = isign(1, idir), iadir = std::abs(idir);
    if (t == 3 || t == 4) {                       /* turbc_extpt */
      double foso = 1.0;
      if (iadir == 1) {
        for (int jc = 1; jc <= je - js + 1; ++jc) {
          int j = (idir == 1) ? je - jc + 1 : js + jc - 1; int j1 = j + iadd, j2 = j1 + iadd;
          for (int k = ks; k <= ke; ++k) q(j, k, n5) = (1. + foso) * q(j1, k, n5) - foso * q(j2, k, n5);
        }
      } else if (iadir == 2) {
        for (int kc = 1; kc <= ke - ks + 1; ++kc) {
          int k = (idir == 2) ? ke - kc + 1 : ks + kc - 1; int k1 = k + iadd, k2 = k1 + iadd;
          for (int j = js; j <= je; ++j) q(j, k, n5) = (1. + foso) * q(j, k1, n5) - foso * q(j, k2, n5);
        }
      }
    } else if (t == 5) {                          /* turbc_wall (idir = +-2) */
      double foso = 1.0;
      if (iadir == 2) {
        int k = (idir == 2) ? ke : ks; int k1 = k + iadd;
        for (int j = js; j <= je; ++j) q(j, k, n5) = -q(j, k1, n5);
        for (int kc = 1; kc <= ke - ks; ++kc) {
          k = (idir == 2) ? ke - kc : ks + kc; k1 = k + iadd; int k2 = k1 + iadd;
          for (int j = js; j <= je; ++j) q(j, k, n5) = (1. + foso) * q(j, k1, n5) - foso * q(j, k2, n5);
        }
      } else {
        std::fprintf(stderr, "oracle: turbc_wall idir=+-1 not restated\n"); std::abort();
      }
    } else if (t == 10 || t == 11) {              /* turbc_sym */
      if (iadir == 1) {
        for (int jc = 1; jc <= je - js + 1; ++jc) {
          int j, j1;
          if (idir == 1) { j = je - jc + 1; j1 = je + jc; } else { j = js + jc - 1; j1 = js - jc; }
          for (int k = ks; k <= ke; ++k) q(j, k, n5) = q(j1, k, n5);
        }
      } else if (iadir == 2) {
        for (int kc = 1; kc <= ke - ks + 1; ++kc) {
          int k, k1;
          if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
          for (int j = js; j <= je; ++j) q(j, k, n5) = q(j, k1, n5);
        }
      }
    } else if (t == 22) {                         /* turbc_periodic */
      if (idir == 1 || idir == -1) {
        int jj = je - js + 1;
        for (int j = js; j <= je; ++j) {
          int jc = (idir == 1) ? jd - 2 * jj + (j - js + 1) : 1 + 2 * jj - (je - j + 1);
          for (int k = ks; k <= ke; ++k) q(j, k, n5) = q(jc, k, n5);
        }
      } else {
        int kk = ke - ks + 1;
        for (int k = ks; k <= ke; ++k) {
          int kc = (idir == 2) ? kd - 2 * kk + (k - ks + 1) : 1 + 2 * kk - (ke - k + 1);
          for (int j = js; j <= je; ++j) q(j, k, n5) = q(j, kc, n5);
        }
      }
    } else if (t == 51) {                         /* turbc_wake */
      if (iadir == 2) {
        for (int kc = 1; kc <= ke - ks + 1; ++kc) {
          int k, k1;
          if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
          for (int j = js; j <= je; ++j) {
            int jj = jd - j + 1;
            q(j, k, n5) = q(jj, k1, n5);
            q(jj, k, n5) = q(j, k1, n5);
          }
        }
      }
    } else if (t == 46) {                         /* turbc_inf */
      for (int k = ks; k <= ke; ++k) for (int j = js; j <= je; ++j) q(j, k, n5) = p.vnuinf;
    } else if (t == 47) {                         /* turbc_out */
      if (iadir == 1) {
        int j = (idir == 1) ? je : js; int j1 = j + iadd;
        for (int k = ks; k <= ke; ++k) {
          q(j, k, n5) = p.vnuinf;
          double uu = (u(j, k) - ug(j, k) + u(j1, k) - ug(j1, k)) * xx(j, k);
          uu = uu + (v(j, k) - vg(j, k) + v(j1, k) - vg(j1, k)) * xy(j, k);
          uu = uu * iadd;
          if (uu < 0.) q(j, k, n5) = q(j1, k, n5);
        }
        for (int jc = 1; jc <= je - js; ++jc) {
          j = (idir == 1) ? je - jc : js + jc; j1 = j + iadd;
          for (int k = ks; k <= ke; ++k) q(j, k, n5) = q(j1, k, n5);
        }
      } else if (iadir == 2) {
        int k = (idir == 2) ? ke : ks; int k1 = k + iadd;
        for (int j = js; j <= je; ++j) {
          q(j, k, n5) = p.vnuinf;
          double uu = (u(j, k) - ug(j, k) + u(j, k1) - ug(j, k1)) * yx(j, k);
          uu = uu + (v(j, k) - vg(j, k) + v(j, k1) - vg(j, k1)) * yy(j, k);
          uu = uu * iadd;
          if (uu < 0.) q(j, k, n5) = q(j, k1, n5);
        }
        for (int kc = 1; kc <= ke - ks; ++kc) {
          k = (idir == 2) ? ke - kc : ks + kc; k1 = k + iadd;
          for (int j = js; j <= je; ++j) q(j, k, n5) = q(j, k1, n5);
        }
      }
    }
  }
}

/* samodel2d.f:1306-1344 */
static void lsolvej(A2 a, A2 b, A2 c, A2 s, int js, int je, int ks, int ke) {
  for (int k = ks; k <= ke; ++k) { double bb = 1. / b(js, k); s(js, k) = s(js, k) * bb; c(js, k) = c(js, k) * bb; }
  for (int j = js + 1; j <= je; ++j) for (int k = ks; k <= ke; ++k) {
    double bb = 1. / (b(j, k) - a(j, k) * c(j - 1, k));
    s(j, k) = (s(j, k) - a(j, k) * s(j - 1, k)) * bb;
    c(j, k) = c(j, k) * bb;
  }
  for (int j = je - 1; j >= js; --j) for (int k = ks; k <= ke; ++k) s(j, k) = s(j, k) - c(j, k) * s(j + 1, k);
}

/* samodel2d.f:1347-1385 */
static void lsolvek(A2 a, A2 b, A2 c, A2 s, int js, int je, int ks, int ke) {
  for (int j = js; j <= je; ++j) { double bb = 1. / b(j, ks); s(j, ks) = s(j, ks) * bb; c(j, ks) = c(j, ks) * bb; }
  for (int k = ks + 1; k <= ke; ++k) for (int j = js; j <= je; ++j) {
    double bb = 1. / (b(j, k) - a(j, k) * c(j, k - 1));
    s(j, k) = (s(j, k) - a(j, k) * s(j, k - 1)) * bb;
    c(j, k) = c(j, k) * bb;
  }
  for (int k = ke - 1; k >= ks; --k) for (int j = js; j <= je; ++j) s(j, k) = s(j, k) - c(j, k) * s(j, k + 1);
}

/* samodel2d.f:2-197 (nturiter = nhuang = 1, relfac = 1, no transition) */
void vmu_sa(const P& p, A3 q, A3 s, A2 turmu, A2 x, A2 y, const double* xv, const double* yv,
            A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 tscale, I2 iblank, double* resl2_out) {
  const int jd = p.jd, kd = p.kd, nq = p.nq, n5 = p.nmv + 1;
  const int js = p.jbeg, je = p.jend, ks = p.kbeg, ke = p.kend;
  size_t n2 = (size_t)jd * kd;
  std::vector<double> buf(n2 * 16, 0.0);
  auto mk = [&](int i) { return A2{buf.data() + n2 * i, jd}; };
  A2 sjmat = mk(0), bjmat = mk(1), aj = mk(2), bj = mk(3), cj = mk(4), ak = mk(5), bk = mk(6), ck = mk(7);
  A2 vmul = mk(8), vort = mk(9), sn = mk(10), u = mk(11), v = mk(12), s1 = mk(13), s2 = mk(14);
  const double vnulim = 1.0e-20, relfac = 1.0;
  lamvis(p, q, vmul);
  for (int k = 1; k <= kd; ++k) for (int j = 1; j <= jd; ++j) {
    u(j, k) = q(j, k, 2) / q(j, k, 1); v(j, k) = q(j, k, 3) / q(j, k, 1);
    sjmat(j, k) = 0.0; vort(j, k) = 0.0; sn(j, k) = 1.e10;
    aj(j, k) = 0.; bj(j, k) = 0.; cj(j, k) = 0.; ak(j, k) = 0.; bk(j, k) = 0.; ck(j, k) = 0.; bjmat(j, k) = 0.;
  }
  turbc(p, q, u, v, ug, vg, xx, xy, yx, yy);
  bool bodyflag = false;
  for (int ib = 0; ib < p.nbc; ++ib) if (p.ibtyp[ib] == 5) bodyflag = true;
  if (bodyflag) {
    vortic(vort, u, v, xx, xy, yx, yy, js, je, ks, ke);
    dist(p, sn, x, y, xv, yv);
  }
  c_turm(p, q, turmu, vmul);
  /* rhslhs, samodel2d.f:402-450 */
  for (int k = 1; k <= kd; ++k) for (int j = 1; j <= jd; ++j) {
    aj(j, k) = 0.0; bj(j, k) = 0.0; cj(j, k) = 0.0; ak(j, k) = 0.0; bk(j, k) = 0.0; ck(j, k) = 0.0;
    sjmat(j, k) = s(j, k, n5);
  }
  convec(p, q, u, v, sjmat, xx, xy, yx, yy, ug, vg, aj, bj, cj, ak, bk, ck, js, je, ks, ke);
  diffus(p, q, sjmat, vmul, xx, xy, yx, yy, aj, bj, cj, ak, bk, ck, js, je, ks, ke);
  source(p, q, sn, sjmat, vmul, vort, bk, js, je, ks, ke);
  for (int k = ks; k <= ke; ++k) for (int j = js; j <= je; ++j) {
    double tscal = tscale(j, k);
    if (p.cfltur > 1 && p.idual_turb == 1) {
      double dtpseudo_turb = p.cfltur / (bj(j, k) + bk(j, k));
      tscal = dtpseudo_turb * (double)iblank(j, k);
      tscal = tscal / (1. + tscal / p.h);
    }
    if (p.timeac == 1) {
      double dtpseudo_turb = 1.0;
      double ib = (double)(iblank(j, k) > 0 ? iblank(j, k) : 0);
      tscal = ib * (1.0 + 0.002 * std::sqrt(q(j, k, nq))) / (1. + std::sqrt(q(j, k, nq)));
      tscal = tscal * dtpseudo_turb;
      tscal = tscal / (1. + tscal / p.h);
    }
    sjmat(j, k) = sjmat(j, k) * tscal;
    aj(j, k) = aj(j, k) * tscal; cj(j, k) = cj(j, k) * tscal;
    ak(j, k) = ak(j, k) * tscal; ck(j, k) = ck(j, k) * tscal;
    bjmat(j, k) = 1. + (bj(j, k) + bk(j, k)) * tscal;
    s1(j, k) = 0.; s2(j, k) = 0.;
  }
  lsolvej(aj, bjmat, cj, sjmat, js, je, ks, ke);
  for (int k = ks; k <= ke; ++k) for (int j = js; j <= je; ++j) {
    s1(j, k) = s1(j, k) + sjmat(j, k);
    sjmat(j, k) = (s1(j, k) - s2(j, k)) * bjmat(j, k);
  }
  lsolvek(ak, bjmat, ck, sjmat, js, je, ks, ke);
  for (int k = ks; k <= ke; ++k) for (int j = js; j <= je; ++j) {
    s2(j, k) = s2(j, k) + sjmat(j, k);
    sjmat(j, k) = s2(j, k);
  }
  double resl2 = 0.0;
  for (int k = ks; k <= ke; ++k) for (int j = js; j <= je; ++j) {
    sjmat(j, k) = relfac * sjmat(j, k);
    resl2 = resl2 + sjmat(j, k) * sjmat(j, k);
  }
  resl2 = std::sqrt(resl2 / jd / kd);
  if (resl2_out) *resl2_out = resl2;
  for (int k = ks; k <= ke; ++k) for (int j = js; j <= je; ++j) {
    double ib = (double)(iblank(j, k) > 0 ? iblank(j, k) : 0);
    q(j, k, n5) = fmax2((q(j, k, n5) + sjmat(j, k) * ib), vnulim);
  }
  turbc(p, q, u, v, ug, vg, xx, xy, yx, yy);
  c_turm(p, q, turmu, vmul);
}

}  // namespace oro

/* Test hook: the source terms of samodel2d.f:691-824 alone over the interior
 * cells (jbeg..jend, kbeg..kend), so that a test can hold them against the
 * published model.  q(jd,kd,nq) of one instance; sjmat and bk accumulate. */
extern "C" void oro_sa_source(const oro::P* p, double* q, double* sn, double* vmul, double* vort, double* sjmat,
                              double* bk) {
  using namespace oro;
  const A3 qq{q, p->jd, (size_t)p->jd * p->kd};
  source(*p, qq, A2{sn, p->jd}, A2{sjmat, p->jd}, A2{vmul, p->jd}, A2{vort, p->jd}, A2{bk, p->jd}, p->jbeg,
         p->jend, p->kbeg, p->kend);
}
