/*
 * oracle_sst.cpp -- TEST INFRASTRUCTURE ONLY (see oracle_common.h).
 * FP64 restatement of the Menter k-omega SST solve komegasst and its helpers
 * (src/komegasst.f:2-1520, constants src/komega.h:1-8), without the
 * transition model (itrans = 0).
 *
 * Arrays the reference allocates and fills only on the interior
 * (strain, F1, F2, cdkw, the stresses and gradients) are read on the halo by
 * findturm (all cells) and komegadiffus (the half-points at js-1 / ks-1);
 * the Fortran leaves those halo values undefined.  Here they are 0, which is
 * what the reference reads whenever the allocation comes from fresh pages
 * (arrays above glibc's mmap threshold, e.g. every mesh from 129x65 up).
 */
#include <cstdio>
#include <cstdlib>
#include "oracle.h"

namespace oro {

/* komega.h:1-8 (decimal literals are doubles under -r8) */
static const double sigmak1 = 0.85, sigmaw1 = 0.5, beta1 = 0.075, sigmak2 = 1.0, sigmaw2 = 0.856,
                    beta2 = 0.0828, betastar = 0.09;
static const double gamma1 = 5. / 9, gamma2 = 0.44;

/* komegasst.f:190-215 (all cells) */
static void findturm(const P& p, A3 q, A2 rho, A2 strain, A2 F2, A2 turmu) {
  const double a1 = 0.31, rei = 1. / p.rey;
  const int nmv = p.nmv;
  for (int k = 1; k <= p.kd; ++k) for (int j = 1; j <= p.jd; ++j) {
    turmu(j, k) = a1 * rho(j, k) * q(j, k, nmv + 1) / fmax2(a1 * q(j, k, nmv + 2), F2(j, k) * rho(j, k) * strain(j, k) * rei);
    turmu(j, k) = fmax2(turmu(j, k), 1e-20);
  }
}

/* komegasst.f:270-318 */
static void kwvortic(A2 vort, A2 strain, A2 u, A2 v, A2 xx, A2 xy, A2 yx, A2 yy, int js, int je, int ks, int ke) {
  for (int j = js; j <= je; ++j) for (int k = ks; k <= ke; ++k) {
    double usi = 0.5 * (u(j + 1, k) - u(j - 1, k)), vsi = 0.5 * (v(j + 1, k) - v(j - 1, k));
    double ueta = 0.5 * (u(j, k + 1) - u(j, k - 1)), veta = 0.5 * (v(j, k + 1) - v(j, k - 1));
    double ux = xx(j, k) * usi + yx(j, k) * ueta, uy = xy(j, k) * usi + yy(j, k) * ueta;
    double vx = xx(j, k) * vsi + yx(j, k) * veta, vy = xy(j, k) * vsi + yy(j, k) * veta;
    double sxx = ux, sxy = 0.5 * (uy + vx), syy = vy;
    vort(j, k) = std::fabs(uy - vx);
    strain(j, k) = std::sqrt(2. * (sxx * sxx + 2. * sxy * sxy + syy * syy));
  }
}

/* komegasst.f:321-371 */
static void turbstress(const P& p, A3 q, A2 turmu, A2 tauxx, A2 tauxy, A2 tauyy, A2 u, A2 v, A2 ux, A2 uy, A2 vx,
                       A2 vy, A2 xx, A2 xy, A2 yx, A2 yy, int js, int je, int ks, int ke) {
  const double rei = 1. / p.rey;
  const int nmv = p.nmv;
  for (int j = js; j <= je; ++j) for (int k = ks; k <= ke; ++k) {
    double usi = 0.5 * (u(j + 1, k) - u(j - 1, k)), vsi = 0.5 * (v(j + 1, k) - v(j - 1, k));
    double ueta = 0.5 * (u(j, k + 1) - u(j, k - 1)), veta = 0.5 * (v(j, k + 1) - v(j, k - 1));
    ux(j, k) = xx(j, k) * usi + yx(j, k) * ueta;
    uy(j, k) = xy(j, k) * usi + yy(j, k) * ueta;
    vx(j, k) = xx(j, k) * vsi + yx(j, k) * veta;
    vy(j, k) = xy(j, k) * vsi + yy(j, k) * veta;
    double sfdiv = 2. / 3 * (ux(j, k) + vy(j, k));
    tauxx(j, k) = turmu(j, k) * rei * (2.0 * ux(j, k) - sfdiv) - 2. / 3 * q(j, k, nmv + 1);
    tauyy(j, k) = turmu(j, k) * rei * (2.0 * vy(j, k) - sfdiv) - 2. / 3 * q(j, k, nmv + 1);
    tauxy(j, k) = turmu(j, k) * rei * (uy(j, k) + vx(j, k));
  }
}

/* komegasst.f:374-414 */
static void crossdiff(const P& p, A3 q, A2 rho, A2 cdkw, A2 xx, A2 xy, A2 yx, A2 yy, int js, int je, int ks, int ke) {
  const int nmv = p.nmv;
  for (int j = js; j <= je; ++j) for (int k = ks; k <= ke; ++k) {
    const int jp = j + 1, jm1 = j - 1, kp = k + 1, km1 = k - 1;
    double ksi = 0.5 * (q(jp, k, nmv + 1) / rho(jp, k) - q(jm1, k, nmv + 1) / rho(jm1, k));
    double keta = 0.5 * (q(j, kp, nmv + 1) / rho(j, kp) - q(j, km1, nmv + 1) / rho(j, km1));
    double omegasi = 0.5 * (q(jp, k, nmv + 2) / rho(jp, k) - q(jm1, k, nmv + 2) / rho(jm1, k));
    double omegaeta = 0.5 * (q(j, kp, nmv + 2) / rho(j, kp) - q(j, km1, nmv + 2) / rho(j, km1));
    double kx = ksi * xx(j, k) + keta * yx(j, k), ky = ksi * xy(j, k) + keta * yy(j, k);
    double omegax = omegasi * xx(j, k) + omegaeta * yx(j, k), omegay = omegasi * xy(j, k) + omegaeta * yy(j, k);
    cdkw(j, k) = kx * omegax + ky * omegay;
    cdkw(j, k) = cdkw(j, k) * 2 * sigmaw2 * rho(j, k) * rho(j, k) / q(j, k, nmv + 2);
  }
}

/* komegasst.f:417-461 (itrans = 0) */
static void blend(const P& p, A3 q, A2 rho, A2 vmul, A2 cdkw, A2 sn, A2 F1, A2 F2, int js, int je, int ks, int ke) {
  const double rei = 1. / p.rey;
  const int nmv = p.nmv;
  for (int j = js; j <= je; ++j) for (int k = ks; k <= ke; ++k) {
    double a1 = rei * std::sqrt(q(j, k, nmv + 1) * rho(j, k)) / (0.09 * q(j, k, nmv + 2) * sn(j, k));
    double a2 = 500 * rei * rei * vmul(j, k) / (q(j, k, nmv + 2) * p2(sn(j, k)));
    double cd = fmax2(cdkw(j, k), 1e-10);
    double a3 = 4 * q(j, k, nmv + 1) * sigmaw2 / (cd * p2(sn(j, k)));
    double arg1 = fmin2(fmax2(a1, a2), a3);
    double arg2 = fmax2(2 * a1, a2);
    F1(j, k) = std::tanh(p2(p2(arg1)));
    F2(j, k) = std::tanh(p2(arg2));
  }
}

/* komegasst.f:847-903 (itrans = 0) */
static void komegasource(const P& p, A3 q, A2 rho, A2 turmu, A2 tauxx, A2 tauxy, A2 tauyy, A2 cdkw, A2 ux, A2 uy,
                         A2 vx, A2 vy, A2 F1, A2* bjmat, A2* sjmat, int js, int je, int ks, int ke) {
  const double rei = 1. / p.rey, rey = p.rey;
  const int nmv = p.nmv;
  for (int k = ks; k <= ke; ++k) for (int j = js; j <= je; ++j) {
    double prod = tauxx(j, k) * ux(j, k) + tauxy(j, k) * (uy(j, k) + vx(j, k)) + tauyy(j, k) * vy(j, k);
    double kdes = betastar * rey * q(j, k, nmv + 2) * q(j, k, nmv + 1) / rho(j, k);
    double ksust = betastar * rey * p.tkeinf * p.tomegainf * rho(j, k);
    double prodlim = 10. * kdes;
    prod = fmin2(prod, prodlim);
    double kprod = prod;
    double beta = F1(j, k) * beta1 + (1 - F1(j, k)) * beta2;
    double omegades = beta * rey * q(j, k, nmv + 2) * q(j, k, nmv + 2) / rho(j, k);
    double omegasust = beta * rey * p2(p.tomegainf) * rho(j, k);
    double omegacrossdiff = (1 - F1(j, k)) * cdkw(j, k) * rei;
    sjmat[0](j, k) = sjmat[0](j, k) + kprod - kdes + ksust;
    double gammap = F1(j, k) * gamma1 + (1 - F1(j, k)) * gamma2;
    sjmat[1](j, k) = sjmat[1](j, k) + gammap * rho(j, k) / turmu(j, k) * prod - omegades + omegacrossdiff + omegasust;
    bjmat[0](j, k) = bjmat[0](j, k) + kdes / q(j, k, nmv + 1);
    bjmat[1](j, k) = bjmat[1](j, k) + (2 * omegades + std::fabs(omegacrossdiff)) / q(j, k, nmv + 2);
  }
}

/* komegasst.f:593-844.  The two-equation bands: aj..ck[n], bjmat[n],
 * sjmat[n] for n = 0 (k) and 1 (omega). */
static void komegadiffus(const P& p, A3 q, A2 rho, A2 vmul, A2 turmu, A2 F1, A2 xx, A2 xy, A2 yx, A2 yy, A2* aj,
                         A2* bjmat, A2* cj, A2* ak, A2* ck, A2* sjmat, int js, int je, int ks, int ke) {
  const int jd = p.jd, kd = p.kd, nmv = p.nmv;
  const size_t n2 = (size_t)jd * kd;
  std::vector<double> b_(n2 * 4, 0.0);
  A2 chp{b_.data(), jd}, dnuhp{b_.data() + n2, jd}, dmxh{b_.data() + 2 * n2, jd}, dmyh{b_.data() + 3 * n2, jd};
  const double rei = 1. / p.rey;
  /* j-direction half-point coefficients (:620-625) */
  for (int j = js - 1; j <= je; ++j) for (int k = ks - 1; k <= ke + 1; ++k) {
    dmxh(j, k) = 0.5 * (xx(j, k) + xx(j + 1, k));
    dmyh(j, k) = 0.5 * (xy(j, k) + xy(j + 1, k));
  }
  for (int n = 0; n < 2; ++n) {
    /* j-direction fluxes of equation n (:629-670 k, :679-720 omega) */
    const double sg1 = n == 0 ? sigmak1 : sigmaw1, sg2 = n == 0 ? sigmak2 : sigmaw2;
    for (int j = js - 1; j <= je; ++j) for (int k = ks - 1; k <= ke + 1; ++k) {
      double vnulh = 0.5 * (vmul(j, k) + vmul(j + 1, k));
      double vnuh = 0.5 * (turmu(j, k) + turmu(j + 1, k));
      double sig = F1(j, k) * sg1 + (1. - F1(j, k)) * sg2;
      chp(j, k) = rei * (vnulh + sig * vnuh);
      dnuhp(j, k) = q(j + 1, k, nmv + 1 + n) / rho(j + 1, k) - q(j, k, nmv + 1 + n) / rho(j, k);
    }
    for (int j = js; j <= je; ++j) for (int k = ks - 1; k <= ke + 1; ++k) {
      double dxp = dmxh(j, k) * xx(j, k) + dmyh(j, k) * xy(j, k);
      double dxm = dmxh(j - 1, k) * xx(j, k) + dmyh(j - 1, k) * xy(j, k);
      double dcp = dxp * (chp(j, k)), dcm = dxm * (chp(j - 1, k));
      double ax = 0.0, cx = 0.0;
      if (k != ke + 1 && k != ks - 1) { ax = fmax2(dcm, 0.0); cx = fmax2(dcp, 0.0); }
      sjmat[n](j, k) = sjmat[n](j, k) - ax * dnuhp(j - 1, k) + cx * dnuhp(j, k);
      aj[n](j, k) = aj[n](j, k) - ax / rho(j - 1, k);
      cj[n](j, k) = cj[n](j, k) - cx / rho(j + 1, k);
      bjmat[n](j, k) = bjmat[n](j, k) + (ax + cx) / rho(j, k);
    }
    for (int k = 1; k <= kd; ++k) { aj[n](je + 1, k) = 0.0; cj[n](js - 1, k) = 0.0; }
  }
  /* k-direction half-point coefficients (:727-732) */
  for (int k = ks - 1; k <= ke; ++k) for (int j = js - 1; j <= je + 1; ++j) {
    dmxh(j, k) = 0.5 * (yx(j, k) + yx(j, k + 1));
    dmyh(j, k) = 0.5 * (yy(j, k) + yy(j, k + 1));
  }
  for (int n = 0; n < 2; ++n) {
    /* k-direction fluxes of equation n (:736-784 k, :788-838 omega) */
    const double sg1 = n == 0 ? sigmak1 : sigmaw1, sg2 = n == 0 ? sigmak2 : sigmaw2;
    for (int k = ks - 1; k <= ke; ++k) for (int j = js - 1; j <= je + 1; ++j) {
      double vnulh = 0.5 * (vmul(j, k) + vmul(j, k + 1));
      double vnuh = 0.5 * (turmu(j, k) + turmu(j, k + 1));
      double sig = F1(j, k) * sg1 + (1. - F1(j, k)) * sg2;
      chp(j, k) = rei * (vnulh + sig * vnuh);
      dnuhp(j, k) = q(j, k + 1, nmv + 1 + n) / rho(j, k + 1) - q(j, k, nmv + 1 + n) / rho(j, k);
    }
    for (int k = ks; k <= ke; ++k) for (int j = js - 1; j <= je + 1; ++j) {
      double dyp = dmxh(j, k) * yx(j, k) + dmyh(j, k) * yy(j, k);
      double dym = dmxh(j, k - 1) * yx(j, k) + dmyh(j, k - 1) * yy(j, k);
      double dcp = dyp * (chp(j, k)), dcm = dym * (chp(j, k - 1));
      double ay = 0.0, cy = 0.0;
      if (j != js - 1 && j != je + 1) { ay = fmax2(dcm, 0.0); cy = fmax2(dcp, 0.0); }
      sjmat[n](j, k) = sjmat[n](j, k) - ay * dnuhp(j, k - 1) + cy * dnuhp(j, k);
      ak[n](j, k) = ak[n](j, k) - ay / rho(j, k - 1);
      ck[n](j, k) = ck[n](j, k) - cy / rho(j, k + 1);
      bjmat[n](j, k) = bjmat[n](j, k) + (ay + cy) / rho(j, k);
    }
    /* the reference runs this loop over j = 1..kd (:779-782, :833-836) */
    for (int j = 1; j <= kd && j <= jd; ++j) { ak[n](j, ke + 1) = 0.0; ck[n](j, ks - 1) = 0.0; }
  }
}

/* komegasst.f:464-590 */
static void komegarhslhs(const P& p, A3 q, A3 s, A2 vmul, A2 turmu, A2 tauxx, A2 tauxy, A2 tauyy, A2 cdkw, A2 ux,
                         A2 uy, A2 vx, A2 vy, A2 F1, A2 rho, A2 u, A2 v, A2 ug, A2 vg, A2 xx, A2 xy, A2 yx, A2 yy,
                         A2* aj, A2* bjmat, A2* cj, A2* ak, A2* ck, A2* sjmat, int js, int je, int ks, int ke) {
  const int jd = p.jd, kd = p.kd, nmv = p.nmv;
  for (int k = 1; k <= kd; ++k) for (int j = 1; j <= jd; ++j)
    for (int n = 0; n < 2; ++n) {
      aj[n](j, k) = 0.0; bjmat[n](j, k) = 0.0; cj[n](j, k) = 0.0; ak[n](j, k) = 0.0; ck[n](j, k) = 0.0;
      sjmat[n](j, k) = s(j, k, n + 1 + nmv);
    }
  /* convection, j lines (:507-543) */
  std::vector<double> up(jd + 2), um(jd + 2), vp(kd + 2), vm(kd + 2);
  for (int k = ks; k <= ke; ++k) {
    for (int j = js - 1; j <= je + 1; ++j) {
      double uu = xx(j, k) * (u(j, k) - ug(j, k)) + xy(j, k) * (v(j, k) - vg(j, k));
      up[j] = 0.5 * (uu + std::fabs(uu));
      um[j] = 0.5 * (uu - std::fabs(uu));
    }
    for (int j = js; j <= je; ++j) {
      const int jp = j + 1, jm1 = j - 1;
      for (int n = 0; n < 2; ++n)
        sjmat[n](j, k) = sjmat[n](j, k) - up[j] * (q(j, k, nmv + 1 + n) - q(jm1, k, nmv + 1 + n)) -
                         um[j] * (q(jp, k, nmv + 1 + n) - q(j, k, nmv + 1 + n));
      for (int n = 0; n < 2; ++n) {
        aj[n](j, k) = aj[n](j, k) - up[j];
        cj[n](j, k) = cj[n](j, k) + um[j];
        bjmat[n](j, k) = bjmat[n](j, k) + up[j] - um[j];
      }
    }
  }
  /* convection, k lines (:545-580) */
  for (int j = js; j <= je; ++j) {
    for (int k = ks - 1; k <= ke + 1; ++k) {
      double vv = yx(j, k) * (u(j, k) - ug(j, k)) + yy(j, k) * (v(j, k) - vg(j, k));
      vp[k] = 0.5 * (vv + std::fabs(vv));
      vm[k] = 0.5 * (vv - std::fabs(vv));
    }
    for (int k = ks; k <= ke; ++k) {
      const int kp = k + 1, km1 = k - 1;
      for (int n = 0; n < 2; ++n)
        sjmat[n](j, k) = sjmat[n](j, k) - vp[k] * (q(j, k, nmv + 1 + n) - q(j, km1, nmv + 1 + n)) -
                         vm[k] * (q(j, kp, nmv + 1 + n) - q(j, k, nmv + 1 + n));
      for (int n = 0; n < 2; ++n) {
        ak[n](j, k) = ak[n](j, k) - vp[k];
        ck[n](j, k) = ck[n](j, k) + vm[k];
        bjmat[n](j, k) = bjmat[n](j, k) + vp[k] - vm[k];
      }
    }
  }
  komegasource(p, q, rho, turmu, tauxx, tauxy, tauyy, cdkw, ux, uy, vx, vy, F1, bjmat, sjmat, js, je, ks, ke);
  komegadiffus(p, q, rho, vmul, turmu, F1, xx, xy, yx, yy, aj, bjmat, cj, ak, ck, sjmat, js, je, ks, ke);
}

/* komegasst.f:906-974 with the per-type routines :977-1432 */
static void komegabc(const P& p, A3 q, A2 vmul, A2 rho, A2 x, A2 y, const double* xv_, const double* yv_, A2 u, A2 v,
                     A2 ug, A2 vg, A2 xx, A2 xy, A2 yx, A2 yy) {
  const int jd = p.jd, kd = p.kd, nmv = p.nmv, jmax = p.jmax, nhalo = p.nhalo;
  const int n5 = nmv + 1, n6 = nmv + 2;
  auto xv = [&](int j, int k) { return xv_[(size_t)(k - 1) * jmax + (j - 1)]; };
  auto yv = [&](int j, int k) { return yv_[(size_t)(k - 1) * jmax + (j - 1)]; };
  for (int ib = 0; ib < p.nbc; ++ib) {
    int js, je, ks, ke;
    bc_range(p, ib, js, je, ks, ke);
    const int idir = p.ibdir[ib], t = p.ibtyp[ib];
    const int iadd = isign(1, idir), iadir = idir < 0 ? -idir : idir;
    if (t == 3 || t == 4) {
      /* komegabc_extpt, :1079-1129 */
      const double foso = 1.0;
      if (iadir == 1) {
        for (int jc = 1; jc <= je - js + 1; ++jc) {
          int j = (idir == 1) ? je - jc + 1 : js + jc - 1, j1 = j + iadd, j2 = j1 + iadd;
          for (int k = ks; k <= ke; ++k) {
            q(j, k, n5) = (1. + foso) * q(j1, k, n5) - foso * q(j2, k, n5);
            q(j, k, n6) = (1. + foso) * q(j1, k, n6) - foso * q(j2, k, n6);
          }
        }
      } else if (iadir == 2) {
        for (int kc = 1; kc <= ke - ks + 1; ++kc) {
          int k = (idir == 2) ? ke - kc + 1 : ks + kc - 1, k1 = k + iadd, k2 = k1 + iadd;
          for (int j = js; j <= je; ++j) {
            q(j, k, n5) = (1. + foso) * q(j, k1, n5) - foso * q(j, k2, n5);
            q(j, k, n6) = (1. + foso) * q(j, k1, n6) - foso * q(j, k2, n6);
          }
        }
      }
    } else if (t == 5) {
      /* komegabc_wall, :977-1076 */
      const double foso = 1.0, rei = 1. / p.rey;
      double tt = ((double)p.istep0 - 1.) / 30.;
      if (tt > 1. || p.iread > 0) tt = 1.;
      const double scal = (10. - 15. * tt + 6. * tt * tt) * p3(tt);
      if (iadir == 1) {
        int j = (idir == 1) ? je : js;
        const int j1 = j + iadd, jv = j1 - nhalo;
        for (int k = ks; k <= ke; ++k) {
          const int kv = k - nhalo;
          double dely2 = p2(x(j1, k) - 0.5 * (xv(jv, kv) + xv(jv, kv + 1))) + p2(y(j1, k) - 0.5 * (yv(jv, kv) + yv(jv, kv + 1)));
          double vmulwall = 0.5 * (vmul(j1, k) + vmul(j, k));
          double omegawall = 60. * vmulwall * rei * rei / (beta1 * dely2);
          double qwall5 = -q(j1, k, n5);
          double qwall6 = 2 * omegawall - 6. * vmul(j1, k) * rei * rei / (beta1 * dely2);
          q(j, k, n5) = scal * qwall5 + (1. - scal) * q(j, k, n5);
          q(j, k, n6) = scal * qwall6 + (1. - scal) * q(j, k, n6);
        }
        /* :1024-1036 -- with nhalo = 1, je - js = 0 and this never runs */
        for (int jc = 1; jc <= je - js; ++jc) {
          fprintf(stderr, "oracle komegabc_wall: multi-cell j halo not supported\n");
          abort();
        }
      } else if (iadir == 2) {
        const int k = (idir == 2) ? ke : ks, k1 = k + iadd, kv = k1 - nhalo;
        for (int j = js; j <= je; ++j) {
          const int jv = j - nhalo;
          double dely2 = p2(x(j, k1) - 0.5 * (xv(jv, kv) + xv(jv + 1, kv))) + p2(y(j, k1) - 0.5 * (yv(jv, kv) + yv(jv + 1, kv)));
          double vmulwall = 0.5 * (vmul(j, k1) + vmul(j, k1));
          double omegawall = 60. * vmulwall * rei * rei / (beta1 * dely2);
          double qwall5 = -q(j, k1, n5);
          double qwall6 = 2 * omegawall - 6. * vmul(j, k1) * rei * rei / (beta1 * dely2);
          q(j, k, n5) = scal * qwall5 + (1. - scal) * q(j, k, n5);
          q(j, k, n6) = scal * qwall6 + (1. - scal) * q(j, k, n6);
        }
        for (int kc = 1; kc <= ke - ks; ++kc) {
          int kk = (idir == 2) ? ke - kc : ks + kc, kk1 = kk + iadd, kk2 = kk1 + iadd;
          for (int j = js; j <= je; ++j) {
            q(j, kk, n5) = (1. + foso) * q(j, kk1, n5) - foso * q(j, kk2, n5);
            q(j, kk, n6) = (1. + foso) * q(j, kk1, n6) - foso * q(j, kk2, n6);
          }
        }
      }
    } else if (t == 10 || t == 11) {
      /* komegabc_sym, :1132-1180 */
      if (iadir == 1) {
        for (int jc = 1; jc <= je - js + 1; ++jc) {
          int j, j1;
          if (idir == 1) { j = je - jc + 1; j1 = je + jc; } else { j = js + jc - 1; j1 = js - jc; }
          for (int k = ks; k <= ke; ++k) { q(j, k, n5) = q(j1, k, n5); q(j, k, n6) = q(j1, k, n6); }
        }
      } else if (iadir == 2) {
        for (int kc = 1; kc <= ke - ks + 1; ++kc) {
          int k, k1;
          if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
          for (int j = js; j <= je; ++j) { q(j, k, n5) = q(j, k1, n5); q(j, k, n6) = q(j, k1, n6); }
        }
      }
    } else if (t == 22) {
      /* komegabc_periodic, :1183-1251 */
      if (idir == 1 || idir == -1) {
        const int jj = je - js + 1;
        for (int j = js; j <= je; ++j) {
          const int jj1 = (idir == 1) ? j - js + 1 : je - j + 1;
          const int jc = (idir == 1) ? jd - 2 * jj + jj1 : 1 + 2 * jj - jj1;
          for (int k = ks; k <= ke; ++k) { q(j, k, n5) = q(jc, k, n5); q(j, k, n6) = q(jc, k, n6); }
        }
      } else {
        const int kk = ke - ks + 1;
        for (int k = ks; k <= ke; ++k) {
          const int kk1 = (idir == 2) ? k - ks + 1 : ke - k + 1;
          const int kc = (idir == 2) ? kd - 2 * kk + kk1 : 1 + 2 * kk - kk1;
          for (int j = js; j <= je; ++j) { q(j, k, n5) = q(j, kc, n5); q(j, k, n6) = q(j, kc, n6); }
        }
      }
    } else if (t == 51) {
      /* komegabc_wake, :1254-1295 */
      if (iadir == 2) {
        for (int kc = 1; kc <= ke - ks + 1; ++kc) {
          int k, k1;
          if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
          for (int j = js; j <= je; ++j) {
            const int jj = jd - j + 1;
            q(j, k, n5) = q(jj, k1, n5);
            q(j, k, n6) = q(jj, k1, n6);
            q(jj, k, n5) = q(j, k1, n5);
            q(jj, k, n6) = q(j, k1, n6);
          }
        }
      }
    } else if (t == 46) {
      /* komegabc_inf, :1298-1332 */
      for (int k = ks; k <= ke; ++k) for (int j = js; j <= je; ++j) {
        q(j, k, n5) = p.tkeinf * rho(j, k);
        q(j, k, n6) = p.tomegainf * rho(j, k);
      }
    } else if (t == 47) {
      /* komegabc_out, :1335-1432 */
      if (iadir == 1) {
        const int j = (idir == 1) ? je : js, j1 = j + iadd;
        for (int k = ks; k <= ke; ++k) {
          q(j, k, n5) = p.tkeinf * rho(j, k);
          q(j, k, n6) = p.tomegainf * rho(j, k);
          double uu = (u(j, k) - ug(j, k) + u(j1, k) - ug(j1, k)) * xx(j, k);
          uu = uu + (v(j, k) - vg(j, k) + v(j1, k) - vg(j1, k)) * xy(j, k);
          uu = uu * iadd;
          if (uu < 0.) { q(j, k, n5) = q(j1, k, n5); q(j, k, n6) = q(j1, k, n6); }
        }
        for (int jc = 1; jc <= je - js; ++jc) {
          const int jj = (idir == 1) ? je - jc : js + jc, jj1 = jj + iadd;
          for (int k = ks; k <= ke; ++k) { q(jj, k, n5) = q(jj1, k, n5); q(jj, k, n6) = q(jj1, k, n6); }
        }
      } else if (iadir == 2) {
        const int k = (idir == 2) ? ke : ks, k1 = k + iadd;
        for (int j = js; j <= je; ++j) {
          q(j, k, n5) = p.tkeinf * rho(j, k);
          q(j, k, n6) = p.tomegainf * rho(j, k);
          double uu = (u(j, k) - ug(j, k) + u(j, k1) - ug(j, k1)) * yx(j, k);
          uu = uu + (v(j, k) - vg(j, k) + v(j, k1) - vg(j, k1)) * yy(j, k);
          uu = uu * iadd;
          if (uu < 0.) { q(j, k, n5) = q(j, k1, n5); q(j, k, n6) = q(j, k1, n6); }
        }
        for (int kc = 1; kc <= ke - ks; ++kc) {
          const int kk = (idir == 2) ? ke - kc : ks + kc, kk1 = kk + iadd;
          for (int j = js; j <= je; ++j) { q(j, kk, n5) = q(j, kk1, n5); q(j, kk, n6) = q(j, kk1, n6); }
        }
      }
    }
  }
}

/* komegasst.f:1435-1475 (one equation) */
static void lsolvej2(A2 a, A2 b, A2 c, A2 s, int js, int je, int ks, int ke) {
  for (int k = ks; k <= ke; ++k) { double bb = 1. / b(js, k); s(js, k) = s(js, k) * bb; c(js, k) = c(js, k) * bb; }
  for (int j = js + 1; j <= je; ++j) for (int k = ks; k <= ke; ++k) {
    double bb = 1. / (b(j, k) - a(j, k) * c(j - 1, k));
    s(j, k) = (s(j, k) - a(j, k) * s(j - 1, k)) * bb;
    c(j, k) = c(j, k) * bb;
  }
  for (int j = je - 1; j >= js; --j) for (int k = ks; k <= ke; ++k) s(j, k) = s(j, k) - c(j, k) * s(j + 1, k);
}

/* komegasst.f:1478-1518 (one equation) */
static void lsolvek2(A2 a, A2 b, A2 c, A2 s, int js, int je, int ks, int ke) {
  for (int j = js; j <= je; ++j) { double bb = 1. / b(j, ks); s(j, ks) = s(j, ks) * bb; c(j, ks) = c(j, ks) * bb; }
  for (int k = ks + 1; k <= ke; ++k) for (int j = js; j <= je; ++j) {
    double bb = 1. / (b(j, k) - a(j, k) * c(j, k - 1));
    s(j, k) = (s(j, k) - a(j, k) * s(j, k - 1)) * bb;
    c(j, k) = c(j, k) * bb;
  }
  for (int k = ke - 1; k >= ks; --k) for (int j = js; j <= je; ++j) s(j, k) = s(j, k) - c(j, k) * s(j, k + 1);
}

/* komegasst.f:2-187 (itrans = 0) */
void komegasst(const P& p, A3 q, A3 s, A2 turmu, A2 x, A2 y, const double* xv, const double* yv, A2 xx, A2 xy,
               A2 yx, A2 yy, A2 ug, A2 vg, A2 tscale, I2 iblank, double* res_out) {
  const int jd = p.jd, kd = p.kd, nq = p.nq, nmv = p.nmv;
  const int js = p.jbeg, je = p.jend, ks = p.kbeg, ke = p.kend;
  const size_t n2 = (size_t)jd * kd;
  std::vector<double> buf(n2 * 34, 0.0);
  int slot = 0;
  auto mk = [&]() { return A2{buf.data() + n2 * (slot++), jd}; };
  A2 bjmat[2] = {mk(), mk()}, sjmat[2] = {mk(), mk()}, aj[2] = {mk(), mk()}, cj[2] = {mk(), mk()};
  A2 ak[2] = {mk(), mk()}, ck[2] = {mk(), mk()};
  A2 rho = mk(), u = mk(), v = mk(), vmul = mk(), tauxx = mk(), tauxy = mk(), tauyy = mk();
  A2 ux = mk(), uy = mk(), vx = mk(), vy = mk(), cdkw = mk(), F1 = mk(), F2 = mk(), sn = mk();
  A2 vort = mk(), strain = mk();
  const double tkelim = 1e-20, tomegalim = 1e-20;
  lamvis(p, q, vmul);
  for (int k = 1; k <= kd; ++k) for (int j = 1; j <= jd; ++j) {
    rho(j, k) = q(j, k, 1) * q(j, k, nq);
    u(j, k) = q(j, k, 2) / q(j, k, 1);
    v(j, k) = q(j, k, 3) / q(j, k, 1);
    sn(j, k) = 1.e10;
  }
  komegabc(p, q, vmul, rho, x, y, xv, yv, u, v, ug, vg, xx, xy, yx, yy);
  bool bodyflag = false;
  for (int ib = 0; ib < p.nbc; ++ib) if (p.ibtyp[ib] == 5) bodyflag = true;
  if (bodyflag) dist(p, sn, x, y, xv, yv);
  kwvortic(vort, strain, u, v, xx, xy, yx, yy, js, je, ks, ke);
  turbstress(p, q, turmu, tauxx, tauxy, tauyy, u, v, ux, uy, vx, vy, xx, xy, yx, yy, js, je, ks, ke);
  crossdiff(p, q, rho, cdkw, xx, xy, yx, yy, js, je, ks, ke);
  blend(p, q, rho, vmul, cdkw, sn, F1, F2, js, je, ks, ke);
  findturm(p, q, rho, strain, F2, turmu);
  komegarhslhs(p, q, s, vmul, turmu, tauxx, tauxy, tauyy, cdkw, ux, uy, vx, vy, F1, rho, u, v, ug, vg, xx, xy, yx,
               yy, aj, bjmat, cj, ak, ck, sjmat, js, je, ks, ke);
  /* time accuracy factor and scaling (:100-131) */
  double oat = 1.0;
  if (p.ntac == -2) oat = 0.5;
  if (p.ntac >= 2 && p.istep > 1) oat = 2. / 3.;
  if (p.ntac == 3 && p.istep > 2) oat = 6. / 11.;
  for (int k = ks; k <= ke; ++k) for (int j = js; j <= je; ++j) {
    double tscal = tscale(j, k);
    if (p.timeac == 1) {
      const double dtpseudo_turb = 10.0;
      const double ib = (double)(iblank(j, k) > 0 ? iblank(j, k) : 0);
      tscal = ib * (1.0 + 0.002 * std::sqrt(q(j, k, nq))) / (1. + std::sqrt(q(j, k, nq)));
      tscal = tscal * dtpseudo_turb;
      tscal = tscal / (1. + tscal / p.h / oat);
    }
    for (int n = 0; n < 2; ++n) {
      aj[n](j, k) = aj[n](j, k) * tscal;
      cj[n](j, k) = cj[n](j, k) * tscal;
      ak[n](j, k) = ak[n](j, k) * tscal;
      ck[n](j, k) = ck[n](j, k) * tscal;
      bjmat[n](j, k) = 1. + bjmat[n](j, k) * tscal;
      sjmat[n](j, k) = sjmat[n](j, k) * tscal;
    }
  }
  for (int n = 0; n < 2; ++n) lsolvej2(aj[n], bjmat[n], cj[n], sjmat[n], js, je, ks, ke);
  for (int k = ks; k <= ke; ++k) for (int j = js; j <= je; ++j)
    for (int n = 0; n < 2; ++n) sjmat[n](j, k) = sjmat[n](j, k) * bjmat[n](j, k);
  for (int n = 0; n < 2; ++n) lsolvek2(ak[n], bjmat[n], ck[n], sjmat[n], js, je, ks, ke);
  /* update (:135-165) */
  const double relfac = 1.;
  double restke = 0.0, restomega = 0.0;
  for (int k = ks; k <= ke; ++k) for (int j = js; j <= je; ++j) {
    s(j, k, nmv + 1) = relfac * sjmat[0](j, k);
    s(j, k, nmv + 2) = relfac * sjmat[1](j, k);
    const double ib = (double)(iblank(j, k) > 0 ? iblank(j, k) : 0);
    q(j, k, nmv + 1) = q(j, k, nmv + 1) + s(j, k, nmv + 1) * ib;
    q(j, k, nmv + 2) = q(j, k, nmv + 2) + s(j, k, nmv + 2) * ib;
    q(j, k, nmv + 1) = fmax2(q(j, k, nmv + 1), tkelim * rho(j, k));
    q(j, k, nmv + 2) = fmax2(q(j, k, nmv + 2), tomegalim * rho(j, k));
    restke = restke + p2(s(j, k, nmv + 1));
    restomega = restomega + p2(s(j, k, nmv + 2));
  }
  if (res_out) {
    res_out[0] = std::sqrt(restke / p.jmax / p.kmax);
    res_out[1] = std::sqrt(restomega / p.jmax / p.kmax);
  }
  komegabc(p, q, vmul, rho, x, y, xv, yv, u, v, ug, vg, xx, xy, yx, yy);
  findturm(p, q, rho, strain, F2, turmu);
}

}  // namespace oro
