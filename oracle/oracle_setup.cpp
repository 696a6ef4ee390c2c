/*
 * oracle_setup.cpp -- TEST INFRASTRUCTURE ONLY (see oracle_common.h).
 * FP64 restatement of the reference's setup path: derived constants
 * (read_inputs), cell centres, finite-volume metrics, freestream state and
 * the time-spectral operator.
 */
#include <cstdlib>
#include <cstring>
#include "oracle.h"

namespace oro {

/* read_inputs: setup.f:960-971 (timespectral/nspec), :982-986 (invisc/lamin),
 * :1162-1204 (freestream and nq/nv), :1230 (h=dt), :1233-1235 (SST
 * freestream), :1262-1265 (nadd); set_pointers_globals: setup.f:73-98;
 * jtail from the wall bc: init.f:59-66; defaults: modules.f:170-190. */
void read_inputs(const ot2d_inputs& in, P& p) {
  std::memset(&p, 0, sizeof(p));
  const double pi = 4.0 * std::atan(1.0);
  p.gamma = 1.4; p.pr = 0.72; p.rmue = 1.0; p.tinf = 400.0;   /* modules.f:172 */
  p.jmax = in.jmax; p.kmax = in.kmax; p.nhalo = in.nhalo; p.half = in.half;
  p.invisc = in.invisc; p.lamin = in.lamin; p.iturb = in.iturb; p.itrans = in.itrans;
  p.irhsy = in.irhsy; p.ilim = in.ilim; p.ilhs = in.ilhs;
  p.iconstant_cfl = in.iconstant_cfl; p.idual = in.idual; p.idual_turb = in.idual_turb;
  p.iunst = in.iunst; p.ntac = in.ntac; p.itnmax = in.itnmax; p.iread = in.iread;
  p.timespectral = in.timespectral; p.nspec = in.nspec; p.motiontype = in.motiontype;
  p.npnorm = in.npnorm;
  p.fsmach = in.fsmach; p.fmtip = in.fmtip; p.alfa = in.alfa; p.rey = in.rey;
  p.vnuinf = in.vnuinf; p.dt = in.dt; p.timeac = in.timeac; p.epse = in.epse;
  p.cfltur = in.cfltur; p.rf = in.rf; p.angmax = in.angmax; p.xac = in.xac; p.yac = in.yac;
  p.Mp = 1.0; p.iprecon = 0; p.dualtime = 1.0;
  p.nbc = in.nbc;
  for (int i = 0; i < OT2D_MAXBC; ++i) {
    p.ibtyp[i] = in.ibtyp[i]; p.ibdir[i] = in.ibdir[i];
    p.jbcs[i] = in.jbcs[i]; p.jbce[i] = in.jbce[i];
    p.kbcs[i] = in.kbcs[i]; p.kbce[i] = in.kbce[i];
  }
  if (p.timespectral) p.iunst = 0; else p.nspec = 1;
  if (p.invisc) { p.rmue = 0.0; p.lamin = 1; }
  if (p.lamin) p.iturb = -1;
  p.gm1 = p.gamma - 1.0;
  p.ggm1 = p.gamma * p.gm1;
  double cs = std::cos(pi * p.alfa / 180.0);
  double ss = std::sin(pi * p.alfa / 180.0);
  p.theta_col = p.alfa;
  p.einf = 1.0 / p.ggm1 + 0.5 * p2(p.fsmach);
  p.pinf = 1.0 / p.gamma;
  p.rinf = 1.0;
  p.ainf = p.gamma * p.pinf / p.rinf;
  p.htinf = p.gamma * p.einf / p.rinf - 0.5 * p.gm1 * p2(p.fsmach);
  p.nq = 5; p.nv = 4; p.nmv = 4; p.nturb = 0;
  if (p.iturb == 1) { p.nturb = 1; p.nq += 1; p.nv += 1; }
  else if (p.iturb == 2) { p.nturb = 2; p.nq += 2; p.nv += 2; }
  p.uinf = p.fsmach * cs;
  p.vinf = p.fsmach * ss;
  if (p.fsmach != 0) p.rey = p.rey / p.fsmach; else p.rey = p.rey / p.fmtip;
  p.h = p.dt;
  p.tkeinf = 1e-6 * p2(p.fsmach);
  p.tomegainf = 5 * p.fsmach / p.rey;
  p.nadd = 2 * p.nhalo - 1;
  p.jd = p.jmax + p.nadd; p.kd = p.kmax + p.nadd;
  /* set_pointers_globals */
  p.jbeg = p.nhalo + 1; p.kbeg = p.nhalo + 1;
  p.jend = p.jd - p.nhalo; p.kend = p.kd - p.nhalo;
  int jtail = 1;
  for (int ib = 0; ib < p.nbc; ++ib) if (p.ibtyp[ib] == 5) jtail = p.jbcs[ib];
  p.jtail1 = jtail + p.nhalo;
  if (p.half == 0) { p.jle = (p.jd + 1) / 2; p.jtail2 = p.jd - p.jtail1 + 1; }
  else { p.jle = p.jd - 1; p.jtail2 = p.jd - 1; }
  if (p.rf != 0) p.rotf = 1 * p.rf;
  p.istep = 0; p.istep0 = 0; p.itn = 1;
}

/* setup.f:111-345 */
void find_cellcenter(const P& p, A2 x, A2 y, const double* xv_, const double* yv_) {
  const int jd = p.jd, kd = p.kd, jmax = p.jmax, nhalo = p.nhalo;
  const int jbeg = p.jbeg, jend = p.jend, kbeg = p.kbeg, kend = p.kend;
  auto xv = [&](int j, int k) { return xv_[(size_t)(k - 1) * jmax + (j - 1)]; };
  auto yv = [&](int j, int k) { return yv_[(size_t)(k - 1) * jmax + (j - 1)]; };
  for (int k = 1; k <= kd; ++k) for (int j = 1; j <= jd; ++j) { x(j, k) = 0.; y(j, k) = 0.; }
  for (int j = jbeg; j <= jend; ++j)
    for (int k = kbeg; k <= kend; ++k) {
      int jv = j - nhalo + 1, kv = k - nhalo + 1;
      x(j, k) = 0.25 * (xv(jv, kv) + xv(jv - 1, kv) + xv(jv, kv - 1) + xv(jv - 1, kv - 1));
      y(j, k) = 0.25 * (yv(jv, kv) + yv(jv - 1, kv) + yv(jv, kv - 1) + yv(jv - 1, kv - 1));
    }
  int j = jbeg - 1, k;
  for (k = kbeg; k <= kend; ++k) {
    int jv = j - nhalo + 1, kv = k - nhalo + 1;
    x(j, k) = x(j + 1, k) - 0.5 * (xv(jv + 1, kv) - xv(jv, kv) + xv(jv + 1, kv - 1) - xv(jv, kv - 1));
    y(j, k) = y(j + 1, k) - 0.5 * (yv(jv + 1, kv) - yv(jv, kv) + yv(jv + 1, kv - 1) - yv(jv, kv - 1));
  }
  j = jend + 1;
  for (k = kbeg; k <= kend; ++k) {
    int jv = j - nhalo + 1, kv = k - nhalo + 1;
    x(j, k) = x(j - 1, k) - 0.5 * (xv(jv - 2, kv) - xv(jv - 1, kv) + xv(jv - 2, kv - 1) - xv(jv - 1, kv - 1));
    y(j, k) = y(j - 1, k) - 0.5 * (yv(jv - 2, kv) - yv(jv - 1, kv) + yv(jv - 2, kv - 1) - yv(jv - 1, kv - 1));
  }
  k = kbeg - 1;
  for (j = jbeg; j <= jend; ++j) {
    int jv = j - nhalo + 1, kv = k - nhalo + 1;
    x(j, k) = x(j, k + 1) - 0.5 * (xv(jv, kv + 1) - xv(jv, kv) + xv(jv - 1, kv + 1) - xv(jv - 1, kv));
    y(j, k) = y(j, k + 1) - 0.5 * (yv(jv, kv + 1) - yv(jv, kv) + yv(jv - 1, kv + 1) - yv(jv - 1, kv));
  }
  k = kend + 1;
  for (j = jbeg; j <= jend; ++j) {
    int jv = j - nhalo + 1, kv = k - nhalo + 1;
    x(j, k) = x(j, k - 1) - 0.5 * (xv(jv, kv - 2) - xv(jv, kv - 1) + xv(jv - 1, kv - 2) - xv(jv - 1, kv - 1));
    y(j, k) = y(j, k - 1) - 0.5 * (yv(jv, kv - 2) - yv(jv, kv - 1) + yv(jv - 1, kv - 2) - yv(jv - 1, kv - 1));
  }
  j = jbeg - 1; k = kbeg - 1;
  x(j, k) = 2 * x(j + 1, k) - x(j + 2, k); y(j, k) = 2 * y(j + 1, k) - y(j + 2, k);
  k = kend + 1;
  x(j, k) = 2 * x(j + 1, k) - x(j + 2, k); y(j, k) = 2 * y(j + 1, k) - y(j + 2, k);
  j = jend + 1; k = kbeg - 1;
  x(j, k) = 2 * x(j, k + 1) - x(j, k + 2); y(j, k) = 2 * y(j, k + 1) - y(j, k + 2);
  k = kend + 1;
  x(j, k) = 2 * x(j, k - 1) - x(j, k - 2); y(j, k) = 2 * y(j, k - 1) - y(j, k - 2);
  for (int nh = 2; nh <= nhalo; ++nh) {
    j = jbeg - nh;
    for (k = kbeg - nh + 1; k <= kend + nh - 1; ++k) { x(j, k) = 2 * x(j + 1, k) - x(j + 2, k); y(j, k) = 2 * y(j + 1, k) - y(j + 2, k); }
    j = jend + nh;
    for (k = kbeg - nh + 1; k <= kend + nh - 1; ++k) { x(j, k) = 2 * x(j - 1, k) - x(j - 2, k); y(j, k) = 2 * y(j - 1, k) - y(j - 2, k); }
    k = kbeg - nh;
    for (j = jbeg - nh + 1; j <= jend + nh - 1; ++j) { x(j, k) = 2 * x(j, k + 1) - x(j, k + 2); y(j, k) = 2 * y(j, k + 1) - y(j, k + 2); }
    k = kend + nh;
    for (j = jbeg - nh + 1; j <= jend + nh - 1; ++j) { x(j, k) = 2 * x(j, k - 1) - x(j, k - 2); y(j, k) = 2 * y(j, k - 1) - y(j, k - 2); }
    j = jbeg - nh; k = kbeg - nh;
    x(j, k) = 2 * x(j + 1, k) - x(j + 2, k); y(j, k) = 2 * y(j + 1, k) - y(j + 2, k);
    k = kend + nh;
    x(j, k) = 2 * x(j + 1, k) - x(j + 2, k); y(j, k) = 2 * y(j + 1, k) - y(j + 2, k);
    j = jend + nh; k = kbeg - nh;
    x(j, k) = 2 * x(j, k + 1) - x(j, k + 2); y(j, k) = 2 * y(j, k + 1) - y(j, k + 2);
    k = kend + nh;
    x(j, k) = 2 * x(j, k - 1) - x(j, k - 2); y(j, k) = 2 * y(j, k - 1) - y(j, k - 2);
  }
  for (int ib = 0; ib < p.nbc; ++ib) {
    int js, je, ks, ke; bc_range(p, ib, js, je, ks, ke);
    int idir = p.ibdir[ib], iadir = std::abs(idir);
    if (p.ibtyp[ib] == 22) {
      if (idir == 1) {
        int jj = je - js + 1;
        for (j = js; j <= je; ++j) { int jj1 = j - js + 1, jc = jd - 2 * jj + jj1;
          for (k = ks; k <= ke; ++k) { x(j, k) = x(jc, k); y(j, k) = y(jc, k); } }
      } else if (idir == -1) {
        int jj = je - js + 1;
        for (j = js; j <= je; ++j) { int jj1 = je - j + 1, jc = 1 + 2 * jj - jj1;
          for (k = ks; k <= ke; ++k) { x(j, k) = x(jc, k); y(j, k) = y(jc, k); } }
      } else if (idir == 2) {
        int kk = ke - ks + 1;
        for (k = ks; k <= ke; ++k) { int kk1 = k - ks + 1, kc = kd - 2 * kk + kk1;
          for (j = js; j <= je; ++j) { x(j, k) = x(j, kc); y(j, k) = y(j, kc); } }
      } else if (idir == -2) {
        int kk = ke - ks + 1;
        for (k = ks; k <= ke; ++k) { int kk1 = ke - k + 1, kc = 1 + 2 * kk - kk1;
          for (j = js; j <= je; ++j) { x(j, k) = x(j, kc); y(j, k) = y(j, kc); } }
      }
    } else if (p.ibtyp[ib] == 51 && iadir == 2) {
      for (int kc = 1; kc <= ke - ks + 1; ++kc) {
        int k1;
        if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
        for (j = js; j <= je; ++j) {
          int jj = jd - j + 1;
          x(j, k) = x(jj, k1); y(j, k) = y(jj, k1);
          x(jj, k) = x(j, k1); y(jj, k) = y(j, k1);
        }
      }
    }
  }
}

/* setup.f:440-724 */
int metfv(const P& p, A3 q, const double* xv_, const double* yv_, A2 xx, A2 xy, A2 yx, A2 yy) {
  const int jd = p.jd, kd = p.kd, jmax = p.jmax, kmax = p.kmax, nhalo = p.nhalo, nq = p.nq;
  const int jbeg = p.jbeg, jend = p.jend, kbeg = p.kbeg, kend = p.kend;
  auto xv = [&](int j, int k) { return xv_[(size_t)(k - 1) * jmax + (j - 1)]; };
  auto yv = [&](int j, int k) { return yv_[(size_t)(k - 1) * jmax + (j - 1)]; };
  for (int k = 2; k <= kmax; ++k)
    for (int j = 2; j <= jmax; ++j) {
      int jc = j + nhalo - 1, kc = k + nhalo - 1;
      double dx1 = xv(j, k) - xv(j - 1, k - 1);
      double dy1 = yv(j, k) - yv(j - 1, k - 1);
      double dx2 = xv(j - 1, k) - xv(j, k - 1);
      double dy2 = yv(j - 1, k) - yv(j, k - 1);
      double a3 = 0.5 * (dx1 * dy2 - dx2 * dy1);
      q(jc, kc, nq) = 1. / a3;
    }
  for (int j = 2; j <= jmax; ++j)
    for (int k = 2; k <= kmax; ++k) {
      int jc = j + nhalo - 1, kc = k + nhalo - 1;
      xx(jc, kc) = 0.5 * (yv(j, k) - yv(j, k - 1) + yv(j - 1, k) - yv(j - 1, k - 1));
      xy(jc, kc) = -0.5 * (xv(j, k) - xv(j, k - 1) + xv(j - 1, k) - xv(j - 1, k - 1));
    }
  for (int k = 2; k <= kmax; ++k)
    for (int j = 2; j <= jmax; ++j) {
      int jc = j + nhalo - 1, kc = k + nhalo - 1;
      yx(jc, kc) = -0.5 * (yv(j, k) - yv(j - 1, k) + yv(j, k - 1) - yv(j - 1, k - 1));
      yy(jc, kc) = 0.5 * (xv(j, k) - xv(j - 1, k) + xv(j, k - 1) - xv(j - 1, k - 1));
    }
  for (int k = kbeg; k <= kend; ++k)
    for (int j = jbeg; j <= jend; ++j) {
      double qj = q(j, k, nq);
      xx(j, k) = qj * (xx(j, k)); xy(j, k) = qj * (xy(j, k));
      yx(j, k) = qj * (yx(j, k)); yy(j, k) = qj * (yy(j, k));
    }
  auto cp = [&](int j, int k, int j1, int k1) {
    q(j, k, nq) = q(j1, k1, nq);
    xx(j, k) = xx(j1, k1); xy(j, k) = xy(j1, k1); yx(j, k) = yx(j1, k1); yy(j, k) = yy(j1, k1);
  };
  for (int nh = 1; nh <= nhalo; ++nh) {
    int j = jbeg - nh, j1 = jbeg + nh - 1;
    for (int k = kbeg - nh + 1; k <= kend + nh - 1; ++k) cp(j, k, j1, k);
    j = jend + nh; j1 = jend - nh + 1;
    for (int k = kbeg - nh + 1; k <= kend + nh - 1; ++k) cp(j, k, j1, k);
    int k = kbeg - nh, k1 = kbeg + nh - 1;
    for (j = jbeg - nh; j <= jend + nh; ++j) cp(j, k, j, k1);
    k = kend + nh; k1 = kend - nh + 1;
    for (j = jbeg - nh; j <= jend + nh; ++j) cp(j, k, j, k1);
  }
  for (int ib = 0; ib < p.nbc; ++ib) {
    int js, je, ks, ke; bc_range(p, ib, js, je, ks, ke);
    int idir = p.ibdir[ib], iadir = std::abs(idir);
    if (p.ibtyp[ib] == 22) {
      if (idir == 1) {
        int jj = je - js + 1;
        for (int j = js; j <= je; ++j) { int jj1 = j - js + 1, jc = jd - 2 * jj + jj1;
          for (int k = ks; k <= ke; ++k) cp(j, k, jc, k); }
      } else if (idir == -1) {
        int jj = je - js + 1;
        for (int j = js; j <= je; ++j) { int jj1 = je - j + 1, jc = 1 + 2 * jj - jj1;
          for (int k = ks; k <= ke; ++k) cp(j, k, jc, k); }
      } else if (idir == 2) {
        int kk = ke - ks + 1;
        for (int k = ks; k <= ke; ++k) { int kk1 = k - ks + 1, kc = kd - 2 * kk + kk1;
          for (int j = js; j <= je; ++j) cp(j, k, j, kc); }
      } else if (idir == -2) {
        int kk = ke - ks + 1;
        for (int k = ks; k <= ke; ++k) { int kk1 = ke - k + 1, kc = 1 + 2 * kk - kk1;
          for (int j = js; j <= je; ++j) cp(j, k, j, kc); }
      }
    } else if (p.ibtyp[ib] == 51 && iadir == 2) {
      for (int kc = 1; kc <= ke - ks + 1; ++kc) {
        int k, k1;
        if (idir == 2) { k = ke - kc + 1; k1 = ke + kc; } else { k = ks + kc - 1; k1 = ks - kc; }
        for (int j = js; j <= je; ++j) {
          int jj = jd - j + 1;
          q(j, k, nq) = q(jj, k1, nq);
          xx(j, k) = -xx(jj, k1); xy(j, k) = -xy(jj, k1); yx(j, k) = -yx(jj, k1); yy(j, k) = -yy(jj, k1);
          q(jj, k, nq) = q(j, k1, nq);
          xx(jj, k) = -xx(j, k1); xy(jj, k) = -xy(j, k1); yx(jj, k) = -yx(j, k1); yy(jj, k) = -yy(j, k1);
        }
      }
    }
  }
  int nneg = 0;
  for (int k = 1; k <= kd; ++k) for (int j = 1; j <= jd; ++j) if (q(j, k, nq) <= 0.0) ++nneg;
  return nneg;
}

/* init.f:209-277 */
void qzero(const P& p, A3 q) {
  double ruinf = p.rinf * p.uinf, rvinf = p.rinf * p.vinf;
  for (int k = 1; k <= p.kd; ++k) for (int j = 1; j <= p.jd; ++j) {
    q(j, k, 1) = p.rinf; q(j, k, 2) = ruinf; q(j, k, 3) = rvinf; q(j, k, 4) = p.einf;
  }
  if (p.iturb == 1) {
    for (int k = 1; k <= p.kd; ++k) for (int j = 1; j <= p.jd; ++j) q(j, k, 5) = p.vnuinf;
  } else if (p.iturb == 2) {
    double rtkeinf = p.rinf * p.tkeinf, rtomegainf = p.rinf * p.tomegainf;
    for (int k = 1; k <= p.kd; ++k) for (int j = 1; j <= p.jd; ++j) { q(j, k, 5) = rtkeinf; q(j, k, 6) = rtomegainf; }
  }
}

/* init.f:180-206 */
void qdivj(const P& p, A3 q) {
  for (int k = 1; k <= p.kd; ++k) for (int j = 1; j <= p.jd; ++j)
    for (int n = 1; n <= 4; ++n) q(j, k, n) = q(j, k, n) / q(j, k, p.nq);
}

/* setup.f:838-873 ; Ds(N,N) column-major */
void computeTScoefs(int N, double* Ds) {
  const double pi = 4. * std::atan(1.);
  for (int i = 1; i <= N; ++i)
    for (int j = 1; j <= N; ++j) {
      double& d = Ds[(size_t)(j - 1) * N + (i - 1)];
      int e = i - j; double sgn = ((e % 2) == 0) ? 1.0 : -1.0;
      if (i == j) d = 0.;
      else if (N % 2 == 0) d = 0.5 * sgn / std::tan(pi * e / N);
      else d = 0.5 * sgn / std::sin(pi * e / N);
    }
}

/* setup.f:396-438 (motiontype=1) */
void find_coord_TS_orig(const P& p, double* xv, double* yv, const double* xv1, const double* yv1, double tspec) {
  const double pi = 4.0 * std::atan(1.0);
  double theta = p.angmax * pi / 180. * std::sin(p.rotf * tspec);
  double ss = std::sin(theta), cs = std::cos(theta);
  size_t n = (size_t)p.jmax * p.kmax;
  for (size_t i = 0; i < n; ++i) {
    xv[i] = (xv1[i] - p.xac) * cs + (yv1[i] - p.yac) * ss + p.xac;
    yv[i] = (yv1[i] - p.yac) * cs - (xv1[i] - p.xac) * ss + p.yac;
  }
}

/* setup.f:789-835 (motiontype=1) */
void find_timemetrics_TS_orig(const P& p, A2 x, A2 y, const double* xv, const double* yv, double tspec,
                              A2 ug, A2 vg, double* ugv, double* vgv) {
  const double pi = 4.0 * std::atan(1.0);
  for (int k = 1; k <= p.kd; ++k) for (int j = 1; j <= p.jd; ++j) {
    ug(j, k) = p.angmax * pi / 180. * p.rotf * (y(j, k) - p.yac) * std::cos(p.rotf * tspec);
    vg(j, k) = -p.angmax * pi / 180. * p.rotf * (x(j, k) - p.xac) * std::cos(p.rotf * tspec);
  }
  size_t n = (size_t)p.jmax * p.kmax;
  for (size_t i = 0; i < n; ++i) {
    ugv[i] = p.angmax * pi / 180. * p.rotf * (yv[i] - p.yac) * std::cos(p.rotf * tspec);
    vgv[i] = -p.angmax * pi / 180. * p.rotf * (xv[i] - p.xac) * std::cos(p.rotf * tspec);
  }
}

}  // namespace oro
