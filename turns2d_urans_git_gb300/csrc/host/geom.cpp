/*
 * geom.cpp -- per-request geometry set-up on the host (FP64), computed once
 * at admission and uploaded:
 *   cell centres      find_cellcenter   src/setup.f:111-345
 *   metrics, J        metfv             src/setup.f:440-724
 *   SA wall distance  dist              src/samodel2d.f:243-293
 *   face normals      rhsup             src/eulerrhs.f:102-116, :209-223
 *   swept-area face speeds of a moving grid (drop-in path)
 *                     rhsup             src/eulerrhs.f:118-139, :224-246
 *   time-spectral pitching grid and grid speeds (sine form)
 *                     find_coord_TS_orig / find_timemetrics_TS_orig
 *                     src/setup.f:396-438, :789-835; tj: eulerrhs.f:140-146
 *   Ds                computeTScoefs    src/setup.f:838-873
 * Built with -ffp-contract=off: every a*b+c rounds twice, as the reference.
 */
#include "geom.h"

#include <cmath>
#include <cstdlib>

namespace ot2d {

namespace {
struct C2 {  // column-major (jd,kd) view, 1-based
  double* p; int jd;
  double& operator()(int j, int k) const { return p[(size_t)(k - 1) * jd + (j - 1)]; }
};
struct V2 {  // vertex (jmax,kmax) view, 1-based
  const double* p; int jm;
  double operator()(int j, int k) const { return p[(size_t)(k - 1) * jm + (j - 1)]; }
};
inline int isgn(int idir) { return idir >= 0 ? 1 : -1; }
}  // namespace

void bc_cells(const ot2d_params& p, int ib, int& js, int& je, int& ks, int& ke) {
  js = p.jbcs[ib]; je = p.jbce[ib]; ks = p.kbcs[ib]; ke = p.kbce[ib];
  if (js < 0) js = p.jmax + js + 1;
  if (ks < 0) ks = p.kmax + ks + 1;
  if (je < 0) je = p.jmax + je + 1;
  if (ke < 0) ke = p.kmax + ke + 1;
  if (js > 1) js += p.nhalo;
  if (ks > 1) ks += p.nhalo;
  if (je < p.jmax) je += p.nhalo - 1;
  if (ke < p.kmax) ke += p.nhalo - 1;
  if (je == p.jmax) je = p.jd;
  if (ke == p.kmax) ke = p.kd;
}

void cell_centres(const ot2d_params& p, const double* xv_, const double* yv_, double* x_, double* y_) {
  const int jd = p.jd, kd = p.kd, nh = p.nhalo;
  const int jb = p.jbeg, je = p.jend, kb = p.kbeg, ke = p.kend;
  C2 x{x_, jd}, y{y_, jd};
  V2 xv{xv_, p.jmax}, yv{yv_, p.jmax};
  for (int k = 1; k <= kd; ++k)
    for (int j = 1; j <= jd; ++j) { x(j, k) = 0.; y(j, k) = 0.; }
  for (int j = jb; j <= je; ++j)
    for (int k = kb; k <= ke; ++k) {
      const int a = j - nh + 1, b = k - nh + 1;
      x(j, k) = 0.25 * (xv(a, b) + xv(a - 1, b) + xv(a, b - 1) + xv(a - 1, b - 1));
      y(j, k) = 0.25 * (yv(a, b) + yv(a - 1, b) + yv(a, b - 1) + yv(a - 1, b - 1));
    }
  // first halo layer from the adjacent cell minus half a cell width
  for (int k = kb; k <= ke; ++k) {
    int j = jb - 1, a = j - nh + 1, b = k - nh + 1;
    x(j, k) = x(j + 1, k) - 0.5 * (xv(a + 1, b) - xv(a, b) + xv(a + 1, b - 1) - xv(a, b - 1));
    y(j, k) = y(j + 1, k) - 0.5 * (yv(a + 1, b) - yv(a, b) + yv(a + 1, b - 1) - yv(a, b - 1));
    j = je + 1; a = j - nh + 1;
    x(j, k) = x(j - 1, k) - 0.5 * (xv(a - 2, b) - xv(a - 1, b) + xv(a - 2, b - 1) - xv(a - 1, b - 1));
    y(j, k) = y(j - 1, k) - 0.5 * (yv(a - 2, b) - yv(a - 1, b) + yv(a - 2, b - 1) - yv(a - 1, b - 1));
  }
  for (int j = jb; j <= je; ++j) {
    int k = kb - 1, a = j - nh + 1, b = k - nh + 1;
    x(j, k) = x(j, k + 1) - 0.5 * (xv(a, b + 1) - xv(a, b) + xv(a - 1, b + 1) - xv(a - 1, b));
    y(j, k) = y(j, k + 1) - 0.5 * (yv(a, b + 1) - yv(a, b) + yv(a - 1, b + 1) - yv(a - 1, b));
    k = ke + 1; b = k - nh + 1;
    x(j, k) = x(j, k - 1) - 0.5 * (xv(a, b - 2) - xv(a, b - 1) + xv(a - 1, b - 2) - xv(a - 1, b - 1));
    y(j, k) = y(j, k - 1) - 0.5 * (yv(a, b - 2) - yv(a, b - 1) + yv(a - 1, b - 2) - yv(a - 1, b - 1));
  }
  // corners by linear extrapolation (nhalo = 1)
  auto ex = [&](int j, int k, int j1, int k1, int j2, int k2) {
    x(j, k) = 2 * x(j1, k1) - x(j2, k2);
    y(j, k) = 2 * y(j1, k1) - y(j2, k2);
  };
  ex(jb - 1, kb - 1, jb, kb - 1, jb + 1, kb - 1);
  ex(jb - 1, ke + 1, jb, ke + 1, jb + 1, ke + 1);
  ex(je + 1, kb - 1, je + 1, kb, je + 1, kb + 1);
  ex(je + 1, ke + 1, je + 1, ke, je + 1, ke - 1);
  // boundary-specific copies: periodic overlap (22) and the wake cut (51)
  for (int ib = 0; ib < p.nbc; ++ib) {
    int js, je2, ks, ke2; bc_cells(p, ib, js, je2, ks, ke2);
    const int idir = p.ibdir[ib], t = p.ibtyp[ib];
    if (t == 22) {
      if (idir == 1 || idir == -1) {
        const int n = je2 - js + 1;
        for (int j = js; j <= je2; ++j) {
          const int jc = (idir == 1) ? jd - 2 * n + (j - js + 1) : 1 + 2 * n - (je2 - j + 1);
          for (int k = ks; k <= ke2; ++k) { x(j, k) = x(jc, k); y(j, k) = y(jc, k); }
        }
      } else {
        const int n = ke2 - ks + 1;
        for (int k = ks; k <= ke2; ++k) {
          const int kc = (idir == 2) ? kd - 2 * n + (k - ks + 1) : 1 + 2 * n - (ke2 - k + 1);
          for (int j = js; j <= je2; ++j) { x(j, k) = x(j, kc); y(j, k) = y(j, kc); }
        }
      }
    } else if (t == 51 && (idir == 2 || idir == -2)) {
      for (int kc = 1; kc <= ke2 - ks + 1; ++kc) {
        const int k = (idir == 2) ? ke2 - kc + 1 : ks + kc - 1;
        const int k1 = (idir == 2) ? ke2 + kc : ks - kc;
        for (int j = js; j <= je2; ++j) {
          const int jj = jd - j + 1;
          x(j, k) = x(jj, k1); y(j, k) = y(jj, k1);
          x(jj, k) = x(j, k1); y(jj, k) = y(j, k1);
        }
      }
    }
  }
}

int metrics(const ot2d_params& p, const double* xv_, const double* yv_, double* J_, double* xx_, double* xy_,
            double* yx_, double* yy_) {
  const int jd = p.jd, kd = p.kd, nh = p.nhalo;
  C2 J{J_, jd}, xx{xx_, jd}, xy{xy_, jd}, yx{yx_, jd}, yy{yy_, jd};
  V2 xv{xv_, p.jmax}, yv{yv_, p.jmax};
  for (int k = 2; k <= p.kmax; ++k)
    for (int j = 2; j <= p.jmax; ++j) {
      const int jc = j + nh - 1, kc = k + nh - 1;
      // cell area from the two diagonals
      const double dx1 = xv(j, k) - xv(j - 1, k - 1), dy1 = yv(j, k) - yv(j - 1, k - 1);
      const double dx2 = xv(j - 1, k) - xv(j, k - 1), dy2 = yv(j - 1, k) - yv(j, k - 1);
      J(jc, kc) = 1. / (0.5 * (dx1 * dy2 - dx2 * dy1));
      xx(jc, kc) = 0.5 * (yv(j, k) - yv(j, k - 1) + yv(j - 1, k) - yv(j - 1, k - 1));
      xy(jc, kc) = -0.5 * (xv(j, k) - xv(j, k - 1) + xv(j - 1, k) - xv(j - 1, k - 1));
      yx(jc, kc) = -0.5 * (yv(j, k) - yv(j - 1, k) + yv(j, k - 1) - yv(j - 1, k - 1));
      yy(jc, kc) = 0.5 * (xv(j, k) - xv(j - 1, k) + xv(j, k - 1) - xv(j - 1, k - 1));
    }
  for (int k = p.kbeg; k <= p.kend; ++k)
    for (int j = p.jbeg; j <= p.jend; ++j) {
      const double qj = J(j, k);
      xx(j, k) = qj * xx(j, k); xy(j, k) = qj * xy(j, k);
      yx(j, k) = qj * yx(j, k); yy(j, k) = qj * yy(j, k);
    }
  auto cp = [&](int j, int k, int j1, int k1, double sgn) {
    J(j, k) = J(j1, k1);
    xx(j, k) = sgn * xx(j1, k1); xy(j, k) = sgn * xy(j1, k1);
    yx(j, k) = sgn * yx(j1, k1); yy(j, k) = sgn * yy(j1, k1);
  };
  for (int k = p.kbeg; k <= p.kend; ++k) { cp(p.jbeg - 1, k, p.jbeg, k, 1.0); cp(p.jend + 1, k, p.jend, k, 1.0); }
  for (int j = p.jbeg - 1; j <= p.jend + 1; ++j) { cp(j, p.kbeg - 1, j, p.kbeg, 1.0); cp(j, p.kend + 1, j, p.kend, 1.0); }
  for (int ib = 0; ib < p.nbc; ++ib) {
    int js, je2, ks, ke2; bc_cells(p, ib, js, je2, ks, ke2);
    const int idir = p.ibdir[ib], t = p.ibtyp[ib];
    if (t == 22) {
      if (idir == 1 || idir == -1) {
        const int n = je2 - js + 1;
        for (int j = js; j <= je2; ++j) {
          const int jc = (idir == 1) ? jd - 2 * n + (j - js + 1) : 1 + 2 * n - (je2 - j + 1);
          for (int k = ks; k <= ke2; ++k) cp(j, k, jc, k, 1.0);
        }
      } else {
        const int n = ke2 - ks + 1;
        for (int k = ks; k <= ke2; ++k) {
          const int kc = (idir == 2) ? kd - 2 * n + (k - ks + 1) : 1 + 2 * n - (ke2 - k + 1);
          for (int j = js; j <= je2; ++j) cp(j, k, j, kc, 1.0);
        }
      }
    } else if (t == 51 && (idir == 2 || idir == -2)) {
      // wake halo: mirrored cell across the cut, metrics negated (setup.f:662-691)
      for (int kc = 1; kc <= ke2 - ks + 1; ++kc) {
        const int k = (idir == 2) ? ke2 - kc + 1 : ks + kc - 1;
        const int k1 = (idir == 2) ? ke2 + kc : ks - kc;
        for (int j = js; j <= je2; ++j) {
          const int jj = jd - j + 1;
          cp(j, k, jj, k1, -1.0);
          cp(jj, k, j, k1, -1.0);
        }
      }
    }
  }
  int nneg = 0;
  for (int k = 1; k <= kd; ++k)
    for (int j = 1; j <= jd; ++j) if (J(j, k) <= 0.0) ++nneg;
  return nneg;
}

void wall_distance(const ot2d_params& p, const double* x_, const double* y_, const double* xv_, const double* yv_,
                   double* sn_) {
  const int jd = p.jd, kd = p.kd, nh = p.nhalo;
  C2 sn{sn_, jd};
  C2 x{const_cast<double*>(x_), jd}, y{const_cast<double*>(y_), jd};
  V2 xv{xv_, p.jmax}, yv{yv_, p.jmax};
  for (int k = 1; k <= kd; ++k)
    for (int j = 1; j <= jd; ++j) sn(j, k) = 1.e10;
  for (int j = p.jtail1; j <= p.jtail2; ++j) {
    sn(j, 1) = 0.0;
    const int a = j - nh;  // wall face of column j: vertices a, a+1 on k=1
    const double fx = 0.5 * (xv(a, 1) + xv(a + 1, 1)), fy = 0.5 * (yv(a, 1) + yv(a + 1, 1));
    for (int k = 2; k <= kd; ++k) {
      const double dx = x(j, k) - fx, dy = y(j, k) - fy;
      sn(j, k) = std::sqrt(dx * dx + dy * dy);
    }
  }
  // wake columns: distance to the trailing-edge vertex
  const int a = p.jtail1 - nh;
  for (int j = 1; j <= jd; ++j) {
    if (j >= p.jtail1 && j <= p.jtail2) continue;
    for (int k = 1; k <= kd; ++k) {
      const double dx = x(j, k) - xv(a, 1), dy = y(j, k) - yv(a, 1);
      sn(j, k) = std::sqrt(dx * dx + dy * dy);
    }
  }
}

void sst_wall_d2(const ot2d_params& p, const double* x_, const double* y_, const double* xv_, const double* yv_,
                 double* wd2_) {
  const int jd = p.jd, kd = p.kd, nh = p.nhalo;
  C2 wd2{wd2_, jd};
  C2 x{const_cast<double*>(x_), jd}, y{const_cast<double*>(y_), jd};
  V2 xv{xv_, p.jmax}, yv{yv_, p.jmax};
  for (int k = 1; k <= kd; ++k)
    for (int j = 1; j <= jd; ++j) wd2(j, k) = 0.0;
  for (int ib = 0; ib < p.nbc; ++ib) {
    if (p.ibtyp[ib] != 5) continue;
    int js, je, ks, ke;
    bc_cells(p, ib, js, je, ks, ke);
    const int idir = p.ibdir[ib], iadd = isgn(idir), iadir = idir < 0 ? -idir : idir;
    if (iadir == 1) {
      const int j = (idir == 1) ? je : js, j1 = j + iadd, jv = j1 - nh;
      for (int k = ks; k <= ke; ++k) {
        const int kv = k - nh;
        const double dx = x(j1, k) - 0.5 * (xv(jv, kv) + xv(jv, kv + 1));
        const double dy = y(j1, k) - 0.5 * (yv(jv, kv) + yv(jv, kv + 1));
        wd2(j, k) = dx * dx + dy * dy;
      }
    } else if (iadir == 2) {
      const int k = (idir == 2) ? ke : ks, k1 = k + iadd, kv = k1 - nh;
      for (int j = js; j <= je; ++j) {
        const int jv = j - nh;
        const double dx = x(j, k1) - 0.5 * (xv(jv, kv) + xv(jv + 1, kv));
        const double dy = y(j, k1) - 0.5 * (yv(jv, kv) + yv(jv + 1, kv));
        wd2(j, k) = dx * dx + dy * dy;
      }
    }
  }
}

void face_normals(const ot2d_params& p, const double* xv_, const double* yv_, const double* ugv_, const double* vgv_,
                  double* fxa_, double* fya_, double* gxa_, double* gya_, double* ftj_, double* gtj_) {
  const int jd = p.jd, nh = p.nhalo;
  C2 fxa{fxa_, jd}, fya{fya_, jd}, gxa{gxa_, jd}, gya{gya_, jd};
  V2 xv{xv_, p.jmax}, yv{yv_, p.jmax};
  for (size_t i = 0; i < (size_t)jd * p.kd; ++i) { fxa_[i] = 0; fya_[i] = 0; gxa_[i] = 0; gya_[i] = 0; }
  if (ftj_) for (size_t i = 0; i < (size_t)jd * p.kd; ++i) { ftj_[i] = 0; gtj_[i] = 0; }
  for (int k = p.kbeg; k <= p.kend; ++k)
    for (int j = p.jbeg - 1; j <= p.jend; ++j) {
      const int a = j - nh + 1, b = k - nh + 1;
      fxa(j, k) = (yv(a, b) - yv(a, b - 1));
      fya(j, k) = -(xv(a, b) - xv(a, b - 1));
      if (ftj_) {
        V2 ugv{ugv_, p.jmax}, vgv{vgv_, p.jmax};
        C2 ftj{ftj_, jd};
        ftj(j, k) = -0.5 * (ugv(a, b) + ugv(a, b - 1)) * fxa(j, k) - 0.5 * (vgv(a, b) + vgv(a, b - 1)) * fya(j, k);
      }
    }
  for (int j = p.jbeg; j <= p.jend; ++j)
    for (int k = p.kbeg - 1; k <= p.kend; ++k) {
      const int a = j - nh + 1, b = k - nh + 1;
      gxa(j, k) = -(yv(a, b) - yv(a - 1, b));
      gya(j, k) = (xv(a, b) - xv(a - 1, b));
      if (gtj_) {
        V2 ugv{ugv_, p.jmax}, vgv{vgv_, p.jmax};
        C2 gtj{gtj_, jd};
        gtj(j, k) = -0.5 * (ugv(a, b) + ugv(a - 1, b)) * gxa(j, k) - 0.5 * (vgv(a, b) + vgv(a - 1, b)) * gya(j, k);
      }
    }
}

void face_speeds_swept(const ot2d_params& p, const double* xv_, const double* yv_, const double* xold_,
                       const double* yold_, const double* xole_, const double* yole_, double* ftj_, double* gtj_) {
  const int jd = p.jd, nh = p.nhalo;
  C2 ftj{ftj_, jd}, gtj{gtj_, jd};
  V2 xv{xv_, p.jmax}, yv{yv_, p.jmax}, xo{xold_, p.jmax}, yo{yold_, p.jmax}, xe{xole_, p.jmax}, ye{yole_, p.jmax};
  for (size_t i = 0; i < (size_t)jd * p.kd; ++i) { ftj_[i] = 0; gtj_[i] = 0; }
  const bool second = p.ntac == 2 && p.istep > 1;
  for (int k = p.kbeg; k <= p.kend; ++k)
    for (int j = p.jbeg - 1; j <= p.jend; ++j) {
      const int a = j - nh + 1, b = k - nh + 1;
      double dx1 = xv(a, b) - xo(a, b - 1), dy1 = yv(a, b) - yo(a, b - 1);
      double dx2 = xo(a, b) - xv(a, b - 1), dy2 = yo(a, b) - yv(a, b - 1);
      double tj = -(0.5 * (dx1 * dy2 - dx2 * dy1) / p.dt);
      if (second) {
        dx1 = xo(a, b) - xe(a, b - 1); dy1 = yo(a, b) - ye(a, b - 1);
        dx2 = xe(a, b) - xo(a, b - 1); dy2 = ye(a, b) - yo(a, b - 1);
        const double temp = -(0.5 * (dx1 * dy2 - dx2 * dy1) / p.dt);
        tj = 1.5 * tj - 0.5 * temp;
      }
      ftj(j, k) = tj;
    }
  for (int j = p.jbeg; j <= p.jend; ++j)
    for (int k = p.kbeg - 1; k <= p.kend; ++k) {
      const int a = j - nh + 1, b = k - nh + 1;
      double dx1 = xv(a, b) - xo(a - 1, b), dy1 = yv(a, b) - yo(a - 1, b);
      double dx2 = xo(a, b) - xv(a - 1, b), dy2 = yo(a, b) - yv(a - 1, b);
      double tj = 0.5 * (dx1 * dy2 - dx2 * dy1) / p.dt;
      if (second) {
        dx1 = xo(a, b) - xe(a - 1, b); dy1 = yo(a, b) - ye(a - 1, b);
        dx2 = xe(a, b) - xo(a - 1, b); dy2 = ye(a, b) - yo(a - 1, b);
        const double temp = 0.5 * (dx1 * dy2 - dx2 * dy1) / p.dt;
        tj = 1.5 * tj - 0.5 * temp;
      }
      gtj(j, k) = tj;
    }
}

void ts_pitch_grid(const ot2d_params& p, const double* xv1, const double* yv1, double tspec, double* xv, double* yv) {
  const double pi = 4.0 * std::atan(1.0);
  const double theta = p.angmax * pi / 180. * std::sin(p.rotf * tspec);
  const double ss = std::sin(theta), cs = std::cos(theta);
  const size_t n = (size_t)p.jmax * p.kmax;
  for (size_t i = 0; i < n; ++i) {
    xv[i] = (xv1[i] - p.xac) * cs + (yv1[i] - p.yac) * ss + p.xac;
    yv[i] = (yv1[i] - p.yac) * cs - (xv1[i] - p.xac) * ss + p.yac;
  }
}

void ts_grid_speed(const ot2d_params& p, const double* x, const double* y, const double* xv, const double* yv,
                   double tspec, double* ug, double* vg, double* ugv, double* vgv) {
  const double pi = 4.0 * std::atan(1.0);
  const size_t n2 = (size_t)p.jd * p.kd, nv = (size_t)p.jmax * p.kmax;
  for (size_t i = 0; i < n2; ++i) {
    ug[i] = p.angmax * pi / 180. * p.rotf * (y[i] - p.yac) * std::cos(p.rotf * tspec);
    vg[i] = -p.angmax * pi / 180. * p.rotf * (x[i] - p.xac) * std::cos(p.rotf * tspec);
  }
  for (size_t i = 0; i < nv; ++i) {
    ugv[i] = p.angmax * pi / 180. * p.rotf * (yv[i] - p.yac) * std::cos(p.rotf * tspec);
    vgv[i] = -p.angmax * pi / 180. * p.rotf * (xv[i] - p.xac) * std::cos(p.rotf * tspec);
  }
}

void ts_operator(int n, double* Ds) {
  const double pi = 4. * std::atan(1.);
  for (int i = 1; i <= n; ++i)
    for (int j = 1; j <= n; ++j) {
      const int e = i - j;
      const double sgn = (e % 2 == 0) ? 1.0 : -1.0;
      double v = 0.;
      if (i != j) v = (n % 2 == 0) ? 0.5 * sgn / std::tan(pi * e / n) : 0.5 * sgn / std::sin(pi * e / n);
      Ds[(size_t)(j - 1) * n + (i - 1)] = v;
    }
}

void freestream(const ot2d_params& p, double* q, size_t qs) {
  const size_t n2 = (size_t)p.jd * p.kd;
  for (size_t i = 0; i < n2; ++i) {
    const double J = q[(p.nq - 1) * qs + i];
    // qzero then qdivj (init.f:229-237, :197-203): Q/J
    q[i] = p.rinf / J;
    q[qs + i] = (p.rinf * p.uinf) / J;
    q[2 * qs + i] = (p.rinf * p.vinf) / J;
    q[3 * qs + i] = p.einf / J;
    if (p.iturb == 1) q[4 * qs + i] = p.vnuinf;
    if (p.iturb == 2) { q[4 * qs + i] = p.rinf * p.tkeinf; q[5 * qs + i] = p.rinf * p.tomegainf; }
  }
}

}  // namespace ot2d
