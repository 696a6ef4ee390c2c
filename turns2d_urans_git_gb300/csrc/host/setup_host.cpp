/*
 * setup_host.cpp -- host-side set-up for the GB300 OVERTURNS-2D hot path.
 *
 *  - ot2d_params_from_inputs: the derived-constant part of read_inputs
 *    (src/setup.f:960-971, :982-986, :1162-1204, :1230-1235, :1262-1265),
 *    set_pointers_globals (src/setup.f:55-108) and the jtail rule of initia
 *    (src/init.f:59-66).
 *  - ot2d_cmesh_bc_table: the five-entry &bcinp table of a single C-mesh
 *    (wall 5, wake cut 51, three characteristic far fields 47).
 *  - ot2d_mesh_naca4_cmesh: the seeded algebraic NACA 4-digit C-mesh that
 *    stands in for the reference's unformatted grid file (fort.1,
 *    src/io.f:343-380).  The reference ships no grids; this generator is new.
 */
#include <cmath>
#include <cstring>
#include <vector>
#include "ot2d.h"

extern "C" int ot2d_params_from_inputs(const ot2d_inputs* in, ot2d_params* out) {
  if (!in || !out) return OT2D_ERR_ARG;
  ot2d_params p;
  std::memset(&p, 0, sizeof(p));
  const double pi = 4.0 * std::atan(1.0);
  /* module defaults, modules.f:170-190 */
  p.gamma = 1.4; p.pr = 0.72; p.rmue = 1.0; p.tinf = 400.0; p.Mp = 1.0; p.dualtime = 1.0;
  p.jmax = in->jmax; p.kmax = in->kmax; p.nhalo = in->nhalo; p.half = in->half;
  p.invisc = in->invisc; p.lamin = in->lamin; p.iturb = in->iturb; p.itrans = in->itrans;
  p.irhsy = in->irhsy; p.ilim = in->ilim; p.ilhs = in->ilhs;
  p.iconstant_cfl = in->iconstant_cfl; p.idual = in->idual; p.idual_turb = in->idual_turb;
  p.iunst = in->iunst; p.ntac = in->ntac; p.itnmax = in->itnmax; p.iread = in->iread;
  p.timespectral = in->timespectral; p.nspec = in->nspec; p.motiontype = in->motiontype;
  p.npnorm = in->npnorm;
  p.fsmach = in->fsmach; p.fmtip = in->fmtip; p.alfa = in->alfa; p.rey = in->rey;
  p.vnuinf = in->vnuinf; p.dt = in->dt; p.timeac = in->timeac; p.epse = in->epse; p.cfltur = in->cfltur;
  p.rf = in->rf; p.angmax = in->angmax; p.xac = in->xac; p.yac = in->yac;
  if (in->nbc < 0 || in->nbc > OT2D_MAXBC) return OT2D_ERR_ARG;
  p.nbc = in->nbc;
  std::memcpy(p.ibtyp, in->ibtyp, sizeof(p.ibtyp)); std::memcpy(p.ibdir, in->ibdir, sizeof(p.ibdir));
  std::memcpy(p.jbcs, in->jbcs, sizeof(p.jbcs)); std::memcpy(p.jbce, in->jbce, sizeof(p.jbce));
  std::memcpy(p.kbcs, in->kbcs, sizeof(p.kbcs)); std::memcpy(p.kbce, in->kbce, sizeof(p.kbce));
  /* read_inputs */
  if (p.timespectral) p.iunst = 0; else p.nspec = 1;
  if (p.nspec < 1) return OT2D_ERR_ARG;
  if (p.invisc) { p.rmue = 0.0; p.lamin = 1; }
  if (p.lamin) p.iturb = -1;
  p.gm1 = p.gamma - 1.0;
  p.ggm1 = p.gamma * p.gm1;
  const double cs = std::cos(pi * p.alfa / 180.0), ss = std::sin(pi * p.alfa / 180.0);
  p.theta_col = p.alfa;
  p.einf = 1.0 / p.ggm1 + 0.5 * (p.fsmach * p.fsmach);
  p.pinf = 1.0 / p.gamma;
  p.rinf = 1.0;
  p.ainf = p.gamma * p.pinf / p.rinf;
  p.htinf = p.gamma * p.einf / p.rinf - 0.5 * p.gm1 * (p.fsmach * p.fsmach);
  p.nq = 5; p.nv = 4; p.nmv = 4; p.nturb = 0;
  if (p.iturb == 1) { p.nturb = 1; p.nq += 1; p.nv += 1; }
  else if (p.iturb == 2) { p.nturb = 2; p.nq += 2; p.nv += 2; }
  p.uinf = p.fsmach * cs;
  p.vinf = p.fsmach * ss;
  p.rey = (p.fsmach != 0) ? p.rey / p.fsmach : p.rey / p.fmtip;
  p.h = p.dt;
  p.tkeinf = 1e-6 * (p.fsmach * p.fsmach);
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
  if (p.rf != 0) p.rotf = p.rf;
  p.istep = 0; p.istep0 = 0; p.itn = 1;
  if (p.jmax < 8 || p.kmax < 8 || p.nhalo != 1) return OT2D_ERR_ARG;
  *out = p;
  return OT2D_OK;
}

extern "C" int ot2d_cmesh_bc_table(ot2d_inputs* in, int32_t jtail) {
  if (!in) return OT2D_ERR_ARG;
  const int32_t jmax = in->jmax, kmax = in->kmax;
  in->nbc = 5;
  /* wall on k=1 between the two trailing-edge vertices */
  in->ibtyp[0] = 5;  in->ibdir[0] = 2;  in->jbcs[0] = jtail; in->jbce[0] = jmax - jtail + 1; in->kbcs[0] = 1; in->kbce[0] = 1;
  /* wake cut on k=1 (lower run; bcwake mirrors it onto the upper run) */
  in->ibtyp[1] = 51; in->ibdir[1] = 2;  in->jbcs[1] = 1; in->jbce[1] = jtail; in->kbcs[1] = 1; in->kbce[1] = 1;
  /* far field: outer boundary, then the two outflow ends */
  in->ibtyp[2] = 47; in->ibdir[2] = -2; in->jbcs[2] = 1; in->jbce[2] = jmax; in->kbcs[2] = kmax; in->kbce[2] = kmax;
  in->ibtyp[3] = 47; in->ibdir[3] = 1;  in->jbcs[3] = 1; in->jbce[3] = 1; in->kbcs[3] = 1; in->kbce[3] = kmax;
  in->ibtyp[4] = 47; in->ibdir[4] = -1; in->jbcs[4] = jmax; in->jbce[4] = jmax; in->kbcs[4] = 1; in->kbce[4] = kmax;
  return OT2D_OK;
}

namespace {
struct Naca4 {
  double m, p, t;
  void at(double x, double& yc, double& dyc, double& yt) const {
    yt = 5.0 * t * (0.2969 * std::sqrt(x) - 0.1260 * x - 0.3516 * x * x + 0.2843 * x * x * x - 0.1036 * x * x * x * x);
    if (m <= 0.0 || p <= 0.0) { yc = 0.0; dyc = 0.0; return; }
    if (x < p) { yc = m / (p * p) * (2 * p * x - x * x); dyc = 2 * m / (p * p) * (p - x); }
    else { yc = m / ((1 - p) * (1 - p)) * ((1 - 2 * p) + 2 * p * x - x * x); dyc = 2 * m / ((1 - p) * (1 - p)) * (p - x); }
  }
};
/* ratio r of a geometric series with first step a and n steps summing to L */
double geometric_ratio(double a, int n, double L) {
  if (a * n >= L) return 1.0;
  double lo = 1.0 + 1e-12, hi = 4.0;
  for (int it = 0; it < 200; ++it) {
    double r = 0.5 * (lo + hi);
    double sum = a * (std::pow(r, n) - 1.0) / (r - 1.0);
    if (sum > L) hi = r; else lo = r;
  }
  return 0.5 * (lo + hi);
}
}  // namespace

/* NACA 4-digit C-mesh, vertices xv,yv(jmax,kmax) column-major.  j runs
 * clockwise: lower wake (outflow to trailing edge), lower surface (TE to LE),
 * upper surface (LE to TE), upper wake; k runs from the wall/cut to the far
 * field.  Surface points are cosine clustered; the wall-normal distribution
 * is geometric with first spacing ds_wall, reaching the far field at r_far
 * chords; lines are cubic Hermite blends between the wall normal and the
 * straight ray to the outer C boundary (orthogonal at the wall). */
extern "C" int ot2d_mesh_naca4_cmesh(int32_t jmax, int32_t kmax, int32_t n_wake, double m, double p, double t,
                                     double ds_wall, double r_far, double* xv, double* yv) {
  if (!xv || !yv || jmax < 9 || kmax < 5 || n_wake < 2) return OT2D_ERR_ARG;
  const int nsurf = jmax - 2 * n_wake;
  if (nsurf < 5 || (nsurf % 2) == 0) return OT2D_ERR_ARG;
  const int half = (nsurf - 1) / 2;
  const double pi = 4.0 * std::atan(1.0);
  Naca4 af{m, p, t};
  std::vector<double> bx(jmax), by(jmax), nx(jmax), ny(jmax), ox(jmax), oy(jmax);
  /* surface: index i = 0..nsurf-1, lower TE -> LE -> upper TE */
  for (int i = 0; i < nsurf; ++i) {
    bool lower = i < half;
    double phi = lower ? (double)(half - i) / half : (double)(i - half) / half;
    double x = 0.5 * (1.0 - std::cos(pi * phi));
    double yc, dyc, yt; af.at(x, yc, dyc, yt);
    double th = std::atan(dyc);
    int j = n_wake + i;
    if (lower) { bx[j] = x + yt * std::sin(th); by[j] = yc - yt * std::cos(th); }
    else { bx[j] = x - yt * std::sin(th); by[j] = yc + yt * std::cos(th); }
    if (i == 0 || i == nsurf - 1) { bx[j] = 1.0; by[j] = 0.0; }
    if (i == half) { bx[j] = 0.0; by[j] = 0.0; }
  }
  /* wake along y = 0, geometric from the trailing edge */
  double ds_te = std::hypot(bx[n_wake + 1] - bx[n_wake], by[n_wake + 1] - by[n_wake]);
  double r_w = geometric_ratio(ds_te, n_wake, r_far);
  double xw = 1.0, step = ds_te;
  std::vector<double> wx(n_wake + 1);
  wx[0] = 1.0;
  for (int i = 1; i <= n_wake; ++i) { xw += step; step *= r_w; wx[i] = xw; }
  double scale = r_far / (wx[n_wake] - 1.0);
  for (int i = 1; i <= n_wake; ++i) wx[i] = 1.0 + (wx[i] - 1.0) * scale;
  for (int i = 1; i <= n_wake; ++i) {
    int jl = n_wake - i, ju = jmax - n_wake - 1 + i;
    bx[jl] = wx[i]; by[jl] = 0.0;
    bx[ju] = wx[i]; by[ju] = 0.0;
  }
  /* wall normals (outward; j runs clockwise).  The wake-cut lines leave the
   * cut in the direction of their side's trailing-edge normal, so that the
   * line directions rotate monotonically along j and neighbouring lines
   * never cross near the sharp trailing edge. */
  for (int j = n_wake; j <= jmax - n_wake - 1; ++j) {
    double tx, ty;
    if (j == n_wake) { tx = bx[j + 1] - bx[j]; ty = by[j + 1] - by[j]; }
    else if (j == jmax - n_wake - 1) { tx = bx[j] - bx[j - 1]; ty = by[j] - by[j - 1]; }
    else { tx = bx[j + 1] - bx[j - 1]; ty = by[j + 1] - by[j - 1]; }
    double l = std::hypot(tx, ty);
    nx[j] = -ty / l; ny[j] = tx / l;
  }
  /* smooth the surface normals (ends held) so that lines leaving concave
   * parts of cambered sections do not cross */
  {
    std::vector<double> tx(jmax), ty(jmax);
    const int passes = 4 * nsurf;
    for (int it = 0; it < passes; ++it) {
      for (int j = n_wake + 1; j < jmax - n_wake - 1; ++j) {
        tx[j] = 0.25 * nx[j - 1] + 0.5 * nx[j] + 0.25 * nx[j + 1];
        ty[j] = 0.25 * ny[j - 1] + 0.5 * ny[j] + 0.25 * ny[j + 1];
      }
      for (int j = n_wake + 1; j < jmax - n_wake - 1; ++j) {
        double l = std::hypot(tx[j], ty[j]);
        nx[j] = tx[j] / l; ny[j] = ty[j] / l;
      }
    }
  }
  for (int j = 0; j < n_wake; ++j) { nx[j] = nx[n_wake]; ny[j] = ny[n_wake]; }
  for (int j = jmax - n_wake; j < jmax; ++j) { nx[j] = nx[jmax - n_wake - 1]; ny[j] = ny[jmax - n_wake - 1]; }
  /* line directions must turn monotonically from the leading edge out to the
   * outflow ends (clockwise along the lower side, anticlockwise along the
   * upper side); concave stretches keep the previous direction instead */
  {
    const int jle0 = n_wake + half;
    double amax = -1e30;
    for (int j = jle0; j >= 0; --j) {
      double a = std::atan2(ny[j], nx[j]);
      if (a > 0.5 * pi) a -= 2.0 * pi;
      if (a < amax) a = amax;
      amax = a;
      nx[j] = std::cos(a); ny[j] = std::sin(a);
    }
    double amin = 1e30;
    for (int j = jle0; j < jmax; ++j) {
      double a = std::atan2(ny[j], nx[j]);
      if (a < -0.5 * pi) a += 2.0 * pi;
      if (a > amin) a = amin;
      amin = a;
      nx[j] = std::cos(a); ny[j] = std::sin(a);
    }
  }
  /* outer C boundary: lines y = -R / +R downstream, semicircle about the TE */
  const double xc = 1.0;
  for (int j = 0; j < jmax; ++j) {
    if (j < n_wake) { ox[j] = bx[j]; oy[j] = -r_far; }
    else if (j > jmax - n_wake - 1) { ox[j] = bx[j]; oy[j] = r_far; }
    else {
      double phi = (double)(j - n_wake) / (nsurf - 1);
      double ang = -0.5 * pi - pi * phi;
      ox[j] = xc + r_far * std::cos(ang); oy[j] = r_far * std::sin(ang);
    }
  }
  /* wall-normal distribution, eta in [0,1] */
  const int K = kmax - 1;
  double a = ds_wall / r_far;
  double rk = geometric_ratio(a, K, 1.0);
  std::vector<double> eta(kmax);
  eta[0] = 0.0; double st = a, acc = 0.0;
  for (int k = 1; k < kmax; ++k) { acc += st; st *= rk; eta[k] = acc; }
  for (int k = 1; k < kmax; ++k) eta[k] /= eta[K];
  for (int j = 0; j < jmax; ++j) {
    double dx = ox[j] - bx[j], dy = oy[j] - by[j];
    double D = std::hypot(dx, dy);
    double t0x = nx[j] * D, t0y = ny[j] * D;
    for (int k = 0; k < kmax; ++k) {
      double e = eta[k], e2 = e * e, e3 = e2 * e;
      double h0 = 2 * e3 - 3 * e2 + 1, h1 = -2 * e3 + 3 * e2, h2 = e3 - 2 * e2 + e, h3 = e3 - e2;
      size_t o = (size_t)k * jmax + j;
      xv[o] = h0 * bx[j] + h1 * ox[j] + h2 * t0x + h3 * dx;
      yv[o] = h0 * by[j] + h1 * oy[j] + h2 * t0y + h3 * dy;
    }
  }
  /* the cut is shared exactly by both wake runs */
  for (int j = 0; j < n_wake + 1; ++j) {
    int jj = jmax - 1 - j;
    xv[jj] = xv[j]; yv[jj] = yv[j];
  }
  /* a symmetric section gets an exactly mirror-symmetric grid */
  if (m <= 0.0 || p <= 0.0) {
    const int mid = (jmax - 1) / 2;
    for (int k = 0; k < kmax; ++k) {
      for (int j = 0; j < mid; ++j) {
        size_t o = (size_t)k * jmax + j, om = (size_t)k * jmax + (jmax - 1 - j);
        xv[om] = xv[o]; yv[om] = -yv[o];
      }
      yv[(size_t)k * jmax + mid] = 0.0;
    }
  }
  return OT2D_OK;
}
