/*
 * oracle_flux.cpp -- TEST INFRASTRUCTURE ONLY (see oracle_common.h).
 * FP64 restatement of the inviscid residual (src/eulerrhs.f) and the
 * viscous residual (src/visrhs.f).
 */
#include <cstdio>
#include <cstdlib>
#include "oracle.h"

namespace oro {

/* Line work arrays, 1-based with index 0 unused: f(i,n) -> F[n][i]. */
struct Line {
  std::vector<double> f[5], ql[5], qr[5], xa, ya, tj;
  std::vector<int> iba;
  explicit Line(int m) {
    for (int n = 1; n <= 4; ++n) { f[n].assign(m + 2, 0.); ql[n].assign(m + 2, 0.); qr[n].assign(m + 2, 0.); }
    xa.assign(m + 2, 0.); ya.assign(m + 2, 0.); tj.assign(m + 2, 0.); iba.assign(m + 2, 0);
  }
};

/* eulerrhs.f:628-681 (ibmin = ibmax = 1 on the path) */
static void iflux(Line& L, int is, int ie, double qt) {
  for (int n = 1; n <= 4; ++n) {
    std::vector<double>& f = L.f[n]; std::vector<double>& ql = L.ql[n]; std::vector<double>& qr = L.qr[n];
    if (qt == 0.0) { for (int i = is; i <= ie; ++i) { ql[i] = f[i]; qr[i] = f[i]; } continue; }
    for (int i = is + 1; i <= ie - 1; ++i) {
      double s1 = f[i] - f[i - 1], s2 = f[i + 1] - f[i];
      double slope = (s1 + s2) / 2;
      ql[i] = f[i] + 0.5 * slope;
      qr[i] = f[i] - 0.5 * slope;
    }
    ql[is] = f[is]; qr[is] = f[is];
    ql[ie] = f[ie]; qr[ie] = f[ie];
  }
}

/* eulerrhs.f:821-912 (ibmin = ibmax = 1 on the path) */
static void muscld_new(Line& L, int is, int imax, int im, double th, double qt, double eps) {
  std::vector<double> f2(imax + 2, 0.);
  if (qt == 0.0) {
    for (int n = 1; n <= 4; ++n) for (int i = is; i <= imax; ++i) { L.ql[n][i] = L.f[n][i]; L.qr[n][i] = L.f[n][i]; }
    return;
  }
  double thm = 1.0 - th, thp = 1.0 + th;
  for (int n = 1; n <= 4; ++n) {
    std::vector<double>& f = L.f[n]; std::vector<double>& ql = L.ql[n]; std::vector<double>& qr = L.qr[n];
    for (int i = is; i <= im; ++i) f2[i] = f[i + 1] - f[i];
    for (int i = is + 1; i <= im; ++i) {
      double f2i = f2[i], f2i1 = f2[i - 1];
      double a1 = 3.0 * (f2i * f2i1 + eps);
      double a2 = 2.0 * p2(f2i - f2i1) + a1;
      double f3i = a1 / a2;
      double f3qt = qt * f3i * (double)L.iba[i] * (double)L.iba[i + 1] * (double)L.iba[i - 1];
      ql[i] = f[i] + f3qt * (thm * f2i1 + thp * f2i);
      qr[i] = f[i] - f3qt * (thp * f2i1 + thm * f2i);
    }
    qr[is] = f[is]; ql[is] = f[is];
    ql[imax] = f[imax]; qr[imax] = f[imax];
  }
}

static inline double ammd(double fl, double fr) {
  return 0.5 * (fsign(1., fl) + fsign(1., fr)) * fmin2(std::fabs(fl), std::fabs(fr));
}

/* eulerrhs.f:1194-1230 */
static double weno5(double a, double b, double c, double d, double e) {
  double b1 = 13. / 12., b2 = 1. / 6., epsw = 1.e-6;
  double djm1 = a - 2. * b + c, ejm1 = a - 4. * b + 3. * c;
  double dj = b - 2. * c + d, ej = b - d;
  double djp1 = c - 2. * d + e, ejp1 = 3. * c - 4. * d + e;
  double dis0 = b1 * djm1 * djm1 + 0.25 * ejm1 * ejm1 + epsw;
  double dis1 = b1 * dj * dj + 0.25 * ej * ej + epsw;
  double dis2 = b1 * djp1 * djp1 + 0.25 * ejp1 * ejp1 + epsw;
  double q30 = 2. * a - 7. * b + 11. * c, q31 = -b + 5. * c + 2. * d, q32 = 2. * c + 5. * d - e;
  double d01 = dis0 / dis1, d02 = dis0 / dis2;
  double a1ba0 = 6. * d01, a2ba0 = 3. * d02;
  double w0 = 1. / (1. + a1ba0 + a2ba0);
  double w1 = a1ba0 * w0;
  double w2 = 1. - w0 - w1;
  return b2 * (w0 * q30 + w1 * q31 + w2 * q32);
}

/* sonic-A slope, eulerrhs.f:1124-1129 */
static inline double sonic_slope(double at, double ati1, double s1) {
  double t1 = ammd(at, ati1);
  return fsign(1., t1) * fmin2(0.5 * std::fabs(at + ati1), fmax2(2. * std::fabs(s1), std::fabs(t1)));
}

/* eulerrhs.f:1011-1192 (ibmin = ibmax = 1).  The reference writes slope(i)
 * with a stale loop index at :1101 and :1116; slope is a scratch value read
 * back at once, so a local scalar gives the same ql/qr. */
static void weno(Line& L, int is, int ie, double qt) {
  std::vector<double> f0(ie + 2), f1(ie + 2), f2(ie + 2), f2m(ie + 2);
  if (qt == 0.0) {
    for (int n = 1; n <= 4; ++n) for (int i = is; i <= ie; ++i) { L.ql[n][i] = L.f[n][i]; L.qr[n][i] = L.f[n][i]; }
    return;
  }
  for (int n = 1; n <= 4; ++n) {
    std::vector<double>& ql = L.ql[n]; std::vector<double>& qr = L.qr[n];
    for (int i = is; i <= ie; ++i) f0[i] = L.f[n][i];
    for (int i = is; i <= ie - 1; ++i) f1[i] = f0[i + 1] - f0[i];
    for (int i = is + 1; i <= ie - 1; ++i) f2[i] = f1[i] - f1[i - 1];
    f2[is] = 2. * f2[is + 1] - f2[is + 2];
    f2[ie] = 2. * f2[ie - 1] - f2[ie - 2];
    for (int i = is; i <= ie - 1; ++i) f2m[i] = ammd(f2[i], f2[i + 1]);
    double at = f1[is] - 0.5 * f2m[is];
    double slope = ammd(at, 2. * f1[is]);
    ql[is] = f0[is] + 0.5 * slope;
    double at1 = f1[ie - 1] + 0.5 * f2m[ie - 1];
    slope = ammd(at1, 2. * f1[ie - 1]);
    qr[ie] = f0[ie] - 0.5 * slope;
    for (int i = is + 1; i <= ie - 1; i += (ie - is - 2)) {
      double a = f1[i] - 0.5 * f2m[i];
      double ai1 = f1[i - 1] + 0.5 * f2m[i - 1];
      double s1 = ammd(f1[i], f1[i - 1]);
      slope = sonic_slope(a, ai1, s1);
      ql[i] = f0[i] + 0.5 * slope;
      qr[i] = f0[i] - 0.5 * slope;
      if (ie - is - 2 <= 0) break;
    }
    for (int i = is + 2; i <= ie - 2; ++i) {
      ql[i] = weno5(f0[i - 2], f0[i - 1], f0[i], f0[i + 1], f0[i + 2]);
      qr[i] = weno5(f0[i + 2], f0[i + 1], f0[i], f0[i - 1], f0[i - 2]);
      double blankv = (double)(L.iba[i] * L.iba[i - 1] * L.iba[i + 1] * L.iba[i - 2] * L.iba[i + 2]);
      ql[i] = ql[i] * blankv + (1. - blankv) * f0[i];
      qr[i] = qr[i] * blankv + (1. - blankv) * f0[i];
    }
    {
      int i = is + 2;
      double a = f1[i] - 0.5 * f2m[i];
      double ai1 = f1[i - 1] + 0.5 * f2m[i - 1];
      double s1 = ammd(f1[i], f1[i - 1]);
      slope = sonic_slope(a, ai1, s1);
      ql[i] = f0[i] + 0.5 * slope;
    }
    {
      int i = ie - 1;
      double a = f1[i] - 0.5 * f2m[i];
      double ai1 = f1[i - 1] + 0.5 * f2m[i - 1];
      double s1 = ammd(f1[i], f1[i - 1]);
      slope = sonic_slope(a, ai1, s1);
      qr[i] = f0[i] - 0.5 * slope;
    }
  }
}

/* eulerrhs.f:283-446 (fssub = 0) */
static void roeflx(const P& p, Line& L, int is, int ie) {
  const double gm1 = p.gm1, eps = 1.e-6;
  for (int i = is; i <= ie; ++i) {
    int i1 = i + 1;
    double rlft = L.ql[1][i], ulft = L.ql[2][i], vlft = L.ql[3][i], plft = L.ql[4][i];
    double rlfti = 1.0 / rlft;
    double rulft = rlft * ulft, rvlft = rlft * vlft;
    double uvl = 0.5 * (ulft * ulft + vlft * vlft);
    double elft = plft / gm1 + rlft * uvl;
    double hlft = (elft + plft) * rlfti;
    double clft = std::sqrt(gm1 * (hlft - uvl));
    double rrht = L.qr[1][i1], urht = L.qr[2][i1], vrht = L.qr[3][i1], prht = L.qr[4][i1];
    double rrhti = 1.0 / rrht;
    double rurht = rrht * urht, rvrht = rrht * vrht;
    double uvr = 0.5 * (urht * urht + vrht * vrht);
    double erht = prht / gm1 + rrht * uvr;
    double hrht = (erht + prht) * rrhti;
    double crht = std::sqrt(gm1 * (hrht - uvr));
    double rat = std::sqrt(rrht * rlfti);
    double rati = 1.0 / (rat + 1.);
    double rav = rat * rlft;
    double uav = (rat * urht + ulft) * rati;
    double vav = (rat * vrht + vlft) * rati;
    double hav = (rat * hrht + hlft) * rati;
    double uv = 0.5 * (uav * uav + vav * vav);
    double cav = std::sqrt(gm1 * (hav - uv));
    double aq1 = rrht - rlft, aq2 = urht - ulft, aq3 = vrht - vlft, aq4 = prht - plft;
    double ri1 = L.xa[i], ri2 = L.ya[i], ri3 = L.tj[i];
    double rr2 = ri1 * ri1 + ri2 * ri2;
    double rr = std::sqrt(rr2);
    double r0 = 1.0 / rr;
    double r1 = ri1 * r0, r2 = ri2 * r0, r3 = ri3 * r0;
    double uu = r1 * uav + r2 * vav + r3;
    double c2 = cav * cav;
    double c2i = 1.0 / c2;
    double auu = std::fabs(uu), aupc = std::fabs(uu + cav), aumc = std::fabs(uu - cav);
    double uulft = r1 * ulft + r2 * vlft + r3;
    double uurht = r1 * urht + r2 * vrht + r3;
    double upclft = uulft + clft, upcrht = uurht + crht;
    double umclft = uulft - clft, umcrht = uurht - crht;
    double dauu = 4. * (uurht - uulft) + eps;
    double dauus = fmax2(dauu, 0.0);
    if (auu <= 0.5 * dauus) auu = auu * auu / dauu + 0.25 * dauu;
    double daupc = 4. * (upcrht - upclft) + eps;
    double daupcs = fmax2(daupc, 0.0);
    if (aupc <= 0.5 * daupcs) aupc = aupc * aupc / daupc + 0.25 * daupc;
    double daumc = 4. * (umcrht - umclft) + eps;
    double daumcs = fmax2(daumc, 0.0);
    if (aumc <= 0.5 * daumcs) aumc = aumc * aumc / daumc + 0.25 * daumc;
    double rcav = rav * cav;
    double aquu = uurht - uulft;
    double c2ih = 0.5 * c2i;
    double ruuav = auu * rav;
    double b1 = auu * (aq1 - c2i * aq4);
    double b2 = c2ih * aupc * (aq4 + rcav * aquu);
    double b3 = c2ih * aumc * (aq4 - rcav * aquu);
    double b4 = b1 + b2 + b3;
    double b5 = cav * (b2 - b3);
    double b6 = ruuav * (aq2 - r1 * aquu);
    double b7 = ruuav * (aq3 - r2 * aquu);
    aq1 = b4;
    aq2 = uav * b4 + r1 * b5 + b6;
    aq3 = vav * b4 + r2 * b5 + b7;
    aq4 = hav * b4 + (uu - r3) * b5 + uav * b6 + vav * b7 - c2 * b1 / gm1;
    double aj = 0.5 * rr;
    double plar = plft + prht;
    double eplft = elft + plft, eprht = erht + prht;
    double fssub = 0.0;
    L.f[1][i] = aj * (rlft * uulft + rrht * uurht - aq1) - fssub * p.rinf;
    L.f[2][i] = aj * (rulft * uulft + rurht * uurht + r1 * plar - aq2) - fssub * p.rinf * p.uinf;
    L.f[3][i] = aj * (rvlft * uulft + rvrht * uurht + r2 * plar - aq3) - fssub * p.rinf * p.vinf;
    L.f[4][i] = aj * (eplft * uulft + eprht * uurht - r3 * plar - aq4) - fssub * p.einf;
  }
}

/* eulerrhs.f:450-625 (roetrklflx): the Roe flux with Turkel's low-Mach
 * preconditioning; b = 1 on every face (eulerrhs.f:78, :185), so
 * bSq = Mp**2 */
static void roetrklflx(const P& p, Line& L, int is, int ie) {
  const double gm1 = p.gm1, eps = 1.e-6;
  const double bt = 1.0;
  const double bSq = (p.Mp * p.Mp) / (bt - (p.Mp * p.Mp) * (bt - 1.));
  for (int i = is; i <= ie; ++i) {
    int i1 = i + 1;
    double rlft = L.ql[1][i], ulft = L.ql[2][i], vlft = L.ql[3][i], plft = L.ql[4][i];
    double rlfti = 1.0 / rlft;
    double rulft = rlft * ulft, rvlft = rlft * vlft;
    double uvl = 0.5 * (ulft * ulft + vlft * vlft);
    double elft = plft / gm1 + rlft * uvl;
    double hlft = (elft + plft) * rlfti;
    double clft = std::sqrt(gm1 * (hlft - uvl));
    double rrht = L.qr[1][i1], urht = L.qr[2][i1], vrht = L.qr[3][i1], prht = L.qr[4][i1];
    double rrhti = 1.0 / rrht;
    double rurht = rrht * urht, rvrht = rrht * vrht;
    double uvr = 0.5 * (urht * urht + vrht * vrht);
    double erht = prht / gm1 + rrht * uvr;
    double hrht = (erht + prht) * rrhti;
    double crht = std::sqrt(gm1 * (hrht - uvr));
    double rat = std::sqrt(rrht * rlfti);
    double rati = 1.0 / (rat + 1.);
    double rav = rat * rlft;
    double uav = (rat * urht + ulft) * rati;
    double vav = (rat * vrht + vlft) * rati;
    double hav = (rat * hrht + hlft) * rati;
    double uv = 0.5 * (uav * uav + vav * vav);
    double cav = std::sqrt(gm1 * (hav - uv));
    double aq1 = rrht - rlft, aq2 = urht - ulft, aq3 = vrht - vlft, aq4 = prht - plft;
    double ri1 = L.xa[i], ri2 = L.ya[i], ri3 = L.tj[i];
    double rr2 = ri1 * ri1 + ri2 * ri2;
    double rr = std::sqrt(rr2);
    double r0 = 1.0 / rr;
    double r1 = ri1 * r0, r2 = ri2 * r0, r3 = ri3 * r0;
    double uumxt = r1 * uav + r2 * vav;
    double uu = uumxt + r3;
    double c2 = cav * cav;
    double c2i = 1.0 / c2;
    double X = std::sqrt((((1. - bSq) * uu) * (1. - bSq)) * uu + ((4. * bSq) * c2));
    double auu = std::fabs(uu);
    double aupc = 0.5 * std::fabs((1. + bSq) * uu + X);
    double aumc = 0.5 * std::fabs((1. + bSq) * uu - X);
    double uulft = r1 * ulft + r2 * vlft + r3;
    double uurht = r1 * urht + r2 * vrht + r3;
    X = std::sqrt(((1. - bSq) * uulft) * ((1. - bSq) * uulft) + ((4. * bSq) * clft) * clft);
    double upclft = 0.5 * ((1. + bSq) * uulft + X);
    double umclft = 0.5 * ((1. + bSq) * uulft - X);
    X = std::sqrt(((1. - bSq) * uurht) * ((1. - bSq) * uurht) + ((4. * bSq) * crht) * crht);
    double upcrht = 0.5 * ((1. + bSq) * uurht + X);
    double umcrht = 0.5 * ((1. + bSq) * uurht - X);
    double dauu = 4. * (uurht - uulft) + eps;
    double dauus = fmax2(dauu, 0.0);
    if (auu <= 0.5 * dauus) auu = auu * auu / dauu + 0.25 * dauu;
    double daupc = 4. * (upcrht - upclft) + eps;
    double daupcs = fmax2(daupc, 0.0);
    if (aupc <= 0.5 * daupcs) aupc = aupc * aupc / daupc + 0.25 * daupc;
    double daumc = 4. * (umcrht - umclft) + eps;
    double daumcs = fmax2(daumc, 0.0);
    if (aumc <= 0.5 * daumcs) aumc = aumc * aumc / daumc + 0.25 * daumc;
    double aquu = uurht - uulft;
    double ruuav = auu * rav;
    X = std::sqrt(((1. - bSq) * uu) * ((1. - bSq) * uu) + ((4. * bSq) * c2));
    double R = 0.5 * ((1. - bSq) * uu + X);
    double S = 0.5 * ((1. - bSq) * uu - X);
    double b1 = auu * (aq1 - c2i * aq4);
    double b2 = aupc * (aq4 / R + rav * aquu) / X;
    double b3 = aumc * (-(aq4 / S) - rav * aquu) / X;
    double b4 = b1 + b2 + b3;
    double b5 = (R * b2 + S * b3);
    double b6 = ruuav * (aq2 - r1 * aquu);
    double b7 = ruuav * (aq3 - r2 * aquu);
    aq1 = b4;
    aq2 = uav * b4 + r1 * b5 + b6;
    aq3 = vav * b4 + r2 * b5 + b7;
    aq4 = hav * b4 + uumxt * b5 + uav * b6 + vav * b7 - c2 * b1 / gm1;
    double aj = 0.5 * rr;
    double plar = plft + prht;
    double eplft = elft + plft, eprht = erht + prht;
    double fssub = 0.0;
    L.f[1][i] = aj * (rlft * uulft + rrht * uurht - aq1) - fssub * p.rinf;
    L.f[2][i] = aj * (rulft * uulft + rurht * uurht + r1 * plar - aq2) - fssub * p.rinf * p.uinf;
    L.f[3][i] = aj * (rvlft * uulft + rvrht * uurht + r2 * plar - aq3) - fssub * p.rinf * p.vinf;
    L.f[4][i] = aj * (eplft * uulft + eprht * uurht - r3 * plar - aq4) - fssub * p.einf;
  }
}

/* tridag, eulerrhs.f:1562-1588: Thomas elimination of the rows ni..nl
 * (a sub-, b main, c super-diagonal, f right-hand side) into z. */
static void tridag(const std::vector<double>& a, const std::vector<double>& b, const std::vector<double>& c,
                   const std::vector<double>& f, std::vector<double>& z, int ni, int nl) {
  std::vector<double> w(nl + 2, 0.), g(nl + 2, 0.);
  w[ni] = c[ni] / b[ni];
  g[ni] = f[ni] / b[ni];
  for (int j = ni + 1; j <= nl; ++j) {
    double d = b[j] - a[j] * w[j - 1];
    double rd = 1.0 / d;
    w[j] = c[j] * rd;
    g[j] = (f[j] - a[j] * g[j - 1]) * rd;
  }
  z[nl] = g[nl];
  for (int j1 = 1; j1 <= nl - ni; ++j1) {
    int j = nl - j1;
    z[j] = g[j] - w[j] * z[j + 1];
  }
}

/* Fortran's amedian statement function of quad (eulerrhs.f:1256-1257):
 * b moved toward c and d by the smaller distance when both lie on one side */
static inline double amedian(double b, double c, double d) {
  return b + 0.5 * (fsign(1., c - b) + fsign(1., d - b)) * fmin2(std::fabs(c - b), std::fabs(d - b));
}

/* the sonic-A limited slope quad uses next to the line ends */
static inline double quad_sonic(double at, double ati1, double sl) {
  double t1 = ammd(at, ati1);
  return fsign(1., t1) * fmin2(0.5 * std::fabs(at + ati1), fmax2(2. * std::fabs(sl), std::fabs(t1)));
}

/* quad, eulerrhs.f:1233-1559 (ibmin = ibmax = 1 on the path): piecewise
 * quadratic reconstruction with compact sixth-order nodal slopes and
 * curvatures (two tridiagonal solves per line and variable), a median
 * correction of their signs and the monotonicity-preserving constraint
 * ("method 2").  cm, a scalar of the reference carried from one cell to the
 * next, starts at 0 for every line here (the reference leaves it
 * undefined; it is only read when amedian's sum rounds to none of its
 * arguments). */
static void quad(Line& L, int is, int ie, double qt) {
  if (qt == 0.0) {
    for (int n = 1; n <= 4; ++n) for (int i = is; i <= ie; ++i) { L.ql[n][i] = L.f[n][i]; L.qr[n][i] = L.f[n][i]; }
    return;
  }
  const int is1 = is + 1, is2 = is + 2, ie2 = ie - 2, ie1 = ie - 1;
  std::vector<double> d1(ie + 2, 0.), d2(ie + 2, 0.), con1(ie + 2, 0.), con2(ie + 2, 0.), con3(ie + 2, 0.);
  std::vector<double> s1(ie + 2, 0.), sf(ie + 2, 0.), sc(ie + 2, 0.), sb(ie + 2, 0.);
  for (int n = 1; n <= 4; ++n) {
    const std::vector<double>& f = L.f[n];
    std::vector<double>& ql = L.ql[n]; std::vector<double>& qr = L.qr[n];
    // slope: the two cells at each end (sonic-A), then the compact system
    int i = is;
    double f1i = f[i + 1] - f[i], f1i1 = f[i + 2] - f[i + 1], f1i2 = f[i + 3] - f[i + 2], f1i3 = f[i + 4] - f[i + 3];
    double f2i1 = f1i1 - f1i, f2i2 = f1i2 - f1i1, f2i3 = f1i3 - f1i2;
    double f2i = 2. * f2i1 - f2i2;
    double f2mi = ammd(f2i, f2i1), f2mi1 = ammd(f2i1, f2i2), f2mi2 = ammd(f2i2, f2i3);
    double at = f1i - 0.5 * f2mi;
    d1[i] = ammd(at, 2. * f1i);
    ql[i] = f[i] + 0.5 * d1[i];
    qr[i] = f[i] - 0.5 * d1[i];
    i = is1;
    d1[i] = quad_sonic(f1i1 - 0.5 * f2mi1, f1i + 0.5 * f2mi, ammd(f1i1, f1i));
    ql[i] = f[i] + 0.5 * d1[i];
    qr[i] = f[i] - 0.5 * d1[i];
    i = is2;
    const double slopes2 = quad_sonic(f1i2 - 0.5 * f2mi2, f1i1 + 0.5 * f2mi1, ammd(f1i2, f1i1));
    con1[i] = 0.25;
    con2[i] = 1.;
    con3[i] = 0.75 * (f[i + 1] - f[i - 1]);
    con3[i] = con3[i] - con1[i] * d1[i - 1];
    for (i = is + 3; i <= ie - 3; ++i) {
      con1[i] = 1. / 3.;
      con2[i] = 1.;
      con3[i] = (f[i + 2] + 28. * f[i + 1] - 28. * f[i - 1] - f[i - 2]) / 36.;
    }
    i = ie;
    f1i1 = f[i] - f[i - 1]; f1i2 = f[i - 1] - f[i - 2]; f1i3 = f[i - 2] - f[i - 3];
    double f1i4 = f[i - 3] - f[i - 4];
    f2i1 = f1i1 - f1i2; f2i2 = f1i2 - f1i3; f2i3 = f1i3 - f1i4;
    f2i = 2. * f2i1 - f2i2;
    f2mi1 = ammd(f2i1, f2i); f2mi2 = ammd(f2i2, f2i1);
    double f2mi3 = ammd(f2i3, f2i2);
    double at1 = f1i1 + 0.5 * f2mi1;
    d1[i] = ammd(at1, 2. * f1i1);
    ql[i] = f[i] + 0.5 * d1[i];
    qr[i] = f[i] - 0.5 * d1[i];
    i = ie1;
    d1[i] = quad_sonic(f1i1 - 0.5 * f2mi1, f1i2 + 0.5 * f2mi2, ammd(f1i1, f1i2));
    ql[i] = f[i] + 0.5 * d1[i];
    qr[i] = f[i] - 0.5 * d1[i];
    i = ie2;
    const double slopee2 = quad_sonic(f1i2 - 0.5 * f2mi2, f1i3 + 0.5 * f2mi3, ammd(f1i2, f1i3));
    con1[i] = 0.25;
    con2[i] = 1.;
    con3[i] = 0.75 * (f[i + 1] - f[i - 1]);
    con3[i] = con3[i] - con1[i] * d1[i + 1];
    tridag(con1, con2, con1, con3, d1, is2, ie2);
    // curvature
    d2[is] = 0.; d2[is1] = 0.;
    i = is2;
    con1[i] = 0.1;
    con2[i] = 1.;
    con3[i] = 1.2 * (f[i + 1] - 2. * f[i] + f[i - 1]);
    con3[i] = con3[i] - con1[i] * d2[i - 1];
    for (i = is + 3; i <= ie - 3; ++i) {
      con1[i] = 2. / 11.;
      con2[i] = 1.;
      con3[i] = (3. * f[i + 2] + 48. * f[i + 1] - 102. * f[i] + 48. * f[i - 1] + 3. * f[i - 2]) / 44.;
    }
    d2[ie] = 0.; d2[ie1] = 0.;
    i = ie2;
    con1[i] = 0.1;
    con2[i] = 1.;
    con3[i] = 1.2 * (f[i + 1] - 2. * f[i] + f[i - 1]);
    con3[i] = con3[i] - con1[i] * d2[i + 1];
    tridag(con1, con2, con1, con3, d2, is2, ie2);
    // signs of the slope and the curvature
    for (i = is1; i <= ie; ++i) s1[i] = f[i] - f[i - 1];
    for (i = is; i <= ie2; ++i) sf[i] = (-f[i + 2] + 4. * f[i + 1] - 3. * f[i]) / 2.;
    for (i = is1; i <= ie1; ++i) sc[i] = (f[i + 1] - f[i - 1]) / 2.;
    for (i = is2; i <= ie; ++i) sb[i] = (f[i - 2] - 4. * f[i - 1] + 3. * f[i]) / 2.;
    double cm = 0.;
    for (i = is2; i <= ie2; ++i) {
      double sm = amedian(sf[i], sc[i], sb[i]);
      if (sm == sf[i]) cm = f[i + 2] - 2. * f[i + 1] + f[i];
      if (sm == sc[i]) cm = f[i + 1] - 2. * f[i] + f[i - 1];
      if (sm == sb[i]) cm = f[i] - 2. * f[i - 1] + f[i - 2];
      d1[i] = amedian(d1[i], sm, sc[i]);
      if (d1[i] == sm) d2[i] = cm;
      if (d1[i] == sc[i]) d2[i] = f[i + 1] - 2. * f[i] + f[i - 1];
    }
    // monotonicity-preserving constraint (method 2) and the quadratic
    for (i = is2; i <= ie2; ++i) {
      double si = d1[i], ci = d2[i], sr, cr, sl, cl;
      const double ad = std::fabs(d1[i]);
      if (ad > 2.0 * std::fabs(s1[i + 1]) && ad > 2.0 * std::fabs(s1[i])) {
        if (ad <= std::fabs(d1[i + 1])) { sr = d1[i]; cr = 2. * (s1[i + 1] - d1[i]); }
        else { sr = 2. * s1[i + 1] - d1[i + 1]; cr = 2. * (-s1[i + 1] + d1[i + 1]); }
        if (ad <= std::fabs(d1[i - 1])) { sl = d1[i]; cl = 2. * (-s1[i] + d1[i]); }
        else { sl = 2. * s1[i] - d1[i - 1]; cl = 2. * (s1[i] - d1[i - 1]); }
        si = ammd(sl, sr);
        ci = ammd(cl, cr);
      } else {
        if (ad > 2.0 * std::fabs(s1[i + 1])) {
          if (ad <= std::fabs(d1[i + 1])) { sr = d1[i]; cr = 2. * (s1[i + 1] - d1[i]); }
          else { sr = 2. * s1[i + 1] - d1[i + 1]; cr = 2. * (-s1[i + 1] + d1[i + 1]); }
          si = ammd(d1[i], sr);
          ci = ammd(d2[i], cr);
        }
        if (ad > 2.0 * std::fabs(s1[i])) {
          if (ad <= std::fabs(d1[i - 1])) { sl = d1[i]; cl = 2. * (-s1[i] + d1[i]); }
          else { sl = 2. * s1[i] - d1[i - 1]; cl = 2. * (s1[i] - d1[i - 1]); }
          si = ammd(sl, d1[i]);
          ci = ammd(cl, d2[i]);
        }
      }
      ql[i] = f[i] + 0.5 * si + ci / 12.;
      qr[i] = f[i] - 0.5 * si + ci / 12.;
    }
    qr[is2] = f[is2] - 0.5 * slopes2;
    ql[ie2] = f[ie2] + 0.5 * slopee2;
  }
}

static void reconstruct(const P& p, Line& L, int n, double th, double qt, double eps, double epsl) {
  int ilima = std::abs(p.ilim);
  if (ilima == 0) iflux(L, 1, n, qt);
  if (ilima == 1) muscld_new(L, 1, n, n - 1, th, qt, epsl);
  if (ilima == 2) quad(L, 1, n, qt);
  if (p.ilim == 4) weno(L, 1, n, qt);
  (void)eps;
}

/* eulerrhs.f:2-280 with nei=1 */
void rhsup(const P& p, A3 q, A3 s, const double* xv_, const double* yv_, I2 iblank,
           const double* ugv_, const double* vgv_, const double* xold_, const double* yold_,
           const double* xole_, const double* yole_) {
  const int jd = p.jd, kd = p.kd, nq = p.nq, jmax = p.jmax, nhalo = p.nhalo;
  auto xv = [&](int j, int k) { return xv_[(size_t)(k - 1) * jmax + (j - 1)]; };
  auto yv = [&](int j, int k) { return yv_[(size_t)(k - 1) * jmax + (j - 1)]; };
  auto ugv = [&](int j, int k) { return ugv_[(size_t)(k - 1) * jmax + (j - 1)]; };
  auto vgv = [&](int j, int k) { return vgv_[(size_t)(k - 1) * jmax + (j - 1)]; };
  int irhs = std::abs(p.irhsy);
  double th = (double)(irhs - 2) / (double)irhs;
  double qt = 0.25; if (irhs == 1) qt = 0.0;
  double eps = 1.e-6;
  double epsj = p3(10. / (double)p.jmax), epsk = p3(10. / (double)p.kmax);
  std::vector<double> ppp_((size_t)jd * kd);
  A2 ppp{ppp_.data(), jd};
  for (int k = 1; k <= kd; ++k)
    for (int j = 1; j <= jd; ++j)
      ppp(j, k) = p.gm1 * (q(j, k, 4) - 0.5 * (p2(q(j, k, 2)) + p2(q(j, k, 3))) / q(j, k, 1));
  int mdim = (jd > kd ? jd : kd);
  Line L(mdim);
  if (p.iunst > 0 && (!xold_ || !yold_ || !xole_ || !yole_)) {
    std::fprintf(stderr, "oracle: iunst>0 needs the previous vertex levels\n"); std::abort();
  }
  auto xold = [&](int j, int k) { return xold_[(size_t)(k - 1) * jmax + (j - 1)]; };
  auto yold = [&](int j, int k) { return yold_[(size_t)(k - 1) * jmax + (j - 1)]; };
  auto xole = [&](int j, int k) { return xole_[(size_t)(k - 1) * jmax + (j - 1)]; };
  auto yole = [&](int j, int k) { return yole_[(size_t)(k - 1) * jmax + (j - 1)]; };
  /* xi fluxes */
  for (int k = p.kbeg; k <= p.kend; ++k) {
    int kv = k - nhalo + 1;
    for (int j = 1; j <= jd; ++j) {
      double rhoi = 1.0 / q(j, k, 1);
      L.f[1][j] = q(j, k, 1) * q(j, k, nq);
      L.f[2][j] = q(j, k, 2) * rhoi;
      L.f[3][j] = q(j, k, 3) * rhoi;
      L.f[4][j] = ppp(j, k) * q(j, k, nq);
      L.iba[j] = std::abs(iblank(j, k));
    }
    reconstruct(p, L, jd, th, qt, eps, epsj);
    for (int j = p.jbeg - 1; j <= p.jend; ++j) {
      int jv = j - nhalo + 1;
      L.xa[j] = (yv(jv, kv) - yv(jv, kv - 1));
      L.ya[j] = -(xv(jv, kv) - xv(jv, kv - 1));
    }
    if (p.iunst > 0) {
      /* eulerrhs.f:118-139: face speed from the area the face sweeps */
      for (int j = p.jbeg - 1; j <= p.jend; ++j) {
        int jv = j - nhalo + 1;
        double dx1 = xv(jv, kv) - xold(jv, kv - 1), dy1 = yv(jv, kv) - yold(jv, kv - 1);
        double dx2 = xold(jv, kv) - xv(jv, kv - 1), dy2 = yold(jv, kv) - yv(jv, kv - 1);
        L.tj[j] = -(0.5 * (dx1 * dy2 - dx2 * dy1) / p.dt);
      }
      if (p.ntac == 2 && p.istep > 1) {
        for (int j = p.jbeg - 1; j <= p.jend; ++j) {
          int jv = j - nhalo + 1;
          double dx1 = xold(jv, kv) - xole(jv, kv - 1), dy1 = yold(jv, kv) - yole(jv, kv - 1);
          double dx2 = xole(jv, kv) - xold(jv, kv - 1), dy2 = yole(jv, kv) - yold(jv, kv - 1);
          double temp = -(0.5 * (dx1 * dy2 - dx2 * dy1) / p.dt);
          L.tj[j] = 1.5 * L.tj[j] - 0.5 * temp;
        }
      }
    } else if (p.timespectral) {
      for (int j = p.jbeg - 1; j <= p.jend; ++j) {
        int jv = j - nhalo + 1;
        L.tj[j] = -0.5 * (ugv(jv, kv) + ugv(jv, kv - 1)) * L.xa[j] - 0.5 * (vgv(jv, kv) + vgv(jv, kv - 1)) * L.ya[j];
      }
    } else {
      for (int j = p.jbeg - 1; j <= p.jend; ++j) L.tj[j] = 0.0;
    }
    if (p.iprecon) roetrklflx(p, L, p.jbeg - 1, p.jend);
    else roeflx(p, L, p.jbeg - 1, p.jend);
    for (int j = p.jbeg; j <= p.jend; ++j)
      for (int n = 1; n <= 4; ++n) s(j, k, n) = s(j, k, n) - (L.f[n][j] - L.f[n][j - 1]);
  }
  /* eta fluxes */
  for (int j = p.jbeg; j <= p.jend; ++j) {
    int jv = j - nhalo + 1;
    for (int k = 1; k <= kd; ++k) {
      double rhoi = 1.0 / q(j, k, 1);
      L.f[1][k] = q(j, k, 1) * q(j, k, nq);
      L.f[2][k] = q(j, k, 2) * rhoi;
      L.f[3][k] = q(j, k, 3) * rhoi;
      L.f[4][k] = ppp(j, k) * q(j, k, nq);
      L.iba[k] = std::abs(iblank(j, k));
    }
    reconstruct(p, L, kd, th, qt, eps, epsk);
    for (int k = p.kbeg - 1; k <= p.kend; ++k) {
      int kv = k - nhalo + 1;
      L.xa[k] = -(yv(jv, kv) - yv(jv - 1, kv));
      L.ya[k] = (xv(jv, kv) - xv(jv - 1, kv));
    }
    if (p.iunst > 0) {
      /* eulerrhs.f:224-246 */
      for (int k = p.kbeg - 1; k <= p.kend; ++k) {
        int kv = k - nhalo + 1;
        double dx1 = xv(jv, kv) - xold(jv - 1, kv), dy1 = yv(jv, kv) - yold(jv - 1, kv);
        double dx2 = xold(jv, kv) - xv(jv - 1, kv), dy2 = yold(jv, kv) - yv(jv - 1, kv);
        L.tj[k] = 0.5 * (dx1 * dy2 - dx2 * dy1) / p.dt;
      }
      if (p.ntac == 2 && p.istep > 1) {
        for (int k = p.kbeg - 1; k <= p.kend; ++k) {
          int kv = k - nhalo + 1;
          double dx1 = xold(jv, kv) - xole(jv - 1, kv), dy1 = yold(jv, kv) - yole(jv - 1, kv);
          double dx2 = xole(jv, kv) - xold(jv - 1, kv), dy2 = yole(jv, kv) - yold(jv - 1, kv);
          double temp = 0.5 * (dx1 * dy2 - dx2 * dy1) / p.dt;
          L.tj[k] = 1.5 * L.tj[k] - 0.5 * temp;
        }
      }
    } else if (p.timespectral) {
      for (int k = p.kbeg - 1; k <= p.kend; ++k) {
        int kv = k - nhalo + 1;
        L.tj[k] = -0.5 * (ugv(jv, kv) + ugv(jv - 1, kv)) * L.xa[k] - 0.5 * (vgv(jv, kv) + vgv(jv - 1, kv)) * L.ya[k];
      }
    } else {
      for (int k = p.kbeg - 1; k <= p.kend; ++k) L.tj[k] = 0.;
    }
    if (p.iprecon) roetrklflx(p, L, p.kbeg - 1, p.kend);
    else roeflx(p, L, p.kbeg - 1, p.kend);
    for (int k = p.kbeg; k <= p.kend; ++k)
      for (int n = 1; n <= 4; ++n) s(j, k, n) = s(j, k, n) - (L.f[n][k] - L.f[n][k - 1]);
  }
}

/* visrhs.f:2-287 */
void visrhs(const P& p, A2 turmu, A3 q, A3 s, A2 xx, A2 xy, A2 yx, A2 yy) {
  const int jd = p.jd, kd = p.kd, nq = p.nq;
  const double gamma = p.gamma, ggm1 = p.ggm1;
  double gkpr = gamma / p.pr, prtr = p.pr / 0.9, dre = .5 / p.rey;
  double c2b = 198.6 / p.tinf, c2bp = c2b + 1.;
  int mdim = (jd > kd ? jd : kd) + 2;
  std::vector<double> f2(mdim), f3(mdim), f4(mdim), f2v(mdim), f3v(mdim), f4v(mdim), u(mdim), v(mdim), e(mdim);
  std::vector<double> a1v(mdim), a2v(mdim), a4v(mdim), a5v(mdim), d1v(mdim), d2v(mdim), d4v(mdim), d5v(mdim), d7v(mdim);
  std::vector<double>& b1v = a1v; std::vector<double>& b2v = a2v; std::vector<double>& b4v = a4v; std::vector<double>& b5v = a5v;
  /* eta direction */
  for (int j = p.jbeg; j <= p.jend; ++j) {
    for (int k = 1; k <= kd; ++k) {
      double ra = 1. / q(j, k, 1);
      u[k] = q(j, k, 2) * ra; v[k] = q(j, k, 3) * ra;
      e[k] = q(j, k, 4) * ra - .5 * (p2(u[k]) + p2(v[k]));
      double tt = ggm1 * e[k];
      double vmue = c2bp * tt * std::sqrt(tt) / (c2b + tt);
      double turm = turmu(j, k);
      double vnu = vmue + turm, gkap = vmue + prtr * turm;
      double rj = 1. / q(j, k, nq), rjm = 1. / q(j - 1, k, nq), rjp = 1. / q(j + 1, k, nq);
      b4v[k] = (p2(yx(j, k)) + p2(yy(j, k))) * rj;
      b1v[k] = (b4v[k] + p2(yx(j, k)) / 3. * rj) * vnu * dre;
      b2v[k] = (b4v[k] + p2(yy(j, k)) / 3. * rj) * vnu * dre;
      b5v[k] = (yx(j, k) * yy(j, k) / 3. * rj) * vnu * dre;
      b4v[k] = b4v[k] * gkpr * gkap * dre;
      d1v[k] = (4. / 3. * xx(j - 1, k) * yx(j - 1, k) + xy(j - 1, k) * yy(j - 1, k)) * rjm;
      d1v[k] = d1v[k] + (4. / 3. * xx(j + 1, k) * yx(j + 1, k) + xy(j + 1, k) * yy(j + 1, k)) * rjp;
      d1v[k] = vnu * dre * d1v[k];
      d2v[k] = (4. / 3. * xy(j - 1, k) * yy(j - 1, k) + xx(j - 1, k) * yx(j - 1, k)) * rjm;
      d2v[k] = d2v[k] + (4. / 3. * xy(j + 1, k) * yy(j + 1, k) + xx(j + 1, k) * yx(j + 1, k)) * rjp;
      d2v[k] = vnu * dre * d2v[k];
      d4v[k] = (xy(j - 1, k) * yy(j - 1, k) + xx(j - 1, k) * yx(j - 1, k)) * rjm;
      d4v[k] = d4v[k] + (xy(j + 1, k) * yy(j + 1, k) + xx(j + 1, k) * yx(j + 1, k)) * rjp;
      d4v[k] = d4v[k] * gkpr * gkap * dre;
      d5v[k] = (-2. / 3. * xy(j - 1, k) * yx(j - 1, k) + xx(j - 1, k) * yy(j - 1, k)) * rjm;
      d5v[k] = d5v[k] + (-2. / 3. * xy(j + 1, k) * yx(j + 1, k) + xx(j + 1, k) * yy(j + 1, k)) * rjp;
      d5v[k] = vnu * dre * d5v[k];
      d7v[k] = (-2. / 3. * xx(j - 1, k) * yy(j - 1, k) + xy(j - 1, k) * yx(j - 1, k)) * rjm;
      d7v[k] = d7v[k] + (-2. / 3. * xx(j + 1, k) * yy(j + 1, k) + xy(j + 1, k) * yx(j + 1, k)) * rjp;
      d7v[k] = vnu * dre * d7v[k];
    }
    for (int k = 1; k <= kd - 1; ++k) {
      int k1 = k + 1;
      double b1 = b1v[k1] + b1v[k], b2 = b2v[k1] + b2v[k], b5 = b5v[k1] + b5v[k], b4 = b4v[k1] + b4v[k];
      (void)b4;
      double d1 = d1v[k], d2 = d2v[k], d4 = d4v[k], d5 = d5v[k], d7 = d7v[k];
      double ujp1 = q(j + 1, k, 2) / q(j + 1, k, 1), ujm1 = q(j - 1, k, 2) / q(j - 1, k, 1);
      double duj = 0.5 * (ujp1 - ujm1);
      double vjp1 = q(j + 1, k, 3) / q(j + 1, k, 1), vjm1 = q(j - 1, k, 3) / q(j - 1, k, 1);
      double dvj = 0.5 * (vjp1 - vjm1);
      double ejp1 = q(j + 1, k, 4) / q(j + 1, k, 1) - .5 * (p2(ujp1) + p2(vjp1));
      double ejm1 = q(j - 1, k, 4) / q(j - 1, k, 1) - .5 * (p2(ujm1) + p2(vjm1));
      double dej = 0.5 * (ejp1 - ejm1);
      double t4 = u[k1] * b1v[k1] + u[k] * b1v[k];
      double t5 = v[k1] * b2v[k1] + v[k] * b2v[k];
      double t6 = u[k1] * b5v[k1] + u[k] * b5v[k];
      double t7 = v[k1] * b5v[k1] + v[k] * b5v[k];
      double t8 = b4v[k1] + b4v[k];
      double du = u[k1] - u[k], dv = v[k1] - v[k], dei = e[k1] - e[k];
      f2[k] = b1 * du + b5 * dv;
      f2v[k] = d1 * duj + d5 * dvj;
      f3[k] = b5 * du + b2 * dv;
      f3v[k] = d7 * duj + d2 * dvj;
      f4[k] = (t4 + t7) * du + (t5 + t6) * dv + t8 * dei;
      f4v[k] = 0.5 * d1 * 0.5 * (p2(ujp1) - p2(ujm1));
      f4v[k] = f4v[k] + 0.5 * d2 * 0.5 * (p2(vjp1) - p2(vjm1));
      f4v[k] = f4v[k] + d5 * 0.5 * (ujp1 + ujm1) * dvj;
      f4v[k] = f4v[k] + d7 * 0.5 * (vjp1 + vjm1) * duj;
      f4v[k] = f4v[k] + d4 * dej;
    }
    int ke;
    if (p.nhalo == 1) {
      ke = p.kend - 1;
      int k = p.kend;
      s(j, k, 2) = s(j, k, 2) + (f2[k] - f2[k - 1]) + 0.5 * (f2v[k - 2] - 4. * f2v[k - 1] + 3 * f2v[k]);
      s(j, k, 3) = s(j, k, 3) + (f3[k] - f3[k - 1]) + 0.5 * (f3v[k - 2] - 4. * f3v[k - 1] + 3 * f3v[k]);
      s(j, k, 4) = s(j, k, 4) + (f4[k] - f4[k - 1]) + 0.5 * (f4v[k - 2] - 4. * f4v[k - 1] + 3. * f4v[k]);
    } else ke = p.kend;
    for (int k = p.kbeg; k <= ke; ++k) {
      s(j, k, 2) = s(j, k, 2) + (f2[k] - f2[k - 1]) + 0.5 * (f2v[k + 1] - f2v[k - 1]);
      s(j, k, 3) = s(j, k, 3) + (f3[k] - f3[k - 1]) + 0.5 * (f3v[k + 1] - f3v[k - 1]);
      s(j, k, 4) = s(j, k, 4) + (f4[k] - f4[k - 1]) + 0.5 * (f4v[k + 1] - f4v[k - 1]);
    }
  }
  /* xi direction */
  for (int k = p.kbeg; k <= p.kend; ++k) {
    for (int j = 1; j <= jd; ++j) {
      double ra = 1. / q(j, k, 1);
      u[j] = q(j, k, 2) * ra; v[j] = q(j, k, 3) * ra;
      e[j] = q(j, k, 4) * ra - .5 * (p2(u[j]) + p2(v[j]));
      double tt = ggm1 * e[j];
      double vmue = c2bp * tt * std::sqrt(tt) / (c2b + tt);
      double turm = turmu(j, k);
      double vnu = vmue + turm, gkap = vmue + prtr * turm;
      double rj = 1. / q(j, k, nq), rkm = 1. / q(j, k - 1, nq), rkp = 1. / q(j, k + 1, nq);
      a4v[j] = (p2(xx(j, k)) + p2(xy(j, k))) * rj;
      a1v[j] = (a4v[j] + p2(xx(j, k)) / 3. * rj) * vnu * dre;
      a2v[j] = (a4v[j] + p2(xy(j, k)) / 3. * rj) * vnu * dre;
      a5v[j] = (xx(j, k) * xy(j, k) / 3. * rj) * vnu * dre;
      a4v[j] = a4v[j] * gkpr * gkap * dre;
      d1v[j] = (4. / 3. * xx(j, k - 1) * yx(j, k - 1) + xy(j, k - 1) * yy(j, k - 1)) * rkm;
      d1v[j] = d1v[j] + (4. / 3. * xx(j, k + 1) * yx(j, k + 1) + xy(j, k + 1) * yy(j, k + 1)) * rkp;
      d1v[j] = vnu * dre * d1v[j];
      d2v[j] = (4. / 3. * xy(j, k - 1) * yy(j, k - 1) + xx(j, k - 1) * yx(j, k - 1)) * rkm;
      d2v[j] = d2v[j] + (4. / 3. * xy(j, k + 1) * yy(j, k + 1) + xx(j, k + 1) * yx(j, k + 1)) * rkp;
      d2v[j] = vnu * dre * d2v[j];
      d4v[j] = (xy(j, k - 1) * yy(j, k - 1) + xx(j, k - 1) * yx(j, k - 1)) * rkm;
      d4v[j] = d4v[j] + (xy(j, k + 1) * yy(j, k + 1) + xx(j, k + 1) * yx(j, k + 1)) * rkp;
      d4v[j] = d4v[j] * gkpr * gkap * dre;
      d5v[j] = (-2. / 3. * xy(j, k - 1) * yx(j, k - 1) + xx(j, k - 1) * yy(j, k - 1)) * rkm;
      d5v[j] = d5v[j] + (-2. / 3. * xy(j, k + 1) * yx(j, k + 1) + xx(j, k + 1) * yy(j, k + 1)) * rkp;
      d5v[j] = vnu * dre * d5v[j];
      d7v[j] = (-2. / 3. * xx(j, k - 1) * yy(j, k - 1) + xy(j, k - 1) * yx(j, k - 1)) * rkm;
      d7v[j] = d7v[j] + (-2. / 3. * xx(j, k + 1) * yy(j, k + 1) + xy(j, k + 1) * yx(j, k + 1)) * rkp;
      d7v[j] = vnu * dre * d7v[j];
    }
    for (int j = 1; j <= jd - 1; ++j) {
      int j1 = j + 1;
      double a1 = a1v[j1] + a1v[j], a2 = a2v[j1] + a2v[j], a5 = a5v[j1] + a5v[j];
      double d1 = d1v[j], d2 = d2v[j], d4 = d4v[j], d5 = d5v[j], d7 = d7v[j];
      double ukp1 = q(j, k + 1, 2) / q(j, k + 1, 1), ukm1 = q(j, k - 1, 2) / q(j, k - 1, 1);
      double duk = 0.5 * (ukp1 - ukm1);
      double vkp1 = q(j, k + 1, 3) / q(j, k + 1, 1), vkm1 = q(j, k - 1, 3) / q(j, k - 1, 1);
      double dvk = 0.5 * (vkp1 - vkm1);
      double ekp1 = q(j, k + 1, 4) / q(j, k + 1, 1) - .5 * (p2(ukp1) + p2(vkp1));
      double ekm1 = q(j, k - 1, 4) / q(j, k - 1, 1) - .5 * (p2(ukm1) + p2(vkm1));
      double dek = 0.5 * (ekp1 - ekm1);
      double t4 = u[j1] * a1v[j1] + u[j] * a1v[j];
      double t5 = v[j1] * a2v[j1] + v[j] * a2v[j];
      double t6 = u[j1] * a5v[j1] + u[j] * a5v[j];
      double t7 = v[j1] * a5v[j1] + v[j] * a5v[j];
      double t8 = a4v[j1] + a4v[j];
      double du = u[j1] - u[j], dv = v[j1] - v[j], dei = e[j1] - e[j];
      f2[j] = a1 * du + a5 * dv;
      f2v[j] = d1 * duk + d7 * dvk;
      f3[j] = a5 * du + a2 * dv;
      f3v[j] = d5 * duk + d2 * dvk;
      f4[j] = (t4 + t7) * du + (t5 + t6) * dv + t8 * dei;
      f4v[j] = 0.5 * d1 * 0.5 * (p2(ukp1) - p2(ukm1));
      f4v[j] = f4v[j] + 0.5 * d2 * 0.5 * (p2(vkp1) - p2(vkm1));
      f4v[j] = f4v[j] + d5 * 0.5 * (vkp1 + vkm1) * duk;
      f4v[j] = f4v[j] + d7 * 0.5 * (ukp1 + ukm1) * dvk;
      f4v[j] = f4v[j] + d4 * dek;
    }
    int je;
    if (p.nhalo == 1) {
      je = p.jend - 1;
      int j = p.jend;
      s(j, k, 2) = s(j, k, 2) + (f2[j] - f2[j - 1]) + 0.5 * (f2v[j - 2] - 4. * f2v[j - 1] + 3 * f2v[j]);
      s(j, k, 3) = s(j, k, 3) + (f3[j] - f3[j - 1]) + 0.5 * (f3v[j - 2] - 4. * f3v[j - 1] + 3 * f3v[j]);
      s(j, k, 4) = s(j, k, 4) + (f4[j] - f4[j - 1]) + 0.5 * (f4v[j - 2] - 4. * f4v[j - 1] + 3 * f4v[j]);
    } else je = p.jend;
    for (int j = p.jbeg; j <= je; ++j) {
      s(j, k, 2) = s(j, k, 2) + (f2[j] - f2[j - 1]) + 0.5 * (f2v[j + 1] - f2v[j - 1]);
      s(j, k, 3) = s(j, k, 3) + (f3[j] - f3[j - 1]) + 0.5 * (f3v[j + 1] - f3v[j - 1]);
      s(j, k, 4) = s(j, k, 4) + (f4[j] - f4[j - 1]) + 0.5 * (f4v[j + 1] - f4v[j - 1]);
    }
  }
}

}  // namespace oro

/* Test hook: roeflx on one face, left state ql and right state qr (the
 * primitives rho, u, v, p), face vector (ri1, ri2), grid-speed term ri3;
 * the four fluxes out in f.  No counterpart in the reference. */
extern "C" void oro_roe_face(double gm1, const double* ql, const double* qr, double ri1, double ri2, double ri3,
                             double* f) {
  oro::P p{};
  p.gm1 = gm1;
  oro::Line L(2);
  for (int n = 1; n <= 4; ++n) { L.ql[n][1] = ql[n - 1]; L.qr[n][2] = qr[n - 1]; }
  L.xa[1] = ri1; L.ya[1] = ri2; L.tj[1] = ri3;
  oro::roeflx(p, L, 1, 1);
  for (int n = 1; n <= 4; ++n) f[n - 1] = L.f[n][1];
}

/* Test hook: quad on one line of primitives f[0..n) (one variable; the
 * other three lines a copy of it), ql/qr out.  No counterpart in the
 * reference. */
extern "C" void oro_quad_line(const double* f, int n, double qt, double* ql, double* qr) {
  oro::Line L(n);
  for (int v = 1; v <= 4; ++v)
    for (int i = 1; i <= n; ++i) L.f[v][i] = f[i - 1];
  oro::quad(L, 1, n, qt);
  for (int i = 1; i <= n; ++i) { ql[i - 1] = L.ql[1][i]; qr[i - 1] = L.qr[1][i]; }
}
