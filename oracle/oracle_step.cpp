/*
 * oracle_step.cpp -- TEST INFRASTRUCTURE ONLY (see oracle_common.h).
 * FP64 restatement of the per-iteration orchestrator (src/step.f), the
 * time-spectral coupling (src/sources.f:2-27), the speed-of-sound monitor,
 * the force integration (src/forces.f), and a driver that mirrors the
 * iteration loop of src/Turns_overset.f:360-505 for single-grid runs.
 * Everything is exported with C linkage (prefix oro_) for the Python tests.
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include "oracle.h"

namespace oro {

/* sources.f:2-27; q, s are the full (jd,kd,nspec,n) arrays */
void timespectralrhs(const P& p, const double* q, double* s, const double* Ds, int nsp) {
  const int jd = p.jd, kd = p.kd, nspec = p.nspec;
  size_t n2 = (size_t)jd * kd;
  for (int n = 1; n <= p.nv; ++n)
    for (int nsp1 = 1; nsp1 <= nspec; ++nsp1) {
      double dsn = Ds[(size_t)(nsp1 - 1) * nspec + (nsp - 1)];
      for (int k = p.kbeg; k <= p.kend; ++k)
        for (int j = p.jbeg; j <= p.jend; ++j) {
          size_t o = (size_t)(k - 1) * jd + (j - 1);
          double& sv = s[((size_t)(n - 1) * nspec + (nsp - 1)) * n2 + o];
          sv = sv - p.rotf * dsn * q[((size_t)(n - 1) * nspec + (nsp1 - 1)) * n2 + o];
        }
    }
}

/* step.f:332-392 */
int monitor(const P& p, A3 q) {
  const double asqmin = 0.002; int nneg = 0;
  for (int k = 1; k <= p.kd; ++k) for (int j = 1; j <= p.jd; ++j) {
    double rho = q(j, k, 1);
    double qq = p2(q(j, k, 2)) + p2(q(j, k, 3));
    double asq = p.ggm1 * (q(j, k, 4) - .5 * qq / rho) / rho;
    if (asq <= asqmin || asq + 1 == asq || asq != asq) ++nneg;
  }
  return nneg;
}

/* forces.f:130-398 ; out = {cfx, cfy, cm0, cpower} */
void force2d(const P& p, A3 q, A2 x, A2 y, const double* xv_, const double* yv_,
             A2 xx, A2 xy, A2 yx, A2 yy, double* out) {
  (void)x; (void)y;
  const int jmax = p.jmax, nhalo = p.nhalo, nq = p.nq; const double gm1 = p.gm1, gamma = p.gamma;
  auto xv = [&](int j, int k) { return xv_[(size_t)(k - 1) * jmax + (j - 1)]; };
  auto yv = [&](int j, int k) { return yv_[(size_t)(k - 1) * jmax + (j - 1)]; };
  int k = p.kbeg, k2 = k + 1, k3 = k2 + 1, j1 = p.jtail1, j2 = p.jtail2;
  double fmm = (p.fsmach != 0) ? p.fsmach : ((p.fmtip != 0) ? p.fmtip : 1.0);
  std::vector<double> zz(p.jd + 2), sxx(p.jd + 2), syy(p.jd + 2);
  for (int j = j1; j <= j2; ++j) {
    double rr = 1. / q(j, k, 1), rho = q(j, k, 1) * q(j, k, nq);
    double u = q(j, k, 2) * rr, v = q(j, k, 3) * rr, e = q(j, k, 4) * q(j, k, nq);
    double vsq = u * u + v * v, pp = gm1 * (e - rho * vsq / 2.), pp1 = pp / p.pinf;
    double cp = 2. * (pp1 - 1.) / (gamma * p2(fmm));
    zz[j] = cp;
    rr = 1. / q(j, k - 1, 1); rho = q(j, k - 1, 1) * q(j, k - 1, nq);
    u = q(j, k - 1, 2) * rr; v = q(j, k - 1, 3) * rr; e = q(j, k - 1, 4) * q(j, k - 1, nq);
    vsq = u * u + v * v; pp = gm1 * (e - rho * vsq / 2.); pp1 = pp / p.pinf;
    cp = 2. * (pp1 - 1.) / (gamma * p2(fmm));
    zz[j] = 0.5 * (zz[j] + cp);
  }
  double cn = 0., cc = 0., cmle = 0., cpinv = 0.;
  for (int j = j1; j <= j2; ++j) {
    int jv = j - nhalo, kv = k - nhalo;
    cn = cn - zz[j] * (xv(jv + 1, kv) - xv(jv, kv));
    cc = cc + zz[j] * (yv(jv + 1, kv) - yv(jv, kv));
    cmle = cmle + zz[j] * (0.5 * (xv(jv + 1, kv) + xv(jv, kv)) * (xv(jv + 1, kv) - xv(jv, kv)) +
                           0.5 * (yv(jv + 1, kv) + yv(jv, kv)) * (yv(jv + 1, kv) - yv(jv, kv)));
    double u = q(j, k, 2) / q(j, k, 1), v = q(j, k, 3) / q(j, k, 1);
    double um = q(j, k - 1, 2) / q(j, k - 1, 1), vm = q(j, k - 1, 3) / q(j, k - 1, 1);
    cpinv = cpinv + 0.5 * (u + um) * zz[j] * (yv(jv + 1, kv) - yv(jv, kv)) - 0.5 * (v + vm) * zz[j] * (xv(jv + 1, kv) - xv(jv, kv));
  }
  double half = (double)p.half;
  cn = cn - half * cn; cmle = cmle - half * cmle; cc = cc + half * cc;
  double cnv = 0., ccv = 0., cmlev = 0., cpv = 0.;
  if (!p.invisc) {
    double alngth = 1., amu = p.rinf * alngth / p.rey, uinf2 = p2(fmm);
    auto wall = [&](int j, double uxi, double vxi) {
      double ueta = -1.5 * q(j, k, 2) / q(j, k, 1) + 2. * q(j, k2, 2) / q(j, k2, 1) - .5 * q(j, k3, 2) / q(j, k3, 1);
      double veta = -1.5 * q(j, k, 3) / q(j, k, 1) + 2. * q(j, k2, 3) / q(j, k2, 1) - .5 * q(j, k3, 3) / q(j, k3, 1);
      double xix = xx(j, k), xiy = xy(j, k), etax = yx(j, k), etay = yy(j, k);
      double sfdiv = 2. / 3 * (uxi * xix + ueta * etax + vxi * xiy + veta * etay);
      sxx[j] = amu * (2. * (uxi * xix + ueta * etax) - sfdiv);
      syy[j] = amu * (2. * (vxi * xiy + veta * etay) - sfdiv);
      double tauw = amu * ((uxi * xiy + ueta * etay) + (vxi * xix + veta * etax));
      sxx[j] = sxx[j] / (.5 * p.rinf * uinf2);
      syy[j] = syy[j] / (.5 * p.rinf * uinf2);
      zz[j] = tauw / (.5 * p.rinf * uinf2);
    };
    {
      int j = j1, jp1 = j + 1;
      double uxi = q(jp1, k, 2) / q(jp1, k, 1) - q(j, k, 2) / q(j, k, 1);
      double vxi = q(jp1, k, 3) / q(jp1, k, 1) - q(j, k, 3) / q(j, k, 1);
      wall(j, uxi, vxi);
    }
    {
      int j = j2, jm1 = j - 1;
      double uxi = q(j, k, 2) / q(j, k, 1) - q(jm1, k, 2) / q(jm1, k, 1);
      double vxi = q(j, k, 3) / q(j, k, 1) - q(jm1, k, 3) / q(jm1, k, 1);
      wall(j, uxi, vxi);
    }
    for (int j = j1 + 1; j <= j2 - 1; ++j) {
      int jp1 = j + 1, jm1 = j - 1;
      double uxi = .5 * (q(jp1, k, 2) / q(jp1, k, 1) - q(jm1, k, 2) / q(jm1, k, 1));
      double vxi = .5 * (q(jp1, k, 3) / q(jp1, k, 1) - q(jm1, k, 3) / q(jm1, k, 1));
      wall(j, uxi, vxi);
    }
    for (int j = j1; j <= j2; ++j) {
      int jv = j - nhalo, kv = k - nhalo;
      double dxv = xv(jv + 1, kv) - xv(jv, kv), dyv = yv(jv + 1, kv) - yv(jv, kv);
      ccv = ccv + zz[j] * (xv(jv + 1, kv) - xv(jv, kv)) - sxx[j] * (yv(jv + 1, kv) - yv(jv, kv));
      cnv = cnv - zz[j] * (yv(jv + 1, kv) - yv(jv, kv)) + syy[j] * (xv(jv + 1, kv) - xv(jv, kv));
      cmlev = cmlev + zz[j] * (0.5 * (xv(jv + 1, kv) + xv(jv, kv)) * (yv(jv + 1, kv) - yv(jv, kv)) +
                               0.5 * (yv(jv + 1, kv) + yv(jv, kv)) * (xv(jv + 1, kv) - xv(jv, kv))) -
              0.5 * (xv(jv + 1, kv) + xv(jv, kv)) * (xv(jv + 1, kv) - xv(jv, kv)) * syy[j] -
              0.5 * (yv(jv + 1, kv) + yv(jv, kv)) * (yv(jv + 1, kv) - yv(jv, kv)) * sxx[j];
      (void)dxv; (void)dyv;
      double u = q(j, k, 2) / q(j, k, 1), v = q(j, k, 3) / q(j, k, 1);
      double um = q(j, k - 1, 2) / q(j, k - 1, 1), vm = q(j, k - 1, 3) / q(j, k - 1, 1);
      cpv = cpv + 0.5 * (u + um) * zz[j] * (xv(jv + 1, kv) - xv(jv, kv)) - 0.5 * (u + um) * sxx[j] * (yv(jv + 1, kv) - yv(jv, kv)) -
            0.5 * (v + vm) * zz[j] * (yv(jv + 1, kv) - yv(jv, kv)) + 0.5 * (v + vm) * syy[j] * (xv(jv + 1, kv) - xv(jv, kv));
    }
    cnv = cnv - half * cnv; cmlev = cmlev - half * cmlev; ccv = ccv + half * ccv;
  }
  out[0] = cc + ccv;
  out[1] = cn + cnv;
  out[2] = cmle + cmlev;
  out[3] = (cpinv + cpv) / fmm;
}

}  // namespace oro

using namespace oro;

/* ------------------------------------------------------------------ */
/* Flat C API for the test harness (ctypes).  Array pointers follow the
 * reference layout; a multi-variable argument points at the first variable
 * of one time instance and strides jd*kd*nspec between variables. */
extern "C" {

static inline A3 v3(const P* p, double* a) { return A3{a, p->jd, (size_t)p->jd * p->kd * p->nspec}; }
static inline A2 v2(const P* p, double* a) { return A2{a, p->jd}; }

void oro_read_inputs(const ot2d_inputs* in, ot2d_params* p) { read_inputs(*in, *p); }
void oro_find_cellcenter(const P* p, double* x, double* y, const double* xv, const double* yv) {
  find_cellcenter(*p, v2(p, x), v2(p, y), xv, yv);
}
int oro_metfv(const P* p, double* q, const double* xv, const double* yv, double* xx, double* xy, double* yx, double* yy) {
  return metfv(*p, v3(p, q), xv, yv, v2(p, xx), v2(p, xy), v2(p, yx), v2(p, yy));
}
void oro_qzero(const P* p, double* q) { qzero(*p, v3(p, q)); }
void oro_qdivj(const P* p, double* q) { qdivj(*p, v3(p, q)); }
void oro_computeTScoefs(int n, double* Ds) { computeTScoefs(n, Ds); }
void oro_timespectralrhs(const P* p, const double* q, double* s, const double* Ds, int nsp) {
  timespectralrhs(*p, q, s, Ds, nsp);
}
void oro_find_coord_TS_orig(const P* p, double* xv, double* yv, const double* xv1, const double* yv1, double tspec) {
  find_coord_TS_orig(*p, xv, yv, xv1, yv1, tspec);
}
void oro_find_timemetrics_TS_orig(const P* p, double* x, double* y, const double* xv, const double* yv, double tspec,
                                  double* ug, double* vg, double* ugv, double* vgv) {
  find_timemetrics_TS_orig(*p, v2(p, x), v2(p, y), xv, yv, tspec, v2(p, ug), v2(p, vg), ugv, vgv);
}
void oro_bc(const P* p, double* q, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg, double* bt) {
  A2 z{nullptr, p->jd};
  bc(*p, v3(p, q), z, z, v2(p, xx), v2(p, xy), v2(p, yx), v2(p, yy), v2(p, ug), v2(p, vg), v2(p, bt));
}
void oro_rbc(const P* p, double* q, double* s) { rbc(*p, v3(p, q), v3(p, s)); }
void oro_rhsup(const P* p, double* q, double* s, const double* xv, const double* yv, const int32_t* iblank,
               const double* ugv, const double* vgv) {
  rhsup(*p, v3(p, q), v3(p, s), xv, yv, I2{iblank, p->jd}, ugv, vgv);
}
void oro_visrhs(const P* p, double* turmu, double* q, double* s, double* xx, double* xy, double* yx, double* yy) {
  visrhs(*p, v2(p, turmu), v3(p, q), v3(p, s), v2(p, xx), v2(p, xy), v2(p, yx), v2(p, yy));
}
void oro_time_step(const P* p, double* q, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg,
                   double* tscale, double* bt, const int32_t* iblank) {
  time_step(*p, v3(p, q), v2(p, xx), v2(p, xy), v2(p, yx), v2(p, yy), v2(p, ug), v2(p, vg), v2(p, tscale), v2(p, bt),
            I2{iblank, p->jd});
}
void oro_ilu2d(const P* p, double* q, double* s, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg,
               double* turmu, double* tscale) {
  ilu2d(*p, v3(p, q), v3(p, s), v2(p, xx), v2(p, xy), v2(p, yx), v2(p, yy), v2(p, ug), v2(p, vg), v2(p, turmu),
        v2(p, tscale));
}
void oro_preilu2d(const P* p, double* q, double* s, double* xx, double* xy, double* yx, double* yy, double* ug,
                  double* vg, double* turmu, double* tscale, double* bt) {
  preilu2d(*p, v3(p, q), v3(p, s), v2(p, xx), v2(p, xy), v2(p, yx), v2(p, yy), v2(p, ug), v2(p, vg), v2(p, turmu),
           v2(p, tscale), v2(p, bt));
}
void oro_rhslom(const P* p, double* q, double* s, double* bt) { rhslom(*p, v3(p, q), v3(p, s), v2(p, bt)); }
double oro_vmu_sa(const P* p, double* q, double* s, double* turmu, double* x, double* y, const double* xv, const double* yv,
                  double* xx, double* xy, double* yx, double* yy, double* ug, double* vg, double* tscale,
                  const int32_t* iblank) {
  double r = 0;
  vmu_sa(*p, v3(p, q), v3(p, s), v2(p, turmu), v2(p, x), v2(p, y), xv, yv, v2(p, xx), v2(p, xy), v2(p, yx), v2(p, yy),
         v2(p, ug), v2(p, vg), v2(p, tscale), I2{iblank, p->jd}, &r);
  return r;
}
void oro_komegasst(const P* p, double* q, double* s, double* turmu, double* x, double* y, const double* xv,
                   const double* yv, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg,
                   double* tscale, const int32_t* iblank, double* res) {
  komegasst(*p, v3(p, q), v3(p, s), v2(p, turmu), v2(p, x), v2(p, y), xv, yv, v2(p, xx), v2(p, xy), v2(p, yx),
            v2(p, yy), v2(p, ug), v2(p, vg), v2(p, tscale), I2{iblank, p->jd}, res);
}
void oro_arc2d(const P* p, double* q, double* s, double* xx, double* xy, double* yx, double* yy, double* ug,
               double* vg, double* turmu, const int32_t* iblank, double* tscale, double* bt) {
  arc2d(*p, v3(p, q), v3(p, s), v2(p, xx), v2(p, xy), v2(p, yx), v2(p, yy), v2(p, ug), v2(p, vg), v2(p, turmu),
        I2{iblank, p->jd}, v2(p, tscale), v2(p, bt));
}
void oro_arc2d_precon(const P* p, double* q, double* s, double* xx, double* xy, double* yx, double* yy, double* ug,
                      double* vg, double* turmu, const int32_t* iblank, double* tscale, double* bt) {
  arc2d(*p, v3(p, q), v3(p, s), v2(p, xx), v2(p, xy), v2(p, yx), v2(p, yy), v2(p, ug), v2(p, vg), v2(p, turmu),
        I2{iblank, p->jd}, v2(p, tscale), v2(p, bt), true);
}
int oro_monitor(const P* p, double* q) {
  int n = 0;
  size_t n2 = (size_t)p->jd * p->kd;
  for (int nsp = 0; nsp < p->nspec; ++nsp) n += monitor(*p, v3(p, q + nsp * n2));
  return n;
}
void oro_force2d(const P* p, double* q, const double* xv, const double* yv, double* xx, double* xy, double* yx, double* yy,
                 double* out) {
  A2 z{nullptr, p->jd};
  force2d(*p, v3(p, q), z, z, xv, yv, v2(p, xx), v2(p, xy), v2(p, yx), v2(p, yy), out);
}

/* step.f:2-218 over all nspec instances.  Arrays are the full reference
 * arrays (jd,kd,nspec[,n]).  norms[3*nsp+{0,1,2}] = rsum, resrho, resmax;
 * loc[3*nsp+{0,1,2}] = j,k,n of resmax.  Returns 0, or 2 when the L2 norm
 * exceeds 1000 (the reference's `stop 'norm'`, step.f:105-110). */
int oro_step_u(const P* pp, double* q, double* s, double* x, double* y, const double* xv, const double* yv,
               const int32_t* iblank, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg,
               const double* ugv, const double* vgv, double* turmu, double* tscale, double* bt, const double* Ds,
               double* norms, int32_t* loc, const double* qnewt, const double* xold, const double* yold,
               const double* xole, const double* yole);

int oro_step(const P* pp, double* q, double* s, double* x, double* y, const double* xv, const double* yv,
             const int32_t* iblank, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg,
             const double* ugv, const double* vgv, double* turmu, double* tscale, double* bt, const double* Ds,
             double* norms, int32_t* loc) {
  return oro_step_u(pp, q, s, x, y, xv, yv, iblank, xx, xy, yx, yy, ug, vg, ugv, vgv, turmu, tscale, bt, Ds, norms,
                    loc, nullptr, nullptr, nullptr, nullptr, nullptr);
}

/* step.f:2-218 with the time-accurate terms: qnewt (jd,kd,nspec,nv) is the
 * Newton target of stqol (used when itnmax > 1, time.f:178-210), xold..yole
 * the previous vertex levels (used when iunst > 0). */
int oro_step_u(const P* pp, double* q, double* s, double* x, double* y, const double* xv, const double* yv,
               const int32_t* iblank, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg,
               const double* ugv, const double* vgv, double* turmu, double* tscale, double* bt, const double* Ds,
               double* norms, int32_t* loc, const double* qnewt, const double* xold, const double* yold,
               const double* xole, const double* yole) {
  const P& p = *pp;
  const int jd = p.jd, kd = p.kd, nspec = p.nspec;
  size_t n2 = (size_t)jd * kd, nv2 = (size_t)jd * kd * nspec;
  size_t nvert = (size_t)p.jmax * p.kmax;
  std::memset(s, 0, sizeof(double) * nv2 * p.nv);
  std::vector<double> ss(nv2 * p.nv, 0.0);
  int status = 0;
  for (int nsp = 1; nsp <= nspec; ++nsp) {
    size_t o = (size_t)(nsp - 1) * n2;
    A3 qn = v3(pp, q + o), sn = v3(pp, s + o);
    A2 z{nullptr, jd};
    bc(p, qn, z, z, v2(pp, xx + o), v2(pp, xy + o), v2(pp, yx + o), v2(pp, yy + o), v2(pp, ug + o), v2(pp, vg + o),
       v2(pp, bt + o));
    const size_t ov = (size_t)(nsp - 1) * nvert;
    rhsup(p, qn, sn, xv + ov, yv + ov, I2{iblank + o, jd}, ugv + ov, vgv + ov, xold ? xold + ov : nullptr,
          yold ? yold + ov : nullptr, xole ? xole + ov : nullptr, yole ? yole + ov : nullptr);
    // compute_residual, step.f:274-285: newton into s, or (time spectral)
    // newtonTS into ss, which is added to s after the norms (step.f:125-131)
    if (p.itnmax > 1) {
      if (!qnewt) { std::fprintf(stderr, "oracle: itnmax>1 needs qnewt\n"); std::abort(); }
      if (p.timespectral) newtonTS(p, qn, qnewt + o, v3(pp, ss.data() + o), v2(pp, tscale + o));
      else newton(p, qn, qnewt + o, sn);
    }
    if (!p.invisc) visrhs(p, v2(pp, turmu + o), qn, sn, v2(pp, xx + o), v2(pp, xy + o), v2(pp, yx + o), v2(pp, yy + o));
    if (p.timespectral) timespectralrhs(p, q, s, Ds, nsp);
  }
  if (!p.timespectral || p.itn == 1) {
    for (int nsp = 1; nsp <= nspec; ++nsp) {
      size_t o = (size_t)(nsp - 1) * n2;
      A3 sn = v3(pp, s + o); I2 ib{iblank + o, jd};
      double rsum = 0., resrho = 0.0, resmax = 0.0; int jd1 = 2, kd1 = 2, nd1 = 1;
      for (int k = p.kbeg; k <= p.kend; ++k) {
        for (int n = 1; n <= p.nmv; ++n)
          for (int j = p.jbeg; j <= p.jend; ++j) {
            double smrs = std::fabs(sn(j, k, n)) * (double)(ib(j, k) > 0 ? ib(j, k) : 0);
            if (smrs > resmax) { jd1 = j; kd1 = k; nd1 = n; resmax = smrs; }
          }
        for (int j = p.jbeg; j <= p.jend; ++j) {
          double m = (double)(ib(j, k) > 0 ? ib(j, k) : 0);
          double s1 = sn(j, k, 1) * m, s2 = sn(j, k, 2) * m, s3 = sn(j, k, 3) * m, s4 = sn(j, k, 4) * m;
          resrho = resrho + p2(sn(j, k, 1));
          rsum = rsum + s1 * s1 + s2 * s2 + s3 * s3 + s4 * s4;
        }
      }
      double volum = (double)(jd * kd);
      resrho = std::sqrt(resrho / volum);
      rsum = std::sqrt(rsum / volum);
      if (norms) { norms[3 * (nsp - 1)] = rsum; norms[3 * (nsp - 1) + 1] = resrho; norms[3 * (nsp - 1) + 2] = resmax; }
      if (loc) { loc[3 * (nsp - 1)] = jd1; loc[3 * (nsp - 1) + 1] = kd1; loc[3 * (nsp - 1) + 2] = nd1; }
      if (rsum > 1000.0 || rsum != rsum) status = 2;
    }
  }
  for (int nsp = 1; nsp <= nspec; ++nsp) {
    size_t o = (size_t)(nsp - 1) * n2;
    A3 qn = v3(pp, q + o), sn = v3(pp, s + o), ssn = v3(pp, ss.data() + o);
    if (p.iprecon) rhslom(p, qn, sn, v2(pp, bt + o));   // step.f:121-123
    for (int k = p.kbeg; k <= p.kend; ++k) for (int j = p.jbeg; j <= p.jend; ++j)
      for (int n = 1; n <= p.nv; ++n) sn(j, k, n) = sn(j, k, n) + ssn(j, k, n);
    rbc(p, qn, sn);
    A2 ts = v2(pp, tscale + o);
    for (int k = 1; k <= kd; ++k) for (int j = 1; j <= jd; ++j)
      for (int n = 1; n <= 4; ++n) sn(j, k, n) = sn(j, k, n) * ts(j, k);
    if (p.ilhs == 1 && p.iprecon) {
      preilu2d(p, qn, sn, v2(pp, xx + o), v2(pp, xy + o), v2(pp, yx + o), v2(pp, yy + o), v2(pp, ug + o),
               v2(pp, vg + o), v2(pp, turmu + o), ts, v2(pp, bt + o));
    } else if (p.ilhs == 1) {
      ilu2d(p, qn, sn, v2(pp, xx + o), v2(pp, xy + o), v2(pp, yx + o), v2(pp, yy + o), v2(pp, ug + o), v2(pp, vg + o),
            v2(pp, turmu + o), ts);
    } else if ((p.ilhs == 2 || p.ilhs == 3) && p.iprecon) {
      arc2d(p, qn, sn, v2(pp, xx + o), v2(pp, xy + o), v2(pp, yx + o), v2(pp, yy + o), v2(pp, ug + o), v2(pp, vg + o),
            v2(pp, turmu + o), I2{iblank + o, jd}, ts, v2(pp, bt + o), true);   // step.f:174-180
    } else if (p.ilhs == 2 || p.ilhs == 3) {
      arc2d(p, qn, sn, v2(pp, xx + o), v2(pp, xy + o), v2(pp, yx + o), v2(pp, yy + o), v2(pp, ug + o), v2(pp, vg + o),
            v2(pp, turmu + o), I2{iblank + o, jd}, ts, v2(pp, bt + o));
    } else {
      std::fprintf(stderr, "oracle: ilhs=%d not restated\n", p.ilhs); std::abort();
    }
  }
  for (int nsp = 1; nsp <= nspec; ++nsp) {
    size_t o = (size_t)(nsp - 1) * n2;
    if (!p.lamin) {
      if (p.iturb == 1) {
        vmu_sa(p, v3(pp, q + o), v3(pp, s + o), v2(pp, turmu + o), v2(pp, x + o), v2(pp, y + o), xv + (nsp - 1) * nvert,
               yv + (nsp - 1) * nvert, v2(pp, xx + o), v2(pp, xy + o), v2(pp, yx + o), v2(pp, yy + o), v2(pp, ug + o),
               v2(pp, vg + o), v2(pp, tscale + o), I2{iblank + o, jd}, nullptr);
      } else if (p.iturb == 2) {
        komegasst(p, v3(pp, q + o), v3(pp, s + o), v2(pp, turmu + o), v2(pp, x + o), v2(pp, y + o),
                  xv + (nsp - 1) * nvert, yv + (nsp - 1) * nvert, v2(pp, xx + o), v2(pp, xy + o), v2(pp, yx + o),
                  v2(pp, yy + o), v2(pp, ug + o), v2(pp, vg + o), v2(pp, tscale + o), I2{iblank + o, jd}, nullptr);
      } else {
        std::fprintf(stderr, "oracle: iturb=%d not restated\n", p.iturb); std::abort();
      }
    }
  }
  for (int nsp = 1; nsp <= nspec; ++nsp) {
    size_t o = (size_t)(nsp - 1) * n2;
    A3 qn = v3(pp, q + o), sn = v3(pp, s + o); I2 ib{iblank + o, jd};
    for (int k = p.kbeg; k <= p.kend; ++k) for (int j = p.jbeg; j <= p.jend; ++j) {
      double m = (double)(ib(j, k) > 0 ? ib(j, k) : 0);
      for (int n = 1; n <= 4; ++n) qn(j, k, n) = qn(j, k, n) + sn(j, k, n) * m;
    }
  }
  return status;
}

/* Single-grid driver mirroring Turns_overset.f:360-505 plus initia
 * (init.f:2-177) for a grid given in memory.  xv,yv: (jmax,kmax) vertices of
 * time instance 1 (the other instances are rotated copies, setup.f:396-438).
 * Runs up to nsteps iterations (stopping early when the L2 norm of every
 * instance has dropped by `orders` decades, if orders > 0).
 * hist[it*nspec+nsp] = rsum; forces[5*nsp+{0..4}] = cl,cd,cm,cpower,- and
 * q_out (jd,kd,nspec,nq) the final state.  Returns the number of iterations
 * run, or the negative iteration count on a monitor / norm stop. */
// The Turns_overset.f time loop from freestream (q_init = nullptr) or, as
// init.f:138-170 does with iread > 0, from a restart state: q_init holds
// q(1:nv) of every instance already divided by J (jd,kd,nspec,nv), and the
// step counter istep0 continues from istep0_init.
int oro_solve_from(const P* pin, const double* xv1, const double* yv1, int nsteps, double orders,
                   const double* q_init, int istep0_init, double* hist, double* forces, double* q_out);

int oro_solve(const P* pin, const double* xv1, const double* yv1, int nsteps, double orders,
              double* hist, double* forces, double* q_out) {
  return oro_solve_from(pin, xv1, yv1, nsteps, orders, nullptr, 0, hist, forces, q_out);
}

int oro_solve_from(const P* pin, const double* xv1, const double* yv1, int nsteps, double orders,
                   const double* q_init, int istep0_init, double* hist, double* forces, double* q_out) {
  P p = *pin;
  // time.f:30-35 sets idual / idual_turb in the module the first time the
  // time step runs; the turbulence model sees them from then on
  if (p.iprecon && (p.timeac == 1 && !p.timespectral)) { p.idual = 1; p.idual_turb = 1; }
  // Turns_overset.f:481: without preconditioning Mp is 1 (the far-field BC
  // reads it)
  if (!p.iprecon) p.Mp = 1.0;
  const int jd = p.jd, kd = p.kd, nspec = p.nspec, jmax = p.jmax, kmax = p.kmax;
  size_t n2 = (size_t)jd * kd, nv2 = n2 * nspec, nvert = (size_t)jmax * kmax;
  std::vector<double> q(nv2 * p.nq), s(nv2 * p.nv), x(nv2), y(nv2), xx(nv2), xy(nv2), yx(nv2), yy(nv2);
  std::vector<double> ug(nv2, 0.), vg(nv2, 0.), turmu(nv2, 0.), tscale(nv2), bt(nv2);
  std::vector<double> xv(nvert * nspec), yv(nvert * nspec), ugv(nvert * nspec, 0.), vgv(nvert * nspec, 0.);
  std::vector<int32_t> iblank(nv2, 1);
  std::vector<double> Ds((size_t)nspec * nspec, 0.0), tspec(nspec, 0.0);
  const double pi = 4.0 * std::atan(1.0);
  if (p.timespectral) computeTScoefs(nspec, Ds.data());
  for (int nsp = 1; nsp <= nspec; ++nsp)
    if (p.rf != 0) tspec[nsp - 1] = 2 * pi * (nsp - 1) / nspec / std::fabs(p.rf);
  std::memcpy(xv.data(), xv1, sizeof(double) * nvert);
  std::memcpy(yv.data(), yv1, sizeof(double) * nvert);
  for (int nsp = 2; nsp <= nspec; ++nsp)
    find_coord_TS_orig(p, xv.data() + (nsp - 1) * nvert, yv.data() + (nsp - 1) * nvert, xv1, yv1, tspec[nsp - 1]);
  for (int nsp = 1; nsp <= nspec; ++nsp) {
    size_t o = (size_t)(nsp - 1) * n2;
    find_cellcenter(p, A2{x.data() + o, jd}, A2{y.data() + o, jd}, xv.data() + (nsp - 1) * nvert, yv.data() + (nsp - 1) * nvert);
    A3 qn{q.data() + o, jd, nv2};
    if (metfv(p, qn, xv.data() + (nsp - 1) * nvert, yv.data() + (nsp - 1) * nvert, A2{xx.data() + o, jd},
              A2{xy.data() + o, jd}, A2{yx.data() + o, jd}, A2{yy.data() + o, jd}) != 0)
      return 0;
    if (p.timespectral)
      find_timemetrics_TS_orig(p, A2{x.data() + o, jd}, A2{y.data() + o, jd}, xv.data() + (nsp - 1) * nvert,
                               yv.data() + (nsp - 1) * nvert, tspec[nsp - 1], A2{ug.data() + o, jd}, A2{vg.data() + o, jd},
                               ugv.data() + (nsp - 1) * nvert, vgv.data() + (nsp - 1) * nvert);
    qzero(p, qn);
    qdivj(p, qn);
  }
  if (q_init)
    for (int n = 0; n < p.nv; ++n) std::memcpy(q.data() + (size_t)n * nv2, q_init + (size_t)n * nv2, sizeof(double) * nv2);
  std::vector<double> norms(3 * nspec), first(nspec, 0.0);
  std::vector<int32_t> loc(3 * nspec);
  // time-accurate state: previous vertex levels (init.f:101-108) and the
  // stqol levels (time.f:110-175)
  const bool moving = p.iunst > 0 && p.motiontype == 1;
  if (p.iunst > 0 && !moving) { std::fprintf(stderr, "oracle: only motiontype 1 (pitch) is restated\n"); std::abort(); }
  std::vector<double> xold(xv), yold(yv), xole(xv), yole(yv);
  std::vector<double> qtn(p.itnmax > 1 ? nv2 * p.nv : 0, 0.0), qtnm1(qtn), qnewt(qtn);
  p.istep0 = q_init ? istep0_init : 0;
  int it = 0, stopped = 0;
  for (int istep = 1; istep <= nsteps; ++istep) {
    p.istep0 += 1; p.istep = istep;
    // Turns_overset.f:365-403
    if (p.iunst != 0) p.totime += p.dt;
    if (moving) {
      pitch(p, A2{x.data(), jd}, A2{y.data(), jd}, xv.data(), yv.data(), xold.data(), yold.data(), xole.data(),
            yole.data(), A2{ug.data(), jd}, A2{vg.data(), jd});
      A3 qn{q.data(), jd, nv2};
      if (metfv(p, qn, xv.data(), yv.data(), A2{xx.data(), jd}, A2{xy.data(), jd}, A2{yx.data(), jd},
                A2{yy.data(), jd}) != 0)
        return -istep;
    }
    if (p.itnmax > 1) stqol(p, q.data(), qtn.data(), qtnm1.data(), qnewt.data());
    for (int itn = 1; itn <= p.itnmax; ++itn) {
      p.itn = itn;
      for (int nsp = 1; nsp <= nspec; ++nsp) {
        size_t o = (size_t)(nsp - 1) * n2;
        time_step(p, A3{q.data() + o, jd, nv2}, A2{xx.data() + o, jd}, A2{xy.data() + o, jd}, A2{yx.data() + o, jd},
                  A2{yy.data() + o, jd}, A2{ug.data() + o, jd}, A2{vg.data() + o, jd}, A2{tscale.data() + o, jd},
                  A2{bt.data() + o, jd}, I2{iblank.data() + o, jd});
      }
      int st = oro_step_u(&p, q.data(), s.data(), x.data(), y.data(), xv.data(), yv.data(), iblank.data(),
                          xx.data(), xy.data(), yx.data(), yy.data(), ug.data(), vg.data(), ugv.data(), vgv.data(),
                          turmu.data(), tscale.data(), bt.data(), Ds.data(), norms.data(), loc.data(),
                          p.itnmax > 1 ? qnewt.data() : nullptr, moving ? xold.data() : nullptr,
                          moving ? yold.data() : nullptr, moving ? xole.data() : nullptr,
                          moving ? yole.data() : nullptr);
      int bad = 0;
      for (int nsp = 0; nsp < nspec; ++nsp) bad += monitor(p, A3{q.data() + nsp * n2, jd, nv2});
      if (st != 0 || bad != 0) stopped = 1;
      if (stopped) break;
    }
    it = istep;
    for (int nsp = 0; nsp < nspec; ++nsp) {
      if (hist) hist[(size_t)(istep - 1) * nspec + nsp] = norms[3 * nsp];
      if (istep == 1) first[nsp] = norms[3 * nsp];
    }
    if (stopped) break;
    if (orders > 0) {
      bool conv = true;
      for (int nsp = 0; nsp < nspec; ++nsp)
        if (!(norms[3 * nsp] <= first[nsp] * std::pow(10.0, -orders))) conv = false;
      if (conv) break;
    }
  }
  if (forces) {
    double ca = std::cos(pi * p.alfa / 180.0), sa = std::sin(pi * p.alfa / 180.0);
    for (int nsp = 0; nsp < nspec; ++nsp) {
      size_t o = (size_t)nsp * n2;
      double out[4];
      A2 z{nullptr, jd};
      force2d(p, A3{q.data() + o, jd, nv2}, z, z, xv.data() + nsp * nvert, yv.data() + nsp * nvert, A2{xx.data() + o, jd},
              A2{xy.data() + o, jd}, A2{yx.data() + o, jd}, A2{yy.data() + o, jd}, out);
      double cfx = out[0], cfy = out[1], cm0 = out[2];
      forces[5 * nsp + 0] = -cfx * sa + cfy * ca;
      forces[5 * nsp + 1] = cfx * ca + cfy * sa;
      forces[5 * nsp + 2] = cm0 - 0.00 * cfx + 0.25 * cfy;
      forces[5 * nsp + 3] = out[3];
      forces[5 * nsp + 4] = 0.0;
    }
  }
  if (q_out) std::memcpy(q_out, q.data(), sizeof(double) * q.size());
  return stopped ? -it : it;
}

}  /* extern "C" */
