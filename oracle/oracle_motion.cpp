/*
 * oracle_motion.cpp -- TEST INFRASTRUCTURE ONLY (CPU FP64 oracle): the
 * time-accurate pieces of the reference's unsteady path, restated in the
 * reference's operation order:
 *   pitch    src/motion.f:546-632   grid rotation, cell grid speeds, the
 *                                   two previous vertex levels
 *   stqol    src/time.f:110-175     target state of the Newton iterations
 *   newton   src/time.f:178-210     physical-time term of the residual
 */
#include <cmath>

#include "oracle.h"

namespace oro {

void pitch(const P& p, A2 x, A2 y, double* xv, double* yv, double* xold, double* yold, double* xole, double* yole,
           A2 ug, A2 vg) {
  const double pi = 4.0 * std::atan(1.0);
  const int istep = p.istep;
  // motion.f:579-583
  const double dtheta = -(p.angmax * (std::cos(p.rotf * (double)istep * p.dt) -
                                      std::cos(p.rotf * (double)(istep - 1) * p.dt)));
  const double sn = std::sin(dtheta * pi / 180.), cn = std::cos(dtheta * pi / 180.);
  const double snold = std::sin(-1. * dtheta * pi / 180.), cnold = std::cos(-1. * dtheta * pi / 180.);
  // motion.f:585-605: cell centres and their grid speeds
  for (int k = 1; k <= p.kd; ++k)
    for (int j = 1; j <= p.jd; ++j) {
      const double xnew = (x(j, k) - p.xac) * cn + (y(j, k) - p.yac) * sn + p.xac;
      const double ynew = -((x(j, k) - p.xac) * sn) + (y(j, k) - p.yac) * cn + p.yac;
      if (p.ntac == 1) {
        ug(j, k) = (xnew - x(j, k)) / p.dt;
        vg(j, k) = (ynew - y(j, k)) / p.dt;
      } else {
        const double xo = (x(j, k) - p.xac) * cnold + (y(j, k) - p.yac) * snold + p.xac;
        const double yo = -((x(j, k) - p.xac) * snold) + (y(j, k) - p.yac) * cnold + p.yac;
        ug(j, k) = (1.5 * xnew - 2. * x(j, k) + 0.5 * xo) / p.dt;
        vg(j, k) = (1.5 * ynew - 2. * y(j, k) + 0.5 * yo) / p.dt;
      }
      x(j, k) = xnew;
      y(j, k) = ynew;
    }
  // motion.f:607-624: vertices
  const size_t nv = (size_t)p.jmax * p.kmax;
  for (size_t i = 0; i < nv; ++i) {
    xole[i] = xold[i];
    yole[i] = yold[i];
    xold[i] = xv[i];
    yold[i] = yv[i];
    xv[i] = (xold[i] - p.xac) * cn + (yold[i] - p.yac) * sn + p.xac;
    yv[i] = -((xold[i] - p.xac) * sn) + (yold[i] - p.yac) * cn + p.yac;
  }
}

void stqol(const P& p, const double* q, double* qtn, double* qtnm1, double* qnewt) {
  const size_t n2s = (size_t)p.jd * p.kd * p.nspec;
  const int istep = p.istep;
  const bool c1 = (p.ntac == 2 && istep > 1) || (p.ntac == 3 && istep == 2);
  const bool c2 = p.ntac == 3 && istep > 2;
  for (int n = 0; n < p.nv; ++n)
    for (size_t i = 0; i < n2s; ++i) {
      const size_t o = (size_t)n * n2s + i;
      double v = q[o];
      if (c1) v = v + (q[o] - qtn[o]) / 3.;
      if (c2) v = v + 7. * (q[o] - qtn[o]) / 11. - 2. * (qtn[o] - qtnm1[o]) / 11.;
      qnewt[o] = v;
      qtnm1[o] = qtn[o];
      qtn[o] = q[o];
    }
}

void newton(const P& p, A3 q, const double* qnewt, A3 s) {
  double oat = 1.0;
  if (p.ntac >= 2 && p.istep > 1) oat = 2. / 3.;
  if (p.ntac == 3 && p.istep > 2) oat = 6. / 11.;
  const double tac = 1. / (oat * p.h);
  // qnewt of this instance: (jd,kd,nv) with the instance stride of q
  A3 qn{const_cast<double*>(qnewt), q.jd, q.ns};
  for (int k = p.kbeg; k <= p.kend; ++k)
    for (int j = p.jbeg; j <= p.jend; ++j)
      for (int n = 1; n <= p.nv; ++n) s(j, k, n) = s(j, k, n) - (q(j, k, n) - qn(j, k, n)) * tac;
}

/* time.f:213-241 (newtonTS): the pseudo-time Newton term of a time-spectral
 * run into ss (added to s after the norms) */
void newtonTS(const P& p, A3 q, const double* qnewt, A3 ss, A2 tscale) {
  A3 qn{const_cast<double*>(qnewt), q.jd, q.ns};
  for (int k = p.kbeg; k <= p.kend; ++k)
    for (int j = p.jbeg; j <= p.jend; ++j)
      if (tscale(j, k) != 0)
        for (int n = 1; n <= p.nv; ++n) ss(j, k, n) = ss(j, k, n) - (q(j, k, n) - qn(j, k, n)) / tscale(j, k);
}

}  // namespace oro
