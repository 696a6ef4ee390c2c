/*
 * oracle_common.h -- TEST INFRASTRUCTURE ONLY.
 *
 * Shared helpers for the CPU FP64 oracle, a line-by-line C++ restatement of
 * the OVERTURNS-2D Fortran hot path.  Only tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / --impl reference leg may load the oracle; the
 * product (turns2d_urans_git_gb300) never links or calls it.
 *
 * Parity status: the reference ships no golden vectors, test data or sample
 * inputs, and no Fortran compiler exists on either machine, so the oracle is
 * "parity unpinned" against the reference itself.  It is pinned instead by
 * the invariants the tests check (freestream preservation, residual mirror
 * symmetry, Ds antisymmetry) and by golden fixtures it generated.
 *
 * Fortran semantics kept throughout (the reference is compiled with -r8 /
 * -fdefault-real-8, configure.ac:27-33):
 *   - every literal is a double (e.g. sigma = 0.6666667, not 2/3);
 *   - SIGN(a,b) follows the IEEE sign bit of b (gfortran semantics);
 *   - x**2 = x*x, x**3 = (x*x)*x, x**6 = x3*x3; real exponents call pow();
 *   - expressions are evaluated left to right as written, no contraction
 *     (build with -ffp-contract=off).
 */
#ifndef OT2D_ORACLE_COMMON_H
#define OT2D_ORACLE_COMMON_H

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <vector>
#include "ot2d_params.h"

namespace oro {

typedef ot2d_params P;

static inline double fsign(double a, double b) { return std::copysign(std::fabs(a), b); }
static inline double fmax2(double a, double b) { return (b > a) ? b : a; }
static inline double fmin2(double a, double b) { return (b < a) ? b : a; }
static inline int isign(int a, int b) { int aa = a < 0 ? -a : a; return b >= 0 ? aa : -aa; }
static inline double p2(double x) { return x * x; }
static inline double p3(double x) { return (x * x) * x; }
static inline double p6(double x) { double t = (x * x) * x; return t * t; }

/* 2-D cell array a(jd,kd) */
struct A2 {
  double* p; int jd;
  inline double& operator()(int j, int k) const { return p[(size_t)(k - 1) * jd + (j - 1)]; }
};
struct I2 {
  const int32_t* p; int jd;
  inline int32_t operator()(int j, int k) const { return p[(size_t)(k - 1) * jd + (j - 1)]; }
};
/* q(jd,kd,[nsp],n): one time instance of a multi-variable array; `ns` is the
 * distance between consecutive variables (jd*kd*nspec in the reference). */
struct A3 {
  double* p; int jd; size_t ns;
  inline double& operator()(int j, int k, int n) const {
    return p[(size_t)(n - 1) * ns + (size_t)(k - 1) * jd + (j - 1)];
  }
};

/* bc.f:20-33 -- convert a &bcinp vertex range to halo-cell indices */
static inline void bc_range(const P& p, int ib, int& js, int& je, int& ks, int& ke) {
  js = p.jbcs[ib]; je = p.jbce[ib]; ks = p.kbcs[ib]; ke = p.kbce[ib];
  if (js < 0) js = p.jmax + js + 1;
  if (ks < 0) ks = p.kmax + ks + 1;
  if (je < 0) je = p.jmax + je + 1;
  if (ke < 0) ke = p.kmax + ke + 1;
  if (js > 1) js = js + p.nhalo;
  if (ks > 1) ks = ks + p.nhalo;
  if (je < p.jmax) je = je + p.nhalo - 1;
  if (ke < p.kmax) ke = ke + p.nhalo - 1;
  if (je == p.jmax) je = p.jd;
  if (ke == p.kmax) ke = p.kd;
}

}  // namespace oro
#endif
