// k_adi.cuh -- the diagonalised ADI operator arc2d with pentadiagonal line
// inversions (src/lhs.f:817-1057 with lhsinv :1536-1816 and pentadag
// :1819-1873; ilhs = 2) or the upwind-split tridiagonal ones (lhsinv_up
// :1333-1533; ilhs = 3).
//
// The reference converts q to primitive variables in place, multiplies s by
// T_xi^-1, inverts a scalar pentadiagonal system per j-line and variable,
// multiplies by N^-1, inverts per k-line, multiplies by T_eta and converts
// q back.  Here q is never rewritten: the primitive values and every
// per-cell factor are kept in scratch arrays (cell-parallel kernels), the
// dissipation coefficients of the line systems are assembled per cell in
// gather form, and each (line, variable) system is solved by one thread with
// a sliding window over the reference's pentadag recurrences.  In FP64 the
// conservative round trip of q (:853-860, :1047-1054) is applied at the end
// so q leaves with the reference's bits.
#pragma once
#include "dev_common.cuh"
#include "launch.h"

namespace ot2d {

// scratch arrays of one slice (stride S.wstride); dm/em: per variable
// i = 1..4 the modified super-diagonals of pentadag's forward sweep
enum ADIw { A_P = 0, A_QX, A_QY, A_CX, A_CY, A_UV, A_VN, A_GE, A_U, A_V, A_E, A_D2P, A_AT, A_BT, A_CT, A_DT, A_ET,
            A_DM, A_EM = A_DM + 4, A_N = A_EM + 4 };
static_assert(A_N <= ADI_NSCRATCH, "ADI scratch layout");

__device__ __forceinline__ bool adi_slice(const ot2d_params& p) { return p.ilhs == 2 || p.ilhs == 3; }

// line view of direction dir (0: j lines, m = j, n = k; 1: k lines, m = k, n = j)
__device__ __forceinline__ int64_t adi_at(int jd, int dir, int m, int n) { return dir == 0 ? at(jd, m, n) : at(jd, n, m); }

// bSq = Mp**2/(bt - Mp**2 (bt-1)) of cell o (arc2d_precon, lhsinv)
template <class R>
__device__ __forceinline__ R adi_bsq(const Slice<R>& S, int64_t o) {
  const R btv = S.bt ? S.bt[o] : (R)1.;
  return S.k_mp2 / (btv - S.k_mp2 * (btv - (R)1));
}

// s *= tscale when `scale` (step.f:141-148), primitive variables (:853-860) and the
// T_xi^-1 multiplication with its per-cell factors (:863-917), on every
// cell of js-1..je+1 x ks-1..ke+1
template <class R>
__device__ void adi_txi_cell(const Slice<R>& S, const ot2d_params& p, int j, int k, int scale) {
  const int64_t o = at(S.jd, j, k), qs = S.qs, ws = S.wstride;
  const R gm1 = S.k_gm1, ggm1 = S.k_ggm1;
  const R q1 = S.q[o], J = S.q[(p.nq - 1) * qs + o];
  const R dj = (R)1.0 / q1;
  const R uu = S.q[qs + o] * dj, vv = S.q[2 * qs + o] * dj, e = S.q[3 * qs + o] * dj;
  const R rho = q1 * J;
  R s1 = S.s[o], s2 = S.s[qs + o], s3 = S.s[2 * qs + o], s4 = S.s[3 * qs + o];
  if (scale) {
    const R ts = S.tscale[o];
    s1 = s1 * ts; s2 = s2 * ts; s3 = s3 * ts; s4 = s4 * ts;
  }
  const R uv2 = (R)0.5 * (uu * uu + vv * vv);
  const R cjkl = sqrt(ggm1 * (e - uv2));
  const R c2i = (R)1.0 / (cjkl * cjkl);
  S.w[A_P * ws + o] = (e - uv2) * gm1 * rho;
  R rj1 = S.xx[o], rj2 = S.xy[o];
  const R ugc = S.ug ? S.ug[o] : (R)0, vgc = S.vg ? S.vg[o] : (R)0;
  // arc2d_precon (:1116, :1125) takes the contravariant velocities relative
  // to the grid before storing them; arc2d (:874-876) subtracts afterwards
  const bool pre = S.k_mp2 >= (R)0;
  const R qq1 = pre ? rj1 * (uu - ugc) + rj2 * (vv - vgc) : rj1 * uu + rj2 * vv;
  S.w[A_QX * ws + o] = pre ? qq1 : qq1 - (rj1 * ugc + rj2 * vgc);
  const R rr1 = sqrt(sq(rj1) + sq(rj2));
  rj1 = rj1 / rr1; rj2 = rj2 / rr1;
  const R rk1 = S.yx[o], rk2 = S.yy[o];
  if (pre) {
    S.w[A_QY * ws + o] = rk1 * (uu - ugc) + rk2 * (vv - vgc);
  } else {
    const R qq2 = rk1 * uu + rk2 * vv;
    S.w[A_QY * ws + o] = qq2 - (rk1 * ugc + rk2 * vgc);
  }
  const R rr2 = sqrt(sq(rk1) + sq(rk2));
  S.w[A_UV * ws + o] = uv2;
  S.w[A_CX * ws + o] = cjkl * rr1;
  S.w[A_CY * ws + o] = cjkl * rr2;
  S.w[A_VN * ws + o] = (S.k_rmue + S.turmu[o]) / (S.k_rey * rho);
  S.w[A_GE * ws + o] = S.k_gamma * e - gm1 * uv2;
  S.w[A_U * ws + o] = uu; S.w[A_V * ws + o] = vv; S.w[A_E * ws + o] = e;
  R a1 = s2 * uu + s3 * vv - s4;
  a1 = a1 * gm1 * c2i;
  a1 = a1 + s1 * ((R)1.0 - uv2 * gm1 * c2i);
  const R a2 = (rj1 * vv - rj2 * uu) * s1 + rj2 * s2 - rj1 * s3;
  R a3 = uv2 * s1 - s2 * uu - s3 * vv + s4;
  a3 = a3 * gm1 * c2i;
  S.s[o] = a1;
  S.s[qs + o] = a2;
  if (pre) {
    // arc2d_precon :1141-1164: the preconditioned acoustic eigenvectors
    const R bSq = adi_bsq(S, o), omb = (R)1. - bSq;
    const R cx = cjkl * rr1;
    const R X = sqrt((omb * qq1) * (omb * qq1) + (R)4. * bSq * cx * cx) / rr1;
    const R Y = (R)0.5 * (omb * qq1 / rr1 + X);
    const R Z = (R)0.5 * (omb * qq1 / rr1 - X);
    const R qqmxt = qq1 + ugc * rj1 * rr1 + vgc * rj2 * rr1;
    R a4 = qqmxt * s1 / rr1 - rj1 * s2 - rj2 * s3;
    a4 = a4 * bSq;
    S.s[2 * qs + o] = -(Z * a3 + a4) / X;
    S.s[3 * qs + o] = (Y * a3 + a4) / X;
    return;
  }
  const R a4 = qq1 * s1 / rr1 - rj1 * s2 - rj2 * s3;
  S.s[2 * qs + o] = (R)0.5 * (a3 - a4 / cjkl);
  S.s[3 * qs + o] = (R)0.5 * (a3 + a4 / cjkl);
}

// pressure switch of line direction dir (:919-935, :977-993): interior of
// the line, 0 at its two ends
template <class R>
__device__ __forceinline__ void adi_d2p_cell(const Slice<R>& S, int dir, int m, int n, int ms, int me) {
  const int jd = S.jd; const int64_t ws = S.wstride;
  const R* P = S.w + A_P * ws;
  R v = (R)0;
  if (m > ms && m < me) {
    const R pp = P[adi_at(jd, dir, m + 1, n)], pc = P[adi_at(jd, dir, m, n)], pm = P[adi_at(jd, dir, m - 1, n)];
    v = fabs(pp - (R)2. * pc + pm);
    v = v / fabs(pp + (R)2. * pc + pm);
  }
  S.w[A_D2P * ws + adi_at(jd, dir, m, n)] = v;
}

// spectral-radius diagonal of lhsinv (:1587-1596): d[0] = diag(m,1) =
// diag(m,2), d[1] = diag(m,3), d[2] = diag(m,4), d[3] = diag(m,nq)
template <class R>
__device__ __forceinline__ void adi_diag(const Slice<R>& S, const ot2d_params& p, int dir, int64_t o, R* d) {
  const int64_t ws = S.wstride;
  const R Mp = (R)p.Mp;
  const R btv = S.bt ? S.bt[o] : (R)1.;
  const R bSq = (Mp * Mp) / (btv - (Mp * Mp) * (btv - (R)1));
  const R qv = S.w[(dir == 0 ? A_QX : A_QY) * ws + o], cv = S.w[(dir == 0 ? A_CX : A_CY) * ws + o];
  const R X = sqrt(((R)1. - bSq) * qv * (((R)1. - bSq) * qv) + (R)4. * bSq * cv * cv);
  d[0] = qv;
  d[1] = (R)0.5 * ((bSq + (R)1.) * qv + X);
  d[2] = (R)0.5 * ((bSq + (R)1.) * qv - X);
  d[3] = (R)0.5 * ((bSq + (R)1.) * fabs(qv) + X) / S.q[(int64_t)(p.nq - 1) * S.qs + o];
}

// Dissipation coefficients atmp..etmp of lhsinv (:1655-1732) at line
// position m, times J (:1734-1740); the entries the reference leaves
// unassigned (both line ends, and the ones its end-point formulas skip) are
// 0.  Requires lines of at least 8 points.
template <class R>
__device__ void adi_coef_cell(const Slice<R>& S, const ot2d_params& p, int dir, int m, int n, int ms, int me) {
  const int jd = S.jd; const int64_t ws = S.wstride, qs = S.qs;
  const R dis2 = (R)10.0, dis4 = (R)0.1;
  R g[5], dn[5];   // positions m-2 .. m+2
  for (int t = 0; t < 5; ++t) {
    const int mm = m - 2 + t;
    if (mm < ms || mm > me) { g[t] = (R)0; dn[t] = (R)0; continue; }
    const int64_t oo = adi_at(jd, dir, mm, n);
    g[t] = S.w[A_D2P * ws + oo];
    R d[4];
    adi_diag(S, p, dir, oo, d);
    dn[t] = d[3];
  }
  auto G = [&](int dm) { return g[dm + 2]; };
  auto D = [&](int dm) { return dn[dm + 2]; };
  R at = (R)0, bt = (R)0, ct = (R)0, dt = (R)0, et = (R)0;
  if (m == me - 1) {
    const R c2 = ((G(0))) * dis2, c2m = (R)0.5 * ((G(0) + G(-1))) * dis2;
    const R c4 = (dis4 - fmin2(dis4, (R)1. * c2)), c4m = (dis4 - fmin2(dis4, (R)1. * c2m));
    const R c4m2 = (dis4 - fmin2(dis4, (R).5 * dis2 * (G(-2) + G(-1))));
    ct = +((D(-1) + D(0)) * ((R)3. * c4m + c2m) + (R)2. * (D(0)) * ((R)2. * c4 + c2));
    dt = -((D(-2) + D(-1)) * c4m2 + (D(0) + D(-1)) * ((R)3. * c4m + c2m));
    et = (D(-1) + D(-2)) * c4m2;
  } else if (m == me - 2) {
    const R c2 = (R)0.5 * ((G(0) + G(1))) * dis2, c2m = (R)0.5 * ((G(0) + G(-1))) * dis2;
    const R c4p = (dis4 - fmin2(dis4, (R)1. * dis2 * (G(1))));
    const R c4 = (dis4 - fmin2(dis4, (R)1. * c2)), c4m = (dis4 - fmin2(dis4, (R)1. * c2m));
    const R c4m2 = (dis4 - fmin2(dis4, (R).5 * dis2 * (G(-2) + G(-1))));
    bt = -((R)2. * (D(1)) * c4p + (D(1) + D(0)) * ((R)3. * c4 + c2));
    ct = ((D(-1) + D(0)) * ((R)3. * c4m + c2m) + (D(1) + D(0)) * ((R)2. * c4 + c2));
    dt = -((D(-2) + D(-1)) * c4m2 + (D(0) + D(-1)) * ((R)3. * c4m + c2m));
    et = (D(-1) + D(-2)) * c4m2;
  } else if (m == ms + 1) {
    const R c2 = (R)0.5 * ((G(0) + G(1))) * dis2, c2m = ((G(0))) * dis2;
    const R c4p = (dis4 - fmin2(dis4, (R).5 * dis2 * (G(2) + G(1))));
    const R c4 = (dis4 - fmin2(dis4, (R)1. * c2)), c4m = (dis4 - fmin2(dis4, (R)1. * c2m));
    at = (D(1) + D(2)) * c4p;
    bt = -((D(2) + D(1)) * c4p + (D(1) + D(0)) * ((R)3. * c4 + c2));
    ct = ((R)2. * (D(0)) * ((R)2. * c4m + c2m) + (D(1) + D(0)) * ((R)3. * c4 + c2));
  } else if (m == ms + 2) {
    const R c2 = (R)0.5 * ((G(0) + G(1))) * dis2, c2m = (R)0.5 * ((G(0) + G(-1))) * dis2;
    const R c4p = (dis4 - fmin2(dis4, (R).5 * dis2 * (G(2) + G(1))));
    const R c4 = (dis4 - (R)1. * fmin2(dis4, c2)), c4m = (dis4 - fmin2(dis4, (R)1. * c2m));
    const R c4m2 = (dis4 - fmin2(dis4, (R)1. * dis2 * (G(-1))));
    at = (D(1) + D(2)) * c4p;
    bt = -((D(2) + D(1)) * c4p + (D(1) + D(0)) * ((R)3. * c4 + c2));
    ct = ((D(-1) + D(0)) * ((R)3. * c4m + c2m) + (D(1) + D(0)) * ((R)3. * c4 + c2));
    dt = -(((R)2. * D(-1)) * c4m2 + (D(0) + D(-1)) * ((R)3. * c4m + c2m));
  } else if (m >= ms + 3 && m <= me - 3) {
    const R c2 = (R)0.5 * ((G(0) + G(1))) * dis2, c2m = (R)0.5 * ((G(0) + G(-1))) * dis2;
    const R c4p = (dis4 - fmin2(dis4, (R).5 * dis2 * (G(2) + G(1))));
    const R c4 = (dis4 - fmin2(dis4, (R)1. * c2)), c4m = (dis4 - fmin2(dis4, (R)1. * c2m));
    const R c4m2 = (dis4 - fmin2(dis4, (R).5 * dis2 * (G(-2) + G(-1))));
    at = (D(1) + D(2)) * c4p;
    bt = -((D(2) + D(1)) * c4p + (D(1) + D(0)) * ((R)3. * c4 + c2));
    ct = +((D(-1) + D(0)) * ((R)3. * c4m + c2m) + (D(1) + D(0)) * ((R)3. * c4 + c2));
    dt = -((D(-2) + D(-1)) * c4m2 + (D(0) + D(-1)) * ((R)3. * c4m + c2m));
    et = (D(-1) + D(-2)) * c4m2;
  }
  const int64_t o = adi_at(jd, dir, m, n);
  const R J = S.q[(int64_t)(p.nq - 1) * qs + o];
  S.w[A_AT * ws + o] = at * J;
  S.w[A_BT * ws + o] = bt * J;
  S.w[A_CT * ws + o] = ct * J;
  S.w[A_DT * ws + o] = dt * J;
  S.w[A_ET * ws + o] = et * J;
}

// The five scaled bands a1..e1 of lhsinv (:1742-1785) for variable i at
// line position m
template <class R>
struct AdiRow { R a, b, c, d, e; };
template <class R>
__device__ __forceinline__ AdiRow<R> adi_row(const Slice<R>& S, const ot2d_params& p, int dir, int i, int m, int n,
                                            int ms, int me) {
  const int jd = S.jd; const int64_t ws = S.wstride, qs = S.qs;
  const int64_t o = adi_at(jd, dir, m, n);
  const R* ts = S.tscale;
  R dg[4];
  adi_diag(S, p, dir, o, dg);
  const R di = (i <= 2) ? dg[0] : (i == 3 ? dg[1] : dg[2]);
  R v1 = (R)0, v2 = (R)0, v3 = (R)0;
  if (m > ms && m < me) {
    const R* xn = dir == 0 ? S.xx : S.yx;
    const R* yn = dir == 0 ? S.xy : S.yy;
    const R* Jq = S.q + (int64_t)(p.nq - 1) * qs;
    const int64_t op = adi_at(jd, dir, m + 1, n), om = adi_at(jd, dir, m - 1, n);
    const R vnu = S.w[A_VN * ws + o];
    v1 = (xn[o] * xn[o] + yn[o] * yn[o]) / Jq[o];
    v1 = v1 + (xn[op] * xn[op] + yn[op] * yn[op]) / Jq[op];
    v1 = v1 * Jq[o] * vnu;
    v3 = (xn[o] * xn[o] + yn[o] * yn[o]) / Jq[o];
    v3 = v3 + (xn[om] * xn[om] + yn[om] * yn[om]) / Jq[om];
    v3 = v3 * Jq[o] * vnu;
    v2 = (R)0.5 * (v1 + v3);
  }
  AdiRow<R> r;
  auto T = [&](int mm) { return ts[adi_at(jd, dir, mm, n)]; };
  if (p.ilhs == 3) {
    // lhsinv_up (lhs.f:1387-1501): upwind split eigenvalues, tridiagonal
    const R* xn = dir == 0 ? S.xx : S.yx;
    const R* yn = dir == 0 ? S.xy : S.yy;
    const R eps = (R)0.05 * sqrt(sq(xn[o]) + sq(yn[o]));
    const R fac = (R)1.05;
    const R dpl = (R)0.5 * (di + fac * sqrt(sq(di) + sq(eps)));
    const R dmi = (R)0.5 * (di - fac * sqrt(sq(di) + sq(eps)));
    r.a = (R)0.; r.b = (R)0.; r.c = (R)0.; r.d = (R)0.; r.e = (R)0.;
    r.b = r.b - dpl;
    r.d = r.d + dmi;
    r.c = r.c + dpl - dmi;
    r.b = r.b - (R)0.5 * v1;
    r.c = r.c + v2;
    r.d = r.d - (R)0.5 * v3;
    r.b = (m <= me - 1) ? r.b * T(m + 1) : r.b * T(m);
    r.d = (m >= ms + 1) ? r.d * T(m - 1) : r.d * T(m);
    r.c = r.c * T(m) + (R)1.0;
    return r;
  }
  r.a = S.w[A_AT * ws + o]; r.b = S.w[A_BT * ws + o]; r.c = S.w[A_CT * ws + o];
  r.d = S.w[A_DT * ws + o]; r.e = S.w[A_ET * ws + o];
  r.b = r.b - di * (R)0.5;
  r.d = r.d + di * (R)0.5;
  r.b = r.b - (R)0.5 * v1;
  r.c = r.c + v2;
  r.d = r.d - (R)0.5 * v3;
  r.a = (m <= me - 2) ? r.a * T(m + 2) : r.a * T(m);
  r.b = (m <= me - 1) ? r.b * T(m + 1) : r.b * T(m);
  r.d = (m >= ms + 1) ? r.d * T(m - 1) : r.d * T(m);
  r.e = (m >= ms + 2) ? r.e * T(m - 2) : r.e * T(m);
  r.c = r.c * T(m) + (R)1.0;
  return r;
}

// One pentadiagonal system (variable i, line n): the reduced system over
// m = ms+1..me-1 with the end corrections of :1787-1797, solved with
// pentadag's recurrences (:1819-1873) in a sliding window; the modified
// super-diagonals go to scratch for the backward sweep, the solution into s.
template <class R>
__device__ void adi_solve_line(const Slice<R>& S, const ot2d_params& p, int dir, int i, int n, int ms, int me) {
  const int jd = S.jd; const int64_t ws = S.wstride, qs = S.qs;
  R* sv = S.s + (int64_t)(i - 1) * qs;
  R* Dm = S.w + (A_DM + i - 1) * ws;
  R* Em = S.w + (A_EM + i - 1) * ws;
  const int N = me - ms - 1;
  auto O = [&](int ii) { return adi_at(jd, dir, ms + ii, n); };   // system index -> cell
  // end rows of the full line
  const AdiRow<R> r0 = adi_row(S, p, dir, i, ms, n, ms, me), rN1 = adi_row(S, p, dir, i, me, n, ms, me);
  const R f1ms = sv[adi_at(jd, dir, ms, n)], f1me = sv[adi_at(jd, dir, me, n)];
  // original bands of system row ii (1..N), with d(1)=e(1)=e(2)=0,
  // b(N)=a(N)=a(N-1)=0, and f with its end corrections
  auto row = [&](int ii) {
    AdiRow<R> r = adi_row(S, p, dir, i, ms + ii, n, ms, me);
    if (ii == 1) { r.d = (R)0; r.e = (R)0; }
    if (ii == 2) r.e = (R)0;
    if (ii == N) { r.b = (R)0; r.a = (R)0; }
    if (ii == N - 1) r.a = (R)0;
    return r;
  };
  auto fval = [&](int ii) {
    R f = sv[O(ii)];
    if (ii == 1) f = f - r0.b * f1ms / r0.c;
    if (ii == N) f = f - rN1.d * f1me / rN1.c;
    return f;
  };
  // i = 1
  AdiRow<R> R1 = row(1), R2 = row(2), R3 = row(3);
  R d0 = (R)1.0 / R1.c;
  R Dn = R2.d * d0;                 // D(2)
  R En1 = R3.e * d0;                // E(3)
  R F1 = fval(1) * d0;
  sv[O(1)] = F1;
  Dm[O(2)] = Dn; Em[O(3)] = En1;
  // i = 2
  R d1 = R1.b;
  d0 = (R)1.0 / (R2.c - d1 * Dn);
  R F2 = (fval(2) - d1 * F1) * d0;
  sv[O(2)] = F2;
  const AdiRow<R> R4 = row(4);
  R Dp = (R3.d - d1 * En1) * d0;    // D(3)
  R Ep = R4.e * d0;                 // E(4)
  Dm[O(3)] = Dp; Em[O(4)] = Ep;
  // window: Dprev = D(i-1), Dcur = D(i), Ecur = E(i), Enext = E(i+1)
  R Dprev = Dn, Dcur = Dp, Ecur = En1, Enext = Ep;
  R Fm2 = F1, Fm1 = F2;
  AdiRow<R> Rm2 = R1, Rm1 = R2, Rc = R3, Rn1 = R4;   // rows i-2, i-1, i, i+1
  for (int ii = 3; ii <= N; ++ii) {
    const AdiRow<R> Rn2 = (ii + 2 <= N) ? row(ii + 2) : AdiRow<R>{(R)0, (R)0, (R)0, (R)0, (R)0};
    d1 = Rm2.a;
    const R d2 = (Rm1.b - Rm2.a * Dprev);
    d0 = (R)1. / (Rc.c - d2 * Dcur - d1 * Ecur);
    const R Fi = (fval(ii) - d2 * Fm1 - d1 * Fm2) * d0;
    sv[O(ii)] = Fi;
    R Dnew = (R)0, Enew = (R)0;
    if (ii <= N - 1) {
      Dnew = (Rn1.d - d2 * Enext) * d0;
      Dm[O(ii + 1)] = Dnew;
      if (ii <= N - 2) { Enew = (Rn2.e) * d0; Em[O(ii + 2)] = Enew; }
    }
    Dprev = Dcur; Dcur = Dnew; Ecur = Enext; Enext = Enew;
    Fm2 = Fm1; Fm1 = Fi;
    Rm2 = Rm1; Rm1 = Rc; Rc = Rn1; Rn1 = Rn2;
  }
  // backward sweep
  R Fa = sv[O(N)];                  // F(i+1)
  R Fb = sv[O(N - 1)] - Dm[O(N)] * Fa;
  sv[O(N - 1)] = Fb;
  R Fc = Fa;                        // F(i+2)
  Fa = Fb;
  for (int ii = N - 2; ii >= 1; --ii) {
    const R Fi = sv[O(ii)] - Dm[O(ii + 1)] * Fa - Em[O(ii + 2)] * Fc;
    sv[O(ii)] = Fi;
    Fc = Fa; Fa = Fi;
  }
}

// N^-1 multiplication (:948-975)
template <class R>
__device__ void adi_ninv_cell(const Slice<R>& S, const ot2d_params& p, int j, int k) {
  const int64_t o = at(S.jd, j, k), qs = S.qs, ws = S.wstride;
  const R cjkl = sqrt(S.k_ggm1 * (S.w[A_E * ws + o] - S.w[A_UV * ws + o]));
  const R rj1 = S.xx[o], rj2 = S.xy[o], rr1 = sqrt(rj1 * rj1 + rj2 * rj2);
  const R rk1 = S.yx[o], rk2 = S.yy[o], rr2 = sqrt(rk1 * rk1 + rk2 * rk2);
  const R a1 = (rj1 * rk1 + rj2 * rk2) / rr1 / rr2;
  const R a2 = (rj1 * rk2 - rj2 * rk1) / rr1 / rr2;
  const R s2 = S.s[qs + o], s3 = S.s[2 * qs + o], s4 = S.s[3 * qs + o];
  if (S.k_mp2 >= (R)0) {
    // arc2d_precon :1207-1231
    const R bSq = adi_bsq(S, o), omb = (R)1.0 - bSq;
    const R qx = S.w[A_QX * ws + o], qy = S.w[A_QY * ws + o], cx = S.w[A_CX * ws + o], cy = S.w[A_CY * ws + o];
    const R X = sqrt((omb * qx) * (omb * qx) + (R)4. * bSq * cx * cx) / rr1;
    const R Y = (R)0.5 * (omb * qx / rr1 + X);
    const R Z = (R)0.5 * (omb * qx / rr1 - X);
    const R X1 = sqrt((omb * qy) * (omb * qy) + (R)4. * bSq * cy * cy) / rr2;
    const R Y1 = (R)0.5 * (omb * qy / rr2 + X1);
    const R Z1 = (R)0.5 * (omb * qy / rr2 - X1);
    S.s[qs + o] = a1 * s2 + (Y * s3 + Z * s4) * a2 / bSq;
    S.s[2 * qs + o] = -(a2 * bSq * s2 - (Y * a1 - Z1) * s3 - (Z * a1 - Z1) * s4) / X1;
    S.s[3 * qs + o] = (a2 * bSq * s2 - (Y * a1 - Y1) * s3 - (Z * a1 - Y1) * s4) / X1;
    return;
  }
  const R a4 = a1 * s2 + (cjkl * s3 - cjkl * s4) * a2;
  const R a5 = (R)-0.5 * (a2 * s2 / cjkl - (a1 + (R)1) * s3 + (a1 - (R)1) * s4);
  const R a6 = (R)0.5 * (a2 * s2 / cjkl - (a1 - (R)1) * s3 + (a1 + (R)1) * s4);
  S.s[qs + o] = a4; S.s[2 * qs + o] = a5; S.s[3 * qs + o] = a6;
}

// T_eta multiplication (:1005-1034), the unsteady rotation term of
// :1036-1045, and (FP64) the conservative round trip of q (:1047-1054)
template <class R>
__device__ void adi_teta_cell(const Slice<R>& S, const ot2d_params& p, int j, int k) {
  const int64_t o = at(S.jd, j, k), qs = S.qs, ws = S.wstride;
  const R uu = S.w[A_U * ws + o], vv = S.w[A_V * ws + o], uv = S.w[A_UV * ws + o], ge = S.w[A_GE * ws + o];
  const R cjkl = sqrt(S.k_ggm1 * (S.w[A_E * ws + o] - uv));
  R rk1 = S.yx[o], rk2 = S.yy[o];
  const R ugc = S.ug ? S.ug[o] : (R)0, vgc = S.vg ? S.vg[o] : (R)0;
  const bool pre = S.k_mp2 >= (R)0;
  const R qq2 = pre ? S.w[A_QY * ws + o] : S.w[A_QY * ws + o] + (rk1 * ugc + rk2 * vgc);
  const R rr2 = sqrt(rk1 * rk1 + rk2 * rk2);
  rk1 = rk1 / rr2; rk2 = rk2 / rr2;
  const R s1 = S.s[o], s2 = S.s[qs + o], s3 = S.s[2 * qs + o], s4 = S.s[3 * qs + o];
  const R a1 = s1 + s3 + s4;
  R a2, a3, a4;
  if (pre) {
    // arc2d_precon :1264-1298
    const R bSq = adi_bsq(S, o), omb = (R)1. - bSq, cy = S.w[A_CY * ws + o];
    const R X = sqrt((omb * qq2) * (omb * qq2) + (R)4. * bSq * cy * cy) / rr2;
    const R Y = (R)0.5 * (omb * qq2 / rr2 + X);
    const R Z = (R)0.5 * (omb * qq2 / rr2 - X);
    const R qqmxt = qq2 + ugc * rk1 * rr2 + vgc * rk2 * rr2;
    a2 = uu * s1 + rk2 * s2 + (uu + rk1 * Y / bSq) * s3;
    a2 = a2 + (uu + rk1 * Z / bSq) * s4;
    a3 = vv * s1 - rk1 * s2 + (vv + rk2 * Y / bSq) * s3;
    a3 = a3 + (vv + rk2 * Z / bSq) * s4;
    a4 = uv * s1 + (rk2 * uu - rk1 * vv) * s2;
    a4 = a4 + (ge + Y * qqmxt / rr2 / bSq) * s3;
    a4 = a4 + (ge + Z * qqmxt / rr2 / bSq) * s4;
  } else {
    a2 = uu * s1 + rk2 * s2 + (uu + rk1 * cjkl) * s3;
    a2 = a2 + (uu - rk1 * cjkl) * s4;
    a3 = vv * s1 - rk1 * s2 + (vv + rk2 * cjkl) * s3;
    a3 = a3 + (vv - rk2 * cjkl) * s4;
    a4 = uv * s1 + (rk2 * uu - rk1 * vv) * s2;
    a4 = a4 + (ge + cjkl * qq2 / rr2) * s3;
    a4 = a4 + (ge - cjkl * qq2 / rr2) * s4;
  }
  R o2 = a2, o3 = a3;
  if (p.iunst == 2) {
    const R tsr = S.tscale[o] * (R)p.rotf;
    const R d = (R)1.0 + sq(S.tscale[o] * (R)p.rotf);
    o2 = (a2 + tsr * a3) / d;
    o3 = (a3 - tsr * a2) / d;
  }
  S.s[o] = a1; S.s[qs + o] = o2; S.s[2 * qs + o] = o3; S.s[3 * qs + o] = a4;
  if constexpr (sizeof(R) == sizeof(double)) {
    double* q = S.q64;
    const double q1 = q[o], J = q[(int64_t)(p.nq - 1) * qs + o];
    const double dj = 1.0 / q1;
    const double u = q[qs + o] * dj, v = q[2 * qs + o] * dj, e = q[3 * qs + o] * dj;
    const double q1n = (q1 * J) / J;
    q[o] = q1n;
    q[qs + o] = u * q1n;
    q[2 * qs + o] = v * q1n;
    q[3 * qs + o] = e * q1n;
  }
}

}  // namespace ot2d
