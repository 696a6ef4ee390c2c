// k_rhs.cuh -- local time step (src/time.f:2-108), inviscid residual
// (src/eulerrhs.f:2-446, 628-912, 1011-1230) and viscous residual
// (src/visrhs.f:2-287), each restated per face / per cell so that every
// face flux is computed once and the per-cell arithmetic follows the
// reference's operation order.
#pragma once
#include "dev_common.cuh"

namespace ot2d {

// ---------------------------------------------------------------- time step
// The local time step of cell o (time.f:2-108) from its state: tscale and
// bt.  J is read only in the Jacobian-scaled form (iconstant_cfl = 0),
// q1..q4 only in the spectral-radius form.
template <class R>
__device__ __forceinline__ void time_step_vals(const Slice<R>& S, const ot2d_params& p, int64_t o, int ibi, R q1,
                                               R q2, R q3, R q4, R J, R oat) {
  const R h = S.k_h, timeac = S.k_timeac;
  R ib = (R)(ibi > 0 ? ibi : 0);
  R jac_factor = p.invisc ? (R)0.01 : (R)0.002;
  if (p.iconstant_cfl == 0) {
    if (p.idual == 0) {
      S.tscale[o] = oat * h * ib * ((R)1.0 + jac_factor * ((R)1. - timeac) * sqrt(J)) / ((R)1.0 + ((R)1. - timeac) * sqrt(J));
      S.bt[o] = (R)1.;
    } else {
      R t = ib * ((R)1.0 + jac_factor * sqrt(J)) / ((R)1.0 + sqrt(J));
      if (p.iprecon) t = (R)100. * ib * ((R)1.0 + (R)0.005 * sqrt(J)) / ((R)1.0 + sqrt(J));   // time.f:62-66
      t = t * S.k_dualtime;
      S.bt[o] = (R)1. / ((R)1. + t / h / oat);
      S.tscale[o] = t / ((R)1. + t / h / oat);
    }
    return;
  }
  R u = q2 / q1, v = q3 / q1, e = q4 / q1;
  R ugc = S.ug ? S.ug[o] : (R)0, vgc = S.vg ? S.vg[o] : (R)0;
  R xx = S.xx[o], xy = S.xy[o], yx = S.yx[o], yy = S.yy[o];
  R uu = (u - ugc) * xx + (v - vgc) * xy;
  R vv = (u - ugc) * yx + (v - vgc) * yy;
  R dxdx = sq(xx) + sq(xy), dydy = sq(yx) + sq(yy);
  R asq = S.k_ggm1 * (e - (R)0.5 * (sq(u) + sq(v)));
  R lam_j = fabs(uu) + sqrt(asq * dxdx);
  R lam_k = fabs(vv) + sqrt(asq * dydy);
  if (p.idual == 0) {
    R t = h / (lam_j + lam_k);
    S.tscale[o] = t * ib;
    S.bt[o] = (R)1.;
  } else {
    R hnew = S.k_dualtime / (lam_j + lam_k);
    R t = hnew * ib;
    t = t / ((R)1. + t / h / oat);
    S.tscale[o] = t;
    S.bt[o] = (R)1. / ((R)1. + t / h / oat);
  }
}
template <class R>
__device__ void time_step_cell(const Slice<R>& S, int j, int k, R oat) {
  const ot2d_params& p = *S.P;
  const int64_t o = at(S.jd, j, k), qs = S.qs;
  const R* q = S.q;
  if (p.iconstant_cfl == 0)
    time_step_vals(S, p, o, S.iblank[o], (R)0, (R)0, (R)0, (R)0, q[(p.nq - 1) * qs + o], oat);
  else
    time_step_vals(S, p, o, S.iblank[o], q[o], q[qs + o], q[2 * qs + o], q[3 * qs + o], (R)0, oat);
}

// ---------------------------------------------------------- reconstruction
// Primitive (rho, u, v, p) of cell i of a line, exactly as rhsup builds f
// (eulerrhs.f:55-61, :71-79).  dir 0: xi line at row `fix`; dir 1: eta line
// at column `fix`.
template <class R>
struct LineRd {
  const R* q; int64_t qs; int jd, nq, fix, dir; R gm1;
  const int32_t* ib;
  const R* qd = nullptr;   // ilim +-2: this direction's quad face states (ql arrays, then qr), stride qn2
  int64_t qn2 = 0;
  __device__ __forceinline__ int64_t off(int i) const { return dir == 0 ? at(jd, i, fix) : at(jd, fix, i); }
  __device__ __forceinline__ R quad_l(int v, int i) const { return qd[v * qn2 + off(i)]; }
  __device__ __forceinline__ R quad_r(int v, int i) const { return qd[(4 + v) * qn2 + off(i)]; }
  __device__ __forceinline__ R f(int i, int n) const {
    int64_t o = off(i);
    R q1 = q[o];
    if (n == 1) return q1 * q[(nq - 1) * qs + o];
    if (n == 2) { R rhoi = (R)1.0 / q1; return q[qs + o] * rhoi; }
    if (n == 3) { R rhoi = (R)1.0 / q1; return q[2 * qs + o] * rhoi; }
    R q2 = q[qs + o], q3 = q[2 * qs + o];
    R ppp = gm1 * (q[3 * qs + o] - (R)0.5 * (sq(q2) + sq(q3)) / q1);
    return ppp * q[(nq - 1) * qs + o];
  }
  __device__ __forceinline__ void f4(int i, R* out) const {
    int64_t o = off(i);
    R q1 = q[o], q2 = q[qs + o], q3 = q[2 * qs + o], q4 = q[3 * qs + o], J = q[(nq - 1) * qs + o];
    R rhoi = (R)1.0 / q1;
    out[0] = q1 * J; out[1] = q2 * rhoi; out[2] = q3 * rhoi;
    R ppp = gm1 * (q4 - (R)0.5 * (sq(q2) + sq(q3)) / q1);
    out[3] = ppp * J;
  }
  __device__ __forceinline__ int iba(int i) const { int v = ib[off(i)]; return v < 0 ? -v : v; }
};

template <class R> __device__ __forceinline__ R ammd(R fl, R fr) {
  return (R)0.5 * (fsign((R)1., fl) + fsign((R)1., fr)) * fmin2(fabs(fl), fabs(fr));
}

// weno5, eulerrhs.f:1194-1230
template <class R> __device__ __forceinline__ R weno5(R a, R b, R c, R d, R e) {
  const R b1 = (R)(13. / 12.), b2 = (R)(1. / 6.), epsw = (R)1.e-6;
  R djm1 = a - (R)2. * b + c, ejm1 = a - (R)4. * b + (R)3. * c;
  R dj = b - (R)2. * c + d, ej = b - d;
  R djp1 = c - (R)2. * d + e, ejp1 = (R)3. * c - (R)4. * d + e;
  R dis0 = b1 * djm1 * djm1 + (R)0.25 * ejm1 * ejm1 + epsw;
  R dis1 = b1 * dj * dj + (R)0.25 * ej * ej + epsw;
  R dis2 = b1 * djp1 * djp1 + (R)0.25 * ejp1 * ejp1 + epsw;
  R q30 = (R)2. * a - (R)7. * b + (R)11. * c, q31 = -b + (R)5. * c + (R)2. * d, q32 = (R)2. * c + (R)5. * d - e;
  R d01 = dis0 / dis1, d02 = dis0 / dis2;
  R a1ba0 = (R)6. * d01, a2ba0 = (R)3. * d02;
  R w0 = (R)1. / ((R)1. + a1ba0 + a2ba0);
  R w1 = a1ba0 * w0;
  R w2 = (R)1. - w0 - w1;
  return b2 * (w0 * q30 + w1 * q31 + w2 * q32);
}

// Left / right states at cell i of a line of n cells, for one variable,
// following the limiter the reference dispatches (eulerrhs.f:85-97):
// ilim 0 -> iflux, |ilim| 1 -> muscld_new, ilim 4 -> weno.  The WENO
// forms take a window w[0..6] = f(i-3..i+3) (entries outside 1..n are not
// read).
template <class R>
struct Recon {
  int ilim; R th, qt, epsl;
  R bsq;   // bSq of the faces with Turkel preconditioning (Mp**2), < 0 without
  // muscld_new, eulerrhs.f:855-873 (is=1, imax=n, im=n-1) on the cells
  // i-1, i, i+1 of the line
  __device__ __forceinline__ void muscl3(R wm, R w0, R wp, int i, int n, int ibm, int ib0, int ibp, R& ql,
                                         R& qr) const {
    if (qt == (R)0.0 || i == 1 || i == n) { ql = w0; qr = w0; return; }
    R thm = (R)1.0 - th, thp = (R)1.0 + th;
    R f2i = wp - w0, f2i1 = w0 - wm;
    R a1 = (R)3.0 * (f2i * f2i1 + epsl);
    R a2 = (R)2.0 * sq(f2i - f2i1) + a1;
    R f3i = a1 / a2;
    R f3qt = qt * f3i * (R)ib0 * (R)ibp * (R)ibm;
    ql = w0 + f3qt * (thm * f2i1 + thp * f2i);
    qr = w0 - f3qt * (thp * f2i1 + thm * f2i);
  }
  // iflux, eulerrhs.f:650-659
  __device__ __forceinline__ void central3(R wm, R w0, R wp, int i, int n, R& ql, R& qr) const {
    if (qt == (R)0.0 || i == 1 || i == n) { ql = w0; qr = w0; return; }
    R s1 = w0 - wm, s2 = wp - w0;
    R slope = (s1 + s2) / (R)2;
    ql = w0 + (R)0.5 * slope;
    qr = w0 - (R)0.5 * slope;
  }
  // weno, eulerrhs.f:1046-1189.  f1(i) = f(i+1)-f(i); f2 with the
  // extrapolated end values; f2m(i) = ammd(f2(i), f2(i+1)).
  __device__ __forceinline__ R f1(const R* w, int i, int c) const { return w[i - c + 4] - w[i - c + 3]; }
  __device__ __forceinline__ R f2(const R* w, int i, int c, int n) const {
    if (i == 1) { R a = f1(w, 2, c) - f1(w, 1, c), b = f1(w, 3, c) - f1(w, 2, c); return (R)2. * a - b; }
    if (i == n) { R a = f1(w, n - 1, c) - f1(w, n - 2, c), b = f1(w, n - 2, c) - f1(w, n - 3, c); return (R)2. * a - b; }
    return f1(w, i, c) - f1(w, i - 1, c);
  }
  __device__ __forceinline__ R f2m(const R* w, int i, int c, int n) const { return ammd(f2(w, i, c, n), f2(w, i + 1, c, n)); }
  __device__ __forceinline__ R sonic(const R* w, int i, int c, int n) const {
    R at = f1(w, i, c) - (R)0.5 * f2m(w, i, c, n);
    R ati1 = f1(w, i - 1, c) + (R)0.5 * f2m(w, i - 1, c, n);
    R s1 = ammd(f1(w, i, c), f1(w, i - 1, c));
    R t1 = ammd(at, ati1);
    return fsign((R)1., t1) * fmin2((R)0.5 * fabs(at + ati1), fmax2((R)2. * fabs(s1), fabs(t1)));
  }
  // window w covers f(c-3..c+3); i is the cell whose state is wanted (== c)
  __device__ __forceinline__ R weno_l(const R* w, int c, int n, int blank) const {
    if (qt == (R)0.0) return w[3];
    if (c == 1) { R at = f1(w, 1, c) - (R)0.5 * f2m(w, 1, c, n); R slope = ammd(at, (R)2. * f1(w, 1, c)); return w[3] + (R)0.5 * slope; }
    if (c == 2 || c == 3 || c == n - 1) return w[3] + (R)0.5 * sonic(w, c, c, n);
    R v = weno5(w[1], w[2], w[3], w[4], w[5]);
    R bv = (R)blank;
    return v * bv + ((R)1. - bv) * w[3];
  }
  __device__ __forceinline__ R weno_r(const R* w, int c, int n, int blank) const {
    if (qt == (R)0.0) return w[3];
    if (c == n) { R at1 = f1(w, n - 1, c) + (R)0.5 * f2m(w, n - 1, c, n); R slope = ammd(at1, (R)2. * f1(w, n - 1, c)); return w[3] - (R)0.5 * slope; }
    if (c == 2 || c == n - 1) return w[3] - (R)0.5 * sonic(w, c, c, n);
    R v = weno5(w[5], w[4], w[3], w[2], w[1]);
    R bv = (R)blank;
    return v * bv + ((R)1. - bv) * w[3];
  }
};

// ---------------------------------------------------------------- Roe flux
// roeflx, eulerrhs.f:283-446 (fssub = 0); left state L, right state Rr,
// face vector (ri1, ri2) and grid speed ri3.
template <class R>
__device__ __forceinline__ void roe(R gm1, const R* L, const R* Rr, R ri1, R ri2, R ri3, R* f) {
  const R eps = (R)1.e-6;
  R rlft = L[0], ulft = L[1], vlft = L[2], plft = L[3];
  R rlfti = (R)1.0 / rlft;
  R rulft = rlft * ulft, rvlft = rlft * vlft;
  R uvl = (R)0.5 * (ulft * ulft + vlft * vlft);
  R elft = plft / gm1 + rlft * uvl;
  R hlft = (elft + plft) * rlfti;
  R clft = sqrt(gm1 * (hlft - uvl));
  R rrht = Rr[0], urht = Rr[1], vrht = Rr[2], prht = Rr[3];
  R rrhti = (R)1.0 / rrht;
  R rurht = rrht * urht, rvrht = rrht * vrht;
  R uvr = (R)0.5 * (urht * urht + vrht * vrht);
  R erht = prht / gm1 + rrht * uvr;
  R hrht = (erht + prht) * rrhti;
  R crht = sqrt(gm1 * (hrht - uvr));
  R rat = sqrt(rrht * rlfti);
  R rati = (R)1.0 / (rat + (R)1.);
  R rav = rat * rlft;
  R uav = (rat * urht + ulft) * rati;
  R vav = (rat * vrht + vlft) * rati;
  R hav = (rat * hrht + hlft) * rati;
  R uv = (R)0.5 * (uav * uav + vav * vav);
  R cav = sqrt(gm1 * (hav - uv));
  R aq1 = rrht - rlft, aq2 = urht - ulft, aq3 = vrht - vlft, aq4 = prht - plft;
  R rr2 = ri1 * ri1 + ri2 * ri2;
  R rr = sqrt(rr2);
  R r0 = (R)1.0 / rr;
  R r1 = ri1 * r0, r2 = ri2 * r0, r3 = ri3 * r0;
  R uu = r1 * uav + r2 * vav + r3;
  R c2 = cav * cav;
  R c2i = (R)1.0 / c2;
  R auu = fabs(uu), aupc = fabs(uu + cav), aumc = fabs(uu - cav);
  R uulft = r1 * ulft + r2 * vlft + r3;
  R uurht = r1 * urht + r2 * vrht + r3;
  R upclft = uulft + clft, upcrht = uurht + crht;
  R umclft = uulft - clft, umcrht = uurht - crht;
  R dauu = (R)4. * (uurht - uulft) + eps;
  R dauus = fmax2(dauu, (R)0.0);
  if (auu <= (R)0.5 * dauus) auu = auu * auu / dauu + (R)0.25 * dauu;
  R daupc = (R)4. * (upcrht - upclft) + eps;
  R daupcs = fmax2(daupc, (R)0.0);
  if (aupc <= (R)0.5 * daupcs) aupc = aupc * aupc / daupc + (R)0.25 * daupc;
  R daumc = (R)4. * (umcrht - umclft) + eps;
  R daumcs = fmax2(daumc, (R)0.0);
  if (aumc <= (R)0.5 * daumcs) aumc = aumc * aumc / daumc + (R)0.25 * daumc;
  R rcav = rav * cav;
  R aquu = uurht - uulft;
  R c2ih = (R)0.5 * c2i;
  R ruuav = auu * rav;
  R b1 = auu * (aq1 - c2i * aq4);
  R b2 = c2ih * aupc * (aq4 + rcav * aquu);
  R b3 = c2ih * aumc * (aq4 - rcav * aquu);
  R b4 = b1 + b2 + b3;
  R b5 = cav * (b2 - b3);
  R b6 = ruuav * (aq2 - r1 * aquu);
  R b7 = ruuav * (aq3 - r2 * aquu);
  aq1 = b4;
  aq2 = uav * b4 + r1 * b5 + b6;
  aq3 = vav * b4 + r2 * b5 + b7;
  aq4 = hav * b4 + (uu - r3) * b5 + uav * b6 + vav * b7 - c2 * b1 / gm1;
  R aj = (R)0.5 * rr;
  R plar = plft + prht;
  R eplft = elft + plft, eprht = erht + prht;
  const R fssub = (R)0.0, z = (R)0;
  f[0] = aj * (rlft * uulft + rrht * uurht - aq1) - fssub * z;
  f[1] = aj * (rulft * uulft + rurht * uurht + r1 * plar - aq2) - fssub * z;
  f[2] = aj * (rvlft * uulft + rvrht * uurht + r2 * plar - aq3) - fssub * z;
  f[3] = aj * (eplft * uulft + eprht * uurht - r3 * plar - aq4) - fssub * z;
}

// roetrklflx, eulerrhs.f:450-625 (fssub = 0): the Roe flux with Turkel's
// low-Mach preconditioning.  bSq is the face's Mp**2/(bt - Mp**2*(bt-1))
// with bt = 1, i.e. Mp**2; the eigenvalues (1+bSq)u/2 +- X/2 with
// X = sqrt(((1-bSq)u)**2 + 4 bSq c**2) replace u +- c, in the same entropy
// fix, and the acoustic waves are split with R and S = ((1-bSq)u +- X)/2.
template <class R>
__device__ __forceinline__ void roe_turkel(R gm1, R bSq, const R* L, const R* Rr, R ri1, R ri2, R ri3, R* f) {
  const R eps = (R)1.e-6;
  R rlft = L[0], ulft = L[1], vlft = L[2], plft = L[3];
  R rlfti = (R)1.0 / rlft;
  R rulft = rlft * ulft, rvlft = rlft * vlft;
  R uvl = (R)0.5 * (ulft * ulft + vlft * vlft);
  R elft = plft / gm1 + rlft * uvl;
  R hlft = (elft + plft) * rlfti;
  R clft = sqrt(gm1 * (hlft - uvl));
  R rrht = Rr[0], urht = Rr[1], vrht = Rr[2], prht = Rr[3];
  R rrhti = (R)1.0 / rrht;
  R rurht = rrht * urht, rvrht = rrht * vrht;
  R uvr = (R)0.5 * (urht * urht + vrht * vrht);
  R erht = prht / gm1 + rrht * uvr;
  R hrht = (erht + prht) * rrhti;
  R crht = sqrt(gm1 * (hrht - uvr));
  R rat = sqrt(rrht * rlfti);
  R rati = (R)1.0 / (rat + (R)1.);
  R rav = rat * rlft;
  R uav = (rat * urht + ulft) * rati;
  R vav = (rat * vrht + vlft) * rati;
  R hav = (rat * hrht + hlft) * rati;
  R uv = (R)0.5 * (uav * uav + vav * vav);
  R cav = sqrt(gm1 * (hav - uv));
  R aq1 = rrht - rlft, aq2 = urht - ulft, aq3 = vrht - vlft, aq4 = prht - plft;
  R rr2 = ri1 * ri1 + ri2 * ri2;
  R rr = sqrt(rr2);
  R r0 = (R)1.0 / rr;
  R r1 = ri1 * r0, r2 = ri2 * r0, r3 = ri3 * r0;
  R uumxt = r1 * uav + r2 * vav;
  R uu = uumxt + r3;
  R c2 = cav * cav;
  R c2i = (R)1.0 / c2;
  const R omb = (R)1. - bSq, opb = (R)1. + bSq, fb = (R)4. * bSq;
  R X = sqrt(((omb * uu) * omb) * uu + fb * c2);
  R auu = fabs(uu);
  R aupc = (R)0.5 * fabs(opb * uu + X);
  R aumc = (R)0.5 * fabs(opb * uu - X);
  R uulft = r1 * ulft + r2 * vlft + r3;
  R uurht = r1 * urht + r2 * vrht + r3;
  X = sqrt((omb * uulft) * (omb * uulft) + (fb * clft) * clft);
  R upclft = (R)0.5 * (opb * uulft + X);
  R umclft = (R)0.5 * (opb * uulft - X);
  X = sqrt((omb * uurht) * (omb * uurht) + (fb * crht) * crht);
  R upcrht = (R)0.5 * (opb * uurht + X);
  R umcrht = (R)0.5 * (opb * uurht - X);
  R dauu = (R)4. * (uurht - uulft) + eps;
  R dauus = fmax2(dauu, (R)0.0);
  if (auu <= (R)0.5 * dauus) auu = auu * auu / dauu + (R)0.25 * dauu;
  R daupc = (R)4. * (upcrht - upclft) + eps;
  R daupcs = fmax2(daupc, (R)0.0);
  if (aupc <= (R)0.5 * daupcs) aupc = aupc * aupc / daupc + (R)0.25 * daupc;
  R daumc = (R)4. * (umcrht - umclft) + eps;
  R daumcs = fmax2(daumc, (R)0.0);
  if (aumc <= (R)0.5 * daumcs) aumc = aumc * aumc / daumc + (R)0.25 * daumc;
  R aquu = uurht - uulft;
  R ruuav = auu * rav;
  X = sqrt((omb * uu) * (omb * uu) + fb * c2);
  R Rw = (R)0.5 * (omb * uu + X);
  R Sw = (R)0.5 * (omb * uu - X);
  R b1 = auu * (aq1 - c2i * aq4);
  R b2 = aupc * (aq4 / Rw + rav * aquu) / X;
  R b3 = aumc * (-(aq4 / Sw) - rav * aquu) / X;
  R b4 = b1 + b2 + b3;
  R b5 = (Rw * b2 + Sw * b3);
  R b6 = ruuav * (aq2 - r1 * aquu);
  R b7 = ruuav * (aq3 - r2 * aquu);
  aq1 = b4;
  aq2 = uav * b4 + r1 * b5 + b6;
  aq3 = vav * b4 + r2 * b5 + b7;
  aq4 = hav * b4 + uumxt * b5 + uav * b6 + vav * b7 - c2 * b1 / gm1;
  R aj = (R)0.5 * rr;
  R plar = plft + prht;
  R eplft = elft + plft, eprht = erht + prht;
  f[0] = aj * (rlft * uulft + rrht * uurht - aq1);
  f[1] = aj * (rulft * uulft + rurht * uurht + r1 * plar - aq2);
  f[2] = aj * (rvlft * uulft + rvrht * uurht + r2 * plar - aq3);
  f[3] = aj * (eplft * uulft + eprht * uurht - r3 * plar - aq4);
}

// Inviscid flux through one face between cells i and i+1 of a line.  L
// supplies f4(c, out) (the primitive f of cell c) and iba(c), and for quad
// the states quad_l / quad_r k_quad left.  LIM is the limiter family (0
// central, 1 MUSCL, 2 quad, 4 WENO) so that the central and MUSCL
// forms index their window with constants only (the window stays in
// registers); face_flux() dispatches on rc.ilim.  PRE: Turkel's
// preconditioned flux (roetrklflx) in place of roeflx.
template <int LIM, class R, class Line, bool PRE = false>
__device__ __forceinline__ void face_flux_t(const Line& L, const Recon<R>& rc, int i, int n, R ri1, R ri2, R ri3,
                                            R* fout) {
  R ql[4], qr[4];
  if constexpr (LIM == 4) {
    // window cells i-3 .. i+4 (two overlapping 7-point windows for i and i+1)
    R w8[4][8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const int c = i - 3 + m;
      R t[4] = {(R)0, (R)0, (R)0, (R)0};
      if (c >= 1 && c <= n) L.f4(c, t);
#pragma unroll
      for (int v = 0; v < 4; ++v) w8[v][m] = t[v];
    }
    int blank_l = 1, blank_r = 1;
    if (i >= 3 && i + 2 <= n) blank_l = L.iba(i) * L.iba(i - 1) * L.iba(i + 1) * L.iba(i - 2) * L.iba(i + 2);
    if (i + 1 >= 3 && i + 3 <= n) blank_r = L.iba(i + 1) * L.iba(i) * L.iba(i + 2) * L.iba(i - 1) * L.iba(i + 3);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      ql[v] = rc.weno_l(&w8[v][0], i, n, blank_l);
      qr[v] = rc.weno_r(&w8[v][1], i + 1, n, blank_r);
    }
  } else if constexpr (LIM == 2) {
    // quad: ql of cell i and qr of cell i+1, reconstructed over the whole line
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      ql[v] = L.quad_l(v, i);
      qr[v] = L.quad_r(v, i + 1);
    }
  } else {
    // cells i-1 .. i+2 (w4[m] = f(i-1+m)); MUSCL / central read only these
    R w4[4][4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int c = i - 1 + m;
      R t[4] = {(R)0, (R)0, (R)0, (R)0};
      if (c >= 1 && c <= n) L.f4(c, t);
#pragma unroll
      for (int v = 0; v < 4; ++v) w4[v][m] = t[v];
    }
    if constexpr (LIM == 1) {
      const int bm = (i - 1 >= 1) ? L.iba(i - 1) : 0, b0 = L.iba(i), bp = L.iba(i + 1);
      const int bp2 = (i + 2 <= n) ? L.iba(i + 2) : 0;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        R dummy;
        // muscl reads w[2..4] around its cell: cell i -> w4[v][0..2], cell i+1 -> w4[v][1..3]
        rc.muscl3(w4[v][0], w4[v][1], w4[v][2], i, n, bm, b0, bp, ql[v], dummy);
        rc.muscl3(w4[v][1], w4[v][2], w4[v][3], i + 1, n, b0, bp, bp2, dummy, qr[v]);
      }
    } else {
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        R dummy;
        rc.central3(w4[v][0], w4[v][1], w4[v][2], i, n, ql[v], dummy);
        rc.central3(w4[v][1], w4[v][2], w4[v][3], i + 1, n, dummy, qr[v]);
      }
    }
  }
  if constexpr (PRE) roe_turkel(L.gm1, rc.bsq, ql, qr, ri1, ri2, ri3, fout);
  else roe(L.gm1, ql, qr, ri1, ri2, ri3, fout);
}

// the flux of one face with the limiter of rc.ilim; PRE fixed at compile
// time (the fused residual is instantiated once per flux)
template <bool PRE, class R, class Line>
__device__ __forceinline__ void face_flux_p(const Line& L, const Recon<R>& rc, int i, int n, R ri1, R ri2, R ri3,
                                            R* fout) {
  const int ilm = rc.ilim < 0 ? -rc.ilim : rc.ilim;
  if (rc.ilim == 4) face_flux_t<4, R, Line, PRE>(L, rc, i, n, ri1, ri2, ri3, fout);
  else if (ilm == 1) face_flux_t<1, R, Line, PRE>(L, rc, i, n, ri1, ri2, ri3, fout);
  else if (ilm == 2) face_flux_t<2, R, Line, PRE>(L, rc, i, n, ri1, ri2, ri3, fout);
  else face_flux_t<0, R, Line, PRE>(L, rc, i, n, ri1, ri2, ri3, fout);
}

// eulerrhs.f:155-159, :263-267: roetrklflx with iprecon, roeflx without
template <class R, class Line>
__device__ __forceinline__ void face_flux(const Line& L, const Recon<R>& rc, int i, int n, R ri1, R ri2, R ri3,
                                          R* fout) {
  if (rc.bsq >= (R)0) face_flux_p<true>(L, rc, i, n, ri1, ri2, ri3, fout);
  else face_flux_p<false>(L, rc, i, n, ri1, ri2, ri3, fout);
}

template <class R>
__device__ __forceinline__ Recon<R> make_recon(const ot2d_params& p, int dir) {
  Recon<R> rc;
  int irhs = p.irhsy < 0 ? -p.irhsy : p.irhsy;
  rc.th = (R)((double)(irhs - 2) / (double)irhs);
  rc.qt = (irhs == 1) ? (R)0.0 : (R)0.25;
  double ep = (dir == 0) ? 10. / (double)p.jmax : 10. / (double)p.kmax;
  rc.epsl = (R)((ep * ep) * ep);
  rc.ilim = p.ilim;
  rc.bsq = p.iprecon ? (R)(p.Mp * p.Mp) : (R)-1;
  return rc;
}

// xi face (j+1/2, k), j in [jbeg-1, jend], k in [kbeg, kend]; flux into F
// (4 arrays of stride wstride: F(j,k) = flux through face j+1/2 of row k)
template <class R>
__device__ void xi_face(const Slice<R>& S, int j, int k, R* F) {
  const ot2d_params& p = *S.P;
  LineRd<R> L{S.q, S.qs, S.jd, p.nq, k, 0, S.k_gm1, S.iblank};
  if (S.quad) { L.qd = S.quad; L.qn2 = (int64_t)S.jd * S.kd; }
  Recon<R> rc = make_recon<R>(p, 0);
  int64_t o = at(S.jd, j, k);
  R f[4];
  face_flux(L, rc, j, S.jd, S.fxa[o], S.fya[o], S.ftj ? S.ftj[o] : (R)0.0, f);
#pragma unroll
  for (int v = 0; v < 4; ++v) F[v * S.wstride + o] = f[v];
}

// eta face (j, k+1/2), j in [jbeg, jend], k in [kbeg-1, kend]
template <class R>
__device__ void eta_face(const Slice<R>& S, int j, int k, R* G) {
  const ot2d_params& p = *S.P;
  LineRd<R> L{S.q, S.qs, S.jd, p.nq, j, 1, S.k_gm1, S.iblank};
  if (S.quad) { L.qd = S.quad + 8 * (int64_t)S.jd * S.kd; L.qn2 = (int64_t)S.jd * S.kd; }
  Recon<R> rc = make_recon<R>(p, 1);
  int64_t o = at(S.jd, j, k);
  R f[4];
  face_flux(L, rc, k, S.kd, S.gxa[o], S.gya[o], S.gtj ? S.gtj[o] : (R)0.0, f);
#pragma unroll
  for (int v = 0; v < 4; ++v) G[v * S.wstride + o] = f[v];
}

// ---------------------------------------------------------------- viscous
// Per-cell viscous coefficients of visrhs (visrhs.f:48-60, :168-180).
template <class R>
struct ViscCell { R u, v, e, vnu, gkap, rj; };

template <class R>
__device__ __forceinline__ ViscCell<R> visc_cell(const Slice<R>& S, const ot2d_params& p, int j, int k) {
  const int64_t o = at(S.jd, j, k), qs = S.qs;
  const R c2b = S.k_c2b, c2bp = S.k_c2bp, prtr = S.k_prtr;
  ViscCell<R> c;
  R ra = (R)1. / S.q[o];
  c.u = S.q[qs + o] * ra; c.v = S.q[2 * qs + o] * ra;
  c.e = S.q[3 * qs + o] * ra - (R).5 * (sq(c.u) + sq(c.v));
  R tt = S.k_ggm1 * c.e;
  R vmue = c2bp * tt * sqrt(tt) / (c2b + tt);
  R turm = S.turmu[o];
  c.vnu = vmue + turm; c.gkap = vmue + prtr * turm;
  c.rj = (R)1. / S.q[(p.nq - 1) * qs + o];
  return c;
}

// eta-direction viscous face quantities of column j: f2,f3,f4 at face k+1/2
// and f2v,f3v,f4v at cell k (visrhs.f:46-131), k in [1, kd-1]
template <class R>
__device__ void visc_eta_face(const Slice<R>& S, int j, int k, R* V) {
  const ot2d_params& p = *S.P;
  const int jd = S.jd; const int64_t qs = S.qs;
  const R gkpr = S.k_gkpr, dre = S.k_dre;
  auto M = [&](const R* a, int jj, int kk) { return a[at(jd, jj, kk)]; };
  R bv[2][4], uu[2], vv[2], ee[2];
  R d1 = 0, d2 = 0, d4 = 0, d5 = 0, d7 = 0;
  for (int m = 0; m < 2; ++m) {
    int kk = k + m;
    ViscCell<R> c = visc_cell(S, p, j, kk);
    uu[m] = c.u; vv[m] = c.v; ee[m] = c.e;
    R yx = M(S.yx, j, kk), yy = M(S.yy, j, kk);
    R b4 = (sq(yx) + sq(yy)) * c.rj;
    bv[m][0] = (b4 + sq(yx) / (R)3. * c.rj) * c.vnu * dre;
    bv[m][1] = (b4 + sq(yy) / (R)3. * c.rj) * c.vnu * dre;
    bv[m][3] = (yx * yy / (R)3. * c.rj) * c.vnu * dre;
    bv[m][2] = b4 * gkpr * c.gkap * dre;
    if (m == 0) {
      R rjm = (R)1. / S.q[(p.nq - 1) * qs + at(jd, j - 1, kk)], rjp = (R)1. / S.q[(p.nq - 1) * qs + at(jd, j + 1, kk)];
      R xxm = M(S.xx, j - 1, kk), xym = M(S.xy, j - 1, kk), yxm = M(S.yx, j - 1, kk), yym = M(S.yy, j - 1, kk);
      R xxp = M(S.xx, j + 1, kk), xyp = M(S.xy, j + 1, kk), yxp = M(S.yx, j + 1, kk), yyp = M(S.yy, j + 1, kk);
      d1 = ((R)(4. / 3.) * xxm * yxm + xym * yym) * rjm;
      d1 = d1 + ((R)(4. / 3.) * xxp * yxp + xyp * yyp) * rjp;
      d1 = c.vnu * dre * d1;
      d2 = ((R)(4. / 3.) * xym * yym + xxm * yxm) * rjm;
      d2 = d2 + ((R)(4. / 3.) * xyp * yyp + xxp * yxp) * rjp;
      d2 = c.vnu * dre * d2;
      d4 = (xym * yym + xxm * yxm) * rjm;
      d4 = d4 + (xyp * yyp + xxp * yxp) * rjp;
      d4 = d4 * gkpr * c.gkap * dre;
      d5 = ((R)(-2. / 3.) * xym * yxm + xxm * yym) * rjm;
      d5 = d5 + ((R)(-2. / 3.) * xyp * yxp + xxp * yyp) * rjp;
      d5 = c.vnu * dre * d5;
      d7 = ((R)(-2. / 3.) * xxm * yym + xym * yxm) * rjm;
      d7 = d7 + ((R)(-2. / 3.) * xxp * yyp + xyp * yxp) * rjp;
      d7 = c.vnu * dre * d7;
    }
  }
  R b1 = bv[1][0] + bv[0][0], b2 = bv[1][1] + bv[0][1], b5 = bv[1][3] + bv[0][3];
  const int64_t op = at(jd, j + 1, k), om = at(jd, j - 1, k);
  R ujp1 = S.q[qs + op] / S.q[op], ujm1 = S.q[qs + om] / S.q[om];
  R duj = (R)0.5 * (ujp1 - ujm1);
  R vjp1 = S.q[2 * qs + op] / S.q[op], vjm1 = S.q[2 * qs + om] / S.q[om];
  R dvj = (R)0.5 * (vjp1 - vjm1);
  R ejp1 = S.q[3 * qs + op] / S.q[op] - (R).5 * (sq(ujp1) + sq(vjp1));
  R ejm1 = S.q[3 * qs + om] / S.q[om] - (R).5 * (sq(ujm1) + sq(vjm1));
  R dej = (R)0.5 * (ejp1 - ejm1);
  R t4 = uu[1] * bv[1][0] + uu[0] * bv[0][0];
  R t5 = vv[1] * bv[1][1] + vv[0] * bv[0][1];
  R t6 = uu[1] * bv[1][3] + uu[0] * bv[0][3];
  R t7 = vv[1] * bv[1][3] + vv[0] * bv[0][3];
  R t8 = bv[1][2] + bv[0][2];
  R du = uu[1] - uu[0], dv = vv[1] - vv[0], dei = ee[1] - ee[0];
  const int64_t o = at(jd, j, k), ws = S.wstride;
  V[0 * ws + o] = b1 * du + b5 * dv;
  V[1 * ws + o] = b5 * du + b2 * dv;
  V[2 * ws + o] = (t4 + t7) * du + (t5 + t6) * dv + t8 * dei;
  V[3 * ws + o] = d1 * duj + d5 * dvj;
  V[4 * ws + o] = d7 * duj + d2 * dvj;
  R f4v = (R)0.5 * d1 * (R)0.5 * (sq(ujp1) - sq(ujm1));
  f4v = f4v + (R)0.5 * d2 * (R)0.5 * (sq(vjp1) - sq(vjm1));
  f4v = f4v + d5 * (R)0.5 * (ujp1 + ujm1) * dvj;
  f4v = f4v + d7 * (R)0.5 * (vjp1 + vjm1) * duj;
  f4v = f4v + d4 * dej;
  V[5 * ws + o] = f4v;
}

// xi-direction viscous face quantities of row k: face j+1/2 and cell j
// (visrhs.f:166-251), j in [1, jd-1]
template <class R>
__device__ void visc_xi_face(const Slice<R>& S, int j, int k, R* V) {
  const ot2d_params& p = *S.P;
  const int jd = S.jd; const int64_t qs = S.qs;
  const R gkpr = S.k_gkpr, dre = S.k_dre;
  auto M = [&](const R* a, int jj, int kk) { return a[at(jd, jj, kk)]; };
  R av[2][4], uu[2], vv[2], ee[2];
  R d1 = 0, d2 = 0, d4 = 0, d5 = 0, d7 = 0;
  for (int m = 0; m < 2; ++m) {
    int jj = j + m;
    ViscCell<R> c = visc_cell(S, p, jj, k);
    uu[m] = c.u; vv[m] = c.v; ee[m] = c.e;
    R xx = M(S.xx, jj, k), xy = M(S.xy, jj, k);
    R a4 = (sq(xx) + sq(xy)) * c.rj;
    av[m][0] = (a4 + sq(xx) / (R)3. * c.rj) * c.vnu * dre;
    av[m][1] = (a4 + sq(xy) / (R)3. * c.rj) * c.vnu * dre;
    av[m][3] = (xx * xy / (R)3. * c.rj) * c.vnu * dre;
    av[m][2] = a4 * gkpr * c.gkap * dre;
    if (m == 0) {
      R rkm = (R)1. / S.q[(p.nq - 1) * qs + at(jd, jj, k - 1)], rkp = (R)1. / S.q[(p.nq - 1) * qs + at(jd, jj, k + 1)];
      R xxm = M(S.xx, jj, k - 1), xym = M(S.xy, jj, k - 1), yxm = M(S.yx, jj, k - 1), yym = M(S.yy, jj, k - 1);
      R xxp = M(S.xx, jj, k + 1), xyp = M(S.xy, jj, k + 1), yxp = M(S.yx, jj, k + 1), yyp = M(S.yy, jj, k + 1);
      d1 = ((R)(4. / 3.) * xxm * yxm + xym * yym) * rkm;
      d1 = d1 + ((R)(4. / 3.) * xxp * yxp + xyp * yyp) * rkp;
      d1 = c.vnu * dre * d1;
      d2 = ((R)(4. / 3.) * xym * yym + xxm * yxm) * rkm;
      d2 = d2 + ((R)(4. / 3.) * xyp * yyp + xxp * yxp) * rkp;
      d2 = c.vnu * dre * d2;
      d4 = (xym * yym + xxm * yxm) * rkm;
      d4 = d4 + (xyp * yyp + xxp * yxp) * rkp;
      d4 = d4 * gkpr * c.gkap * dre;
      d5 = ((R)(-2. / 3.) * xym * yxm + xxm * yym) * rkm;
      d5 = d5 + ((R)(-2. / 3.) * xyp * yxp + xxp * yyp) * rkp;
      d5 = c.vnu * dre * d5;
      d7 = ((R)(-2. / 3.) * xxm * yym + xym * yxm) * rkm;
      d7 = d7 + ((R)(-2. / 3.) * xxp * yyp + xyp * yxp) * rkp;
      d7 = c.vnu * dre * d7;
    }
  }
  R a1 = av[1][0] + av[0][0], a2 = av[1][1] + av[0][1], a5 = av[1][3] + av[0][3];
  const int64_t op = at(jd, j, k + 1), om = at(jd, j, k - 1);
  R ukp1 = S.q[qs + op] / S.q[op], ukm1 = S.q[qs + om] / S.q[om];
  R duk = (R)0.5 * (ukp1 - ukm1);
  R vkp1 = S.q[2 * qs + op] / S.q[op], vkm1 = S.q[2 * qs + om] / S.q[om];
  R dvk = (R)0.5 * (vkp1 - vkm1);
  R ekp1 = S.q[3 * qs + op] / S.q[op] - (R).5 * (sq(ukp1) + sq(vkp1));
  R ekm1 = S.q[3 * qs + om] / S.q[om] - (R).5 * (sq(ukm1) + sq(vkm1));
  R dek = (R)0.5 * (ekp1 - ekm1);
  R t4 = uu[1] * av[1][0] + uu[0] * av[0][0];
  R t5 = vv[1] * av[1][1] + vv[0] * av[0][1];
  R t6 = uu[1] * av[1][3] + uu[0] * av[0][3];
  R t7 = vv[1] * av[1][3] + vv[0] * av[0][3];
  R t8 = av[1][2] + av[0][2];
  R du = uu[1] - uu[0], dv = vv[1] - vv[0], dei = ee[1] - ee[0];
  const int64_t o = at(jd, j, k), ws = S.wstride;
  V[0 * ws + o] = a1 * du + a5 * dv;
  V[1 * ws + o] = a5 * du + a2 * dv;
  V[2 * ws + o] = (t4 + t7) * du + (t5 + t6) * dv + t8 * dei;
  V[3 * ws + o] = d1 * duk + d7 * dvk;
  V[4 * ws + o] = d5 * duk + d2 * dvk;
  R f4v = (R)0.5 * d1 * (R)0.5 * (sq(ukp1) - sq(ukm1));
  f4v = f4v + (R)0.5 * d2 * (R)0.5 * (sq(vkp1) - sq(vkm1));
  f4v = f4v + d5 * (R)0.5 * (vkp1 + vkm1) * duk;
  f4v = f4v + d7 * (R)0.5 * (ukp1 + ukm1) * dvk;
  f4v = f4v + d4 * dek;
  V[5 * ws + o] = f4v;
}

// Residual of interior cell (j,k): out4 (the incoming s) - dF_xi - dF_eta
// (+ viscous eta, + viscous xi) in the reference's accumulation order
// (eulerrhs.f:162-167, :263-268, visrhs.f:133-161, :254-284).  F, G:
// inviscid face fluxes (null: skip); VE, VX: viscous (null: skip).
template <class R>
__device__ void assemble_cell(const Slice<R>& S, int j, int k, const R* F, const R* G, const R* VE, const R* VX,
                              R* out4) {
  const ot2d_params& p = *S.P;
  const int jd = S.jd; const int64_t ws = S.wstride;
  const int64_t o = at(jd, j, k), oj = at(jd, j - 1, k), ok = at(jd, j, k - 1);
  R s[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) s[v] = out4[v];
  if (F) {
#pragma unroll
    for (int v = 0; v < 4; ++v) s[v] = s[v] - (F[v * ws + o] - F[v * ws + oj]);
#pragma unroll
    for (int v = 0; v < 4; ++v) s[v] = s[v] - (G[v * ws + o] - G[v * ws + ok]);
  }
  if (VE) {
    // eta viscous: (f(k)-f(k-1)) + 0.5*(fv(k+1)-fv(k-1)), one-sided at kend
    for (int v = 0; v < 3; ++v) {
      R a = VE[v * ws + o] - VE[v * ws + ok];
      R b;
      if (k == p.kend) b = (R)0.5 * (VE[(v + 3) * ws + at(jd, j, k - 2)] - (R)4. * VE[(v + 3) * ws + ok] + (R)3 * VE[(v + 3) * ws + o]);
      else b = (R)0.5 * (VE[(v + 3) * ws + at(jd, j, k + 1)] - VE[(v + 3) * ws + ok]);
      s[v + 1] = s[v + 1] + a + b;
    }
    for (int v = 0; v < 3; ++v) {
      R a = VX[v * ws + o] - VX[v * ws + oj];
      R b;
      if (j == p.jend) b = (R)0.5 * (VX[(v + 3) * ws + at(jd, j - 2, k)] - (R)4. * VX[(v + 3) * ws + oj] + (R)3 * VX[(v + 3) * ws + o]);
      else b = (R)0.5 * (VX[(v + 3) * ws + at(jd, j + 1, k)] - VX[(v + 3) * ws + oj]);
      s[v + 1] = s[v + 1] + a + b;
    }
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) out4[v] = s[v];
}

}  // namespace ot2d
