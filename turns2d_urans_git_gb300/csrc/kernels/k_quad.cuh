// k_quad.cuh -- rhsup's piecewise quadratic reconstruction, ilim = +-2:
// quad (src/eulerrhs.f:1233-1559) with tridag (:1562-1588).
//
// quad takes a whole grid line at a time: the nodal slopes and curvatures
// come from two compact (tridiagonal) systems along the line, then a median
// correction of their signs and the monotonicity-preserving constraint.
// So it runs before the fused residual, one thread per (line, variable) of
// both directions, and leaves the left / right states ql(i), qr(i) of every
// cell of every line in the slice's quad arrays; a face of the residual
// (face_flux_t<2>) reads ql of the cell before it and qr of the cell after
// it.  The arithmetic per line is quad's, in its order, so the FP64 path
// gives the oracle's bits.
#pragma once
#include "dev_common.cuh"
#include "k_rhs.cuh"

namespace ot2d {

// Arrays of a slice's quad block (jd*kd elements of R each, cell (j,k) at
// at(jd, j, k)): out(dir, side, v) = 16 arrays of face states (side 0 ql, 1
// qr); then work(dir, v, a) = 24 line work arrays (a 0 slope, 1 curvature,
// 2 elimination factors of the tridiagonal solve).
template <class R>
__device__ __forceinline__ R* quad_out(const Slice<R>& S, int dir, int side, int v) {
  return S.quad + (int64_t)((dir * 2 + side) * 4 + v) * S.jd * S.kd;
}
template <class R>
__device__ __forceinline__ R* quad_work(const Slice<R>& S, int dir, int v, int a) {
  return S.quad + (int64_t)(16 + (dir * 4 + v) * 3 + a) * S.jd * S.kd;
}

// amedian of quad: b moved toward c and d by the smaller distance when both
// lie on the same side of it
template <class R>
__device__ __forceinline__ R quad_median(R b, R c, R d) {
  return b + (R)0.5 * (fsign((R)1., c - b) + fsign((R)1., d - b)) * fmin2(fabs(c - b), fabs(d - b));
}
// the limited slope quad uses next to the line ends
template <class R>
__device__ __forceinline__ R quad_sonic(R at, R ati1, R sl) {
  const R t1 = ammd(at, ati1);
  return fsign((R)1., t1) * fmin2((R)0.5 * fabs(at + ati1), fmax2((R)2. * fabs(sl), fabs(t1)));
}

// Right-hand side of the compact system of the slope (curv = false) or the
// curvature (curv = true) at interior line position i, is2 < i < ie2.
template <class R>
__device__ __forceinline__ R quad_rhs(const LineRd<R>& L, int v, int i, bool curv) {
  if (!curv) return (L.f(i + 2, v) + (R)28. * L.f(i + 1, v) - (R)28. * L.f(i - 1, v) - L.f(i - 2, v)) / (R)36.;
  return ((R)3. * L.f(i + 2, v) + (R)48. * L.f(i + 1, v) - (R)102. * L.f(i, v) + (R)48. * L.f(i - 1, v) +
          (R)3. * L.f(i - 2, v)) / (R)44.;
}

// tridag over positions is2..ie2 of one line: sub- and super-diagonal c1,
// diagonal 1, right-hand side rhs(i); solution into D (the elimination's g
// first, overwritten in place by the back substitution), factors w into W.
// c1e / rhse: the end rows' coefficient and right-hand side.
template <class R, class Rhs>
__device__ __forceinline__ void quad_tridag(const LineRd<R>& L, R* D, R* W, int is2, int ie2, R c1i, R c1e,
                                            R rhs_s, R rhs_e, Rhs rhs) {
  // row is2: w = c/b, g = f/b with b = 1
  R w = c1e / (R)1., g = rhs_s / (R)1.;
  W[L.off(is2)] = w; D[L.off(is2)] = g;
  for (int j = is2 + 1; j <= ie2; ++j) {
    const R a = j == ie2 ? c1e : c1i;
    const R f = j == ie2 ? rhs_e : rhs(j);
    const R d = (R)1. - a * w;
    const R rd = (R)1.0 / d;
    w = a * rd;
    g = (f - a * g) * rd;
    W[L.off(j)] = w; D[L.off(j)] = g;
  }
  R z = g;   // z(ie2) = g(ie2)
  for (int j = ie2 - 1; j >= is2; --j) {
    const int64_t o = L.off(j);
    z = D[o] - W[o] * z;
    D[o] = z;
  }
}

// quad on variable v (1..4) of one line of n cells (is = 1, ie = n), ibmin =
// ibmax = 1 as rhsup calls it.  cm, a scalar the reference carries from one
// cell to the next, starts at 0 on every line (the reference leaves it
// undefined; it is read only when amedian's sum rounds to none of its
// arguments).
template <class R>
__device__ void quad_line(const Slice<R>& S, const LineRd<R>& L, int dir, int v, int n, R qt) {
  R* QL = quad_out(S, dir, 0, v - 1);
  R* QR = quad_out(S, dir, 1, v - 1);
  if (qt == (R)0.) {
    for (int i = 1; i <= n; ++i) { const R f = L.f(i, v); QL[L.off(i)] = f; QR[L.off(i)] = f; }
    return;
  }
  R* D1 = quad_work(S, dir, v - 1, 0);
  R* D2 = quad_work(S, dir, v - 1, 1);
  R* W = quad_work(S, dir, v - 1, 2);
  const int is = 1, is1 = 2, is2 = 3, ie = n, ie1 = n - 1, ie2 = n - 2;
  auto f = [&](int i) { return L.f(i, v); };
  // slope at the two cells of each end (sonic-A) and the end rows
  R f1i = f(is + 1) - f(is), f1i1 = f(is + 2) - f(is + 1), f1i2 = f(is + 3) - f(is + 2), f1i3 = f(is + 4) - f(is + 3);
  R f2i1 = f1i1 - f1i, f2i2 = f1i2 - f1i1, f2i3 = f1i3 - f1i2;
  R f2i = (R)2. * f2i1 - f2i2;
  R f2mi = ammd(f2i, f2i1), f2mi1 = ammd(f2i1, f2i2), f2mi2 = ammd(f2i2, f2i3);
  const R d1s = ammd(f1i - (R)0.5 * f2mi, (R)2. * f1i);
  const R d1s1 = quad_sonic(f1i1 - (R)0.5 * f2mi1, f1i + (R)0.5 * f2mi, ammd(f1i1, f1i));
  const R slopes2 = quad_sonic(f1i2 - (R)0.5 * f2mi2, f1i1 + (R)0.5 * f2mi1, ammd(f1i2, f1i1));
  R rs = (R)0.75 * (f(is2 + 1) - f(is2 - 1));
  rs = rs - (R)0.25 * d1s1;
  f1i1 = f(ie) - f(ie - 1); f1i2 = f(ie - 1) - f(ie - 2); f1i3 = f(ie - 2) - f(ie - 3);
  const R f1i4 = f(ie - 3) - f(ie - 4);
  f2i1 = f1i1 - f1i2; f2i2 = f1i2 - f1i3; f2i3 = f1i3 - f1i4;
  f2i = (R)2. * f2i1 - f2i2;
  f2mi1 = ammd(f2i1, f2i); f2mi2 = ammd(f2i2, f2i1);
  const R f2mi3 = ammd(f2i3, f2i2);
  const R d1e = ammd(f1i1 + (R)0.5 * f2mi1, (R)2. * f1i1);
  const R d1e1 = quad_sonic(f1i1 - (R)0.5 * f2mi1, f1i2 + (R)0.5 * f2mi2, ammd(f1i1, f1i2));
  const R slopee2 = quad_sonic(f1i2 - (R)0.5 * f2mi2, f1i3 + (R)0.5 * f2mi3, ammd(f1i2, f1i3));
  R re = (R)0.75 * (f(ie2 + 1) - f(ie2 - 1));
  re = re - (R)0.25 * d1e1;
  D1[L.off(is)] = d1s; D1[L.off(is1)] = d1s1; D1[L.off(ie1)] = d1e1; D1[L.off(ie)] = d1e;
  quad_tridag(L, D1, W, is2, ie2, (R)(1. / 3.), (R)0.25, rs, re, [&](int i) { return quad_rhs(L, v, i, false); });
  // curvature (zero at the two cells of each end)
  R cs = (R)1.2 * (f(is2 + 1) - (R)2. * f(is2) + f(is2 - 1));
  cs = cs - (R)0.1 * (R)0.;
  R ce = (R)1.2 * (f(ie2 + 1) - (R)2. * f(ie2) + f(ie2 - 1));
  ce = ce - (R)0.1 * (R)0.;
  D2[L.off(is)] = (R)0.; D2[L.off(is1)] = (R)0.; D2[L.off(ie1)] = (R)0.; D2[L.off(ie)] = (R)0.;
  quad_tridag(L, D2, W, is2, ie2, (R)(2. / 11.), (R)0.1, cs, ce, [&](int i) { return quad_rhs(L, v, i, true); });
  // signs of the slope and the curvature
  R cm = (R)0.;
  for (int i = is2; i <= ie2; ++i) {
    const R fm2 = f(i - 2), fm1 = f(i - 1), f0 = f(i), fp1 = f(i + 1), fp2 = f(i + 2);
    const R sf = (-fp2 + (R)4. * fp1 - (R)3. * f0) / (R)2.;
    const R sc = (fp1 - fm1) / (R)2.;
    const R sb = (fm2 - (R)4. * fm1 + (R)3. * f0) / (R)2.;
    const R sm = quad_median(sf, sc, sb);
    if (sm == sf) cm = fp2 - (R)2. * fp1 + f0;
    if (sm == sc) cm = fp1 - (R)2. * f0 + fm1;
    if (sm == sb) cm = f0 - (R)2. * fm1 + fm2;
    const int64_t o = L.off(i);
    const R d1 = quad_median(D1[o], sm, sc);
    D1[o] = d1;
    if (d1 == sm) D2[o] = cm;
    if (d1 == sc) D2[o] = fp1 - (R)2. * f0 + fm1;
  }
  // monotonicity-preserving constraint (quad's "method 2") and the
  // quadratic's face values
  for (int i = is2; i <= ie2; ++i) {
    const int64_t o = L.off(i);
    const R f0 = f(i);
    const R s1i = f0 - f(i - 1), s1p = f(i + 1) - f0;
    const R d1 = D1[o], d1m = D1[L.off(i - 1)], d1p = D1[L.off(i + 1)], d2 = D2[o];
    R si = d1, ci = d2, sr, cr, sl, cl;
    const R ad = fabs(d1);
    if (ad > (R)2.0 * fabs(s1p) && ad > (R)2.0 * fabs(s1i)) {
      if (ad <= fabs(d1p)) { sr = d1; cr = (R)2. * (s1p - d1); }
      else { sr = (R)2. * s1p - d1p; cr = (R)2. * (-s1p + d1p); }
      if (ad <= fabs(d1m)) { sl = d1; cl = (R)2. * (-s1i + d1); }
      else { sl = (R)2. * s1i - d1m; cl = (R)2. * (s1i - d1m); }
      si = ammd(sl, sr);
      ci = ammd(cl, cr);
    } else {
      if (ad > (R)2.0 * fabs(s1p)) {
        if (ad <= fabs(d1p)) { sr = d1; cr = (R)2. * (s1p - d1); }
        else { sr = (R)2. * s1p - d1p; cr = (R)2. * (-s1p + d1p); }
        si = ammd(d1, sr);
        ci = ammd(d2, cr);
      }
      if (ad > (R)2.0 * fabs(s1i)) {
        if (ad <= fabs(d1m)) { sl = d1; cl = (R)2. * (-s1i + d1); }
        else { sl = (R)2. * s1i - d1m; cl = (R)2. * (s1i - d1m); }
        si = ammd(sl, d1);
        ci = ammd(cl, d2);
      }
    }
    QL[o] = f0 + (R)0.5 * si + ci / (R)12.;
    QR[o] = f0 - (R)0.5 * si + ci / (R)12.;
  }
  // the end cells from their sonic-A slopes, and quad's consistency of the
  // third cell from each end with them
  const int ends[4] = {is, is1, ie1, ie};
  const R dend[4] = {d1s, d1s1, d1e1, d1e};
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int64_t o = L.off(ends[e]);
    const R f0 = f(ends[e]);
    QL[o] = f0 + (R)0.5 * dend[e];
    QR[o] = f0 - (R)0.5 * dend[e];
  }
  QR[L.off(is2)] = f(is2) - (R)0.5 * slopes2;
  QL[L.off(ie2)] = f(ie2) + (R)0.5 * slopee2;
}

// One thread per (direction, line, variable) of a slice (grid.y = slice):
// the xi lines k = kbeg..kend (cells j = 1..jd) and the eta lines j =
// jbeg..jend (cells k = 1..kd) rhsup reconstructs; consecutive threads take
// consecutive lines.
template <class R>
__global__ void __launch_bounds__(128) k_quad(const Slice<R>* __restrict__ sl) {
  const Slice<R>& S = sl[blockIdx.y];
  if (S.lim != 2 || !S.quad) return;
  const ot2d_params& p = *S.P;
  const int jd = S.jd, kd = S.kd;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nx = 4 * kd;
  if (t >= nx + 4 * jd) return;
  const int dir = t < nx ? 0 : 1;
  const int r = dir == 0 ? t : t - nx;
  const int nl = dir == 0 ? kd : jd;
  const int v = r / nl + 1, line = r % nl + 1;
  if (dir == 0 ? (line < p.kbeg || line > p.kend) : (line < p.jbeg || line > p.jend)) return;
  const LineRd<R> L{S.q, S.qs, jd, p.nq, line, dir, S.k_gm1, S.iblank};
  quad_line(S, L, dir, v, dir == 0 ? jd : kd, S.k_qt);
}

}  // namespace ot2d
