// k_sa.cuh -- Spalart-Allmaras solve vmu_sa (src/samodel2d.f:2-1385,
// constants src/sadata.h:2-4).  The reference scatters Jacobian-band
// contributions from each cell into its neighbours; here every interior cell
// gathers its own band entries from the neighbours' values, adding them in
// the reference's order, so each band entry carries the same bits.
#pragma once
#include "dev_common.cuh"

namespace ot2d {

// sadata.h:2-4 (decimal literals are doubles under -r8)
struct SAc {
  static constexpr double cb1 = 0.1355, sigma = 0.6666667, cb2 = 0.622, akt = 0.41, cw1 = 3.2390678;
  static constexpr double cw2 = 0.3, cw3 = 2., cv1 = 7.1, ct3 = 1.2, ct4 = 0.5;
};

// The transcendental terms of the SA source (samodel2d.f:767-778): libm's
// pow in the FP64 path, as the reference; in the f32 path the hardware
// exp2 / log2 form (a few ulp) and r**5. as products.  (The transition
// term's exponential multiplies fturf = 0 and is not evaluated.)
// x**y for x > 0
template <class R> __device__ __forceinline__ R sa_pow_pos(R x, R y) {
  if constexpr (sizeof(R) == sizeof(float)) return __powf(x, y);
  else return pow(x, y);
}
template <class R> __device__ __forceinline__ R sa_pow5(R x) {
  if constexpr (sizeof(R) == sizeof(float)) { const R x2 = x * x; return (x2 * x2) * x; }
  else return pow(x, (R)5.);
}

// scratch arrays of one slice (stride S.wstride)
enum SAw { W_VMUL = 0, W_U, W_V, W_SJ, W_AJ, W_CJ, W_AK, W_CK, W_BJ, W_NSA };

// lamvis (samodel2d.f:200-240) and the u,v of samodel2d.f:74-76, all cells
template <class R>
__device__ __forceinline__ void sa_prep_cell(const Slice<R>& S, const ot2d_params& p, int j, int k) {
  const int64_t o = at(S.jd, j, k), qs = S.qs, ws = S.wstride;
  const R c2b = S.k_c2b, c2bp = S.k_c2bp;
  R q1 = S.q[o], q2 = S.q[qs + o], q3 = S.q[2 * qs + o], q4 = S.q[3 * qs + o];
  R ra = (R)1. / q1;
  R uvel = q2 * ra, vvel = q3 * ra;
  R ei = q4 * ra - (R)0.5 * (sq(uvel) + sq(vvel));
  R tt = S.k_ggm1 * ei;
  S.w[W_VMUL * ws + o] = c2bp * tt * sqrt(tt) / (c2b + tt);
  S.w[W_U * ws + o] = q2 / q1;
  S.w[W_V * ws + o] = q3 / q1;
}

template <class R>
struct SAnb {  // convec upwind split at one cell (samodel2d.f:477-484)
  R up, um, vp, vm;
};
template <class R>
__device__ __forceinline__ SAnb<R> sa_split_of(R u, R v, R ugc, R vgc, R xx, R xy, R yx, R yy) {
  R uu = xx * (u - ugc) + xy * (v - vgc);
  R vv = yx * (u - ugc) + yy * (v - vgc);
  SAnb<R> r;
  r.up = (R)0.5 * (uu + fabs(uu)); r.um = (R)0.5 * (uu - fabs(uu));
  r.vp = (R)0.5 * (vv + fabs(vv)); r.vm = (R)0.5 * (vv - fabs(vv));
  return r;
}

// The values sa_rhs_cell reads at a cell and its four neighbours, staged
// for a tile of cells in shared memory (k_sa_rhs): the velocities of
// sa_prep, the grid speeds (zero on a fixed grid), the metrics, nu_tilde
// and the laminar kinematic viscosity vmul/q1/J.
enum SAst { SA_U = 0, SA_V, SA_XX, SA_XY, SA_YX, SA_YY, SA_Q5, SA_NUL, SA_UG, SA_VG, SA_NST };
template <class R>
struct SaTile {
  const R* sm; int nr, rw, jr, kr; bool gs;   // region origin (jr, kr); gs: grid speeds staged
  __device__ __forceinline__ R g(int a, int j, int k) const { return sm[a * nr + (k - kr) * rw + (j - jr)]; }
  __device__ __forceinline__ R u(int j, int k) const { return g(SA_U, j, k); }
  __device__ __forceinline__ R v(int j, int k) const { return g(SA_V, j, k); }
  __device__ __forceinline__ R xx(int j, int k) const { return g(SA_XX, j, k); }
  __device__ __forceinline__ R xy(int j, int k) const { return g(SA_XY, j, k); }
  __device__ __forceinline__ R yx(int j, int k) const { return g(SA_YX, j, k); }
  __device__ __forceinline__ R yy(int j, int k) const { return g(SA_YY, j, k); }
  __device__ __forceinline__ R q5(int j, int k) const { return g(SA_Q5, j, k); }
  __device__ __forceinline__ R nul(int j, int k) const { return g(SA_NUL, j, k); }
  __device__ __forceinline__ SAnb<R> split(int j, int k) const {
    return sa_split_of(u(j, k), v(j, k), gs ? g(SA_UG, j, k) : (R)0, gs ? g(SA_VG, j, k) : (R)0, xx(j, k), xy(j, k),
                       yx(j, k), yy(j, k));
  }
};

// RHS and bands of one interior cell: rhslhs (samodel2d.f:402-450) with
// convec (:453-542), diffus (:545-688), source (:691-824), then the time
// scaling of vmu_sa (:96-134).  Writes sjmat, aj, cj, ak, ck, bjmat.
template <class R, class A>
__device__ void sa_rhs_cell(const Slice<R>& S, const ot2d_params& p, int j, int k, bool bodyflag,
                            const A& a) {
  const int jd = S.jd; const int64_t qs = S.qs, ws = S.wstride;
  const int n5 = p.nmv + 1, nq = p.nq;
  const int js = p.jbeg, je = p.jend, ks = p.kbeg, ke = p.kend;
  auto Q = [&](int jj, int kk, int n) { return S.q[(int64_t)(n - 1) * qs + at(jd, jj, kk)]; };
  const int64_t o = at(jd, j, k);
  const R rey = S.k_rey;
  // ---- convec
  SAnb<R> c0 = a.split(j, k), cjm = a.split(j - 1, k), cjp = a.split(j + 1, k);
  SAnb<R> ckm = a.split(j, k - 1), ckp = a.split(j, k + 1);
  R q5 = a.q5(j, k);
  R sj = S.s[(int64_t)(n5 - 1) * qs + o];
  sj = sj - c0.up * (q5 - a.q5(j - 1, k)) - c0.um * (a.q5(j + 1, k) - q5);
  sj = sj - c0.vp * (q5 - a.q5(j, k - 1)) - c0.vm * (a.q5(j, k + 1) - q5);
  R aj = (R)0., cj = (R)0., ak = (R)0., ck = (R)0.;
  if (j >= js + 1) aj = aj - ((c0.up > (R)1.0e-12) ? (R)1.0 : (R)0.0) * (cjm.up + cjm.um);
  if (j <= je - 1) cj = cj + ((c0.um < (R)-1.0e-12) ? (R)1.0 : (R)0.0) * (cjp.up + cjp.um);
  R bj = (R)0. + c0.up - c0.um;
  if (k >= ks + 1) ak = ak - ((c0.vp > (R)1.0e-12) ? (R)1.0 : (R)0.0) * (ckm.vp + ckm.vm);
  if (k <= ke - 1) ck = ck + ((c0.vm < (R)-1.0e-12) ? (R)1.0 : (R)0.0) * (ckp.vp + ckp.vm);
  R bk = (R)0. + c0.vp - c0.vm;
  // ---- diffus
  const R chpc = (R)((1. + SAc::cb2) / SAc::sigma) / rey;
  const R c2c = (R)(SAc::cb2 / SAc::sigma) / rey;
  auto nul = [&](int jj, int kk) { return a.nul(jj, kk); };
  {
    // half points j-1/2 (index j-1) and j+1/2 (index j)
    R dmxh_m = (R)0.5 * (a.xx(j - 1, k) + a.xx(j, k)), dmyh_m = (R)0.5 * (a.xy(j - 1, k) + a.xy(j, k));
    R dmxh_p = (R)0.5 * (a.xx(j, k) + a.xx(j + 1, k)), dmyh_p = (R)0.5 * (a.xy(j, k) + a.xy(j + 1, k));
    R n0 = nul(j, k), nm = nul(j - 1, k), np = nul(j + 1, k);
    R chp_m = chpc * ((R)0.5 * (nm + n0) + (R)0.5 * (a.q5(j - 1, k) + q5));
    R chp_p = chpc * ((R)0.5 * (n0 + np) + (R)0.5 * (q5 + a.q5(j + 1, k)));
    R dn_m = q5 - a.q5(j - 1, k), dn_p = a.q5(j + 1, k) - q5;
    R dxp = dmxh_p * a.xx(j, k) + dmyh_p * a.xy(j, k);
    R dxm = dmxh_m * a.xx(j, k) + dmyh_m * a.xy(j, k);
    R c2 = c2c * (n0 + q5);
    R dcp = dxp * (chp_p - c2), dcm = dxm * (chp_m - c2);
    R ax = fmax2(dcm, (R)0.0), cx = fmax2(dcp, (R)0.0);
    sj = sj - ax * dn_m + cx * dn_p;
    aj = aj - ax; cj = cj - cx; bj = bj + ax + cx;
  }
  {
    R dmxh_m = (R)0.5 * (a.yx(j, k - 1) + a.yx(j, k)), dmyh_m = (R)0.5 * (a.yy(j, k - 1) + a.yy(j, k));
    R dmxh_p = (R)0.5 * (a.yx(j, k) + a.yx(j, k + 1)), dmyh_p = (R)0.5 * (a.yy(j, k) + a.yy(j, k + 1));
    R n0 = nul(j, k), nm = nul(j, k - 1), np = nul(j, k + 1);
    R chp_m = chpc * ((R)0.5 * (nm + n0) + (R)0.5 * (a.q5(j, k - 1) + q5));
    R chp_p = chpc * ((R)0.5 * (n0 + np) + (R)0.5 * (q5 + a.q5(j, k + 1)));
    R dn_m = q5 - a.q5(j, k - 1), dn_p = a.q5(j, k + 1) - q5;
    R dyp = dmxh_p * a.yx(j, k) + dmyh_p * a.yy(j, k);
    R dym = dmxh_m * a.yx(j, k) + dmyh_m * a.yy(j, k);
    R c2 = c2c * (n0 + q5);
    R dcp = dyp * (chp_p - c2), dcm = dym * (chp_m - c2);
    R ay = fmax2(dcm, (R)0.0), cy = fmax2(dcp, (R)0.0);
    sj = sj - ay * dn_m + cy * dn_p;
    ak = ak - ay; ck = ck - cy; bk = bk + ay + cy;
  }
  // ---- source (isour = 0, fturf = 0, no transition)
  {
    const R cb1 = (R)SAc::cb1, akt = (R)SAc::akt, cw1 = (R)SAc::cw1, cw2 = (R)SAc::cw2, cw3 = (R)SAc::cw3;
    const R cv1 = (R)SAc::cv1, ct3 = (R)SAc::ct3, ct4 = (R)SAc::ct4;
    const R d2min = (R)1.e-12, rmax = (R)10.0, stilim = (R)1.e-12, fturf = (R)0.0;
    R vort = (R)0.0, d = (R)1.e10;
    if (bodyflag) {
      const R dx2 = (R)0.5, dy2 = (R)0.5;
      R ux = (a.u(j + 1, k) - a.u(j - 1, k)) * dx2, vx = (a.v(j + 1, k) - a.v(j - 1, k)) * dx2;
      R uy = (a.u(j, k + 1) - a.u(j, k - 1)) * dy2, vy = (a.v(j, k + 1) - a.v(j, k - 1)) * dy2;
      R tx = a.xy(j, k) * ux - a.xx(j, k) * vx + a.yy(j, k) * uy - a.yx(j, k) * vy;
      vort = fabs(tx);
      d = S.sn[o];
    }
    R vnul = a.nul(j, k);
    R chi = q5 / vnul;
    chi = fmax2(chi, (R)1.e-12);
    R fv1 = (cube(chi)) / (cube(chi) + cube(cv1));
    R fv2 = (R)1. - chi / ((R)1. + chi * fv1);
    R fv3 = (R)1.0;
    // ft2 = fturf * ct3 * exp(-ct4 chi^2) with fturf = 0: +0 exactly (the
    // exponential is finite and positive), so it is not evaluated
    R ft2 = (R)0.0;
    (void)fturf; (void)ct3;
    R dchi = (R)1. / vnul;
    R dfv1 = ((R)3. * cube(cv1)) * (sq(chi)) * dchi * sq((R)1. / (cube(chi) + cube(cv1)));
    R dfv2 = (fv2 - (R)1.) / chi / vnul + ((R)1. - fv2) * ((R)1 - fv2) * (dfv1 + fv1 / chi / vnul);
    R dfv3 = (R)0.0;
    R dft2 = ((R)-2. * ct4) * chi * dchi * ft2;
    R d2 = fmax2(sq(d), d2min);
    R stilda = vort * fv3 + vnul / (d2 * akt * akt * rey) * chi * fv2;
    stilda = fmax2(stilda, stilim);
    R r = q5 / (d2 * akt * akt * rey) / stilda;
    r = fmin2(r, rmax);
    R g = r + cw2 * (pow6(r) - r);
    // ((1 + cw3^6) / (g^6 + cw3^6))^(1/6), which fw and its derivative
    // both take (samodel2d.f:767-778): one power for the two
    const R fw6 = sa_pow_pos(((R)1. + pow6(cw3)) / (pow6(g) + pow6(cw3)), (R)(1. / 6.));
    R fw = g * fw6;
    R dstild = vort * dfv3 + vnul * (dchi * fv2 + chi * dfv2) / (d2 * akt * akt * rey);
    R dr = vnul * (dchi - chi * dstild / stilda) / stilda / (d2 * akt * akt * rey);
    R dg = dr * ((R)1. + cw2 * ((R)6. * sa_pow5(r) - (R)1.));
    R dfw = fw6;
    dfw = dfw * dg * ((R)1. - pow6(g) / (pow6(g) + pow6(cw3)));
    R pro = cb1 * stilda * ((R)1. - ft2);
    R des = (cw1 * fw - cb1 / (akt * akt) * ft2) / d2 / rey;
    R prod = cb1 * stilda * ((R)1. - ft2) * q5;
    R dest = (cw1 * fw - cb1 / (akt * akt) * ft2) * q5 * q5 / d2 / rey;
    R dpro = pro * dstild / stilda - cb1 * stilda * dft2;
    R ddes = (cw1 * dfw - cb1 / (akt * akt) * dft2) / d2 / rey * vnul * chi;
    ddes = ddes + des;
    ddes = ddes * q5;
    dpro = dpro * q5;
    sj = sj + prod - dest;
    R tk1 = fmax2(des * q5 - pro, (R)0.0);
    R tk2 = fmax2(ddes - dpro, (R)0.0);
    bk = bk + tk1 + tk2;
  }
  // ---- time scaling (vmu_sa, samodel2d.f:104-134)
  R tscal = S.tscale[o];
  int ibi = S.iblank[o];
  if (p.cfltur > 1 && p.idual_turb == 1) {
    R dtp = S.k_cfltur / (bj + bk);
    tscal = dtp * (R)ibi;
    tscal = tscal / ((R)1. + tscal / S.k_h);
  }
  if (p.timeac == 1) {
    R ib = (R)(ibi > 0 ? ibi : 0);
    R J = Q(j, k, nq);
    tscal = ib * ((R)1.0 + (R)0.002 * sqrt(J)) / ((R)1. + sqrt(J));
    tscal = tscal * (R)1.0;
    tscal = tscal / ((R)1. + tscal / S.k_h);
  }
  S.w[W_SJ * ws + o] = sj * tscal;
  S.w[W_AJ * ws + o] = aj * tscal;
  S.w[W_CJ * ws + o] = cj * tscal;
  S.w[W_AK * ws + o] = ak * tscal;
  S.w[W_CK * ws + o] = ck * tscal;
  S.w[W_BJ * ws + o] = (R)1. + (bj + bk) * tscal;
}

// lsolvej (samodel2d.f:1306-1344) on one k-line, then s1 = x,
// sjmat = (s1 - s2)*bjmat with s2 = 0 (samodel2d.f:150-153)
template <class R>
__device__ void sa_lsolvej_line(const Slice<R>& S, const ot2d_params& p, int k) {
  const int jd = S.jd; const int64_t ws = S.wstride;
  R* a = S.w + W_AJ * ws; R* c = S.w + W_CJ * ws; R* s = S.w + W_SJ * ws; const R* b = S.w + W_BJ * ws;
  const int js = p.jbeg, je = p.jend;
  int64_t o = at(jd, js, k);
  R bb = (R)1. / b[o];
  R sp = s[o] * bb, cp = c[o] * bb;
  s[o] = sp; c[o] = cp;
  for (int j = js + 1; j <= je; ++j) {
    o = at(jd, j, k);
    bb = (R)1. / (b[o] - a[o] * cp);
    sp = (s[o] - a[o] * sp) * bb;
    cp = c[o] * bb;
    s[o] = sp; c[o] = cp;
  }
  R snext = sp;
  s[o] = ((snext + (R)0.) - (R)0.) * b[o];
  for (int j = je - 1; j >= js; --j) {
    o = at(jd, j, k);
    R x = s[o] - c[o] * snext;
    snext = x;
    s[o] = ((x + (R)0.) - (R)0.) * b[o];
  }
}

// lsolvej for 32 consecutive k-lines by a CTA of two warps.  The lines run
// along j, the fast index of the arrays, so 32 x 32 tiles are staged
// through shared memory (one row of a tile per copy, then one line per
// lane).  Warp 0 eliminates: lane l walks line kline0+l through the tile
// with the arithmetic of sa_lsolvej_line, in its order, and reads and
// writes only shared memory.  Warp 1 moves the data through three buffers:
// while warp 0 works on tile t it stores the results of tile t-1 and
// fetches tile t+2 (cp.async) into that buffer, so the recurrence neither
// waits on global memory nor spends its issue slots on copies.  The two
// warps meet at one named barrier per tile.
// smem: LJ_SMEM elements of R.
constexpr int LJ_TILE = 32 * 33;
constexpr int LJ_NBUF = 3;
constexpr int LJ_SMEM = LJ_NBUF * 4 * LJ_TILE;
constexpr int LJ_THREADS = 64;

template <class R>
__device__ __forceinline__ void lj_cp_async(R* dst, const R* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src), "n"((int)sizeof(R)));
}
__device__ __forceinline__ void lj_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void lj_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }
// the two warps of the CTA meet (named barrier 1, 64 threads)
__device__ __forceinline__ void lj_meet() { asm volatile("bar.sync 1, 64;" ::: "memory"); }

// The bands are the scratch slots sa, sb, sc, ss.  SAOUT: the result is
// ((x + 0) - 0) * b as vmu_sa forms it (samodel2d.f:150-153); otherwise
// x * b as komegasst does (komegasst.f:134-139).
template <class R, bool SAOUT = true>
__device__ void sa_lsolvej_group(const Slice<R>& S, const ot2d_params& p, int kline0, R* sm, int sa = W_AJ,
                                 int sb = W_BJ, int sc = W_CJ, int ss = W_SJ) {
  const int lane = threadIdx.x & 31;
  const bool mover = (threadIdx.x >> 5) == 1;
  const int jd = S.jd; const int64_t ws = S.wstride;
  const R* ga = S.w + sa * ws; R* gc = S.w + sc * ws; R* gs = S.w + ss * ws; const R* gb = S.w + sb * ws;
  const int js = p.jbeg, je = p.jend, ks = p.kbeg, ke = p.kend;
  const int ntile = (je - js + 1 + 31) / 32;
  const bool mine = ks + kline0 + lane <= ke;
  // buffer b of array m: sm + (b*4 + m)*LJ_TILE; element (row r, column c) at r*33 + c
  auto buf = [&](int b, int m) { return sm + (b * 4 + m) * LJ_TILE; };
  // mover: issue the copies of tile t (columns j0..j0+31) of {a,} b, c, s
  // into buffer b as one cp.async group.  Each lane copies column lane of
  // every row, the same elements it stores below.
  auto fetch = [&](int t, int b, bool fwd) {
    const int j = js + 32 * t + lane;
    for (int r = 0; r < 32; ++r) {
      const int kr = ks + kline0 + r;
      if (kr <= ke && j <= je) {
        const int64_t o = at(jd, j, kr);
        if (fwd) lj_cp_async(buf(b, 0) + r * 33 + lane, ga + o);
        lj_cp_async(buf(b, 1) + r * 33 + lane, gb + o);
        lj_cp_async(buf(b, 2) + r * 33 + lane, gc + o);
        lj_cp_async(buf(b, 3) + r * 33 + lane, gs + o);
      }
    }
    lj_commit();
  };
  // mover: store tile t's results from buffer b (forward: c and s; backward: s)
  auto store = [&](int t, int b, bool fwd) {
    const int j = js + 32 * t + lane;
    const R *Cm = buf(b, 2), *Sm = buf(b, 3);
    for (int r = 0; r < 32; ++r) {
      const int kr = ks + kline0 + r;
      if (kr <= ke && j <= je) {
        const int64_t o = at(jd, j, kr);
        if (fwd) gc[o] = Cm[r * 33 + lane];
        gs[o] = Sm[r * 33 + lane];
      }
    }
  };
  // ---- forward elimination.  Round t: warp 0 eliminates tile t (buffer
  // t%3); warp 1 stores tile t-1 and then fetches tile t+2 into the buffer
  // tile t-1 used (the stores read it before the copies overwrite it), and
  // waits for tile t+1.
  R cp = (R)0, sp = (R)0;
  if (mover) {
    fetch(0, 0, true);
    if (ntile > 1) { fetch(1, 1, true); lj_wait<1>(); }
    else lj_wait<0>();
  }
  lj_meet();
  for (int t = 0; t < ntile; ++t) {
    const int b = t % LJ_NBUF;
    if (!mover) {
      if (mine) {
        const R *A = buf(b, 0), *B = buf(b, 1);
        R *Cm = buf(b, 2), *Sm = buf(b, 3);
        const int j0 = js + 32 * t;
        for (int jj = 0; jj < 32 && j0 + jj <= je; ++jj) {
          const int i = lane * 33 + jj;
          R bb;
          if (j0 + jj == js) { bb = (R)1. / B[i]; sp = Sm[i] * bb; cp = Cm[i] * bb; }
          else { bb = (R)1. / (B[i] - A[i] * cp); sp = (Sm[i] - A[i] * sp) * bb; cp = Cm[i] * bb; }
          Sm[i] = sp; Cm[i] = cp;
        }
      }
    } else {
      const int bf = (t + 2) % LJ_NBUF;   // = (t - 1) % 3
      if (t >= 1) store(t - 1, bf, true);
      __syncwarp();
      if (t + 2 < ntile) { fetch(t + 2, bf, true); lj_wait<1>(); }
      else lj_wait<0>();
    }
    lj_meet();
  }
  // ---- back substitution; output x * bjmat (samodel2d.f:150-153).  Round
  // n (tile t = ntile-1-n, buffer n%3): warp 1 stores tile t+1 and fetches
  // tile t-2.
  if (mover) {
    store(ntile - 1, (ntile - 1) % LJ_NBUF, true);
    // the stores are read back below by the same lanes (same element ->
    // lane mapping); order them before the asynchronous copies
    __threadfence_block();
    fetch(ntile - 1, 0, false);
    if (ntile > 1) { fetch(ntile - 2, 1, false); lj_wait<1>(); }
    else lj_wait<0>();
  }
  lj_meet();
  R snext = sp;
  for (int t = ntile - 1, n = 0; t >= 0; --t, ++n) {
    const int b = n % LJ_NBUF;
    if (!mover) {
      if (mine) {
        const R *B = buf(b, 1), *Cm = buf(b, 2);
        R* Sm = buf(b, 3);
        const int j0 = js + 32 * t;
        const int jjmax = (je - j0 < 31) ? je - j0 : 31;
        for (int jj = jjmax; jj >= 0; --jj) {
          const int i = lane * 33 + jj;
          R x = (j0 + jj == je) ? Sm[i] : Sm[i] - Cm[i] * snext;
          snext = x;
          if constexpr (SAOUT) Sm[i] = ((x + (R)0.) - (R)0.) * B[i];
          else Sm[i] = x * B[i];
        }
      }
    } else {
      const int bf = (n + 2) % LJ_NBUF;   // = (n - 1) % 3
      if (n >= 1) store(t + 1, bf, false);
      __syncwarp();
      if (t - 2 >= 0) { fetch(t - 2, bf, false); lj_wait<1>(); }
      else lj_wait<0>();
    }
    lj_meet();
  }
  if (mover) store(0, (ntile - 1) % LJ_NBUF, false);
}

// lsolvek (samodel2d.f:1347-1385) on one j-line, then s2 = x and the
// update q5 = max(q5 + x*max(iblank,0), 1e-20) (samodel2d.f:184-188) in FP64
// and c_turm of the cell (samodel2d.f:193; the second turbc only changes
// halo cells, so mu_t here equals the reference's).  The line is walked in
// chunks of LK_U cells whose loads are issued one chunk ahead, before the
// stores of the current chunk, so the recurrence does not wait on memory.
template <class R>
__device__ void sa_lsolvek_line(const Slice<R>& S, const ot2d_params& p, int j) {
  constexpr int LK_U = sizeof(R) == 4 ? 8 : 4;
  const int jd = S.jd; const int64_t ws = S.wstride, qs = S.qs;
  R* a = S.w + W_AK * ws; R* c = S.w + W_CK * ws; R* s = S.w + W_SJ * ws; const R* b = S.w + W_BJ * ws;
  const R* vmul = S.w + W_VMUL * ws;
  const int ks = p.kbeg, ke = p.kend, n5 = p.nmv + 1;
  const R cv1 = (R)SAc::cv1;
  int64_t o = at(jd, j, ks);
  R bb = (R)1. / b[o];
  R sp = s[o] * bb, cp = c[o] * bb;
  s[o] = sp; c[o] = cp;
  // forward elimination
  {
    R na[LK_U], nb[LK_U], nc[LK_U], ns[LK_U];
    auto load = [&](int k0) {
#pragma unroll
      for (int u = 0; u < LK_U; ++u)
        if (k0 + u <= ke) { const int64_t ou = at(jd, j, k0 + u); na[u] = a[ou]; nb[u] = b[ou]; nc[u] = c[ou]; ns[u] = s[ou]; }
    };
    load(ks + 1);
    for (int k0 = ks + 1; k0 <= ke; k0 += LK_U) {
      R ra[LK_U], rb[LK_U], rc[LK_U], rs[LK_U];
#pragma unroll
      for (int u = 0; u < LK_U; ++u) { ra[u] = na[u]; rb[u] = nb[u]; rc[u] = nc[u]; rs[u] = ns[u]; }
      if (k0 + LK_U <= ke) load(k0 + LK_U);
#pragma unroll
      for (int u = 0; u < LK_U; ++u) {
        if (k0 + u <= ke) {
          o = at(jd, j, k0 + u);
          bb = (R)1. / (rb[u] - ra[u] * cp);
          sp = (rs[u] - ra[u] * sp) * bb;
          cp = rc[u] * bb;
          s[o] = sp; c[o] = cp;
        }
      }
    }
  }
  // back substitution + update + mu_t
  double* q5 = S.q64 + (int64_t)(n5 - 1) * qs;
  R nc[LK_U], ns[LK_U], nq1[LK_U], nJ[LK_U], nvm[LK_U];
  double nq5[LK_U];
  int nib[LK_U];
  auto load = [&](int k0) {  // cells k0, k0-1, ..., k0-LK_U+1
#pragma unroll
    for (int u = 0; u < LK_U; ++u)
      if (k0 - u >= ks) {
        const int64_t ou = at(jd, j, k0 - u);
        nc[u] = c[ou]; ns[u] = s[ou]; nq1[u] = S.q[ou]; nJ[u] = S.q[(int64_t)(p.nq - 1) * qs + ou];
        nvm[u] = vmul[ou]; nq5[u] = q5[ou]; nib[u] = S.iblank[ou];
      }
  };
  auto upd = [&](int64_t oo, R x, double q5o, int ibi, R q1, R J, R vm) {
    R x2 = (R)0. + x;            // s2 = s2 + sjmat, s2 = 0 on entry
    R relx = (R)1.0 * x2;        // relfac * sjmat
    s[oo] = relx;
    double v;
    R qv;
    if constexpr (sizeof(R) == sizeof(double)) {
      double ib = (double)(ibi > 0 ? ibi : 0);
      v = q5o + (double)relx * ib;
      v = (1.0e-20 > v) ? 1.0e-20 : v;
      qv = (R)v;
    } else {
      // The same values with one FP64 operation (GB300's FP64 pipe is
      // narrow): relx * max(iblank, 0) is exact for iblank 0 (a signed zero,
      // or NaN for a non-finite relx) and 1, so it is formed in f32 and
      // widened on the integer pipe; the clamp compares IEEE bit patterns;
      // the narrowing is the f32 path's round-to-nearest with flush to zero.
      double dx;
      if (ibi == 1) dx = f2d_bits_ftz(relx);
      else if (ibi <= 0) dx = f2d_bits_ftz(relx * 0.0f);
      else dx = (double)relx * (double)ibi;
      v = q5o + dx;
      const uint64_t vb = (uint64_t)__double_as_longlong(v), mag = vb & 0x7fffffffffffffffull;
      // 1e-20 > v: v negative (not NaN), or positive below 1e-20
      const bool below = (vb >> 63) ? mag <= 0x7ff0000000000000ull
                                    : vb < (uint64_t)__double_as_longlong(1.0e-20);
      if (below) v = 1.0e-20;
      qv = d2f_bits_rn_ftz(v);
    }
    q5[oo] = v;
    if constexpr (sizeof(R) != sizeof(double)) S.q[(int64_t)(n5 - 1) * qs + oo] = qv;
    // c_turm (samodel2d.f:372-399) with q5 as just stored
    const R rhoJ = q1 * J;
    const R vnul = vm / rhoJ;
    const R chi = qv / vnul;
    const R fv1 = cube(chi) / (cube(chi) + cube(cv1));
    S.turmu[oo] = rhoJ * qv * fv1;
  };
  R snext = sp;
  load(ke);
  for (int k0 = ke; k0 >= ks; k0 -= LK_U) {
    R rc[LK_U], rs[LK_U], rq1[LK_U], rJ[LK_U], rvm[LK_U];
    double rq5[LK_U];
    int rib[LK_U];
#pragma unroll
    for (int u = 0; u < LK_U; ++u) {
      rc[u] = nc[u]; rs[u] = ns[u]; rq1[u] = nq1[u]; rJ[u] = nJ[u]; rvm[u] = nvm[u]; rq5[u] = nq5[u]; rib[u] = nib[u];
    }
    if (k0 - LK_U >= ks) load(k0 - LK_U);
#pragma unroll
    for (int u = 0; u < LK_U; ++u) {
      const int k = k0 - u;
      if (k >= ks) {
        o = at(jd, j, k);
        const R x = (k == ke) ? snext : rs[u] - rc[u] * snext;
        snext = x;
        upd(o, x, rq5[u], rib[u], rq1[u], rJ[u], rvm[u]);
      }
    }
  }
}

// c_turm, samodel2d.f:372-399 (all cells)
template <class R>
__device__ __forceinline__ void sa_turm_cell(const Slice<R>& S, const ot2d_params& p, int j, int k) {
  const int64_t o = at(S.jd, j, k), qs = S.qs, ws = S.wstride;
  const R cv1 = (R)SAc::cv1;
  R rhoJ = S.q[o] * S.q[(p.nq - 1) * qs + o];
  R vnul = S.w[W_VMUL * ws + o] / rhoJ;
  R q5 = S.q[(int64_t)p.nmv * qs + o];
  R chi = q5 / vnul;
  R fv1 = cube(chi) / (cube(chi) + cube(cv1));
  S.turmu[o] = rhoJ * q5 * fv1;
}

}  // namespace ot2d
