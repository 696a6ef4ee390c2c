// k_resid.cuh -- the fused residual: rhsup (src/eulerrhs.f:2-280) +
// visrhs (src/visrhs.f:2-287) + timespectralrhs (src/sources.f:2-27) + the
// L2 / max norms of step.f:58-93, one CTA per tile of TJ x TK interior
// cells, one thread per cell (16x16, 32x8, 8x32 or 32x16: rt_shape_dims,
// chosen per batch).
//
// A tile stages its cells plus a 3-cell halo in shared memory once
// (primitive variables, viscous cell factors, metrics), computes every
// inviscid and viscous face flux of the tile exactly once, and assembles the
// residual in the reference's accumulation order.  Per face and per cell the
// arithmetic is the same as the reference's, so the FP64 path reproduces the
// oracle bit for bit.
#pragma once
#include "dev_common.cuh"
#include "k_rhs.cuh"
#include "k_misc.cuh"
#include "launch.h"

namespace ot2d {

constexpr int RT_BS = 256;   // threads of the 256-cell tiles
// staged per-cell arrays
enum { RS_RHO = 0, RS_U, RS_V, RS_P, RS_E, RS_VNU, RS_GKAP, RS_RJ, RS_UD, RS_VD, RS_ED, RS_XX, RS_XY, RS_YX, RS_YY, RS_N };

// Geometry of a TJ x TK tile (TJ * TK cells, one per thread in the
// assembly): the staged region with its 3-cell halo and the face arrays.
template <int TJ, int TK>
struct RtGeo {
  static constexpr int BS = TJ * TK;                      // threads: one cell each
  static_assert(BS % 32 == 0 && BS <= 1024, "whole warps");
  static constexpr int H = 3;                             // staged halo width
  static constexpr int RW = TJ + 2 * H, RH = TK + 2 * H;  // staged region
  static constexpr int NR = RW * RH;
  static constexpr int NF = 4 * TK * (TJ + 1);            // F: xi faces j0-1..j1, rows k0..k1
  static constexpr int NG = 4 * (TK + 1) * TJ;            // G: eta faces k0-1..k1, columns j0..j1
  static constexpr int VEH = TK + 3, VXW = TJ + 3;
  static constexpr int NVE = 6 * VEH * TJ;                // eta viscous, k0-2..k1+1
  static constexpr int NVX = 6 * TK * VXW;                // xi viscous, j0-2..j1+1
};

// |iblank| of the staged cells is kept as one byte (values above 255 are
// clamped; the reference's blanking values are -1, 0 and 1).  The norm
// partials of the tile reuse the staged region at the end (k_resid).
template <class R, int TJ, int TK>
__host__ __device__ constexpr size_t rt_smem_bytes() {
  using G = RtGeo<TJ, TK>;
  return ((sizeof(R) * ((size_t)RS_N * G::NR + G::NF + G::NG + G::NVE + G::NVX) + G::NR + 15) / 16) * 16;
}

template <class R, int TJ, int TK>
struct RtSmem {
  using G = RtGeo<TJ, TK>;
  static constexpr int RW = G::RW, NR = G::NR;
  R* c;          // [RS_N][NR]
  R *F, *G_, *VE, *VX;
  uint8_t* iba;  // [NR]
  __device__ RtSmem(unsigned char* base) {
    c = (R*)base;
    F = c + (size_t)RS_N * G::NR;
    G_ = F + G::NF;
    VE = G_ + G::NG;
    VX = VE + G::NVE;
    iba = (uint8_t*)(VX + G::NVX);
  }
  __device__ __forceinline__ R& at(int a, int r) const { return c[(size_t)a * G::NR + r]; }
};

// Phase B-D work in warp tasks of 32 items: the inviscid faces (the xi
// faces of the tile's rows, then the eta faces of its columns: one kind,
// since the same reconstruction and flux code serves a line of either
// direction) and the viscous terms (eta, then xi).  Tasks are dealt to the
// warps longest first, each to the least loaded warp, with a face task
// counted as three viscous ones: no warp mixes face and viscous code, and
// the slowest warp carries about the mean load.  code[w] lists warp w's
// tasks, 7 bits each (task + 1), first task in the lowest bits.
template <int TJ, int TK>
struct RtTasks {
  using G = RtGeo<TJ, TK>;
  static constexpr int NW = G::BS / 32;
  static constexpr int FB = TK * (TJ + 1);                    // xi faces
  static constexpr int NF = FB + (TK + 1) * TJ;               // + eta faces
  static constexpr int NFT = (NF + 31) / 32;
  static constexpr int NVT = (G::VEH * TJ + TK * G::VXW + 31) / 32;
  uint64_t code[NW];
  int most;                                                   // most tasks of a warp
};
template <int TJ, int TK>
__host__ __device__ constexpr RtTasks<TJ, TK> rt_tasks() {
  using T = RtTasks<TJ, TK>;
  T s{};
  int load[T::NW] = {}, cnt[T::NW] = {};
  for (int task = 0; task < T::NFT + T::NVT; ++task) {
    int w = 0;
    for (int i = 1; i < T::NW; ++i)
      if (load[i] < load[w]) w = i;
    if (cnt[w] < 9) s.code[w] |= (uint64_t)(task + 1) << (7 * cnt[w]);
    ++cnt[w];
    load[w] += task < T::NFT ? 3 : 1;
  }
  for (int i = 0; i < T::NW; ++i)
    if (cnt[i] > s.most) s.most = cnt[i];
  return s;
}

// Stage A: cell (j,k) of the staged region -> primitive f of rhsup
// (eulerrhs.f:55-61, :71-79), viscous cell factors of visrhs
// (visrhs.f:48-60), the q2/q1-style divided velocities of its cross terms
// (visrhs.f:77-89), metrics and |iblank|.  Split in a load (RtRaw) and a
// convert-and-store so that a thread issues the loads of all its staged
// cells before it waits for the first.
template <class R>
struct RtRaw {
  R q1, q2, q3, q4, J, turm, xx, xy, yx, yy;
  int ib;
};

template <class R>
__device__ __forceinline__ void rt_load_cell(const Slice<R>& S, const ot2d_params& p, int j, int k, bool visc,
                                             RtRaw<R>& a) {
  const int64_t o = at(S.jd, j, k), qs = S.qs;
  a.q1 = S.q[o]; a.q2 = S.q[qs + o]; a.q3 = S.q[2 * qs + o]; a.q4 = S.q[3 * qs + o];
  a.J = S.q[(p.nq - 1) * qs + o];
  if (visc) {
    a.turm = S.turmu[o];
    a.xx = S.xx[o]; a.xy = S.xy[o]; a.yx = S.yx[o]; a.yy = S.yy[o];
  }
  a.ib = S.iblank[o];
}

template <class R, class SM>
__device__ __forceinline__ void rt_store_cell(const Slice<R>& S, const SM& sm, int r, const RtRaw<R>& a,
                                              bool visc) {
  const R q1 = a.q1, q2 = a.q2, q3 = a.q3, q4 = a.q4, J = a.J;
  const R gm1 = S.k_gm1;
  const R rhoi = (R)1.0 / q1;
  sm.at(RS_RHO, r) = q1 * J;
  const R u = q2 * rhoi, v = q3 * rhoi;
  sm.at(RS_U, r) = u;
  sm.at(RS_V, r) = v;
  const R ppp = gm1 * (q4 - (R)0.5 * (sq(q2) + sq(q3)) / q1);
  sm.at(RS_P, r) = ppp * J;
  if (visc) {
    const R c2b = S.k_c2b, c2bp = S.k_c2bp, prtr = S.k_prtr;
    const R e = q4 * rhoi - (R).5 * (sq(u) + sq(v));
    const R tt = S.k_ggm1 * e;
    const R vmue = c2bp * tt * sqrt(tt) / (c2b + tt);
    const R turm = a.turm;
    sm.at(RS_E, r) = e;
    sm.at(RS_VNU, r) = vmue + turm;
    sm.at(RS_GKAP, r) = vmue + prtr * turm;
    sm.at(RS_RJ, r) = (R)1. / J;
    const R ud = q2 / q1, vd = q3 / q1;
    sm.at(RS_UD, r) = ud;
    sm.at(RS_VD, r) = vd;
    sm.at(RS_ED, r) = q4 / q1 - (R).5 * (sq(ud) + sq(vd));
    sm.at(RS_XX, r) = a.xx; sm.at(RS_XY, r) = a.xy; sm.at(RS_YX, r) = a.yx; sm.at(RS_YY, r) = a.yy;
  }
  const int ia = a.ib < 0 ? -a.ib : a.ib;
  sm.iba[r] = (uint8_t)(ia > 255 ? 255 : ia);
}

// A grid line read from the staged region: line position c sits at region
// index o0 + c*stride; positions outside [lo, hi] were not staged (and are
// never read by the reconstruction that uses them).
template <class R, class SM>
struct RtLine {
  const SM* sm; int o0, stride, lo, hi; R gm1;
  // ilim +-2: this direction's quad face states in global memory (ql
  // arrays, then qr; stride qn2); cell c of the line at g0 + c*gs
  const R* qd = nullptr;
  int64_t qn2 = 0, g0 = 0, gs = 0;
  __device__ __forceinline__ R quad_l(int v, int c) const { return qd[v * qn2 + g0 + c * gs]; }
  __device__ __forceinline__ R quad_r(int v, int c) const { return qd[(4 + v) * qn2 + g0 + c * gs]; }
  __device__ __forceinline__ void f4(int c, R* out) const {
    if (c < lo || c > hi) { out[0] = out[1] = out[2] = out[3] = (R)0; return; }
    const int r = o0 + c * stride;
    out[0] = sm->at(RS_RHO, r); out[1] = sm->at(RS_U, r); out[2] = sm->at(RS_V, r); out[3] = sm->at(RS_P, r);
  }
  __device__ __forceinline__ int iba(int c) const { return (c < lo || c > hi) ? 0 : sm->iba[o0 + c * stride]; }
};

// eta-direction viscous quantities at column j, index k (visrhs.f:46-131):
// face k+1/2 (f2, f3, f4) and cell k (f2v, f3v, f4v); r = region index of
// (j,k); the cell above is r + SM::RW, the side neighbours r -+ 1.
template <class R, class SM>
__device__ __forceinline__ void rt_visc_eta(const SM& sm, int r, R gkpr, R dre, R* out) {
  R bv[2][4], uu[2], vv[2], ee[2];
  for (int m = 0; m < 2; ++m) {
    const int rr = r + m * SM::RW;
    const R rj = sm.at(RS_RJ, rr), vnu = sm.at(RS_VNU, rr), gkap = sm.at(RS_GKAP, rr);
    uu[m] = sm.at(RS_U, rr); vv[m] = sm.at(RS_V, rr); ee[m] = sm.at(RS_E, rr);
    const R yx = sm.at(RS_YX, rr), yy = sm.at(RS_YY, rr);
    const R b4 = (sq(yx) + sq(yy)) * rj;
    bv[m][0] = (b4 + sq(yx) / (R)3. * rj) * vnu * dre;
    bv[m][1] = (b4 + sq(yy) / (R)3. * rj) * vnu * dre;
    bv[m][3] = (yx * yy / (R)3. * rj) * vnu * dre;
    bv[m][2] = b4 * gkpr * gkap * dre;
  }
  const int rm = r - 1, rp = r + 1;
  const R vnu = sm.at(RS_VNU, r), gkap = sm.at(RS_GKAP, r);
  const R rjm = sm.at(RS_RJ, rm), rjp = sm.at(RS_RJ, rp);
  const R xxm = sm.at(RS_XX, rm), xym = sm.at(RS_XY, rm), yxm = sm.at(RS_YX, rm), yym = sm.at(RS_YY, rm);
  const R xxp = sm.at(RS_XX, rp), xyp = sm.at(RS_XY, rp), yxp = sm.at(RS_YX, rp), yyp = sm.at(RS_YY, rp);
  R d1 = ((R)(4. / 3.) * xxm * yxm + xym * yym) * rjm;
  d1 = d1 + ((R)(4. / 3.) * xxp * yxp + xyp * yyp) * rjp;
  d1 = vnu * dre * d1;
  R d2 = ((R)(4. / 3.) * xym * yym + xxm * yxm) * rjm;
  d2 = d2 + ((R)(4. / 3.) * xyp * yyp + xxp * yxp) * rjp;
  d2 = vnu * dre * d2;
  R d4 = (xym * yym + xxm * yxm) * rjm;
  d4 = d4 + (xyp * yyp + xxp * yxp) * rjp;
  d4 = d4 * gkpr * gkap * dre;
  R d5 = ((R)(-2. / 3.) * xym * yxm + xxm * yym) * rjm;
  d5 = d5 + ((R)(-2. / 3.) * xyp * yxp + xxp * yyp) * rjp;
  d5 = vnu * dre * d5;
  R d7 = ((R)(-2. / 3.) * xxm * yym + xym * yxm) * rjm;
  d7 = d7 + ((R)(-2. / 3.) * xxp * yyp + xyp * yxp) * rjp;
  d7 = vnu * dre * d7;
  const R b1 = bv[1][0] + bv[0][0], b2 = bv[1][1] + bv[0][1], b5 = bv[1][3] + bv[0][3];
  const R ujp1 = sm.at(RS_UD, rp), ujm1 = sm.at(RS_UD, rm);
  const R duj = (R)0.5 * (ujp1 - ujm1);
  const R vjp1 = sm.at(RS_VD, rp), vjm1 = sm.at(RS_VD, rm);
  const R dvj = (R)0.5 * (vjp1 - vjm1);
  const R dej = (R)0.5 * (sm.at(RS_ED, rp) - sm.at(RS_ED, rm));
  const R t4 = uu[1] * bv[1][0] + uu[0] * bv[0][0];
  const R t5 = vv[1] * bv[1][1] + vv[0] * bv[0][1];
  const R t6 = uu[1] * bv[1][3] + uu[0] * bv[0][3];
  const R t7 = vv[1] * bv[1][3] + vv[0] * bv[0][3];
  const R t8 = bv[1][2] + bv[0][2];
  const R du = uu[1] - uu[0], dv = vv[1] - vv[0], dei = ee[1] - ee[0];
  out[0] = b1 * du + b5 * dv;
  out[1] = b5 * du + b2 * dv;
  out[2] = (t4 + t7) * du + (t5 + t6) * dv + t8 * dei;
  out[3] = d1 * duj + d5 * dvj;
  out[4] = d7 * duj + d2 * dvj;
  R f4v = (R)0.5 * d1 * (R)0.5 * (sq(ujp1) - sq(ujm1));
  f4v = f4v + (R)0.5 * d2 * (R)0.5 * (sq(vjp1) - sq(vjm1));
  f4v = f4v + d5 * (R)0.5 * (ujp1 + ujm1) * dvj;
  f4v = f4v + d7 * (R)0.5 * (vjp1 + vjm1) * duj;
  f4v = f4v + d4 * dej;
  out[5] = f4v;
}

// xi-direction viscous quantities at row k, index j (visrhs.f:166-251):
// face j+1/2 and cell j; the cell to the right is r + 1, the neighbours
// below / above r -+ SM::RW.
template <class R, class SM>
__device__ __forceinline__ void rt_visc_xi(const SM& sm, int r, R gkpr, R dre, R* out) {
  R av[2][4], uu[2], vv[2], ee[2];
  for (int m = 0; m < 2; ++m) {
    const int rr = r + m;
    const R rj = sm.at(RS_RJ, rr), vnu = sm.at(RS_VNU, rr), gkap = sm.at(RS_GKAP, rr);
    uu[m] = sm.at(RS_U, rr); vv[m] = sm.at(RS_V, rr); ee[m] = sm.at(RS_E, rr);
    const R xx = sm.at(RS_XX, rr), xy = sm.at(RS_XY, rr);
    const R a4 = (sq(xx) + sq(xy)) * rj;
    av[m][0] = (a4 + sq(xx) / (R)3. * rj) * vnu * dre;
    av[m][1] = (a4 + sq(xy) / (R)3. * rj) * vnu * dre;
    av[m][3] = (xx * xy / (R)3. * rj) * vnu * dre;
    av[m][2] = a4 * gkpr * gkap * dre;
  }
  const int rm = r - SM::RW, rp = r + SM::RW;
  const R vnu = sm.at(RS_VNU, r), gkap = sm.at(RS_GKAP, r);
  const R rkm = sm.at(RS_RJ, rm), rkp = sm.at(RS_RJ, rp);
  const R xxm = sm.at(RS_XX, rm), xym = sm.at(RS_XY, rm), yxm = sm.at(RS_YX, rm), yym = sm.at(RS_YY, rm);
  const R xxp = sm.at(RS_XX, rp), xyp = sm.at(RS_XY, rp), yxp = sm.at(RS_YX, rp), yyp = sm.at(RS_YY, rp);
  R d1 = ((R)(4. / 3.) * xxm * yxm + xym * yym) * rkm;
  d1 = d1 + ((R)(4. / 3.) * xxp * yxp + xyp * yyp) * rkp;
  d1 = vnu * dre * d1;
  R d2 = ((R)(4. / 3.) * xym * yym + xxm * yxm) * rkm;
  d2 = d2 + ((R)(4. / 3.) * xyp * yyp + xxp * yxp) * rkp;
  d2 = vnu * dre * d2;
  R d4 = (xym * yym + xxm * yxm) * rkm;
  d4 = d4 + (xyp * yyp + xxp * yxp) * rkp;
  d4 = d4 * gkpr * gkap * dre;
  R d5 = ((R)(-2. / 3.) * xym * yxm + xxm * yym) * rkm;
  d5 = d5 + ((R)(-2. / 3.) * xyp * yxp + xxp * yyp) * rkp;
  d5 = vnu * dre * d5;
  R d7 = ((R)(-2. / 3.) * xxm * yym + xym * yxm) * rkm;
  d7 = d7 + ((R)(-2. / 3.) * xxp * yyp + xyp * yxp) * rkp;
  d7 = vnu * dre * d7;
  const R a1 = av[1][0] + av[0][0], a2 = av[1][1] + av[0][1], a5 = av[1][3] + av[0][3];
  const R ukp1 = sm.at(RS_UD, rp), ukm1 = sm.at(RS_UD, rm);
  const R duk = (R)0.5 * (ukp1 - ukm1);
  const R vkp1 = sm.at(RS_VD, rp), vkm1 = sm.at(RS_VD, rm);
  const R dvk = (R)0.5 * (vkp1 - vkm1);
  const R dek = (R)0.5 * (sm.at(RS_ED, rp) - sm.at(RS_ED, rm));
  const R t4 = uu[1] * av[1][0] + uu[0] * av[0][0];
  const R t5 = vv[1] * av[1][1] + vv[0] * av[0][1];
  const R t6 = uu[1] * av[1][3] + uu[0] * av[0][3];
  const R t7 = vv[1] * av[1][3] + vv[0] * av[0][3];
  const R t8 = av[1][2] + av[0][2];
  const R du = uu[1] - uu[0], dv = vv[1] - vv[0], dei = ee[1] - ee[0];
  out[0] = a1 * du + a5 * dv;
  out[1] = a5 * du + a2 * dv;
  out[2] = (t4 + t7) * du + (t5 + t6) * dv + t8 * dei;
  out[3] = d1 * duk + d7 * dvk;
  out[4] = d5 * duk + d2 * dvk;
  R f4v = (R)0.5 * d1 * (R)0.5 * (sq(ukp1) - sq(ukm1));
  f4v = f4v + (R)0.5 * d2 * (R)0.5 * (sq(vkp1) - sq(vkm1));
  f4v = f4v + d5 * (R)0.5 * (vkp1 + vkm1) * duk;
  f4v = f4v + d7 * (R)0.5 * (ukp1 + ukm1) * dvk;
  f4v = f4v + d4 * dek;
  out[5] = f4v;
}

// rhslom (sources.f:97-148) on one interior cell: s(1:4) times Turkel's
// low-Mach preconditioner, (I + gm1 (bSq-1)/a**2 * [u,v,ge]^T
// [phi**2, -u, -v, 1]) s, with bSq = Mp**2/(bt - Mp**2 (bt-1)) of the cell.
template <class R>
__device__ __forceinline__ void rhslom_cell(const Slice<R>& S, const ot2d_params& p, int64_t o, R* s) {
  const int64_t qs = S.qs;
  const R q1 = S.q[o], gm1 = S.k_gm1, gamma = S.k_gamma, mp2 = S.k_mp2;
  const R u = S.q[qs + o] / q1;
  const R v = S.q[2 * qs + o] / q1;
  const R phiSq = (R)0.5 * (u * u + v * v);
  const R ge = S.q[3 * qs + o] / q1 * gamma - phiSq * gm1;
  const R aSq = (S.q[3 * qs + o] / q1 - phiSq) * gm1 * gamma;
  const R t1 = s[0], t2 = s[1], t3 = s[2], t4 = s[3];
  const R a = phiSq * t1 - u * t2 - v * t3 + t4;
  const R btv = S.bt[o];
  const R bSq = mp2 / (btv - mp2 * (btv - (R)1));
  const R f = gm1 * (bSq - (R)1.) / aSq;
  s[0] = a * f + t1;
  s[1] = (u * a) * f + t2;
  s[2] = (v * a) * f + t3;
  s[3] = (ge * a) * f + t4;
}

// One tile of the residual (step.f:41-93 for the cells of the tile): tile
// `tile` of the slice covers interior cells j0..j1 x k0..k1.  flags as for
// the cell-parallel assembly (AS_*).  Without AS_ACC the tile also zeroes s
// on the halo cells next to it (step.f:41 zeroes s everywhere).  np receives
// the thread's norm partial.  PRE: the slice runs with Turkel's low-Mach
// preconditioning -- roetrklflx fluxes, and in the full residual (AS_NORM)
// rhslom applied to each cell after its norm terms (step.f:121-123).
template <class R, bool PRE, int LIM, int TJ, int TK>
__device__ void resid_tile(const Slice<R>& S, const RtSmem<R, TJ, TK>& sm, int tile, int flags,
                           NormPartR<R>& np) {
  using G = RtGeo<TJ, TK>;
  using SM = RtSmem<R, TJ, TK>;
  const ot2d_params& p = *S.P;
  const int jd = S.jd, kd = S.kd, t = threadIdx.x;
  const int ntj = (p.jend - p.jbeg + TJ) / TJ;
  const int j0 = p.jbeg + (tile % ntj) * TJ, k0 = p.kbeg + (tile / ntj) * TK;
  const int j1 = min(j0 + TJ - 1, p.jend), k1 = min(k0 + TK - 1, p.kend);
  const int jr = j0 - G::H, kr = k0 - G::H;
  const bool visc = (flags & AS_VISC) && !p.invisc;
  const bool inv = flags & AS_INV;
  const R gm1 = S.k_gm1;
  const Recon<R> rx{p.ilim, S.k_th, S.k_qt, S.k_epsl_x, S.k_mp2}, ry{p.ilim, S.k_th, S.k_qt, S.k_epsl_y, S.k_mp2};
  // A: stage the region.  A thread issues the loads of all its staged cells
  // before it converts and stores the first, so that their latencies
  // overlap (one round trip to memory per thread instead of one per cell).
  {
    constexpr int NST = (G::NR + G::BS - 1) / G::BS;
    RtRaw<R> raw[NST];
#pragma unroll
    for (int i = 0; i < NST; ++i) {
      const int r = t + i * G::BS;
      const int j = jr + r % G::RW, k = kr + r / G::RW;
      if (r < G::NR && j >= 1 && j <= jd && k >= 1 && k <= kd) rt_load_cell(S, p, j, k, visc, raw[i]);
    }
#pragma unroll
    for (int i = 0; i < NST; ++i) {
      const int r = t + i * G::BS;
      const int j = jr + r % G::RW, k = kr + r / G::RW;
      if (r < G::NR && j >= 1 && j <= jd && k >= 1 && k <= kd) rt_store_cell(S, sm, r, raw[i], visc);
    }
  }
  __syncthreads();
  // B-D: every face quantity of the tile, in warp tasks (RtTasks)
  using TS = RtTasks<TJ, TK>;
  constexpr TS tasks = rt_tasks<TJ, TK>();
  static_assert(tasks.most <= 9, "a warp's task list must fit 63 bits");
  const int nD1 = visc ? G::VEH * TJ : 0, nD2 = visc ? TK * G::VXW : 0;
  const R gkpr = S.k_gkpr, dre = S.k_dre;
  const int lane = t & 31;
  uint64_t code = 0;
#pragma unroll
  for (int i = 0; i < TS::NW; ++i)
    if (i == (t >> 5)) code = tasks.code[i];
  for (; code; code >>= 7) {
    const int task = (int)(code & 127) - 1;
    if (task < TS::NFT) {
      if (!inv) continue;
      const int f = task * 32 + lane;
      if (f >= TS::NF) continue;
      // B: xi face j+1/2 of row k, j in j0-1..j1 (eulerrhs.f:69-167);
      // C: eta face k+1/2 of column j, k in k0-1..k1 (eulerrhs.f:170-268)
      const bool xi = f < TS::FB;
      const int g = xi ? f : f - TS::FB;
      const int j = xi ? j0 - 1 + g % (TJ + 1) : j0 + g % TJ;
      const int k = xi ? k0 + g / (TJ + 1) : k0 - 1 + g / TJ;
      if (j > j1 || k > k1) continue;
      RtLine<R, SM> L = xi ? RtLine<R, SM>{&sm, (k - kr) * G::RW - jr, 1, max(1, jr), min(jd, jr + G::RW - 1), gm1}
                           : RtLine<R, SM>{&sm, (j - jr) - kr * G::RW, G::RW, max(1, kr), min(kd, kr + G::RH - 1), gm1};
      if constexpr (LIM == 2) {
        const int64_t n2 = (int64_t)jd * kd;
        L.qd = S.quad + (xi ? 0 : 8) * n2;
        L.qn2 = n2;
        L.g0 = xi ? (int64_t)(k - 1) * jd - 1 : (int64_t)(j - 1) - jd;
        L.gs = xi ? 1 : jd;
      }
      const Recon<R> rc = xi ? rx : ry;
      const int64_t o = at(jd, j, k);
      const R* ma = xi ? S.fxa : S.gxa;
      const R* mb = xi ? S.fya : S.gya;
      const R* mc = xi ? S.ftj : S.gtj;
      R fl[4];
      face_flux_t<LIM, R, RtLine<R, SM>, PRE>(L, rc, xi ? j : k, xi ? jd : kd, ma[o], mb[o], mc ? mc[o] : (R)0.0, fl);
      R* dst = xi ? sm.F + g : sm.G_ + g;
      const int vs = xi ? TS::FB : (TK + 1) * TJ;
#pragma unroll
      for (int v = 0; v < 4; ++v) dst[v * vs] = fl[v];
    } else {
      const int d = (task - TS::NFT) * 32 + lane;
      if (d < nD1) {
        // D1: eta viscous terms at k0-2..k1+1 of columns j0..j1
        const int f = d;
        const int kf = f / TJ, jj = f % TJ;
        const int j = j0 + jj, k = k0 - 2 + kf;
        if (j > j1 || k < 1 || k > kd - 1 || k > k1 + 1) continue;
        R out[6];
        rt_visc_eta(sm, (k - kr) * G::RW + (j - jr), gkpr, dre, out);
#pragma unroll
        for (int v = 0; v < 6; ++v) sm.VE[v * (G::VEH * TJ) + f] = out[v];
      } else if (d < nD1 + nD2) {
        // D2: xi viscous terms at j0-2..j1+1 of rows k0..k1
        const int f = d - nD1;
        const int kk = f / G::VXW, jf = f % G::VXW;
        const int j = j0 - 2 + jf, k = k0 + kk;
        if (k > k1 || j < 1 || j > jd - 1 || j > j1 + 1) continue;
        R out[6];
        rt_visc_xi(sm, (k - kr) * G::RW + (j - jr), gkpr, dre, out);
#pragma unroll
        for (int v = 0; v < 6; ++v) sm.VX[v * (TK * G::VXW) + f] = out[v];
      }
    }
  }
  __syncthreads();
  // E: per-cell assembly in the reference's order, then the time-spectral
  // term, the norm partial and the store
  const int jj = t % TJ, kk = t / TJ;
  const int j = j0 + jj, k = k0 + kk;
  const int nv = p.nv;
  const bool acc = flags & AS_ACC;
  if (j <= j1 && k <= k1) {
    const int64_t o = at(jd, j, k);
    R s[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) s[n] = (R)0.0;
    if (acc) {
#pragma unroll
      for (int n = 0; n < 8; ++n)
        if (n < nv) s[n] = S.s[(int64_t)n * S.qs + o];
    }
    if (inv) {
      const R* F = sm.F + kk * (TJ + 1) + jj;
      const R* G = sm.G_ + kk * TJ + jj;
#pragma unroll
      for (int v = 0; v < 4; ++v) s[v] = s[v] - (F[v * (TK * (TJ + 1)) + 1] - F[v * (TK * (TJ + 1))]);
#pragma unroll
      for (int v = 0; v < 4; ++v) s[v] = s[v] - (G[v * ((TK + 1) * TJ) + TJ] - G[v * ((TK + 1) * TJ)]);
    }
    if (S.qnewt && !p.timespectral) {
      // newton (time.f:195-206): the physical-time term, added between the
      // inviscid and the viscous parts as compute_residual does
      // (step.f:274-285); 1/(oat*h) of this step in red[8]
      const double tac = S.red[8];
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        if (n >= nv) continue;
        const int64_t on = (int64_t)n * S.qs + o;
        s[n] = s[n] - (R)((S.q64[on] - S.qnewt[on]) * tac);
      }
    }
    if (visc) {
      // VE row of cell k is kk+2; VX column of cell j is jj+2
      const R* VE = sm.VE + (kk + 2) * TJ + jj;
      for (int v = 0; v < 3; ++v) {
        const R* a0 = VE + v * (G::VEH * TJ);
        const R* b0 = VE + (v + 3) * (G::VEH * TJ);
        const R a = a0[0] - a0[-TJ];
        R b;
        if (k == p.kend) b = (R)0.5 * (b0[-2 * TJ] - (R)4. * b0[-TJ] + (R)3 * b0[0]);
        else b = (R)0.5 * (b0[TJ] - b0[-TJ]);
        s[v + 1] = s[v + 1] + a + b;
      }
      const R* VX = sm.VX + kk * G::VXW + jj + 2;
      for (int v = 0; v < 3; ++v) {
        const R* a0 = VX + v * (TK * G::VXW);
        const R* b0 = VX + (v + 3) * (TK * G::VXW);
        const R a = a0[0] - a0[-1];
        R b;
        if (j == p.jend) b = (R)0.5 * (b0[-2] - (R)4. * b0[-1] + (R)3 * b0[0]);
        else b = (R)0.5 * (b0[1] - b0[-1]);
        s[v + 1] = s[v + 1] + a + b;
      }
    }
    if (S.sinf) {
      // f32 path: remove the f32 residual of the uniform freestream on this
      // mesh (exactly 0 in real arithmetic: closed cells, uniform state);
      // what remains of it in f32 is metric / state rounding that would
      // otherwise set the floor of the residual
#pragma unroll
      for (int v = 0; v < 4; ++v) s[v] = s[v] - S.sinf[(int64_t)v * S.qs + o];
    }
    if ((flags & AS_TS) && p.timespectral && S.Ds) {
      // timespectralrhs (sources.f:16-24): s(n) -= rotf*Ds(nsp,m)*q(m)
      const int64_t n2 = (int64_t)jd * kd;
      const R rotf = (R)p.rotf;
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        if (n >= nv) continue;
        R a = s[n];
        for (int m = 1; m <= S.nspec; ++m) {
          const R dsn = (R)S.Ds[(int64_t)(m - 1) * S.nspec + (S.nsp - 1)];
          const R qm = S.q[(int64_t)n * S.qs + (int64_t)(m - S.nsp) * n2 + o];
          a = a - rotf * dsn * qm;
        }
        s[n] = a;
      }
    }
    if (flags & AS_NORM) {
      // norms (step.f:67-88): the per-cell terms in R, the reduction in f64.
      // The first variable of the cell's maximum |s| carries the smallest
      // loop-order key, as in the reference's scan.
      const int ibi = S.iblank[o];
      const R m = (R)(ibi > 0 ? ibi : 0);
      R best = (R)-1;
      int bn = 1;
#pragma unroll
      for (int n = 1; n <= 8; ++n) {
        if (n > p.nmv) continue;
        const R smrs = fabs(s[n - 1]) * m;
        if (smrs > best) { best = smrs; bn = n; }
      }
      np.resmax = best;
      np.key = ((long long)(k - 1) * (p.nmv + 1) + bn) * (long long)jd + (j - 1);
      const R s1 = s[0] * m, s2 = s[1] * m, s3 = s[2] * m, s4 = s[3] * m;
      np.resrho = to_d(s[0] * s[0]);
      np.rsum = to_d(s1 * s1 + s2 * s2 + s3 * s3 + s4 * s4);
    }
    if constexpr (PRE) {
      if (flags & AS_NORM) rhslom_cell(S, p, o, s);
    }
    if (S.qnewt && p.timespectral && (flags & AS_NORM)) {
      // newtonTS (time.f:213-241): the pseudo-time Newton term of a
      // time-spectral run, gathered in ss and added after the norms and
      // rhslom (step.f:125-131)
      const R ts = S.tscale[o];
      if (ts != (R)0) {
#pragma unroll
        for (int n = 0; n < 8; ++n) {
          if (n >= nv) continue;
          const int64_t on = (int64_t)n * S.qs + o;
          const double ssv = 0.0 - (S.q64[on] - S.qnewt[on]) / (double)ts;
          s[n] = s[n] + (R)ssv;
        }
      }
    }
#pragma unroll
    for (int n = 0; n < 8; ++n)
      if (n < nv) S.s[(int64_t)n * S.qs + o] = s[n];
  }
  if (!acc) {
    // halo cells bordering the tile
    const int jlo = (j0 == p.jbeg) ? 1 : j0, jhi = (j1 == p.jend) ? jd : j1;
    const int klo = (k0 == p.kbeg) ? 1 : k0, khi = (k1 == p.kend) ? kd : k1;
    const int nw = jhi - jlo + 1, nbox = nw * (khi - klo + 1);
    if (nbox > (j1 - j0 + 1) * (k1 - k0 + 1))
      for (int i = t; i < nbox; i += G::BS) {
        const int hj = jlo + i % nw, hk = klo + i / nw;
        if (hj >= p.jbeg && hj <= p.jend && hk >= p.kbeg && hk <= p.kend) continue;
        const int64_t o = at(jd, hj, hk);
        for (int n = 1; n <= nv; ++n) S.s[(int64_t)(n - 1) * S.qs + o] = (R)0.0;
      }
  }
}

}  // namespace ot2d
