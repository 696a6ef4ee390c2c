// k_lusgs.cuh -- LU-SGS hyperplane operator ilu2d (src/lhs.f:470-814).
//
// The reference sweeps i+j hyperplanes; cell (j,k) of the forward sweep
// needs the already-updated s(j-1,k) and s(j,k-1) (backward: j+1, k+1).
// GB300 design:
//  1. k_lu_prep (fully parallel): every interior cell computes what the
//     sweeps need from it -- its scaled residual, tscale/2, the diagonal d
//     and the primitive / metric / spectral-radius factors of its outgoing
//     contributions (lhs.f:524-563, :626-653) -- and stores them in a
//     "skewed band" record: rows are grouped in bands of 32 (one warp, one
//     row per lane) and the record of step t of a band holds, for every
//     lane l, the cell at column t-l.  One wavefront step of a warp is then
//     one contiguous chunk (24 fields x 32 lanes).
//  2. k_lu_edges: point-Jacobi scaling of the halo residuals (lhs.f:567-598),
//     their contributions to the first/last interior row and column, and
//     (FP64) the reference's conservative->primitive->conservative round trip
//     of q (lhs.f:524-531, :805-811).
//  3. k_lu_sweep<FWD> (one CTA per slice, warp w = band w): the warps
//     advance in a skewed lockstep; each warp streams its chunks into a
//     shared-memory ring with cp.async.bulk (TMA) completing on mbarriers,
//     the (j-1,k) contribution stays in registers, the (j,k-1) one arrives
//     from the neighbouring lane by shuffle and across bands through a
//     double-buffered shared slot.  Every cell sees exactly the operands of
//     the reference's hyperplane order, so the sweep equals the sequential
//     one operation for operation.
#pragma once
#include "dev_common.cuh"

namespace ot2d {

// A (band, step) chunk holds the records of the band's 32 lanes one after
// another (lane-major): lane l's 24 fields are contiguous, so a lane reads
// four consecutive fields with one (f32) or two (f64) 16-byte shared loads.
// Each record is padded to LS elements so that the eight lanes of a load
// phase hit disjoint banks (f32: 112-byte stride, f64: 208-byte stride).
// (Interleaving 16-byte field groups over the lanes instead was measured
// slower in the backward sweep.)  With Turkel preconditioning (PRE, the
// preilu2d operator of lhs.f:2-467) a record carries 8 more fields: the
// chk*qq products of both sweeps and the preconditioner factor.
template <class R, bool PRE = false>
struct LuLay {
  static constexpr int NF = PRE ? 32 : 24;                                   // fields per record
  static constexpr int LS = sizeof(R) == 4 ? (PRE ? 36 : 28) : (PRE ? 34 : 26);   // elements per lane record
  static constexpr int CH = 32 * LS;                                         // elements per chunk
};
// record fields
enum {
  LF_S = 0,    // 0..3: residual (forward input, then forward result)
  LF_SV = 4, LF_D = 5, LF_UU = 6, LF_VV = 7, LF_UV2 = 8, LF_GE = 9,
  LF_RI1 = 10, LF_RI2 = 11, LF_RK1 = 12, LF_RK2 = 13, LF_QX = 14, LF_QY = 15,
  LF_FCX = 16, LF_FSX = 17, LF_FCY = 18, LF_FSY = 19,  // forward chk / spec (xi, eta)
  LF_BCX = 20, LF_BSX = 21, LF_BCY = 22, LF_BSY = 23,  // backward chk / spec
  // preconditioned records only: chk*qq (xi, eta) and gm1 (bSq-1)/c**2 of
  // the forward (24..27) and the backward (28..31) sweep
  LF_PF = 24, LF_PB = 28
};
// element offset of field f of lane l within a chunk
template <class R, bool PRE = false>
__host__ __device__ __forceinline__ int lu_idx(int f, int l) {
  return l * LuLay<R, PRE>::LS + f;
}

__host__ __device__ __forceinline__ int lu_nrow(int kd) { return kd - 2; }
__host__ __device__ __forceinline__ int lu_ncol(int jd) { return jd - 2; }
__host__ __device__ __forceinline__ int lu_nband(int kd) { return (kd - 2 + 31) / 32; }
__host__ __device__ __forceinline__ int lu_nstep(int jd) { return jd - 2 + 31; }
// elements of one slice's record (element size esize bytes): chunks + 4
// halo-contribution arrays, sized for the larger (preconditioned) layout so
// that a slice can use either
__host__ __device__ __forceinline__ int64_t lu_rec_elems(int jd, int kd, int esize) {
  const int ch = esize == 4 ? LuLay<float, true>::CH : LuLay<double, true>::CH;
  return (int64_t)lu_nband(kd) * lu_nstep(jd) * ch + 8 * (int64_t)(lu_nrow(kd) + lu_ncol(jd)) + 64;
}

// fields f..f+3 of lane l of a chunk (f a multiple of 4) as 16-byte accesses
template <class R>
struct Lu4 { R x, y, z, w; };
template <bool PRE = false>
__device__ __forceinline__ Lu4<float> lu_ld4(const float* ch, int f, int l) {
  const float4 v = *reinterpret_cast<const float4*>(ch + lu_idx<float, PRE>(f, l));
  return {v.x, v.y, v.z, v.w};
}
template <bool PRE = false>
__device__ __forceinline__ Lu4<double> lu_ld4(const double* ch, int f, int l) {
  const double2 a = *reinterpret_cast<const double2*>(ch + lu_idx<double, PRE>(f, l));
  const double2 b = *reinterpret_cast<const double2*>(ch + lu_idx<double, PRE>(f + 2, l));
  return {a.x, a.y, b.x, b.y};
}
template <bool PRE = false>
__device__ __forceinline__ void lu_st4(float* ch, int f, int l, float a, float b, float c, float d) {
  *reinterpret_cast<float4*>(ch + lu_idx<float, PRE>(f, l)) = make_float4(a, b, c, d);
}
template <bool PRE = false>
__device__ __forceinline__ void lu_st4(double* ch, int f, int l, double a, double b, double c, double d) {
  *reinterpret_cast<double2*>(ch + lu_idx<double, PRE>(f, l)) = make_double2(a, b);
  *reinterpret_cast<double2*>(ch + lu_idx<double, PRE>(f + 2, l)) = make_double2(c, d);
}

// four consecutive values at a 16-byte aligned shared address (the
// cross-band ring slots and the staged halo contributions)
__device__ __forceinline__ Lu4<float> lu_ldv(const float* a) {
  const float4 v = *reinterpret_cast<const float4*>(a);
  return {v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ Lu4<double> lu_ldv(const double* a) {
  const double2 x = *reinterpret_cast<const double2*>(a), y = *reinterpret_cast<const double2*>(a + 2);
  return {x.x, x.y, y.x, y.y};
}
__device__ __forceinline__ void lu_stv(float* a, const float* v) {
  *reinterpret_cast<float4*>(a) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void lu_stv(double* a, const double* v) {
  *reinterpret_cast<double2*>(a) = make_double2(v[0], v[1]);
  *reinterpret_cast<double2*>(a + 2) = make_double2(v[2], v[3]);
}

template <class R>
struct LuCell {
  R uu, vv, uv2, ge, ri1, ri2, rk1, rk2, qx, cx, qy, cy, vn, ugc, vgc, d;
  R bsq, term;   // preconditioned: bSq of the cell, gm1 (bSq-1)/c**2
};

// lhs.f:524-531 (conservative -> primitive) and :535-563 (diagonal); PRE:
// preilu2d's diagonal (lhs.f:60-101) from the preconditioned spectral radii
// 0.5 ((bSq+1)|qq| + sqrt(((1-bSq) qq)**2 + 4 bSq cc**2)) of both directions
template <class R, bool PRE = false>
__device__ __forceinline__ LuCell<R> lu_cell(const Slice<R>& S, const ot2d_params& p, int j, int k, R epsv) {
  const int64_t o = at(S.jd, j, k), qs = S.qs;
  LuCell<R> c;
  R q1 = S.q[o];
  R dj = (R)1.0 / q1;
  c.uu = S.q[qs + o] * dj;
  c.vv = S.q[2 * qs + o] * dj;
  R e = S.q[3 * qs + o] * dj;
  R rho = q1 * S.q[(p.nq - 1) * qs + o];
  c.uv2 = (R)0.5 * (c.uu * c.uu + c.vv * c.vv);
  R cjkl = sqrt(S.k_ggm1 * (e - c.uv2));
  c.ri1 = S.xx[o]; c.ri2 = S.xy[o]; c.rk1 = S.yx[o]; c.rk2 = S.yy[o];
  c.ugc = S.ug ? S.ug[o] : (R)0; c.vgc = S.vg ? S.vg[o] : (R)0;
  R qq1 = c.ri1 * c.uu + c.ri2 * c.vv;
  R qqx = fabs(-c.ri1 * c.ugc - c.ri2 * c.vgc + qq1);
  R rr1 = sqrt(sq(c.ri1) + sq(c.ri2));
  R qq2 = c.rk1 * c.uu + c.rk2 * c.vv;
  R qqy = fabs(-c.rk1 * c.ugc - c.rk2 * c.vgc + qq2);
  R rr2 = sqrt(sq(c.rk1) + sq(c.rk2));
  R vnu = (R)2.0 * rr2 * rr2 * (S.k_rmue + S.turmu[o]) / (S.k_rey * rho);
  R svt = S.tscale[o];
  c.qx = qq1; c.cx = cjkl * rr1; c.qy = qq2; c.cy = cjkl * rr2; c.vn = vnu;
  c.ge = S.k_gamma * e - S.k_gm1 * c.uv2;
  if constexpr (PRE) {
    const R btv = S.bt[o], mp2 = S.k_mp2;
    const R bSq = mp2 / (btv - mp2 * (btv - (R)1));
    const R omb = (R)1. - bSq, opb = bSq + (R)1., fb = (R)4. * bSq;
    const R X = sqrt((omb * qqx) * (omb * qqx) + (fb * c.cx) * c.cx);
    R term = (R)0.5 * (opb * qqx + X);
    const R Y = sqrt((omb * qqy) * (omb * qqy) + (fb * c.cy) * c.cy);
    term = term + (R)0.5 * (opb * qqy + Y);
    c.d = (R)1.0 / ((R)1.0 + svt * (term * epsv + vnu));
    c.bsq = bSq;
    c.term = S.k_gm1 * (bSq - (R)1.) / (cjkl * cjkl);
  } else {
    c.d = (R)1.0 / ((R)1.0 + svt * ((qqx + qqy + cjkl * (rr1 + rr2)) * epsv + vnu));
    c.bsq = (R)0; c.term = (R)0;
  }
  return c;
}

// chk / spec of one direction (lhs.f:636-640, :667-671, :735-739, :765-769)
template <class R, bool XI, bool FWD>
__device__ __forceinline__ void lu_chkspec(const LuCell<R>& c, R eps2, R& chk, R& spec) {
  R ri1 = XI ? c.ri1 : c.rk1, ri2 = XI ? c.ri2 : c.rk2, qq = XI ? c.qx : c.qy, cc = XI ? c.cx : c.cy;
  R qqn = -ri1 * c.ugc - ri2 * c.vgc + qq;
  R sp1 = fabs(qqn) + cc;
  R sm2 = eps2 * sp1;
  if (FWD) {
    chk = (R)0.5 + fsign((R)0.5, qqn + cc);
    spec = XI ? chk * (qqn + sp1) + sm2 : chk * (qqn + sp1) + c.vn + sm2;
  } else {
    chk = (R)0.5 - fsign((R)0.5, qqn - cc);
    spec = XI ? chk * (qqn - sp1) - sm2 : chk * (qqn - sp1) - c.vn - sm2;
  }
}

// contribution of a cell with correction s to its neighbour (lhs.f:643-653)
template <class R>
__device__ __forceinline__ void lu_apply(R chk, R spec, R ri1, R ri2, R qq, R uu, R vv, R uv2, R ge, R gm1,
                                         const R* s, R* a) {
  R s1 = s[0], s2 = s[1], s3 = s[2], s4 = s[3];
  R a4 = chk * (ri1 * s2 + ri2 * s3 - qq * s1);
  R a2 = chk * gm1 * (uv2 * s1 - (uu * s2 + vv * s3) + s4);
  a[0] = a4 + spec * s1;
  a[1] = ri1 * a2 + uu * a4 + spec * s2;
  a[2] = ri2 * a2 + vv * a4 + spec * s3;
  a[3] = qq * a2 + ge * a4 + spec * s4;
}

// preilu2d's chk / spec and chk*qq of one direction (lhs.f:160-179,
// :221-241, :321-340, :382-402): the convective split of the preconditioned
// eigenvalues (bSq+1) qq/2 +- X/2, X = sqrt(((1-bSq) qq)**2 + 4 bSq cc**2)
template <class R, bool XI, bool FWD>
__device__ __forceinline__ void lu_chkspec_pre(const LuCell<R>& c, R eps2, R& chk, R& cq, R& spec) {
  R ri1 = XI ? c.ri1 : c.rk1, ri2 = XI ? c.ri2 : c.rk2, qq = XI ? c.qx : c.qy, cc = XI ? c.cx : c.cy;
  R qqn = -ri1 * c.ugc - ri2 * c.vgc + qq;
  const R bSq = c.bsq, omb = (R)1. - bSq, opb = bSq + (R)1.;
  R X = sqrt((omb * qqn) * (omb * qqn) + (((R)4. * bSq) * cc) * cc);
  if (FWD) chk = (R)0.5 + fsign((R)0.5, opb * qqn + X);
  else chk = (R)0.5 - fsign((R)0.5, opb * qqn - X);
  R sp1 = (R)0.5 * (opb * fabs(qqn) + X);
  R sm2 = eps2 * sp1;
  spec = XI ? chk * sp1 + sm2 : chk * sp1 + c.vn + sm2;
  cq = chk * qqn;
}

// preconditioned contribution of a cell with correction s to its neighbour
// (lhs.f:181-208): the split flux t, then t + term * [u,v,ge]^T
// [uv2, -u, -v, 1] t (the preconditioner), then +- spec * s
template <class R, bool FWD>
__device__ __forceinline__ void lu_apply_pre(R chk, R cq, R spec, R term, R ri1, R ri2, R qq, R uu, R vv, R uv2,
                                             R ge, R gm1, const R* s, R* a) {
  R s1 = s[0], s2 = s[1], s3 = s[2], s4 = s[3];
  R a4 = chk * (ri1 * s2 + ri2 * s3 - qq * s1);
  R a2 = chk * gm1 * (uv2 * s1 - (uu * s2 + vv * s3) + s4);
  const R t1 = a4 + cq * s1;
  const R t2 = ri1 * a2 + uu * a4 + cq * s2;
  const R t3 = ri2 * a2 + vv * a4 + cq * s3;
  const R t4 = qq * a2 + ge * a4 + cq * s4;
  const R r1 = uv2 * t1 - uu * t2 - vv * t3 + t4;
  const R p1 = r1 * term + t1, p2 = (uu * r1) * term + t2, p3 = (vv * r1) * term + t3, p4 = (ge * r1) * term + t4;
  if (FWD) {
    a[0] = p1 + spec * s1; a[1] = p2 + spec * s2; a[2] = p3 + spec * s3; a[3] = p4 + spec * s4;
  } else {
    a[0] = p1 - spec * s1; a[1] = p2 - spec * s2; a[2] = p3 - spec * s3; a[3] = p4 - spec * s4;
  }
}

template <class R, bool XI, bool FWD, bool PRE = false>
__device__ __forceinline__ void lu_contrib(const LuCell<R>& c, const R* s, R gm1, R eps2, R* a) {
  if constexpr (PRE) {
    R chk, cq, spec;
    lu_chkspec_pre<R, XI, FWD>(c, eps2, chk, cq, spec);
    lu_apply_pre<R, FWD>(chk, cq, spec, c.term, XI ? c.ri1 : c.rk1, XI ? c.ri2 : c.rk2, XI ? c.qx : c.qy, c.uu, c.vv,
                         c.uv2, c.ge, gm1, s, a);
  } else {
    R chk, spec;
    lu_chkspec<R, XI, FWD>(c, eps2, chk, spec);
    lu_apply(chk, spec, XI ? c.ri1 : c.rk1, XI ? c.ri2 : c.rk2, XI ? c.qx : c.qy, c.uu, c.vv, c.uv2, c.ge, gm1, s, a);
  }
}

// ---- kernel 1: records of the interior cells (one thread per (band, step, lane))
// The record of lane l of chunk (band, t) into ch, the chunk as the warp
// stages it in shared memory (k_lu_prep stores the staged chunk with
// contiguous 16-byte accesses).
template <class R, bool PRE = false>
__device__ __forceinline__ void lu_prep_cell(const Slice<R>& S, const ot2d_params& p, int band, int t, int l, int scale,
                                             R* ch) {
  const int nrow = lu_nrow(S.kd), ncol = lu_ncol(S.jd);
  const int r = 32 * band + l, c = t - l;
  if (r >= nrow || c < 0 || c >= ncol) {
    const R z = (R)0;
#pragma unroll
    for (int f = 0; f < LuLay<R, PRE>::NF; f += 4) lu_st4<PRE>(ch, f, l, z, z, z, z);
    return;
  }
  const int j = p.jbeg + c, k = p.kbeg + r;
  const R eps2 = S.k_eps2, epsv = S.k_epsv;
  const int64_t o = at(S.jd, j, k);
  LuCell<R> cl = lu_cell<R, PRE>(S, p, j, k, epsv);
  const R ts = S.tscale[o];
  R sv[4];
#pragma unroll
  for (int n = 0; n < 4; ++n) {
    R v = S.s[n * S.qs + o];
    sv[n] = scale ? v * ts : v;
  }
  lu_st4<PRE>(ch, LF_S, l, sv[0], sv[1], sv[2], sv[3]);
  lu_st4<PRE>(ch, LF_SV, l, ts * (R)0.5, cl.d, cl.uu, cl.vv);
  lu_st4<PRE>(ch, LF_UV2, l, cl.uv2, cl.ge, cl.ri1, cl.ri2);
  lu_st4<PRE>(ch, LF_RK1, l, cl.rk1, cl.rk2, cl.qx, cl.qy);
  R a, b, a2, b2;
  if constexpr (PRE) {
    R q1, q2;
    lu_chkspec_pre<R, true, true>(cl, eps2, a, q1, b);
    lu_chkspec_pre<R, false, true>(cl, eps2, a2, q2, b2);
    lu_st4<PRE>(ch, LF_FCX, l, a, b, a2, b2);
    lu_st4<PRE>(ch, LF_PF, l, q1, q2, cl.term, (R)0);
    lu_chkspec_pre<R, true, false>(cl, eps2, a, q1, b);
    lu_chkspec_pre<R, false, false>(cl, eps2, a2, q2, b2);
    lu_st4<PRE>(ch, LF_BCX, l, a, b, a2, b2);
    lu_st4<PRE>(ch, LF_PB, l, q1, q2, cl.term, (R)0);
  } else {
    lu_chkspec<R, true, true>(cl, eps2, a, b);
    lu_chkspec<R, false, true>(cl, eps2, a2, b2);
    lu_st4(ch, LF_FCX, l, a, b, a2, b2);
    lu_chkspec<R, true, false>(cl, eps2, a, b);
    lu_chkspec<R, false, false>(cl, eps2, a2, b2);
    lu_st4(ch, LF_BCX, l, a, b, a2, b2);
  }
}

// halo-contribution arrays after the chunks: A forward [nrow][4], A backward,
// B forward [ncol][4], B backward
template <class R, bool PRE = false>
__device__ __forceinline__ R* lu_halo(const Slice<R>& S, int which) {
  const int nrow = lu_nrow(S.kd), ncol = lu_ncol(S.jd);
  R* base = S.lurec + (int64_t)lu_nband(S.kd) * lu_nstep(S.jd) * LuLay<R, PRE>::CH;
  switch (which) {
    case 0: return base;
    case 1: return base + 4 * nrow;
    case 2: return base + 8 * nrow;
    default: return base + 8 * nrow + 4 * ncol;
  }
}

// ---- kernel 2: halo edges (one thread per cell of the slice)
template <class R, bool PRE = false>
__device__ __forceinline__ void lu_edge_cell(const Slice<R>& S, const ot2d_params& p, int j, int k, int scale) {
  const int js = p.jbeg, je = p.jend, ks = p.kbeg, ke = p.kend;
  const bool ij = j >= js && j <= je, ik = k >= ks && k <= ke;
  const int64_t o = at(S.jd, j, k);
  const R eps2 = S.k_eps2, epsv = S.k_epsv, gm1 = S.k_gm1;
  if (!(ij && ik)) {
    R sv[4];
    const R ts = S.tscale[o];
#pragma unroll
    for (int n = 0; n < 4; ++n) sv[n] = scale ? S.s[n * S.qs + o] * ts : S.s[n * S.qs + o];
    const bool edge = (ik && (j == js - 1 || j == je + 1)) || (ij && (k == ks - 1 || k == ke + 1));
    if (edge) {
      LuCell<R> c = lu_cell<R, PRE>(S, p, j, k, epsv);
#pragma unroll
      for (int n = 0; n < 4; ++n) sv[n] = sv[n] * c.d;
      R a[4];
      R* dst = nullptr;
      if (j == js - 1) { lu_contrib<R, true, true, PRE>(c, sv, gm1, eps2, a); dst = lu_halo<R, PRE>(S, 0) + 4 * (k - ks); }
      else if (j == je + 1) { lu_contrib<R, true, false, PRE>(c, sv, gm1, eps2, a); dst = lu_halo<R, PRE>(S, 1) + 4 * (k - ks); }
      else if (k == ks - 1) { lu_contrib<R, false, true, PRE>(c, sv, gm1, eps2, a); dst = lu_halo<R, PRE>(S, 2) + 4 * (j - js); }
      else { lu_contrib<R, false, false, PRE>(c, sv, gm1, eps2, a); dst = lu_halo<R, PRE>(S, 3) + 4 * (j - js); }
#pragma unroll
      for (int n = 0; n < 4; ++n) dst[n] = a[n];
    }
#pragma unroll
    for (int n = 0; n < 4; ++n) S.s[n * S.qs + o] = sv[n];
  }
  // FP64 plain path: q leaves ilu2d round-tripped (lhs.f:524-531, :805-811)
  if constexpr (sizeof(R) == sizeof(double)) {
    const int64_t qs = S.qs;
    double q1 = S.q[o], J = S.q[(p.nq - 1) * qs + o];
    double dj = 1.0 / q1;
    double u = S.q[qs + o] * dj, v = S.q[2 * qs + o] * dj, e = S.q[3 * qs + o] * dj;
    double q1n = (q1 * J) / J;
    S.q[o] = q1n;
    S.q[qs + o] = u * q1n;
    S.q[2 * qs + o] = v * q1n;
    S.q[3 * qs + o] = e * q1n;
  }
}

// ---- kernel 3: the sweeps --------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Polls a sweep wait makes before it gives up (the status word of the slice
// records the timeout).  The solver can lower it (OT2D_OPT_POLL_LIMIT) to
// make the waits run out on purpose; the drain of copies still in flight
// after a give-up always uses this default bound.
constexpr uint32_t LU_POLL_DEFAULT = 1u << 22;

// Bounded wait on a ring slot; false after `lim` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t lim = LU_POLL_DEFAULT) {
  for (uint32_t it = 0; it < lim; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Progress counters in shared memory: the producer publishes with a release
// store, the consumer reads with an acquire load (CTA scope), so the data
// written before the store is visible after the load.
__device__ __forceinline__ int lu_ld_acquire(const int* cnt) {
  int v;
  asm volatile("ld.acquire.cta.shared::cta.s32 %0, [%1];" : "=r"(v) : "r"(smem_u32(cnt)) : "memory");
  return v;
}
__device__ __forceinline__ void lu_st_release(int* cnt, int v) {
  asm volatile("st.release.cta.shared::cta.s32 [%0], %1;" ::"r"(smem_u32(cnt)), "r"(v) : "memory");
}
// Bounded wait until *cnt >= need; `seen` caches the last value read, so a
// counter already known to be far enough ahead is not read again.
__device__ __forceinline__ bool lu_wait_ge(const int* cnt, int need, int& seen, uint32_t lim) {
  if (seen >= need) return true;
  for (uint32_t it = 0; it < lim; ++it) {
    seen = lu_ld_acquire(cnt);
    if (seen >= need) return true;
  }
  return false;
}

// Cross-band ring: the boundary lane of band w hands its outgoing (j,k-1)
// contribution of local step t to the next band in sweep order through
// slot t % LU_XB; the consumer reads it at its step t - 31.
constexpr int LU_XB = 128;   // a power of two

// Shared memory of the sweep kernel: per warp a ring of two groups of G
// chunks, its two barriers, its cross-band ring and its progress counter;
// then the first-row halo contributions of the slice (4 per column, at most
// maxcol columns).
template <class R, bool PRE = false>
__host__ __device__ __forceinline__ size_t lu_smem_bytes(int nwarp, int G, int maxcol) {
  return (size_t)nwarp * 2 * G * LuLay<R, PRE>::CH * sizeof(R) + (size_t)nwarp * 2 * sizeof(uint64_t) +
         (size_t)nwarp * LU_XB * 4 * sizeof(R) + (size_t)nwarp * sizeof(int) + 16 +
         (size_t)4 * maxcol * sizeof(R);
}

// One sweep of one slice.  Warp w owns band w (rows 32w..32w+31, lane l ->
// row 32w+l) and walks its nst local steps; at local step t lane l is on
// column t-l (forward) or ncol-1-(t-(31-l)) (backward), so the lanes of a
// warp are on 32 consecutive hyperplanes and the in-band dependency (the
// neighbouring row) arrives by shuffle from the previous step.  The
// dependency across bands -- lane 31 of band w-1 feeds lane 0 of band w
// 31 steps later (backward: lane 0 of band w+1 feeds lane 31 of band w) --
// goes through the cross-band ring guarded by per-warp progress counters,
// so the warps run without block-wide barriers.  The records stream in
// through cp.async.bulk, G chunks per copy, double-buffered.
// PRE: the preilu2d records and contributions.
template <class R, bool FWD, int G, bool PRE = false>
__device__ void lu_sweep_slice(const Slice<R>& S, int nwarp, unsigned char* smem, uint32_t lim, int lag) {
  const ot2d_params& p = *S.P;
  const int nrow = lu_nrow(S.kd), ncol = lu_ncol(S.jd), nb = lu_nband(S.kd), nst = lu_nstep(S.jd);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const R gm1 = S.k_gm1;
  R* rings = (R*)smem;
  constexpr int CH = LuLay<R, PRE>::CH;
  uint64_t* bars = (uint64_t*)(smem + (size_t)nwarp * 2 * G * CH * sizeof(R));
  R* xrings = (R*)(bars + (size_t)nwarp * 2);
  int* prog = (int*)(xrings + (size_t)nwarp * LU_XB * 4);
  // halo contributions into the first (forward) / last (backward) row,
  // read once per step by one lane: staged in shared memory
  R* bhs = (R*)(((uintptr_t)(prog + nwarp) + 15) & ~(uintptr_t)15);
  R* ring = rings + (size_t)w * 2 * G * CH;
  uint64_t* bar = bars + (size_t)w * 2;
  const bool wok = w < nb;
  const R* rec_w = S.lurec + (int64_t)w * nst * CH;
  R* recw = S.lurec + (int64_t)w * nst * CH;
  const int ngrp = (nst + G - 1) / G;
  // group g of the sweep covers local steps g*G .. g*G+G-1; its chunks are
  // contiguous in memory starting at chunk c0(g) (ascending)
  auto c0 = [&](int g) -> int { return FWD ? g * G : max(0, nst - (g + 1) * G); };
  auto gsize = [&](int g) -> int { return min(G, nst - g * G); };
  auto issue = [&](int g) {
    const uint32_t bytes = (uint32_t)gsize(g) * CH * sizeof(R);
    fence_proxy_async_smem();
    mbar_expect_tx(&bar[g & 1], bytes);
    bulk_g2s(ring + (size_t)(g & 1) * G * CH, rec_w + (int64_t)c0(g) * CH, bytes, &bar[g & 1]);
  };
  if (l == 0) {
    if (wok) { mbar_init(&bar[0], 1); mbar_init(&bar[1], 1); }
    prog[w] = 0;
  }
  {
    const R* Bg = lu_halo<R, PRE>(S, FWD ? 2 : 3);
    for (int i = threadIdx.x; i < 4 * ncol; i += blockDim.x) bhs[i] = Bg[i];
  }
  __syncthreads();
  if (!wok) return;
  if (l == 0) {
    issue(0);
    if (ngrp > 1) issue(1);
  }
  const R* Ah = lu_halo<R, PRE>(S, FWD ? 0 : 1);
  const R* Bh = bhs;
  // neighbouring bands in sweep order and the boundary lanes
  const int wprev = FWD ? w - 1 : w + 1, wnext = FWD ? w + 1 : w - 1;
  const bool has_prev = FWD ? w > 0 : w + 1 < nb, has_next = FWD ? w + 1 < nb : w > 0;
  const int lout = FWD ? 31 : 0;
  R* xout = xrings + (size_t)w * LU_XB * 4;
  const R* xin = xrings + (size_t)(has_prev ? wprev : w) * LU_XB * 4;
  const int r = 32 * w + l;
  // this lane's row of s (backward sweep output), indexed by column
  R* srow = S.s + (int64_t)(p.kbeg + r - 1) * S.jd + (p.jbeg - 1);
  R aprev[4] = {0, 0, 0, 0}, bout[4] = {0, 0, 0, 0};
  int seen_prev = 0, seen_next = 0;   // cached progress of the neighbouring bands
  bool bad = false;
  int gfail = -1;
  // Band lag: start `lag` steps after the neighbouring band's first
  // contribution is due, so that in the steady state the cross-band value
  // is already there and the cached progress spares most polls (the
  // operands of every cell are the same whatever the lag).
  if (has_prev && lag > 0) {
    if (l == 0 && !lu_wait_ge(&prog[wprev], min(32 + lag, nst), seen_prev, lim)) bad = true;
    seen_prev = __shfl_sync(0xffffffffu, seen_prev, 0);
  }
  // This lane's record: residual, (tscale/2, d, u, v), (uv2, ge, xi
  // metrics), (eta metrics, qx, qy), this sweep's (chk, spec) pairs.
  struct Rec { Lu4<R> r0, r1, r2, r3, r4; };
  auto ldrec = [&](const R* ch) -> Rec {
    return {lu_ld4<PRE>(ch, LF_S, l), lu_ld4<PRE>(ch, LF_SV, l), lu_ld4<PRE>(ch, LF_UV2, l),
            lu_ld4<PRE>(ch, LF_RK1, l), lu_ld4<PRE>(ch, FWD ? LF_FCX : LF_BCX, l)};
  };
  // The new correction of this lane's cell from its record and the summed
  // neighbour contributions, its store (forward: into the record for the
  // backward sweep; backward: into s), and its outgoing contributions:
  // xi into aprev (the same lane's next step), eta into bout (the next lane).
  auto cell = [&](const R* ch, const Rec& rc, int tl, int c, const R* bin) {
    const Lu4<R>&r0 = rc.r0, &r1 = rc.r1, &r2 = rc.r2, &r3 = rc.r3, &r4 = rc.r4;
    const R sv = r1.x, di = r1.y;
    const R st[4] = {r0.x, r0.y, r0.z, r0.w};
    R sn[4];
#pragma unroll
    for (int n = 0; n < 4; ++n)
      sn[n] = FWD ? (st[n] + sv * (aprev[n] + bin[n])) * di : st[n] - sv * (aprev[n] + bin[n]) * di;
    if (FWD) {
      lu_st4<PRE>(recw + (int64_t)tl * CH, LF_S, l, sn[0], sn[1], sn[2], sn[3]);
    } else {
#pragma unroll
      for (int n = 0; n < 4; ++n) srow[n * S.qs + c] = sn[n];
    }
    // xi: (chk, spec) = r4.x, r4.y with ri1, ri2, qx; eta: r4.z, r4.w
    // with rk1, rk2, qy; u, v, uv2, ge shared
    if constexpr (PRE) {
      // (chk*qq xi, chk*qq eta, preconditioner factor)
      const Lu4<R> r5 = lu_ld4<PRE>(ch, FWD ? LF_PF : LF_PB, l);
      lu_apply_pre<R, FWD>(r4.x, r5.x, r4.y, r5.z, r2.z, r2.w, r3.z, r1.z, r1.w, r2.x, r2.y, gm1, sn, aprev);
      lu_apply_pre<R, FWD>(r4.z, r5.y, r4.w, r5.z, r3.x, r3.y, r3.w, r1.z, r1.w, r2.x, r2.y, gm1, sn, bout);
    } else {
      lu_apply(r4.x, r4.y, r2.z, r2.w, r3.z, r1.z, r1.w, r2.x, r2.y, gm1, sn, aprev);
      lu_apply(r4.z, r4.w, r3.x, r3.y, r3.w, r1.z, r1.w, r2.x, r2.y, gm1, sn, bout);
    }
  };
  // Steady groups: a band of 32 rows, G steps all inside columns 1..ncol-1
  // of every lane (local steps 32 .. ncol-1), so every lane is active, no
  // lane is on the first column, and the waits on the neighbouring bands
  // are made once per group -- for the last step's cross-band input and the
  // last step's ring slot -- with the progress published once at the end.
  // Its steps have no waits and no boundary cases (the boundary lane's
  // input and output are predicated accesses); the cells see the same
  // operands as in the per-step form below.
  const bool full = 32 * (w + 1) <= nrow;
  const int lin = FWD ? 0 : 31;
  const bool pout = l == lout && has_next;
  for (int g = 0; g < ngrp; ++g) {
    const bool ok = mbar_wait_bounded(&bar[g & 1], (uint32_t)((g >> 1) & 1), lim);
    if (__any_sync(0xffffffffu, !ok || bad)) { gfail = g; break; }
    const int gs = gsize(g);
    const R* gring = ring + (size_t)(g & 1) * G * CH;
    const int t0 = g * G;
    if (full && gs == G && t0 >= 32 && t0 + G <= ncol) {
      if (has_prev && l == lin && !lu_wait_ge(&prog[wprev], t0 + G - 1 + 32, seen_prev, lim)) bad = true;
      if (pout && !lu_wait_ge(&prog[wnext], t0 + G - 1 - LU_XB + 32, seen_next, lim)) bad = true;
      if (__any_sync(0xffffffffu, bad)) { gfail = g; break; }
#pragma unroll
      for (int u = 0; u < G; ++u) {
        const int tl = t0 + u;
        const R* ch = gring + (FWD ? u : G - 1 - u) * CH;
        const Rec rc = ldrec(ch);
        R bin[4];
#pragma unroll
        for (int n = 0; n < 4; ++n)
          bin[n] = FWD ? __shfl_up_sync(0xffffffffu, bout[n], 1) : __shfl_down_sync(0xffffffffu, bout[n], 1);
        const int c = FWD ? tl - l : ncol - 1 - (tl - (31 - l));
        // lane lin: from band wprev's step tl + 31, or the halo row
        const R* xs = has_prev ? xin + ((tl + 31) & (LU_XB - 1)) * 4 : Bh + 4 * c;
        if (l == lin) {
          const Lu4<R> x = lu_ldv(xs);
          bin[0] = x.x; bin[1] = x.y; bin[2] = x.z; bin[3] = x.w;
        }
        cell(ch, rc, tl, c, bin);
        if (pout) lu_stv(xout + (tl & (LU_XB - 1)) * 4, bout);
      }
      if (l == lout) lu_st_release(&prog[w], t0 + G);
    } else {
#pragma unroll 4
      for (int u = 0; u < gs; ++u) {
        const int tl = t0 + u;
        // (loading the next step's record ahead of this step's arithmetic
        // was measured slower: 0.81 against 0.71 ms at batch 64)
        const R* ch = gring + (FWD ? u : gs - 1 - u) * CH;
        const Rec rc = ldrec(ch);
        R bin[4];
#pragma unroll
        for (int n = 0; n < 4; ++n)
          bin[n] = FWD ? __shfl_up_sync(0xffffffffu, bout[n], 1) : __shfl_down_sync(0xffffffffu, bout[n], 1);
        const int c = FWD ? tl - l : ncol - 1 - (tl - (31 - l));
        const bool act = r < nrow && c >= 0 && c < ncol;
        if (act) {
          if (FWD ? c == 0 : c == ncol - 1) {
#pragma unroll
            for (int n = 0; n < 4; ++n) aprev[n] = Ah[4 * r + n];
          }
          // the (j,k-1) / (j,k+1) neighbour from outside the band
          if (FWD ? l == 0 : (l == 31 || r == nrow - 1)) {
            if (!has_prev || (!FWD && r == nrow - 1)) {
#pragma unroll
              for (int n = 0; n < 4; ++n) bin[n] = Bh[4 * c + n];
            } else if (lu_wait_ge(&prog[wprev], tl + 32, seen_prev, lim)) {
              // produced by band wprev at its step tl + 31
              const R* x = xin + ((tl + 31) & (LU_XB - 1)) * 4;
#pragma unroll
              for (int n = 0; n < 4; ++n) bin[n] = x[n];
            } else {
              bad = true;
            }
          }
          cell(ch, rc, tl, c, bin);
        }
        // hand the boundary contribution to the next band (its slot must have
        // been read: the consumer is at least at step tl - LU_XB + 32), then
        // publish this band's progress
        if (l == lout) {
          if (act && has_next) {
            if (lu_wait_ge(&prog[wnext], tl - LU_XB + 32, seen_next, lim)) {
              R* x = xout + (tl & (LU_XB - 1)) * 4;
#pragma unroll
              for (int n = 0; n < 4; ++n) x[n] = bout[n];
            } else {
              bad = true;
            }
          }
          lu_st_release(&prog[w], tl + 1);
        }
      }
    }
    // group done: refill its buffer with group g + 2
    __syncwarp();
    if (l == 0 && g + 2 < ngrp) issue(g + 2);
  }
  if (__any_sync(0xffffffffu, bad) && gfail < 0) gfail = ngrp;
  if (gfail >= 0) {
    if (l == lout) lu_st_release(&prog[w], 1 << 30);  // release a waiting neighbour
    if (l == 0) {
      // copies issued and not consumed: groups gfail .. gfail+1; wait
      // (bounded) before the CTA's shared memory goes away, then flag
      for (int g = gfail; g < gfail + 2 && g < ngrp; ++g) mbar_wait_bounded(&bar[g & 1], (uint32_t)((g >> 1) & 1));
      if (S.ist) atomicOr(&S.ist[2], 4);
    }
  }
}

}  // namespace ot2d
