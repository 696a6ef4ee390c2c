// k_lusgs.cuh -- LU-SGS hyperplane operator ilu2d (src/lhs.f:470-814).
//
// The reference sweeps i+j hyperplanes; cell (j,k) of the forward sweep
// needs the already-updated s(j-1,k) and s(j,k-1) (backward: j+1, k+1).
// Here one CTA owns one slice; warp w owns rows k = ks+32w .. ks+32w+31
// (lane l -> one row) and all warps advance in a skewed lockstep: at global
// step t lane l of warp w updates column j = js + t - 32w - l.  The (j-1,k)
// contribution stays in the lane's registers, the (j,k-1) contribution
// arrives from lane l-1 by __shfl_up_sync, and across warps through a
// double-buffered shared-memory slot.  Every cell sees exactly the operands
// of the reference's hyperplane order, so the result equals the sequential
// sweep operation for operation.
#pragma once
#include "dev_common.cuh"

namespace ot2d {

template <class R>
struct LuCell {
  R uu, vv, uv2, ge, ri1, ri2, rk1, rk2, qx, cx, qy, cy, vn, ugc, vgc, d;
};

// lhs.f:524-531 (conservative -> primitive) and :535-563 (diagonal)
template <class R>
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
  R cjkl = sqrt((R)p.ggm1 * (e - c.uv2));
  c.ri1 = S.xx[o]; c.ri2 = S.xy[o]; c.rk1 = S.yx[o]; c.rk2 = S.yy[o];
  c.ugc = S.ug ? S.ug[o] : (R)0; c.vgc = S.vg ? S.vg[o] : (R)0;
  R qq1 = c.ri1 * c.uu + c.ri2 * c.vv;
  R qqx = fabs(-c.ri1 * c.ugc - c.ri2 * c.vgc + qq1);
  R rr1 = sqrt(sq(c.ri1) + sq(c.ri2));
  R qq2 = c.rk1 * c.uu + c.rk2 * c.vv;
  R qqy = fabs(-c.rk1 * c.ugc - c.rk2 * c.vgc + qq2);
  R rr2 = sqrt(sq(c.rk1) + sq(c.rk2));
  R vnu = (R)2.0 * rr2 * rr2 * ((R)p.rmue + S.turmu[o]) / ((R)p.rey * rho);
  R svt = S.tscale[o];
  c.d = (R)1.0 / ((R)1.0 + svt * ((qqx + qqy + cjkl * (rr1 + rr2)) * epsv + vnu));
  c.qx = qq1; c.cx = cjkl * rr1; c.qy = qq2; c.cy = cjkl * rr2; c.vn = vnu;
  c.ge = (R)p.gamma * e - (R)p.gm1 * c.uv2;
  return c;
}

// Contribution of cell c with correction s to its neighbour, lhs.f:626-653
// (xi, forward), :656-683 (eta, forward), :725-752 / :755-782 (backward).
template <class R, bool XI, bool FWD>
__device__ __forceinline__ void lu_contrib(const LuCell<R>& c, const R* s, R gm1, R eps2, R* a) {
  R ri1 = XI ? c.ri1 : c.rk1, ri2 = XI ? c.ri2 : c.rk2, qq = XI ? c.qx : c.qy, cc = XI ? c.cx : c.cy;
  R qqn = -ri1 * c.ugc - ri2 * c.vgc + qq;
  R sp1 = fabs(qqn) + cc;
  R sm2 = eps2 * sp1;
  R chk, spec;
  if (FWD) {
    chk = (R)0.5 + fsign((R)0.5, qqn + cc);
    spec = XI ? chk * (qqn + sp1) + sm2 : chk * (qqn + sp1) + c.vn + sm2;
  } else {
    chk = (R)0.5 - fsign((R)0.5, qqn - cc);
    spec = XI ? chk * (qqn - sp1) - sm2 : chk * (qqn - sp1) - c.vn - sm2;
  }
  R s1 = s[0], s2 = s[1], s3 = s[2], s4 = s[3];
  R a4 = chk * (ri1 * s2 + ri2 * s3 - qq * s1);
  R a2 = chk * gm1 * (c.uv2 * s1 - (c.uu * s2 + c.vv * s3) + s4);
  a[0] = a4 + spec * s1;
  a[1] = ri1 * a2 + c.uu * a4 + spec * s2;
  a[2] = ri2 * a2 + c.vv * a4 + spec * s3;
  a[3] = qq * a2 + c.ge * a4 + spec * s4;
}

// Point-Jacobi scaling of the four halo edges (lhs.f:567-598); all threads
// of the CTA.
template <class R>
__device__ void lu_halo_scale(const Slice<R>& S, const ot2d_params& p, R epsv) {
  const int js = p.jbeg, je = p.jend, ks = p.kbeg, ke = p.kend;
  const int nk = ke - ks + 1, nj = je - js + 1;
  const int tot = 2 * nk + 2 * nj;
  for (int i = threadIdx.x; i < tot; i += blockDim.x) {
    int j, k;
    if (i < nk) { j = js - 1; k = ks + i; }
    else if (i < 2 * nk) { j = je + 1; k = ks + i - nk; }
    else if (i < 2 * nk + nj) { j = js + i - 2 * nk; k = ks - 1; }
    else { j = js + i - 2 * nk - nj; k = ke + 1; }
    LuCell<R> c = lu_cell(S, p, j, k, epsv);
    const int64_t o = at(S.jd, j, k);
#pragma unroll
    for (int n = 0; n < 4; ++n) S.s[n * S.qs + o] = S.s[n * S.qs + o] * c.d;
  }
}

// One sweep of one slice.  FWD: lhs.f:611-714, else :716-800.
template <class R, bool FWD>
__device__ void lu_sweep(const Slice<R>& S, R (*xbuf)[4]) {
  const ot2d_params& p = *S.P;
  const int js = p.jbeg, je = p.jend, ks = p.kbeg, ke = p.kend;
  const int ncol = je - js + 1, nrow = ke - ks + 1;
  const int nw = (nrow + 31) >> 5;
  const R eps2 = (R)(p.epse * 2.), epsv = (R)1. + eps2, gm1 = (R)p.gm1;
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const int r = 32 * w + l;                       // row offset from the sweep start
  const bool rowok = (w < nw) && (r < nrow);
  const int k = FWD ? ks + r : ke - r;
  const int T = ncol + 31 + 32 * (nw - 1);
  R aprev[4] = {0, 0, 0, 0};                      // contribution of (j-+1, k) for this lane
  R bout[4] = {0, 0, 0, 0};                       // this lane's last contribution to row k+-1
  const int64_t qs = S.qs;
  for (int t = 0; t < T; ++t) {
    // contribution from the row below (FWD) / above, computed one step ago
    R bin[4];
#pragma unroll
    for (int n = 0; n < 4; ++n) bin[n] = __shfl_up_sync(0xffffffffu, bout[n], 1);
    const int tl = t - 32 * w;
    const int jo = tl - l;                        // column offset from the sweep start
    const bool act = rowok && jo >= 0 && jo < ncol;
    if (act) {
      const int j = FWD ? js + jo : je - jo;
      if (l == 0) {
        if (w == 0) {
          // neighbour is the halo row ks-1 (FWD) / ke+1 (backward)
          const int kh = FWD ? ks - 1 : ke + 1;
          LuCell<R> hc = lu_cell(S, p, j, kh, epsv);
          R sh[4];
          const int64_t oh = at(S.jd, j, kh);
#pragma unroll
          for (int n = 0; n < 4; ++n) sh[n] = S.s[n * qs + oh];
          lu_contrib<R, false, FWD>(hc, sh, gm1, eps2, bin);
        } else {
#pragma unroll
          for (int n = 0; n < 4; ++n) bin[n] = xbuf[2 * (w - 1) + ((t - 1) & 1)][n];
        }
      }
      if (jo == 0) {
        const int jh = FWD ? js - 1 : je + 1;
        LuCell<R> hc = lu_cell(S, p, jh, k, epsv);
        R sh[4];
        const int64_t oh = at(S.jd, jh, k);
#pragma unroll
        for (int n = 0; n < 4; ++n) sh[n] = S.s[n * qs + oh];
        lu_contrib<R, true, FWD>(hc, sh, gm1, eps2, aprev);
      }
      LuCell<R> c = lu_cell(S, p, j, k, epsv);
      const int64_t o = at(S.jd, j, k);
      const R sv = S.tscale[o] * (R)0.5, di = c.d;
      R sn[4];
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        R st = S.s[n * qs + o];
        sn[n] = FWD ? (st + sv * (aprev[n] + bin[n])) * di : st - sv * (aprev[n] + bin[n]) * di;
        S.s[n * qs + o] = sn[n];
      }
      lu_contrib<R, true, FWD>(c, sn, gm1, eps2, aprev);
      lu_contrib<R, false, FWD>(c, sn, gm1, eps2, bout);
      if (l == 31 && w + 1 < nw) {
#pragma unroll
        for (int n = 0; n < 4; ++n) xbuf[2 * w + (t & 1)][n] = bout[n];
      }
    }
    __syncthreads();
  }
}

// FP64 plain path: the reference leaves q round-tripped through
// (rho*J, u, v, e) and back (lhs.f:524-531, :805-811); reproduce it.
template <class R>
__device__ void lu_roundtrip(const Slice<R>& S, const ot2d_params& p) {
  if constexpr (sizeof(R) != sizeof(double)) {
    return;
  } else {
    const int jd = p.jd, kd = p.kd; const int64_t qs = S.qs;
    const int js = p.jbeg - 1, je = p.jend + 1, ks = p.kbeg - 1, ke = p.kend + 1;
    const int nj = je - js + 1, tot = nj * (ke - ks + 1);
    (void)jd; (void)kd;
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
      int j = js + i % nj, k = ks + i / nj;
      const int64_t o = at(S.jd, j, k);
      double q1 = S.q[o], J = S.q[(p.nq - 1) * qs + o];
      double dj = 1.0 / q1;
      double u = S.q[qs + o] * dj, v = S.q[2 * qs + o] * dj, e = S.q[3 * qs + o] * dj;
      double r = q1 * J;
      double q1n = r / J;
      S.q[o] = q1n;
      S.q[qs + o] = u * q1n;
      S.q[2 * qs + o] = v * q1n;
      S.q[3 * qs + o] = e * q1n;
    }
  }
}

}  // namespace ot2d
