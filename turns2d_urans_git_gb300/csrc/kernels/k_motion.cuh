// k_motion.cuh -- the time-accurate moving-grid step of the reference's
// unsteady path (iunst = 1, motiontype = 1), once per physical time step,
// before its Newton iterations (src/Turns_overset.f:362-403):
//   pitch   src/motion.f:546-632  rotate cell centres and vertices by the
//                                 step's increment about (xac, yac); cell
//                                 grid speeds (first / second order); shift
//                                 the two previous vertex levels
//   stqol   src/time.f:110-175    Newton target qnewt and the stored levels
//   metfv   src/setup.f:440-724   J and the J-scaled metrics of the moved
//                                 grid, halo copies and the wake mirror
//   rhsup   src/eulerrhs.f:102-139, :209-246  face normals and the face
//                                 speeds from the areas the faces sweep
//   dist    src/samodel2d.f:243-293  SA wall distance of the moved centres
//   komegabc wall term            komegasst.f:1000-1007, :1042-1049
// All geometry is FP64 (the compute copies of the mixed path are rounded
// from it), evaluated in the reference's operation order; the sines and
// cosines of the increments come from a per-step table computed on the host
// (the same libm values the host oracle uses).
#pragma once
#include "dev_common.cuh"

namespace ot2d {

// 1-based (jd,kd) and (jmax,kmax) offsets
__device__ __forceinline__ int64_t mv_at(int jm, int j, int k) { return (int64_t)(k - 1) * jm + (j - 1); }

// Does this slice start a physical time step in this iteration?
template <class R>
__device__ __forceinline__ bool mv_new_step(const Slice<R>& S) {
  return S.xc && S.ist && S.ist[4] == 1;
}

// stqol (time.f:128-168) for one element o of q / qtn / qtnm1 / qnewt
__device__ __forceinline__ void mv_stqol_elem(const double* q, double* qtn, double* qtnm1, double* qnewt, int64_t o,
                                              int ntac, int istep) {
  const bool c1 = (ntac == 2 && istep > 1) || (ntac == 3 && istep == 2);
  const bool c2 = ntac == 3 && istep > 2;
  const double qv = q[o], qt = qtn[o];
  double v = qv;
  if (c1) v = v + (qv - qt) / 3.;
  if (c2) v = v + 7. * (qv - qt) / 11. - 2. * (qt - qtnm1[o]) / 11.;
  qnewt[o] = v;
  qtnm1[o] = qt;
  qtn[o] = qv;
}

// Phase A (one thread per cell of the slice; the first jmax*kmax threads
// also own one vertex): pitch and stqol.
template <class R>
__device__ void mv_pitch_cell(const Slice<R>& S, int cid) {
  const ot2d_params& p = *S.P;
  const int istep = S.ist[1];
  if (istep < 1 || istep > S.nmotion) {   // no table entry: flag, leave the grid
    if (cid == 0) atomicOr(&S.ist[2], 8);
    return;
  }
  const double* m = S.motion + 4 * (int64_t)(istep - 1);
  const double sn = m[0], cn = m[1], snold = m[2], cnold = m[3];
  const int64_t n2 = (int64_t)S.jd * S.kd;
  if (cid < n2) {
    // motion.f:585-605
    const double x = S.xc[cid], y = S.yc[cid];
    const double xnew = (x - p.xac) * cn + (y - p.yac) * sn + p.xac;
    const double ynew = -((x - p.xac) * sn) + (y - p.yac) * cn + p.yac;
    double ug, vg;
    if (p.ntac == 1) {
      ug = (xnew - x) / p.dt;
      vg = (ynew - y) / p.dt;
    } else {
      const double xo = (x - p.xac) * cnold + (y - p.yac) * snold + p.xac;
      const double yo = -((x - p.xac) * snold) + (y - p.yac) * cnold + p.yac;
      ug = (1.5 * xnew - 2. * x + 0.5 * xo) / p.dt;
      vg = (1.5 * ynew - 2. * y + 0.5 * yo) / p.dt;
    }
    S.xc[cid] = xnew;
    S.yc[cid] = ynew;
    const_cast<double*>(S.ug64)[cid] = ug;
    const_cast<double*>(S.vg64)[cid] = vg;
    if constexpr (sizeof(R) != sizeof(double)) {
      const_cast<R*>(S.ug)[cid] = (R)ug;
      const_cast<R*>(S.vg)[cid] = (R)vg;
    }
    // stqol, element by element
    if (S.qnewt)
      for (int n = 0; n < p.nv; ++n)
        mv_stqol_elem(S.q64, S.qtn, S.qtnm1, S.qnewt, (int64_t)n * S.qs + cid, p.ntac, istep);
  }
  if (cid < (int64_t)p.jmax * p.kmax) {
    // motion.f:607-624
    const double xo = S.xv[cid], yo = S.yv[cid];
    S.xole[cid] = S.xold[cid];
    S.yole[cid] = S.yold[cid];
    S.xold[cid] = xo;
    S.yold[cid] = yo;
    S.xv[cid] = (xo - p.xac) * cn + (yo - p.yac) * sn + p.xac;
    S.yv[cid] = -((xo - p.xac) * sn) + (yo - p.yac) * cn + p.yac;
  }
}

// Phase B (one thread per cell (j,k)): interior metrics and J, the face
// normals and face speeds whose home cell this is, and the wall distances.
template <class R>
__device__ void mv_geom_cell(const Slice<R>& S, int j, int k) {
  const ot2d_params& p = *S.P;
  const int jd = S.jd, jm = p.jmax, nh = p.nhalo;
  const int64_t o = mv_at(jd, j, k);
  const double* xv = S.xv;
  const double* yv = S.yv;
  auto XV = [&](int a, int b) { return xv[mv_at(jm, a, b)]; };
  auto YV = [&](int a, int b) { return yv[mv_at(jm, a, b)]; };
  // metfv interior (setup.f: J from the cell diagonals, J-scaled metrics)
  if (j >= p.jbeg && j <= p.jend && k >= p.kbeg && k <= p.kend) {
    const int a = j - nh + 1, b = k - nh + 1;
    const double dx1 = XV(a, b) - XV(a - 1, b - 1), dy1 = YV(a, b) - YV(a - 1, b - 1);
    const double dx2 = XV(a - 1, b) - XV(a, b - 1), dy2 = YV(a - 1, b) - YV(a, b - 1);
    const double qj = 1. / (0.5 * (dx1 * dy2 - dx2 * dy1));
    const double xx = qj * (0.5 * (YV(a, b) - YV(a, b - 1) + YV(a - 1, b) - YV(a - 1, b - 1)));
    const double xy = qj * (-(0.5 * (XV(a, b) - XV(a, b - 1) + XV(a - 1, b) - XV(a - 1, b - 1))));
    const double yx = qj * (-(0.5 * (YV(a, b) - YV(a - 1, b) + YV(a, b - 1) - YV(a - 1, b - 1))));
    const double yy = qj * (0.5 * (XV(a, b) - XV(a - 1, b) + XV(a, b - 1) - XV(a - 1, b - 1)));
    S.q64[(int64_t)(p.nq - 1) * S.qs + o] = qj;
    const_cast<double*>(S.xx64)[o] = xx; const_cast<double*>(S.xy64)[o] = xy;
    const_cast<double*>(S.yx64)[o] = yx; const_cast<double*>(S.yy64)[o] = yy;
    if constexpr (sizeof(R) != sizeof(double)) {
      S.q[(int64_t)(p.nq - 1) * S.qs + o] = (R)qj;
      const_cast<R*>(S.xx)[o] = (R)xx; const_cast<R*>(S.xy)[o] = (R)xy;
      const_cast<R*>(S.yx)[o] = (R)yx; const_cast<R*>(S.yy)[o] = (R)yy;
    }
    if (qj <= 0.0) atomicOr(&S.ist[2], 16);   // a folded cell
  }
  const int istep = S.ist[1];
  const bool second = p.ntac == 2 && istep > 1;
  const double* xo = S.xold;
  const double* yo = S.yold;
  const double* xe = S.xole;
  const double* ye = S.yole;
  auto XO = [&](int a, int b) { return xo[mv_at(jm, a, b)]; };
  auto YO = [&](int a, int b) { return yo[mv_at(jm, a, b)]; };
  auto XE = [&](int a, int b) { return xe[mv_at(jm, a, b)]; };
  auto YE = [&](int a, int b) { return ye[mv_at(jm, a, b)]; };
  // xi face (j, k): between cells j and j+1 of row k (eulerrhs.f:102-139)
  if (k >= p.kbeg && k <= p.kend && j >= p.jbeg - 1 && j <= p.jend) {
    const int a = j - nh + 1, b = k - nh + 1;
    const double fx = (YV(a, b) - YV(a, b - 1)), fy = -(XV(a, b) - XV(a, b - 1));
    double tj;
    {
      const double dx1 = XV(a, b) - XO(a, b - 1), dy1 = YV(a, b) - YO(a, b - 1);
      const double dx2 = XO(a, b) - XV(a, b - 1), dy2 = YO(a, b) - YV(a, b - 1);
      tj = -(0.5 * (dx1 * dy2 - dx2 * dy1) / p.dt);
    }
    if (second) {
      const double dx1 = XO(a, b) - XE(a, b - 1), dy1 = YO(a, b) - YE(a, b - 1);
      const double dx2 = XE(a, b) - XO(a, b - 1), dy2 = YE(a, b) - YO(a, b - 1);
      const double temp = -(0.5 * (dx1 * dy2 - dx2 * dy1) / p.dt);
      tj = 1.5 * tj - 0.5 * temp;
    }
    const_cast<R*>(S.fxa)[o] = (R)fx; const_cast<R*>(S.fya)[o] = (R)fy; const_cast<R*>(S.ftj)[o] = (R)tj;
  }
  // eta face (j, k): between cells k and k+1 of column j (eulerrhs.f:209-246)
  if (j >= p.jbeg && j <= p.jend && k >= p.kbeg - 1 && k <= p.kend) {
    const int a = j - nh + 1, b = k - nh + 1;
    const double gx = -(YV(a, b) - YV(a - 1, b)), gy = (XV(a, b) - XV(a - 1, b));
    double tj;
    {
      const double dx1 = XV(a, b) - XO(a - 1, b), dy1 = YV(a, b) - YO(a - 1, b);
      const double dx2 = XO(a, b) - XV(a - 1, b), dy2 = YO(a, b) - YV(a - 1, b);
      tj = 0.5 * (dx1 * dy2 - dx2 * dy1) / p.dt;
    }
    if (second) {
      const double dx1 = XO(a, b) - XE(a - 1, b), dy1 = YO(a, b) - YE(a - 1, b);
      const double dx2 = XE(a, b) - XO(a - 1, b), dy2 = YE(a, b) - YO(a - 1, b);
      const double temp = 0.5 * (dx1 * dy2 - dx2 * dy1) / p.dt;
      tj = 1.5 * tj - 0.5 * temp;
    }
    const_cast<R*>(S.gxa)[o] = (R)gx; const_cast<R*>(S.gya)[o] = (R)gy; const_cast<R*>(S.gtj)[o] = (R)tj;
  }
  // SA wall distance of the moved centres (dist, samodel2d.f:243-293)
  if (!p.lamin && p.iturb == 1) {
    double d;
    if (j >= p.jtail1 && j <= p.jtail2) {
      if (k == 1) {
        d = 0.0;
      } else {
        const int a = j - nh;
        const double fx = 0.5 * (XV(a, 1) + XV(a + 1, 1)), fy = 0.5 * (YV(a, 1) + YV(a + 1, 1));
        const double dx = S.xc[o] - fx, dy = S.yc[o] - fy;
        d = sqrt(dx * dx + dy * dy);
      }
    } else {
      const int a = p.jtail1 - nh;
      const double dx = S.xc[o] - XV(a, 1), dy = S.yc[o] - YV(a, 1);
      d = sqrt(dx * dx + dy * dy);
    }
    const_cast<R*>(S.sn)[o] = (R)d;
  }
}

// Phase B for the SST wall term (one thread per wall halo cell of the
// slice's type-5 boundaries): the same expression as the set-up.
template <class R>
__device__ void mv_sst_wall(const Slice<R>& S, int ib, int i) {
  const ot2d_params& p = *S.P;
  const int jd = S.jd, jm = p.jmax, nh = p.nhalo;
  int js = p.jbcs[ib], je = p.jbce[ib], ks = p.kbcs[ib], ke = p.kbce[ib];
  if (js < 0) js = p.jmax + js + 1;
  if (ks < 0) ks = p.kmax + ks + 1;
  if (je < 0) je = p.jmax + je + 1;
  if (ke < 0) ke = p.kmax + ke + 1;
  if (js > 1) js += nh;
  if (ks > 1) ks += nh;
  if (je < p.jmax) je += nh - 1;
  if (ke < p.kmax) ke += nh - 1;
  if (je == p.jmax) je = jd;
  if (ke == p.kmax) ke = S.kd;
  const int idir = p.ibdir[ib], iadd = idir >= 0 ? 1 : -1, iadir = idir < 0 ? -idir : idir;
  double* wd2 = const_cast<double*>(S.wd2);
  if (iadir == 1) {
    const int k = ks + i;
    if (k > ke) return;
    const int j = (idir == 1) ? je : js, j1 = j + iadd, jv = j1 - nh, kv = k - nh;
    const double dx = S.xc[mv_at(jd, j1, k)] - 0.5 * (S.xv[mv_at(jm, jv, kv)] + S.xv[mv_at(jm, jv, kv + 1)]);
    const double dy = S.yc[mv_at(jd, j1, k)] - 0.5 * (S.yv[mv_at(jm, jv, kv)] + S.yv[mv_at(jm, jv, kv + 1)]);
    wd2[mv_at(jd, j, k)] = dx * dx + dy * dy;
  } else if (iadir == 2) {
    const int j = js + i;
    if (j > je) return;
    const int k = (idir == 2) ? ke : ks, k1 = k + iadd, kv = k1 - nh, jv = j - nh;
    const double dx = S.xc[mv_at(jd, j, k1)] - 0.5 * (S.xv[mv_at(jm, jv, kv)] + S.xv[mv_at(jm, jv + 1, kv)]);
    const double dy = S.yc[mv_at(jd, j, k1)] - 0.5 * (S.yv[mv_at(jm, jv, kv)] + S.yv[mv_at(jm, jv + 1, kv)]);
    wd2[mv_at(jd, j, k)] = dx * dx + dy * dy;
  }
}

// Phase C (one CTA per slice): metfv's halo copies in its order -- the
// first / last interior column, then the first / last interior row over
// the extended column range, then the periodic (22) and wake-mirror (51)
// boundaries -- and the compute copies of the copied cells.
template <class R>
__device__ void mv_metric_halo(const Slice<R>& S) {
  const ot2d_params& p = *S.P;
  const int jd = S.jd, kd = S.kd;
  double* J = S.q64 + (int64_t)(p.nq - 1) * S.qs;
  double* xx = const_cast<double*>(S.xx64);
  double* xy = const_cast<double*>(S.xy64);
  double* yx = const_cast<double*>(S.yx64);
  double* yy = const_cast<double*>(S.yy64);
  auto cp = [&](int j, int k, int j1, int k1, double sgn) {
    const int64_t o = mv_at(jd, j, k), o1 = mv_at(jd, j1, k1);
    J[o] = J[o1];
    xx[o] = sgn * xx[o1]; xy[o] = sgn * xy[o1];
    yx[o] = sgn * yx[o1]; yy[o] = sgn * yy[o1];
    if constexpr (sizeof(R) != sizeof(double)) {
      S.q[(int64_t)(p.nq - 1) * S.qs + o] = (R)J[o];
      const_cast<R*>(S.xx)[o] = (R)xx[o]; const_cast<R*>(S.xy)[o] = (R)xy[o];
      const_cast<R*>(S.yx)[o] = (R)yx[o]; const_cast<R*>(S.yy)[o] = (R)yy[o];
    }
  };
  for (int k = p.kbeg + (int)threadIdx.x; k <= p.kend; k += blockDim.x) {
    cp(p.jbeg - 1, k, p.jbeg, k, 1.0);
    cp(p.jend + 1, k, p.jend, k, 1.0);
  }
  __syncthreads();
  for (int j = p.jbeg - 1 + (int)threadIdx.x; j <= p.jend + 1; j += blockDim.x) {
    cp(j, p.kbeg - 1, j, p.kbeg, 1.0);
    cp(j, p.kend + 1, j, p.kend, 1.0);
  }
  __syncthreads();
  for (int ib = 0; ib < p.nbc; ++ib) {
    int js = p.jbcs[ib], je = p.jbce[ib], ks = p.kbcs[ib], ke = p.kbce[ib];
    if (js < 0) js = p.jmax + js + 1;
    if (ks < 0) ks = p.kmax + ks + 1;
    if (je < 0) je = p.jmax + je + 1;
    if (ke < 0) ke = p.kmax + ke + 1;
    if (js > 1) js += p.nhalo;
    if (ks > 1) ks += p.nhalo;
    if (je < p.jmax) je += p.nhalo - 1;
    if (ke < p.kmax) ke += p.nhalo - 1;
    if (je == p.jmax) je = jd;
    if (ke == p.kmax) ke = kd;
    const int idir = p.ibdir[ib], t = p.ibtyp[ib];
    if (t == 22) {
      if (idir == 1 || idir == -1) {
        const int n = je - js + 1;
        for (int i = threadIdx.x; i < n * (ke - ks + 1); i += blockDim.x) {
          const int j = js + i % n, k = ks + i / n;
          const int jc = (idir == 1) ? jd - 2 * n + (j - js + 1) : 1 + 2 * n - (je - j + 1);
          cp(j, k, jc, k, 1.0);
        }
      } else {
        const int n = ke - ks + 1, nw = je - js + 1;
        for (int i = threadIdx.x; i < n * nw; i += blockDim.x) {
          const int j = js + i % nw, k = ks + i / nw;
          const int kc = (idir == 2) ? kd - 2 * n + (k - ks + 1) : 1 + 2 * n - (ke - k + 1);
          cp(j, k, j, kc, 1.0);
        }
      }
    } else if (t == 51 && (idir == 2 || idir == -2)) {
      // wake halo: the mirrored cell across the cut, metrics negated; the
      // two halves are written in the reference's order (j, then jd-j+1)
      const int nw = je - js + 1;
      for (int kc = 1; kc <= ke - ks + 1; ++kc) {
        const int k = (idir == 2) ? ke - kc + 1 : ks + kc - 1;
        const int k1 = (idir == 2) ? ke + kc : ks - kc;
        for (int i = threadIdx.x; i < nw; i += blockDim.x) {
          const int j = js + i, jj = jd - j + 1;
          cp(j, k, jj, k1, -1.0);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nw; i += blockDim.x) {
          const int j = js + i, jj = jd - j + 1;
          cp(jj, k, j, k1, -1.0);
        }
        __syncthreads();
      }
    }
    __syncthreads();
  }
}

}  // namespace ot2d
