// kernels.cuh -- __global__ entry points over a ragged batch of slices.
// Included by one translation unit per arithmetic type (kernels_fp64.cu,
// kernels_fp32.cu) which instantiates the launchers.
#pragma once
#include "dev_common.cuh"
#include "k_bc.cuh"
#include "k_rhs.cuh"
#include "k_quad.cuh"
#include "k_lusgs.cuh"
#include "k_sa.cuh"
#include "k_sst.cuh"
#include "k_adi.cuh"
#include "k_misc.cuh"
#include "k_motion.cuh"
#include "launch.h"
#include "k_resid.cuh"

namespace ot2d {

// true when the speed of sound squared of state q (Q/J, 4 variables) is at
// or below 0.002 or not finite (the reference's mstop, step.f:366-368);
// evaluated in T (the mixed path checks its f32 copy of the updated state)
template <class T>
__device__ __forceinline__ bool monitor_bad(T ggm1, const T* q) {
  const T q1 = q[0], qq = q[1] * q[1] + q[2] * q[2];
  const T lhs = ggm1 * (q[3] * q1 - (T)0.5 * qq), rhs = (T)0.002 * q1 * q1;
  return !(q1 > (T)0) || !(lhs > rhs) || !isfinite(lhs);
}

// Cell-parallel mapping: slice i owns blocks [first[i], first[i+1]) of
// CELL_BS threads each, covering its jd*kd cells.
// Streaming kernels (a few loads and stores per cell) run CELL_BS / CELL_PT
// threads per block of CELL_BS cells, each thread CELL_PT cells CELL_BS /
// CELL_PT apart (coalesced per pass): the same prefix tables, and CELL_PT
// times the loads in flight per block for the one slice lookup of the
// block.
constexpr int CELL_PT = 4;
#define OT2D_CELL_MAP_PT()                                                    \
  const int si = find_slice(first, nslice, blockIdx.x);                      \
  const Slice<R>& S = sl[si];                                                \
  const int cid0 = (blockIdx.x - first[si]) * CELL_BS + threadIdx.x;         \
  const int ncell = S.jd * S.kd;

#define OT2D_CELL_MAP()                                                      \
  const int si = find_slice(first, nslice, blockIdx.x);                      \
  const Slice<R>& S = sl[si];                                                \
  const int cid = (blockIdx.x - first[si]) * blockDim.x + threadIdx.x;       \
  const int j = cid % S.jd + 1, k = cid / S.jd + 1;                          \
  const bool inside = cid < S.jd * S.kd;

template <class R>
__global__ void __launch_bounds__(CELL_BS / CELL_PT) k_time_step(const Slice<R>* __restrict__ sl,
                                                                 const int32_t* __restrict__ first, int nslice) {
  OT2D_CELL_MAP_PT();
  const ot2d_params& p = *S.P;
  int istep = S.ist ? S.ist[1] : p.istep;   // advanced by k_iter_begin
  R oat = (R)1.0;
  if (p.ntac >= 2 && istep > 1) oat = (R)(2. / 3.);
  if (p.ntac == 3 && istep > 2) oat = (R)(6. / 11.);
#pragma unroll
  for (int u = 0; u < CELL_PT; ++u) {
    const int cid = cid0 + u * (CELL_BS / CELL_PT);
    if (cid < ncell) time_step_cell(S, cid % S.jd + 1, cid / S.jd + 1, oat);
  }
}

// Start of a solver iteration (one thread per slice): the step counters of
// Turns_overset.f:362-364 -- advanced once per physical time step, i.e. at
// the first of the itnmax Newton iterations (:472-474) -- and the
// physical-time factor 1/(oat*h) of newton (time.f:195-200) in red[8].
template <class R>
__device__ __forceinline__ void iter_begin_slice(const Slice<R>& S) {
  if (!S.ist) return;
  const ot2d_params& p = *S.P;
  int itn = 1;
  if (p.itnmax > 1) itn = S.ist[4] % p.itnmax + 1;
  S.ist[4] = itn;
  if (itn == 1) { S.ist[0] += 1; S.ist[1] += 1; }
  const int istep = S.ist[1];
  double oat = 1.0;
  if (p.ntac >= 2 && istep > 1) oat = 2. / 3.;
  if (p.ntac == 3 && istep > 2) oat = 6. / 11.;
  if (S.red) S.red[8] = 1. / (oat * p.h);
}
template <class R>
__global__ void k_iter_begin(const Slice<R>* __restrict__ sl, int nslice) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nslice) iter_begin_slice(sl[i]);
}

// Moving slices at the start of a physical step: pitch + stqol (one thread
// per cell / vertex), then metrics, faces and wall distances (one thread per
// cell), then the metric halo and the SST wall term (one CTA per slice).
template <class R>
__global__ void __launch_bounds__(CELL_BS) k_mv_pitch(const Slice<R>* __restrict__ sl,
                                                      const int32_t* __restrict__ first, int nslice) {
  OT2D_CELL_MAP();
  (void)j; (void)k;
  if (!inside || !mv_new_step(S)) return;
  mv_pitch_cell(S, cid);
}
template <class R>
__global__ void __launch_bounds__(CELL_BS) k_mv_geom(const Slice<R>* __restrict__ sl,
                                                     const int32_t* __restrict__ first, int nslice) {
  OT2D_CELL_MAP();
  if (!inside || !mv_new_step(S)) return;
  mv_geom_cell(S, j, k);
}
template <class R>
__global__ void k_mv_halo(const Slice<R>* __restrict__ sl) {
  const Slice<R>& S = sl[blockIdx.x];
  if (!mv_new_step(S)) return;   // uniform over the CTA
  const ot2d_params& p = *S.P;
  if (!p.lamin && p.iturb == 2 && S.wd2)
    for (int ib = 0; ib < p.nbc; ++ib)
      if (p.ibtyp[ib] == 5)
        for (int i = threadIdx.x; i < S.jd + S.kd; i += blockDim.x) mv_sst_wall(S, ib, i);
  mv_metric_halo(S);
}

// bc.f:2-86, BC entry ib of every slice (grid: blockIdx.y = slice,
// blockIdx.x = part of the entry's cells); slices with fewer entries return
template <class R>
__global__ void __launch_bounds__(BCE_BS) k_bc_entry(const Slice<R>* __restrict__ sl, int ib) {
  const Slice<R>& S = sl[blockIdx.y];
  if (ib >= S.nbc) return;
  const int istep0 = S.ist ? S.ist[0] : S.P->istep0;
  bc_entry(S, istep0, ib, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// after the entries: the compute copy of the halo ring and its monitor
template <class R>
__device__ __forceinline__ void bc_ring_monitor(const Slice<R>& S, int advance);
template <class R>
__global__ void __launch_bounds__(BC_BS) k_bc(const Slice<R>* __restrict__ sl, int advance) {
  bc_ring_monitor(sl[blockIdx.x], advance);
}
// All &bcinp entries of a slice in one CTA, in the reference's order with a
// block barrier between entries (entries share corner cells), then the halo
// ring and its monitor: one launch instead of one per entry for the mixed
// path, whose boundary arithmetic is f32 (the FP64 path keeps several CTAs
// per entry: its boundary arithmetic runs on the narrow FP64 pipe).
template <class R>
__global__ void __launch_bounds__(BC_BS) k_bc_all(const Slice<R>* __restrict__ sl, int advance, int begin) {
  const Slice<R>& S = sl[blockIdx.x];
  if (begin) {
    if (threadIdx.x == 0) iter_begin_slice(S);
    __syncthreads();
  }
  const int istep0 = S.ist ? S.ist[0] : S.P->istep0;
  for (int ib = 0; ib < S.nbc; ++ib) {
    bc_entry(S, istep0, ib, threadIdx.x, blockDim.x);
    __syncthreads();
  }
  bc_ring_monitor(S, advance);
}
template <class R>
__device__ __forceinline__ void bc_ring_monitor(const Slice<R>& S, int advance) {
  widen_ring(S, 1, 4);
  // monitor of the halo ring just set (the interior is checked by k_update)
  if (S.ist && advance) {
    const int jd = S.jd, kd = S.kd, nring = 2 * jd + 2 * (kd - 2);
    bool bad = false;
    for (int i = threadIdx.x; i < nring; i += blockDim.x) {
      int j, k;
      if (i < jd) { j = i + 1; k = 1; }
      else if (i < 2 * jd) { j = i - jd + 1; k = kd; }
      else if (i < 2 * jd + kd - 2) { j = 1; k = i - 2 * jd + 2; }
      else { j = jd; k = i - (2 * jd + kd - 2) + 2; }
      const int64_t o = at(jd, j, k);
      const R qh[4] = {S.q[o], S.q[S.qs + o], S.q[2 * S.qs + o], S.q[3 * S.qs + o]};
      bad = bad || monitor_bad<R>(S.k_ggm1, qh);
    }
    if (bad) atomicOr(&S.ist[2], 2);
  }
}

template <class R>
__global__ void __launch_bounds__(CELL_BS) k_faces(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ first,
                                                   int nslice) {
  OT2D_CELL_MAP();
  if (!inside) return;
  const ot2d_params& p = *S.P;
  R* F = S.w + 0 * S.wstride;
  R* G = S.w + 4 * S.wstride;
  if (k >= p.kbeg && k <= p.kend && j >= p.jbeg - 1 && j <= p.jend) xi_face(S, j, k, F);
  if (j >= p.jbeg && j <= p.jend && k >= p.kbeg - 1 && k <= p.kend) eta_face(S, j, k, G);
}

template <class R>
__global__ void __launch_bounds__(CELL_BS) k_visc(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ first,
                                                  int nslice) {
  OT2D_CELL_MAP();
  if (!inside) return;
  const ot2d_params& p = *S.P;
  if (p.invisc) return;
  if (j >= p.jbeg && j <= p.jend && k <= S.kd - 1) visc_eta_face(S, j, k, S.w + 8 * S.wstride);
  if (k >= p.kbeg && k <= p.kend && j <= S.jd - 1) visc_xi_face(S, j, k, S.w + 14 * S.wstride);
}

// Residual assembly.  flags: AS_ACC start from the incoming s and leave
// halo cells alone (the drop-in rhsup / visrhs / timespectralrhs, which add
// into s); otherwise start from 0 on every cell (step.f:41).  AS_INV adds the
// inviscid face fluxes, AS_VISC the viscous ones (slices with invisc skip
// them), AS_TS the time-spectral term, AS_NORM the per-block norm partials.
template <class R>
__global__ void __launch_bounds__(CELL_BS) k_assemble(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ first,
                                                      int nslice, int flags, NormPart* __restrict__ part) {
  OT2D_CELL_MAP();
  __shared__ NormPart sh[CELL_BS];
  NormPart np{0.0, 0.0, 0.0, 0x7fffffffffffffffLL};
  if (inside) {
    const ot2d_params& p = *S.P;
    const int64_t o = at(S.jd, j, k);
    const int nv = p.nv;
    const bool acc = flags & AS_ACC;
    R s[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) s[n] = (R)0.0;
    const bool interior = j >= p.jbeg && j <= p.jend && k >= p.kbeg && k <= p.kend;
    if (interior) {
      if (acc)
        for (int n = 1; n <= nv; ++n) s[n - 1] = S.s[(int64_t)(n - 1) * S.qs + o];
      const bool visc = (flags & AS_VISC) && !p.invisc;
      const R* F = (flags & AS_INV) ? S.w + 0 * S.wstride : nullptr;
      const R* G = (flags & AS_INV) ? S.w + 4 * S.wstride : nullptr;
      const R* VE = visc ? S.w + 8 * S.wstride : nullptr;
      const R* VX = visc ? S.w + 14 * S.wstride : nullptr;
      assemble_cell(S, j, k, F, G, VE, VX, s);
      if ((flags & AS_TS) && p.timespectral && S.Ds) ts_cell(S, p, S.Ds, j, k, s, nv);
      if (flags & AS_NORM) {
        // norms (step.f:67-88)
        int ibi = S.iblank[o];
        double m = (double)(ibi > 0 ? ibi : 0);
        for (int n = 1; n <= p.nmv; ++n) {
          double smrs = fabs((double)s[n - 1]) * m;
          long long key = ((long long)(k - 1) * (p.nmv + 1) + n) * (long long)S.jd + (j - 1);
          if (smrs > np.resmax || (smrs == np.resmax && key < np.key)) { np.resmax = smrs; np.key = key; }
        }
        double s1 = (double)s[0] * m, s2 = (double)s[1] * m, s3 = (double)s[2] * m, s4 = (double)s[3] * m;
        np.resrho = (double)s[0] * (double)s[0];
        np.rsum = s1 * s1 + s2 * s2 + s3 * s3 + s4 * s4;
      }
    }
    if (interior || !acc)
      for (int n = 1; n <= nv; ++n) S.s[(int64_t)(n - 1) * S.qs + o] = s[n - 1];
  }
  if (!(flags & AS_NORM)) return;
  // deterministic block reduction
  sh[threadIdx.x] = np;
  __syncthreads();
  for (int st = CELL_BS / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) sh[threadIdx.x] = norm_combine(sh[threadIdx.x], sh[threadIdx.x + st]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Fused residual over tiles of TJ x TK interior cells: slice i owns tiles
// [tfirst[i], tfirst[i+1]) (the batch's tile table is built for the same
// shape).  Dynamic shared memory: rt_smem_bytes<R, TJ, TK>().  PRE selects
// the preconditioned slices (k_mp2 >= 0) and LIM the reconstruction family
// (rt_lim_class); a batch launches one instantiation per kind it holds,
// each returning on the other kinds' tiles (a whole block returns, so every
// tile is done exactly once).  One family per kernel keeps the WENO windows
// out of the MUSCL kernel's registers and code.
// Occupancy: 1024 threads per SM (f32, 64 registers a thread) or 512 (f64).
template <class R, bool PRE, int LIM, int TJ, int TK>
__global__ void __launch_bounds__(TJ * TK, (sizeof(R) == 4 ? 1024 : 512) / (TJ * TK))
    k_resid(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ tfirst, int nslice, int flags,
            NormPart* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char rt_raw[];
  const int si = find_slice(tfirst, nslice, blockIdx.x);
  const Slice<R>& S = sl[si];
  if ((S.k_mp2 >= (R)0) != PRE || S.lim != LIM) return;
  RtSmem<R, TJ, TK> sm(rt_raw);
  NormPartR<R> npr{0.0, 0.0, (R)0, 0x7fffffffffffffffLL};
  resid_tile<R, PRE, LIM, TJ, TK>(S, sm, blockIdx.x - tfirst[si], flags, npr);
  if (!(flags & AS_NORM)) return;
  // Deterministic block reduction in a fixed order: every thread leaves its
  // cell's terms in the staged region (only the face passes read it, and
  // they are behind the tile's last barrier), then warp 0 sums the BS/32
  // values of each lane position in thread order and finishes with a
  // shuffle tree.  One warp does the FP64 additions of the whole tile.
  constexpr int BS = TJ * TK;
  static_assert((size_t)BS * (2 * sizeof(double) + sizeof(long long) + sizeof(R)) <=
                    sizeof(R) * (size_t)RS_N * RtGeo<TJ, TK>::NR, "partials fit in the staged region");
  double* prs = (double*)sm.c;
  double* prr = prs + BS;
  long long* pky = (long long*)(prr + BS);
  R* pmx = (R*)(pky + BS);
  const int t = threadIdx.x, lane = t & 31;
  prs[t] = npr.rsum; prr[t] = npr.resrho; pky[t] = npr.key; pmx[t] = npr.resmax;
  __syncthreads();
  if (t < 32) {
    NormPartR<R> a{prs[lane], prr[lane], pmx[lane], pky[lane]};
#pragma unroll
    for (int i = 1; i < BS / 32; ++i) {
      const int u = lane + 32 * i;
      a.rsum = a.rsum + prs[u];
      a.resrho = a.resrho + prr[u];
      const R m = pmx[u];
      const long long ky = pky[u];
      if (m > a.resmax || (m == a.resmax && ky < a.key)) { a.resmax = m; a.key = ky; }
    }
    a = warp_norm_reduce_r(a);
    if (lane == 0) part[blockIdx.x] = NormPart{a.rsum, a.resrho, to_d(a.resmax), a.key};
  }
}

// Per-slice norms from the block partials (fixed order): red[0..3] =
// rsum, resrho, resmax, key; status word on blow-up (step.f:105-110).
template <class R>
__global__ void k_norm_final(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ first, int nslice,
                             const NormPart* __restrict__ part) {
  const int si = blockIdx.x;
  const Slice<R>& S = sl[si];
  // one warp: lane l combines partials l, l+32, ... in order, then a fixed
  // shuffle tree over the lanes (the same order on every run)
  const int lane = threadIdx.x & 31;
  NormPart acc{0.0, 0.0, 0.0, 0x7fffffffffffffffLL};
  for (int b = first[si] + lane; b < first[si + 1]; b += 32) acc = norm_combine(acc, part[b]);
  acc = warp_norm_reduce(acc);
  if (lane != 0) return;
  double volum = (double)(S.jd * S.kd);
  double rsum = sqrt(acc.rsum / volum), resrho = sqrt(acc.resrho / volum);
  S.red[0] = rsum; S.red[1] = resrho; S.red[2] = acc.resmax; S.red[3] = (double)acc.key;
  if (S.ist) {
    const int it = S.ist[1];
    if (!(rsum <= 1000.0)) atomicOr(&S.ist[2], 1);   // L2 norm out of bounds (step.f:105-110)
    if (it == 1) S.red[4] = rsum;                 // first-iteration norm
    S.red[5] = rsum;
    if (rsum > S.red[6]) S.red[6] = rsum;         // running peak
    if (S.ist[3] == 0 && it > 1 && rsum <= S.red[6] * S.red[7]) S.ist[3] = it;  // converged at `it`
  }
}

// rhslom alone (sources.f:97-148): the drop-in routine's interior cells
template <class R>
__global__ void __launch_bounds__(CELL_BS) k_rhslom(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ first,
                                                    int nslice) {
  OT2D_CELL_MAP();
  const ot2d_params& p = *S.P;
  if (!inside || j < p.jbeg || j > p.jend || k < p.kbeg || k > p.kend) return;
  const int64_t o = at(S.jd, j, k);
  R s[4];
#pragma unroll
  for (int n = 0; n < 4; ++n) s[n] = S.s[(int64_t)n * S.qs + o];
  rhslom_cell(S, p, o, s);
#pragma unroll
  for (int n = 0; n < 4; ++n) S.s[(int64_t)n * S.qs + o] = s[n];
}

template <class R>
__global__ void k_rbc(const Slice<R>* __restrict__ sl) {
  const Slice<R>& S = sl[blockIdx.x];
  rbc_slice(S);
}

// ilu2d (lhs.f:470-814), preceded by s *= tscale on all cells when `scale`
// (step.f:141-148).  Records of the interior cells (prefix table lfirst):
// a block of LU_PREP_BS threads builds LU_PREP_CH = 16 consecutive chunks of
// the band layout.  Lane l of chunk (band, t) is cell (row 32 band + l,
// column t - l), so the chunks' lanes walk the grid diagonally; thread i
// computes lane i / 16 of chunk i % 16 instead, which makes sixteen
// consecutive threads read sixteen consecutive cells (64 bytes of each
// array) of one row (the lane-per-thread order would touch a different row,
// and cache line, per thread).  The records go to the block's shared-memory
// copy of its chunks (chunk stride padded by 16 bytes so the chunks of one
// row land in different banks), then each warp stores one chunk with one
// bulk copy.  PRE: the
// preconditioned (preilu2d) records of the slices with k_mp2 >= 0; each
// instantiation returns on the other kind's slices.
constexpr int LU_PREP_CH = LU_PREP_BS / 32;   // chunks per block
template <class R, bool PRE>
__host__ __device__ constexpr int lu_prep_stride() { return LuLay<R, PRE>::CH + (int)(16 / sizeof(R)); }
template <class R, bool PRE>
__global__ void __launch_bounds__(LU_PREP_BS) k_lu_prep(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ lfirst,
                                                     int nslice, int scale, int only_lu) {
  static_assert(LU_PREP_CH * 32 == LU_PREP_BS && (LU_PREP_CH & (LU_PREP_CH - 1)) == 0,
                "thread -> (chunk, lane) map: a power-of-two number of 32-lane chunks");
  extern __shared__ __align__(16) unsigned char lp_smem[];
  const int si = find_slice(lfirst, nslice, blockIdx.x);
  const Slice<R>& S = sl[si];
  if ((S.k_mp2 >= (R)0) != PRE) return;                    // uniform over the block
  if (only_lu && S.P->ilhs != 1) return;                   // uniform over the block
  const int nst = lu_nstep(S.jd), nb = lu_nband(S.kd);
  const int c0 = (blockIdx.x - lfirst[si]) * LU_PREP_CH;   // first chunk of the block
  constexpr int CH = LuLay<R, PRE>::CH, CHS = lu_prep_stride<R, PRE>();
  {
    const int w = threadIdx.x & (LU_PREP_CH - 1), l = threadIdx.x / LU_PREP_CH;
    const int c = c0 + w, band = c / nst, t = c - band * nst;
    if (band < nb) lu_prep_cell<R, PRE>(S, *S.P, band, t, l, scale, (R*)lp_smem + w * CHS);
  }
  __syncthreads();
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const int c = c0 + w, band = c / nst;
  if (band >= nb || l != 0) return;
  // one bulk copy (TMA) per staged chunk, shared -> global: chunk (band, t)
  // is chunk band*nst + t; both ends 16-byte aligned, 16-byte multiple size
  static_assert((CH * sizeof(R)) % 16 == 0 && (CHS * sizeof(R)) % 16 == 0, "bulk copy alignment");
  R* dst = S.lurec + (int64_t)c * CH;
  const R* src = (const R*)lp_smem + w * CHS;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
               "r"((uint32_t)__cvta_generic_to_shared(src)), "r"((uint32_t)(CH * sizeof(R)))
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  // the shared source must be read before the block's shared memory goes
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

template <class R, bool PRE>
__global__ void __launch_bounds__(CELL_BS) k_lu_edges(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ first,
                                                      int nslice, int scale, int only_lu) {
  OT2D_CELL_MAP();
  if (!inside || (only_lu && S.P->ilhs != 1) || (S.k_mp2 >= (R)0) != PRE) return;
  lu_edge_cell<R, PRE>(S, *S.P, j, k, scale);
}

// The same over the halo ring only (one halo layer): the f32 path has no
// q round trip, so only the ring cells have work.  grid: (ring parts, slices)
template <class R, bool PRE>
__global__ void __launch_bounds__(128) k_lu_edges_ring(const Slice<R>* __restrict__ sl, int scale, int only_lu) {
  const Slice<R>& S = sl[blockIdx.y];
  if ((only_lu && S.P->ilhs != 1) || (S.k_mp2 >= (R)0) != PRE) return;
  const int jd = S.jd, kd = S.kd, nring = 2 * jd + 2 * (kd - 2);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nring) return;
  int j, k;
  if (i < jd) { j = i + 1; k = 1; }
  else if (i < 2 * jd) { j = i - jd + 1; k = kd; }
  else if (i < 2 * jd + kd - 2) { j = 1; k = i - 2 * jd + 2; }
  else { j = jd; k = i - (2 * jd + kd - 2) + 2; }
  lu_edge_cell<R, PRE>(S, *S.P, j, k, scale);
}

template <class R, bool FWD, int G, bool PRE>
__global__ void k_lu_sweep(const Slice<R>* __restrict__ sl, int only_lu, uint32_t poll_limit, int lag) {
  extern __shared__ __align__(128) unsigned char lu_smem[];
  if (only_lu && sl[blockIdx.x].P->ilhs != 1) return;
  if ((sl[blockIdx.x].k_mp2 >= (R)0) != PRE) return;
  lu_sweep_slice<R, FWD, G, PRE>(sl[blockIdx.x], blockDim.x >> 5, lu_smem, poll_limit, lag);
}

// vmu_sa's closing turbc (with the velocities k_sa_prep stored at the start
// of the step) and c_turm on the halo ring (the interior was done by the
// k-line solve right after its update; turbc leaves interior cells
// unchanged).  The opening turbc runs inside k_sa_prep_bc.
template <class R>
__global__ void __launch_bounds__(BC_BS) k_turbc(const Slice<R>* __restrict__ sl) {
  const Slice<R>& S = sl[blockIdx.x];
  const ot2d_params& p = *S.P;
  if (p.lamin || p.iturb != 1) return;
  turbc_slice(S, S.w + W_U * S.wstride, S.w + W_V * S.wstride);
  shadow_ring(S, p.nmv + 1, p.nmv + 1);
  __syncthreads();
  const int jd = S.jd, kd = S.kd, nring = 2 * jd + 2 * (kd - 2);
  for (int i = threadIdx.x; i < nring; i += blockDim.x) {
    int j, k;
    if (i < jd) { j = i + 1; k = 1; }
    else if (i < 2 * jd) { j = i - jd + 1; k = kd; }
    else if (i < 2 * jd + kd - 2) { j = 1; k = i - 2 * jd + 2; }
    else { j = jd; k = i - (2 * jd + kd - 2) + 2; }
    sa_turm_cell(S, p, j, k);
  }
}

// k_sa_prep and the first turbc in one launch: blocks 0..nslice-1 apply
// turbc to their slice, with the cell velocities formed from q as k_sa_prep
// forms them, and the other blocks evaluate k_sa_prep's cells.  Neither part
// reads what the other writes (k_sa_prep: laminar viscosity and velocities
// from variables 1-4; turbc: variable n5 on the halo), so they run at once.
template <class R>
__global__ void __launch_bounds__(CELL_BS) k_sa_prep_bc(const Slice<R>* __restrict__ sl,
                                                        const int32_t* __restrict__ first, int nslice) {
  if ((int)blockIdx.x < nslice) {
    const Slice<R>& S = sl[blockIdx.x];
    const ot2d_params& p = *S.P;
    if (p.lamin || p.iturb != 1) return;
    turbc_slice<R>(S, nullptr, nullptr);
    shadow_ring(S, p.nmv + 1, p.nmv + 1);
    return;
  }
  const int bid = (int)blockIdx.x - nslice;
  const int si = find_slice(first, nslice, bid);
  const Slice<R>& S = sl[si];
  const int cid = (bid - first[si]) * blockDim.x + threadIdx.x;
  if (cid >= S.jd * S.kd) return;
  if (S.P->lamin || S.P->iturb != 1) return;
  sa_prep_cell(S, *S.P, cid % S.jd + 1, cid / S.jd + 1);
}

// RHS and bands of the SA solve (samodel2d.f:402-450, :96-134) on tiles of
// TJ x TK interior cells, the residual's tile table: every value read at a
// cell and its four neighbours is staged once per tile (region with a
// one-cell halo) in shared memory, then each thread assembles its cell.
template <class R, int TJ, int TK>
__global__ void __launch_bounds__(TJ * TK, (sizeof(R) == 4 ? 1024 : 512) / (TJ * TK))
    k_sa_rhs(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ tfirst, int nslice) {
  extern __shared__ __align__(16) unsigned char sa_raw[];
  const int si = find_slice(tfirst, nslice, blockIdx.x);
  const Slice<R>& S = sl[si];
  const ot2d_params& p = *S.P;
  if (p.lamin || p.iturb != 1) return;   // uniform over the block
  const int tile = blockIdx.x - tfirst[si];
  const int ntj = (p.jend - p.jbeg + TJ) / TJ;
  const int j0 = p.jbeg + (tile % ntj) * TJ, k0 = p.kbeg + (tile / ntj) * TK;
  const int j1 = min(j0 + TJ - 1, p.jend), k1 = min(k0 + TK - 1, p.kend);
  constexpr int RW = TJ + 2, NR = RW * (TK + 2);
  R* sm = (R*)sa_raw;
  const int jd = S.jd, kd = S.kd, t = threadIdx.x;
  const int64_t ws = S.wstride, n5 = p.nmv + 1, nq = p.nq;
  const bool gs = S.ug != nullptr;
  // every load of a thread's staged cells before the first store
  constexpr int NSTG = (NR + TJ * TK - 1) / (TJ * TK);
  R val[NSTG][SA_NST + 2];
#pragma unroll
  for (int i = 0; i < NSTG; ++i) {
    const int r = t + i * TJ * TK;
    const int j = j0 - 1 + r % RW, k = k0 - 1 + r / RW;
    if (r >= NR || j < 1 || j > jd || k < 1 || k > kd) continue;
    const int64_t o = at(jd, j, k);
    val[i][SA_U] = S.w[W_U * ws + o]; val[i][SA_V] = S.w[W_V * ws + o];
    val[i][SA_XX] = S.xx[o]; val[i][SA_XY] = S.xy[o]; val[i][SA_YX] = S.yx[o]; val[i][SA_YY] = S.yy[o];
    val[i][SA_Q5] = S.q[(n5 - 1) * S.qs + o];
    val[i][SA_NUL] = S.w[W_VMUL * ws + o];      // vmul, q1, J: nul below
    val[i][SA_NST] = S.q[o];
    val[i][SA_NST + 1] = S.q[(nq - 1) * S.qs + o];
    if (gs) { val[i][SA_UG] = S.ug[o]; val[i][SA_VG] = S.vg[o]; }
  }
#pragma unroll
  for (int i = 0; i < NSTG; ++i) {
    const int r = t + i * TJ * TK;
    const int j = j0 - 1 + r % RW, k = k0 - 1 + r / RW;
    if (r >= NR || j < 1 || j > jd || k < 1 || k > kd) continue;
#pragma unroll
    for (int a = 0; a < SA_UG; ++a)
      sm[a * NR + r] = a == SA_NUL ? val[i][SA_NUL] / val[i][SA_NST] / val[i][SA_NST + 1] : val[i][a];
    if (gs) { sm[SA_UG * NR + r] = val[i][SA_UG]; sm[SA_VG * NR + r] = val[i][SA_VG]; }
  }
  __syncthreads();
  bool bodyflag = false;
  for (int ib = 0; ib < p.nbc; ++ib) if (p.ibtyp[ib] == 5) bodyflag = true;
  const int j = j0 + t % TJ, k = k0 + t / TJ;
  if (j <= j1 && k <= k1) sa_rhs_cell(S, p, j, k, bodyflag, SaTile<R>{sm, NR, RW, j0 - 1, k0 - 1, gs});
}
template <class R, int TJ, int TK>
__host__ __device__ constexpr size_t sa_rhs_smem() {
  return sizeof(R) * (size_t)SA_NST * (TJ + 2) * (TK + 2);
}

// line solves: slice i owns lines [lfirst[i], lfirst[i+1]) (one thread each)
template <class R>
__global__ void k_sa_lsolve(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ lfirst, int nslice, int dir) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= lfirst[nslice]) return;
  int lo = 0, hi = nslice - 1;
  while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (lfirst[mid] <= gid) lo = mid; else hi = mid - 1; }
  const Slice<R>& S = sl[lo];
  const ot2d_params& p = *S.P;
  if (p.lamin || p.iturb != 1) return;
  const int line = gid - lfirst[lo];
  if (dir == 0) { int k = p.kbeg + line; if (k <= p.kend) sa_lsolvej_line(S, p, k); }
  else { int j = p.jbeg + line; if (j <= p.jend) sa_lsolvek_line(S, p, j); }
}

// lsolvej by CTAs of 32 k-lines (two warps: elimination and data
// movement); slice i owns groups [gfirst[i], gfirst[i+1])
template <class R>
__global__ void __launch_bounds__(LJ_THREADS) k_sa_lsolvej(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ gfirst,
                                                   int nslice) {
  extern __shared__ __align__(16) unsigned char lj_raw[];
  R* sm = (R*)lj_raw;   // LJ_SMEM elements
  const int si = find_slice(gfirst, nslice, blockIdx.x);
  const Slice<R>& S = sl[si];
  const ot2d_params& p = *S.P;
  if (p.lamin || p.iturb != 1) return;
  sa_lsolvej_group(S, p, 32 * (blockIdx.x - gfirst[si]), sm);
}

// ---- k-omega SST (komegasst.f:2-187) ---------------------------------------
template <class R>
__global__ void __launch_bounds__(CELL_BS) k_sst_prep(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ first,
                                                      int nslice) {
  OT2D_CELL_MAP();
  if (!inside || !sst_slice(*S.P)) return;
  sst_prep_cell(S, *S.P, j, k);
}

// komegabc on one CTA per slice; final pass: the second komegabc followed by
// findturm on the halo ring (the interior was done by the k-line solve)
template <class R>
__global__ void k_sst_bc(const Slice<R>* __restrict__ sl, int final_pass) {
  const Slice<R>& S = sl[blockIdx.x];
  const ot2d_params& p = *S.P;
  if (!sst_slice(p)) return;
  sst_bc_slice(S, S.wd2);
  shadow_ring(S, p.nmv + 1, p.nmv + 2);
  if (final_pass) {
    __syncthreads();
    const int jd = S.jd, kd = S.kd, nring = 2 * jd + 2 * (kd - 2);
    for (int i = threadIdx.x; i < nring; i += blockDim.x) {
      int j, k;
      if (i < jd) { j = i + 1; k = 1; }
      else if (i < 2 * jd) { j = i - jd + 1; k = kd; }
      else if (i < 2 * jd + kd - 2) { j = 1; k = i - 2 * jd + 2; }
      else { j = jd; k = i - (2 * jd + kd - 2) + 2; }
      sst_turm_cell(S, p, j, k);
    }
  }
}

template <class R>
__global__ void __launch_bounds__(CELL_BS) k_sst_fields(const Slice<R>* __restrict__ sl,
                                                        const int32_t* __restrict__ first, int nslice) {
  OT2D_CELL_MAP();
  if (!inside) return;
  const ot2d_params& p = *S.P;
  if (!sst_slice(p) || j < p.jbeg || j > p.jend || k < p.kbeg || k > p.kend) return;
  sst_fields_cell(S, p, j, k);
}

template <class R>
__global__ void __launch_bounds__(CELL_BS) k_sst_turm(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ first,
                                                      int nslice) {
  OT2D_CELL_MAP();
  if (!inside || !sst_slice(*S.P)) return;
  sst_turm_cell(S, *S.P, j, k);
}

template <class R>
__global__ void __launch_bounds__(CELL_BS) k_sst_rhs(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ first,
                                                     int nslice) {
  OT2D_CELL_MAP();
  if (!inside) return;
  const ot2d_params& p = *S.P;
  if (!sst_slice(p) || j < p.jbeg || j > p.jend || k < p.kbeg || k > p.kend) return;
  sst_rhs_cell(S, p, j, k);
}

// lsolvej2 of equation blockIdx.y by warps of 32 k-lines; output x * bjmat
template <class R>
__global__ void __launch_bounds__(LJ_THREADS) k_sst_lsolvej(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ gfirst,
                                                    int nslice) {
  extern __shared__ __align__(16) unsigned char lj_raw[];
  R* sm = (R*)lj_raw;   // LJ_SMEM elements
  const int si = find_slice(gfirst, nslice, blockIdx.x);
  const Slice<R>& S = sl[si];
  const ot2d_params& p = *S.P;
  if (!sst_slice(p)) return;
  const int n = blockIdx.y;
  sa_lsolvej_group<R, false>(S, p, 32 * (blockIdx.x - gfirst[si]), sm, kband(KB_AJ, n), kband(KB_BJ, n),
                             kband(KB_CJ, n), kband(KB_SJ, n));
}

// lsolvek2 + update + findturm, one thread per j-line
template <class R>
__global__ void k_sst_lsolvek(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ lfirst, int nslice) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= lfirst[nslice]) return;
  int lo = 0, hi = nslice - 1;
  while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (lfirst[mid] <= gid) lo = mid; else hi = mid - 1; }
  const Slice<R>& S = sl[lo];
  const ot2d_params& p = *S.P;
  if (!sst_slice(p)) return;
  const int j = p.jbeg + gid - lfirst[lo];
  if (j <= p.jend) sst_lsolvek_line(S, p, j);
}

// ---- ADI operator arc2d (lhs.f:817-1057), ilhs = 2 ------------------------
template <class R>
__global__ void __launch_bounds__(CELL_BS) k_adi_txi(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ first,
                                                     int nslice, int scale, int only) {
  OT2D_CELL_MAP();
  if (!inside || (only && !adi_slice(*S.P))) return;
  adi_txi_cell(S, *S.P, j, k, scale);
}
// line direction dir over all cells: d2p (what = 0) or the coefficients (1)
template <class R>
__global__ void __launch_bounds__(CELL_BS) k_adi_line_cells(const Slice<R>* __restrict__ sl,
                                                            const int32_t* __restrict__ first, int nslice, int dir,
                                                            int what, int only) {
  OT2D_CELL_MAP();
  if (!inside) return;
  const ot2d_params& p = *S.P;
  if (only && !adi_slice(p)) return;
  const int m = dir == 0 ? j : k, n = dir == 0 ? k : j;
  const int ms = dir == 0 ? p.jbeg - 1 : p.kbeg - 1, me = dir == 0 ? p.jend + 1 : p.kend + 1;
  if (what == 0) adi_d2p_cell(S, dir, m, n, ms, me);
  else adi_coef_cell(S, p, dir, m, n, ms, me);
}
// one thread per (line, variable); blockIdx.y = slice
template <class R>
__global__ void k_adi_solve(const Slice<R>* __restrict__ sl, int dir, int only) {
  const Slice<R>& S = sl[blockIdx.y];
  const ot2d_params& p = *S.P;
  if (only && !adi_slice(p)) return;
  const int nlines = dir == 0 ? S.kd : S.jd;   // n = ks-1..ke+1 / js-1..je+1
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4 * nlines) return;
  const int n = 1 + t % nlines, i = 1 + t / nlines;
  const int ms = dir == 0 ? p.jbeg - 1 : p.kbeg - 1, me = dir == 0 ? p.jend + 1 : p.kend + 1;
  adi_solve_line(S, p, dir, i, n, ms, me);
}
template <class R>
__global__ void __launch_bounds__(CELL_BS) k_adi_ninv(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ first,
                                                      int nslice, int only) {
  OT2D_CELL_MAP();
  if (!inside || (only && !adi_slice(*S.P))) return;
  adi_ninv_cell(S, *S.P, j, k);
}
template <class R>
__global__ void __launch_bounds__(CELL_BS) k_adi_teta(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ first,
                                                      int nslice, int only) {
  OT2D_CELL_MAP();
  if (!inside || (only && !adi_slice(*S.P))) return;
  adi_teta_cell(S, *S.P, j, k);
}

// q(1:4) += s*max(iblank,0) on interior cells (step.f:203-213), FP64 state
// TS: also the next iteration's local time step (time.f:2-108) of every
// cell of the slice, from the state just written (interior) or the halo the
// boundary conditions set; the solver folds the time step in here when every
// request of the batch is steady with a first-order time step factor, so
// that nothing between this update and the next iteration's time step
// changes its inputs.
template <class R, bool TS>
__global__ void __launch_bounds__(CELL_BS / CELL_PT) k_update(const Slice<R>* __restrict__ sl,
                                                              const int32_t* __restrict__ first, int nslice) {
  OT2D_CELL_MAP_PT();
  const ot2d_params& p = *S.P;
  // a sweep of this slice gave up (status bit 4): its correction is
  // incomplete, so the state is left as it is until the slice is retired
  if (S.ist && (__ldcg(&S.ist[2]) & 4)) return;
  bool bad = false;
  R oat = (R)1.0;
  if constexpr (TS) {
    const int istep = S.ist ? S.ist[1] : p.istep;
    if (p.ntac >= 2 && istep > 1) oat = (R)(2. / 3.);
    if (p.ntac == 3 && istep > 2) oat = (R)(6. / 11.);
  }
#pragma unroll
  for (int u = 0; u < CELL_PT; ++u) {
    const int cid = cid0 + u * (CELL_BS / CELL_PT);
    const int j = cid % S.jd + 1, k = cid / S.jd + 1;
    if (cid >= ncell) continue;
    if (j < p.jbeg || j > p.jend || k < p.kbeg || k > p.kend) {
      if constexpr (TS) time_step_cell(S, j, k, oat);
      continue;
    }
    const int64_t o = at(S.jd, j, k);
    int ibi = S.iblank[o];
    // max(iblank, 0) as a double, the common values without a conversion
    double m;
    if (ibi == 1) m = 1.0;
    else if (ibi <= 0) m = 0.0;
    else m = (double)ibi;
    // every load before the first store (the state and the residual may not
    // alias, but the compiler cannot know): eight independent loads in flight
    double q0[4];
    R sv[4];
#pragma unroll
    for (int n = 0; n < 4; ++n) { q0[n] = S.q64[n * S.qs + o]; sv[n] = S.s[n * S.qs + o]; }
    R qn[4];
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      double sd;
      if constexpr (sizeof(R) == sizeof(float)) sd = f2d_bits_ftz(sv[n]);
      else sd = (double)sv[n];
      double v = q0[n] + sd * m;
      S.q64[n * S.qs + o] = v;
      if constexpr (sizeof(R) == sizeof(float)) qn[n] = d2f_bits_rn_ftz(v);
      else qn[n] = (R)v;
      if constexpr (sizeof(R) != sizeof(double)) S.q[n * S.qs + o] = qn[n];
    }
    // monitor of the updated cell (step.f:356-370), free of divisions:
    // a^2 <= 0.002  <=>  ggm1*(q4*q1 - qq/2) <= 0.002*q1^2 for q1 > 0
    bad = bad || monitor_bad<R>(S.k_ggm1, qn);
    if constexpr (TS) {
      const R J = p.iconstant_cfl == 0 ? S.q[(int64_t)(p.nq - 1) * S.qs + o] : (R)0;
      time_step_vals(S, p, o, ibi, qn[0], qn[1], qn[2], qn[3], J, oat);
    }
  }
  if (S.ist && bad) atomicOr(&S.ist[2], 2);
}

// compute copy of the whole state from the FP64 master (after the host
// replaced q64); a no-op on the plain FP64 path where they are one array
template <class R>
__global__ void __launch_bounds__(CELL_BS / CELL_PT) k_shadow(const Slice<R>* __restrict__ sl,
                                                              const int32_t* __restrict__ first, int nslice) {
  if constexpr (sizeof(R) == sizeof(double)) {
    return;
  } else {
    OT2D_CELL_MAP_PT();
    const int nq = S.P->nq;
#pragma unroll
    for (int u = 0; u < CELL_PT; ++u) {
      const int cid = cid0 + u * (CELL_BS / CELL_PT);
      if (cid >= ncell) continue;
      for (int n = 0; n < nq; ++n) S.q[n * S.qs + cid] = (R)S.q64[n * S.qs + cid];
    }
  }
}

// monitor (step.f:356-370) on the FP64 state: count of cells with a^2 <=
// 0.002 or a non-finite a^2 -> status bit 2
template <class R>
__global__ void __launch_bounds__(CELL_BS) k_monitor(const Slice<R>* __restrict__ sl, const int32_t* __restrict__ first,
                                                     int nslice) {
  OT2D_CELL_MAP();
  bool bad = false;
  if (inside) {
    const ot2d_params& p = *S.P;
    const int64_t o = at(S.jd, j, k);
    double rho = S.q64[o];
    double qq = sq(S.q64[S.qs + o]) + sq(S.q64[2 * S.qs + o]);
    double asq = p.ggm1 * (S.q64[3 * S.qs + o] - .5 * qq / rho) / rho;
    bad = (asq <= 0.002) || (asq + 1 == asq) || (asq != asq);
  }
  bad = __syncthreads_or(bad);
  if (bad && threadIdx.x == 0 && S.ist) atomicOr(&S.ist[2], 2);
}

// FP64 wall forces of one slice (forces.f:130-398); one CTA per slice,
// integrands in parallel, sums by thread 0 in the reference's j order.
// out[0..3] = cfx, cfy, cm0, cpower
template <class R>
__global__ void k_forces(const Slice<R>* __restrict__ sl, const double* const* __restrict__ xv,
                         const double* const* __restrict__ yv, double* __restrict__ out) {
  extern __shared__ double fsh[];
  const Slice<R>& S = sl[blockIdx.x];
  const ot2d_params& p = *S.P;
  const int jd = S.jd, nq = p.nq, jmax = p.jmax;
  const double* q = S.q64; const int64_t qs = S.qs;
  auto Q = [&](int j, int k, int n) { return q[(int64_t)(n - 1) * qs + at(jd, j, k)]; };
  auto XV = [&](int j, int k) { return xv[blockIdx.x][(int64_t)(k - 1) * jmax + (j - 1)]; };
  auto YV = [&](int j, int k) { return yv[blockIdx.x][(int64_t)(k - 1) * jmax + (j - 1)]; };
  const int k = p.kbeg, k2 = k + 1, k3 = k2 + 1, j1 = p.jtail1, j2 = p.jtail2, nw = j2 - j1 + 1;
  double* zz = fsh; double* sxx = fsh + nw; double* syy = fsh + 2 * nw;
  const double fmm = (p.fsmach != 0) ? p.fsmach : ((p.fmtip != 0) ? p.fmtip : 1.0);
  const double gm1 = p.gm1, gamma = p.gamma;
  for (int j = j1 + threadIdx.x; j <= j2; j += blockDim.x) {
    double rr = 1. / Q(j, k, 1), rho = Q(j, k, 1) * Q(j, k, nq);
    double u = Q(j, k, 2) * rr, v = Q(j, k, 3) * rr, e = Q(j, k, 4) * Q(j, k, nq);
    double vsq = u * u + v * v, pp = gm1 * (e - rho * vsq / 2.), pp1 = pp / p.pinf;
    double cp = 2. * (pp1 - 1.) / (gamma * sq(fmm));
    double z = cp;
    rr = 1. / Q(j, k - 1, 1); rho = Q(j, k - 1, 1) * Q(j, k - 1, nq);
    u = Q(j, k - 1, 2) * rr; v = Q(j, k - 1, 3) * rr; e = Q(j, k - 1, 4) * Q(j, k - 1, nq);
    vsq = u * u + v * v; pp = gm1 * (e - rho * vsq / 2.); pp1 = pp / p.pinf;
    cp = 2. * (pp1 - 1.) / (gamma * sq(fmm));
    zz[j - j1] = 0.5 * (z + cp);
  }
  __syncthreads();
  double cn = 0., cc = 0., cmle = 0., cpinv = 0.;
  if (threadIdx.x == 0) {
    for (int j = j1; j <= j2; ++j) {
      int jv = j - p.nhalo, kv = k - p.nhalo;
      double z = zz[j - j1];
      cn = cn - z * (XV(jv + 1, kv) - XV(jv, kv));
      cc = cc + z * (YV(jv + 1, kv) - YV(jv, kv));
      cmle = cmle + z * (0.5 * (XV(jv + 1, kv) + XV(jv, kv)) * (XV(jv + 1, kv) - XV(jv, kv)) +
                         0.5 * (YV(jv + 1, kv) + YV(jv, kv)) * (YV(jv + 1, kv) - YV(jv, kv)));
      double u = Q(j, k, 2) / Q(j, k, 1), v = Q(j, k, 3) / Q(j, k, 1);
      double um = Q(j, k - 1, 2) / Q(j, k - 1, 1), vm = Q(j, k - 1, 3) / Q(j, k - 1, 1);
      cpinv = cpinv + 0.5 * (u + um) * z * (YV(jv + 1, kv) - YV(jv, kv)) - 0.5 * (v + vm) * z * (XV(jv + 1, kv) - XV(jv, kv));
    }
    double half = (double)p.half;
    cn = cn - half * cn; cmle = cmle - half * cmle; cc = cc + half * cc;
  }
  __syncthreads();
  double cnv = 0., ccv = 0., cmlev = 0., cpv = 0.;
  if (!p.invisc) {
    const double amu = p.rinf * 1. / p.rey, uinf2 = sq(fmm);
    const double *xx = S.xx64, *xy = S.xy64, *yx = S.yx64, *yy = S.yy64;
    for (int j = j1 + threadIdx.x; j <= j2; j += blockDim.x) {
      double uxi, vxi;
      if (j == j1) {
        uxi = Q(j + 1, k, 2) / Q(j + 1, k, 1) - Q(j, k, 2) / Q(j, k, 1);
        vxi = Q(j + 1, k, 3) / Q(j + 1, k, 1) - Q(j, k, 3) / Q(j, k, 1);
      } else if (j == j2) {
        uxi = Q(j, k, 2) / Q(j, k, 1) - Q(j - 1, k, 2) / Q(j - 1, k, 1);
        vxi = Q(j, k, 3) / Q(j, k, 1) - Q(j - 1, k, 3) / Q(j - 1, k, 1);
      } else {
        uxi = .5 * (Q(j + 1, k, 2) / Q(j + 1, k, 1) - Q(j - 1, k, 2) / Q(j - 1, k, 1));
        vxi = .5 * (Q(j + 1, k, 3) / Q(j + 1, k, 1) - Q(j - 1, k, 3) / Q(j - 1, k, 1));
      }
      double ueta = -1.5 * Q(j, k, 2) / Q(j, k, 1) + 2. * Q(j, k2, 2) / Q(j, k2, 1) - .5 * Q(j, k3, 2) / Q(j, k3, 1);
      double veta = -1.5 * Q(j, k, 3) / Q(j, k, 1) + 2. * Q(j, k2, 3) / Q(j, k2, 1) - .5 * Q(j, k3, 3) / Q(j, k3, 1);
      const int64_t o = at(jd, j, k);
      double xix = xx[o], xiy = xy[o], etax = yx[o], etay = yy[o];
      double sfdiv = 2. / 3 * (uxi * xix + ueta * etax + vxi * xiy + veta * etay);
      double a = amu * (2. * (uxi * xix + ueta * etax) - sfdiv);
      double b = amu * (2. * (vxi * xiy + veta * etay) - sfdiv);
      double tauw = amu * ((uxi * xiy + ueta * etay) + (vxi * xix + veta * etax));
      sxx[j - j1] = a / (.5 * p.rinf * uinf2);
      syy[j - j1] = b / (.5 * p.rinf * uinf2);
      zz[j - j1] = tauw / (.5 * p.rinf * uinf2);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int j = j1; j <= j2; ++j) {
        int jv = j - p.nhalo, kv = k - p.nhalo;
        double z = zz[j - j1], sx = sxx[j - j1], sy = syy[j - j1];
        ccv = ccv + z * (XV(jv + 1, kv) - XV(jv, kv)) - sx * (YV(jv + 1, kv) - YV(jv, kv));
        cnv = cnv - z * (YV(jv + 1, kv) - YV(jv, kv)) + sy * (XV(jv + 1, kv) - XV(jv, kv));
        cmlev = cmlev + z * (0.5 * (XV(jv + 1, kv) + XV(jv, kv)) * (YV(jv + 1, kv) - YV(jv, kv)) +
                             0.5 * (YV(jv + 1, kv) + YV(jv, kv)) * (XV(jv + 1, kv) - XV(jv, kv))) -
                0.5 * (XV(jv + 1, kv) + XV(jv, kv)) * (XV(jv + 1, kv) - XV(jv, kv)) * sy -
                0.5 * (YV(jv + 1, kv) + YV(jv, kv)) * (YV(jv + 1, kv) - YV(jv, kv)) * sx;
        double u = Q(j, k, 2) / Q(j, k, 1), v = Q(j, k, 3) / Q(j, k, 1);
        double um = Q(j, k - 1, 2) / Q(j, k - 1, 1), vm = Q(j, k - 1, 3) / Q(j, k - 1, 1);
        cpv = cpv + 0.5 * (u + um) * z * (XV(jv + 1, kv) - XV(jv, kv)) - 0.5 * (u + um) * sx * (YV(jv + 1, kv) - YV(jv, kv)) -
              0.5 * (v + vm) * z * (YV(jv + 1, kv) - YV(jv, kv)) + 0.5 * (v + vm) * sy * (XV(jv + 1, kv) - XV(jv, kv));
      }
      double half = (double)p.half;
      cnv = cnv - half * cnv; cmlev = cmlev - half * cmlev; ccv = ccv + half * ccv;
    }
  }
  if (threadIdx.x == 0) {
    out[4 * blockIdx.x + 0] = cc + ccv;
    out[4 * blockIdx.x + 1] = cn + cnv;
    out[4 * blockIdx.x + 2] = cmle + cmlev;
    out[4 * blockIdx.x + 3] = (cpinv + cpv) / fmm;
  }
}

}  // namespace ot2d
