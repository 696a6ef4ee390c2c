// launchers.cuh -- launcher bodies, instantiated once per arithmetic type.
#pragma once
#include "kernels.cuh"

namespace ot2d {

template <class R>
cudaError_t launch_iter_begin(const Slice<R>* d_sl, const Batch& b, cudaStream_t st) {
  k_iter_begin<R><<<(b.nslice + 127) / 128, 128, 0, st>>>(d_sl, b.nslice);
  if (b.moving) {
    k_mv_pitch<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice);
    k_mv_geom<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice);
    k_mv_halo<R><<<b.nslice, 256, 0, st>>>(d_sl);
  }
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_pitch(const Slice<R>* d_sl, const Batch& b, cudaStream_t st) {
  k_mv_pitch<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice);
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_time_step(const Slice<R>* d_sl, const Batch& b, cudaStream_t st) {
  k_time_step<R><<<b.cell_blocks, CELL_BS / CELL_PT, 0, st>>>(d_sl, b.d_first, b.nslice);
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_bc(const Slice<R>* d_sl, const Batch& b, int advance, cudaStream_t st, int begin) {
  // one launch per &bcinp entry (the reference applies them in order), each
  // spread over enough CTAs per slice to cover the longest boundary
  if constexpr (sizeof(R) == sizeof(float)) {
    k_bc_all<R><<<b.nslice, BC_BS, 0, st>>>(d_sl, advance, begin);
  } else {
    if (begin) k_iter_begin<R><<<(b.nslice + 127) / 128, 128, 0, st>>>(d_sl, b.nslice);
    const int nch = (std::max(b.max_wall, b.max_kd) + BCE_BS - 1) / BCE_BS;
    for (int ib = 0; ib < b.max_nbc; ++ib) k_bc_entry<R><<<dim3(nch, b.nslice), BCE_BS, 0, st>>>(d_sl, ib);
    k_bc<R><<<b.nslice, BC_BS, 0, st>>>(d_sl, advance);
  }
  return cudaGetLastError();
}
// the fused residual tiles: the plain instantiation always, the
// preconditioned one when the batch holds a preconditioned slice
template <class R>
cudaError_t launch_quad(const Slice<R>* d_sl, const Batch& b, cudaStream_t st) {
  // quad's face states of every line of the ilim +-2 slices, before the
  // faces that read them
  if (b.lim_mask & 8)
    k_quad<R><<<dim3((4 * (b.max_kd + b.max_wall) + 127) / 128, b.nslice), 128, 0, st>>>(d_sl);
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_resid_both(const Slice<R>* d_sl, const Batch& b, int flags, cudaStream_t st) {
  if (flags & AS_INV) {
    cudaError_t e = launch_quad(d_sl, b, st);
    if (e != cudaSuccess) return e;
  }
  // the tile shape the batch's tile table was built for (k_resid_launch.cuh,
  // one translation unit per shape and precision)
  switch (b.rt_shape) {
    case 1: return launch_resid_shape<R, 32, 8>(d_sl, b, flags, st);
    case 2: return launch_resid_shape<R, 8, 32>(d_sl, b, flags, st);
    case 3: return launch_resid_shape<R, 32, 16>(d_sl, b, flags, st);
    default: return launch_resid_shape<R, 16, 16>(d_sl, b, flags, st);
  }
}
template <class R>
cudaError_t launch_residual(const Slice<R>* d_sl, const Batch& b, int viscous, cudaStream_t st, int norms) {
  const int flags = AS_INV | AS_TS | AS_NORM | (viscous ? AS_VISC : 0);
  cudaError_t e = launch_resid_both(d_sl, b, flags, st);
  if (e != cudaSuccess || !norms) return e;
  return launch_norm_final(d_sl, b, st);
}
template <class R>
cudaError_t launch_norm_final(const Slice<R>* d_sl, const Batch& b, cudaStream_t st) {
  k_norm_final<R><<<b.nslice, 32, 0, st>>>(d_sl, b.d_tfirst, b.nslice, b.d_part);
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_resid_tiles(const Slice<R>* d_sl, const Batch& b, int flags, cudaStream_t st) {
  return launch_resid_both(d_sl, b, flags & ~AS_NORM, st);
}
template <class R>
cudaError_t launch_faces(const Slice<R>* d_sl, const Batch& b, int inviscid, int viscous, cudaStream_t st) {
  if (inviscid) {
    cudaError_t e = launch_quad(d_sl, b, st);
    if (e != cudaSuccess) return e;
    k_faces<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice);
  }
  if (viscous) k_visc<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice);
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_assemble(const Slice<R>* d_sl, const Batch& b, int flags, cudaStream_t st) {
  k_assemble<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice, flags, b.d_part);
  if (flags & AS_NORM) k_norm_final<R><<<b.nslice, 32, 0, st>>>(d_sl, b.d_first, b.nslice, b.d_part);
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_rbc(const Slice<R>* d_sl, const Batch& b, cudaStream_t st) {
  k_rbc<R><<<b.nslice, 128, 0, st>>>(d_sl);
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_rhslom(const Slice<R>* d_sl, const Batch& b, cudaStream_t st) {
  k_rhslom<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice);
  return cudaGetLastError();
}
// ilu2d part 1: the sweep records and the halo edges (reads q, mu_t, tscale;
// the FP64 path also round-trips q here).  PRE: the preilu2d records of the
// preconditioned slices, launched only when the batch holds one.
template <class R, bool PRE>
cudaError_t launch_lusgs_prep_t(const Slice<R>* d_sl, const Batch& b, int scale, cudaStream_t st, int only_lu,
                                int parts) {
  // one staged chunk per warp (f32 28 / 36 KB, f64 53 / 68 KB per block)
  constexpr size_t prep_smem = (size_t)LU_PREP_CH * lu_prep_stride<R, PRE>() * sizeof(R);
  static DeviceOnce once;
  cudaError_t ae = once.run([&](int&) {
    return cudaFuncSetAttribute(k_lu_prep<R, PRE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)prep_smem);
  });
  if (ae != cudaSuccess) return ae;
  if (parts & 1)
    k_lu_prep<R, PRE><<<b.lu_blocks, LU_PREP_BS, prep_smem, st>>>(d_sl, b.d_lfirst, b.nslice, scale, only_lu);
  if (!(parts & 2)) return cudaGetLastError();
  if constexpr (sizeof(R) == sizeof(double)) {
    // every cell: the FP64 path also round-trips q (lhs.f:524-531, :805-811)
    k_lu_edges<R, PRE><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice, scale, only_lu);
  } else {
    const int nring = 2 * b.max_wall + 2 * b.max_kd;   // >= the ring of every slice
    k_lu_edges_ring<R, PRE><<<dim3((nring + 127) / 128, b.nslice), 128, 0, st>>>(d_sl, scale, only_lu);
  }
  return cudaGetLastError();
}
// parts: 1 the records (k_lu_prep), 2 the halo edges (k_lu_edges*), 3 both
template <class R>
cudaError_t launch_lusgs_prep(const Slice<R>* d_sl, const Batch& b, int scale, cudaStream_t st, int only_lu,
                              int parts = 3) {
  cudaError_t e = launch_lusgs_prep_t<R, false>(d_sl, b, scale, st, only_lu, parts);
  if (e == cudaSuccess && b.precon) e = launch_lusgs_prep_t<R, true>(d_sl, b, scale, st, only_lu, parts);
  return e;
}
// ilu2d part 2: the forward and backward sweeps, launched at the device's
// highest priority (they are the iteration's longest dependency chain and
// run beside the turbulence branch)
template <class R, bool PRE>
cudaError_t launch_lusgs_sweeps_t(const Slice<R>* d_sl, const Batch& b, cudaStream_t st, int only_lu) {
  const int nw = b.max_lu_warps;
  // chunks per bulk copy: as many as ~200 KB of shared memory allows (1..8)
  const int maxcol = b.max_wall;   // >= jd - 2 of every slice
  int G = (b.lu_group == 1 || b.lu_group == 2 || b.lu_group == 4 || b.lu_group == 8) ? b.lu_group : 8;
  while (G > 1 && lu_smem_bytes<R, PRE>(nw, G, maxcol) > 200 * 1024) G >>= 1;
  const size_t smem = lu_smem_bytes<R, PRE>(nw, G, maxcol);
  if (32 * nw > 1024 || smem > (size_t)SMEM_OPTIN_MAX) return cudaErrorInvalidConfiguration;
  static DeviceOnce once;
  int prio = 0;
  cudaError_t ae = once.run(
      [&](int& hi_prio) {
        const void* ks[] = {(const void*)k_lu_sweep<R, true, 8, PRE>, (const void*)k_lu_sweep<R, false, 8, PRE>,
                            (const void*)k_lu_sweep<R, true, 4, PRE>, (const void*)k_lu_sweep<R, false, 4, PRE>,
                            (const void*)k_lu_sweep<R, true, 2, PRE>, (const void*)k_lu_sweep<R, false, 2, PRE>,
                            (const void*)k_lu_sweep<R, true, 1, PRE>, (const void*)k_lu_sweep<R, false, 1, PRE>};
        for (const void* k : ks) {
          cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_OPTIN_MAX);
          if (e != cudaSuccess) return e;
        }
        int lo = 0, hi = 0;
        if (cudaDeviceGetStreamPriorityRange(&lo, &hi) == cudaSuccess) hi_prio = hi;
        return cudaSuccess;
      },
      &prio);
  if (ae != cudaSuccess) return ae;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributePriority;
  at[0].val.priority = prio;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(b.nslice);
  cfg.blockDim = dim3(32 * nw);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  auto run = [&](auto fwd, auto bwd) -> cudaError_t {
    cudaError_t e = cudaLaunchKernelEx(&cfg, fwd, d_sl, only_lu, b.poll_limit, b.lu_lag);
    if (e != cudaSuccess) return e;
    return cudaLaunchKernelEx(&cfg, bwd, d_sl, only_lu, b.poll_limit, b.lu_lag);
  };
  cudaError_t e;
  switch (G) {
    case 8: e = run(k_lu_sweep<R, true, 8, PRE>, k_lu_sweep<R, false, 8, PRE>); break;
    case 4: e = run(k_lu_sweep<R, true, 4, PRE>, k_lu_sweep<R, false, 4, PRE>); break;
    case 2: e = run(k_lu_sweep<R, true, 2, PRE>, k_lu_sweep<R, false, 2, PRE>); break;
    default: e = run(k_lu_sweep<R, true, 1, PRE>, k_lu_sweep<R, false, 1, PRE>); break;
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_lusgs_sweeps(const Slice<R>* d_sl, const Batch& b, cudaStream_t st, int only_lu) {
  cudaError_t e = launch_lusgs_sweeps_t<R, false>(d_sl, b, st, only_lu);
  if (e == cudaSuccess && b.precon) e = launch_lusgs_sweeps_t<R, true>(d_sl, b, st, only_lu);
  return e;
}
template <class R>
cudaError_t launch_lusgs(const Slice<R>* d_sl, const Batch& b, int scale, cudaStream_t st, int only_lu) {
  cudaError_t e = launch_lusgs_prep(d_sl, b, scale, st, only_lu);
  if (e != cudaSuccess) return e;
  return launch_lusgs_sweeps(d_sl, b, st, only_lu);
}
template <class R>
cudaError_t launch_sa(const Slice<R>* d_sl, const Batch& b, cudaStream_t st, int final_bc) {
  // k_sa_prep beside the first turbc
  k_sa_prep_bc<R><<<b.nslice + b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice);
  // on the residual's tiles (tile table of the batch's tile shape)
  switch (b.rt_shape) {
    case 1: k_sa_rhs<R, 32, 8><<<b.tile_blocks, 256, sa_rhs_smem<R, 32, 8>(), st>>>(d_sl, b.d_tfirst, b.nslice); break;
    case 2: k_sa_rhs<R, 8, 32><<<b.tile_blocks, 256, sa_rhs_smem<R, 8, 32>(), st>>>(d_sl, b.d_tfirst, b.nslice); break;
    case 3: k_sa_rhs<R, 32, 16><<<b.tile_blocks, 512, sa_rhs_smem<R, 32, 16>(), st>>>(d_sl, b.d_tfirst, b.nslice); break;
    default: k_sa_rhs<R, 16, 16><<<b.tile_blocks, 256, sa_rhs_smem<R, 16, 16>(), st>>>(d_sl, b.d_tfirst, b.nslice);
  }
  constexpr size_t lj_smem = sizeof(R) * LJ_SMEM;
  static DeviceOnce once;
  cudaError_t ae = once.run([&](int&) {
    return cudaFuncSetAttribute(k_sa_lsolvej<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lj_smem);
  });
  if (ae != cudaSuccess) return ae;
  k_sa_lsolvej<R><<<b.jgroups, LJ_THREADS, lj_smem, st>>>(d_sl, b.d_gfirst, b.nslice);
  k_sa_lsolve<R><<<(b.klines + 63) / 64, 64, 0, st>>>(d_sl, b.d_kfirst, b.nslice, 1);
  if (final_bc) k_turbc<R><<<b.nslice, BC_BS, 0, st>>>(d_sl);
  return cudaGetLastError();
}
// the closing turbc of vmu_sa and c_turm on the halo ring
template <class R>
cudaError_t launch_sa_final_bc(const Slice<R>* d_sl, const Batch& b, cudaStream_t st) {
  k_turbc<R><<<b.nslice, BC_BS, 0, st>>>(d_sl);
  return cudaGetLastError();
}
// komegasst (komegasst.f:2-187) for the SST slices of the batch
template <class R>
cudaError_t launch_sst(const Slice<R>* d_sl, const Batch& b, cudaStream_t st) {
  k_sst_prep<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice);
  k_sst_bc<R><<<b.nslice, 256, 0, st>>>(d_sl, 0);
  k_sst_fields<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice);
  k_sst_turm<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice);
  k_sst_rhs<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice);
  constexpr size_t lj_smem = sizeof(R) * LJ_SMEM;
  static DeviceOnce once;
  cudaError_t ae = once.run([&](int&) {
    return cudaFuncSetAttribute(k_sst_lsolvej<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lj_smem);
  });
  if (ae != cudaSuccess) return ae;
  k_sst_lsolvej<R><<<dim3(b.jgroups, 2), LJ_THREADS, lj_smem, st>>>(d_sl, b.d_gfirst, b.nslice);
  k_sst_lsolvek<R><<<(b.klines + 63) / 64, 64, 0, st>>>(d_sl, b.d_kfirst, b.nslice);
  k_sst_bc<R><<<b.nslice, 256, 0, st>>>(d_sl, 1);
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_adi(const Slice<R>* d_sl, const Batch& b, int scale, cudaStream_t st, int only_adi) {
  k_adi_txi<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice, scale, only_adi);
  for (int dir = 0; dir < 2; ++dir) {
    if (dir == 1) k_adi_ninv<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice, only_adi);
    k_adi_line_cells<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice, dir, 0, only_adi);
    k_adi_line_cells<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice, dir, 1, only_adi);
    const int nl = 4 * (dir == 0 ? b.max_kd : b.max_wall);
    k_adi_solve<R><<<dim3((nl + 63) / 64, b.nslice), 64, 0, st>>>(d_sl, dir, only_adi);
  }
  k_adi_teta<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice, only_adi);
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_update(const Slice<R>* d_sl, const Batch& b, cudaStream_t st) {
  if (b.ts_in_update) k_update<R, true><<<b.cell_blocks, CELL_BS / CELL_PT, 0, st>>>(d_sl, b.d_first, b.nslice);
  else k_update<R, false><<<b.cell_blocks, CELL_BS / CELL_PT, 0, st>>>(d_sl, b.d_first, b.nslice);
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_shadow(const Slice<R>* d_sl, const Batch& b, cudaStream_t st) {
  if (sizeof(R) != sizeof(double)) k_shadow<R><<<b.cell_blocks, CELL_BS / CELL_PT, 0, st>>>(d_sl, b.d_first, b.nslice);
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_monitor(const Slice<R>* d_sl, const Batch& b, cudaStream_t st) {
  k_monitor<R><<<b.cell_blocks, CELL_BS, 0, st>>>(d_sl, b.d_first, b.nslice);
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_forces(const Slice<R>* d_sl, const Batch& b, const double* const* d_xv, const double* const* d_yv,
                          double* d_out, cudaStream_t st) {
  size_t smem = sizeof(double) * 3 * (size_t)b.max_wall;
  if (smem > (size_t)SMEM_OPTIN_MAX) return cudaErrorInvalidConfiguration;
  static DeviceOnce once;
  cudaError_t ae = once.run([&](int&) {
    return cudaFuncSetAttribute(k_forces<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_OPTIN_MAX);
  });
  if (ae != cudaSuccess) return ae;
  k_forces<R><<<b.nslice, 128, smem, st>>>(d_sl, d_xv, d_yv, d_out);
  return cudaGetLastError();
}
template <class R>
cudaError_t launch_iteration(const Slice<R>* d_sl, const Batch& b, int viscous, int turb, int lhs, cudaStream_t st,
                             cudaEvent_t after_rbc) {
  cudaError_t e;
  // Mixed path, LU-SGS with a turbulence model: the side kernels (the norm
  // reduction, read only by the host, and the LU-SGS halo edges, read only
  // by the sweeps; the f32 edges touch the halo ring alone) run on the
  // branch stream beside rbc and the record kernel, and the iteration's
  // start is applied by the boundary kernel when nothing comes between.
  const bool side = sizeof(R) == sizeof(float) && lhs == 1 && turb;
  const bool begin_in_bc = sizeof(R) == sizeof(float) && b.ts_in_update && !b.moving;
  Branch* br = nullptr;
  if ((lhs == 1 && turb) && (e = branch_of_device(br)) != cudaSuccess) return e;
  if (!begin_in_bc && (e = launch_iter_begin(d_sl, b, st)) != cudaSuccess) return e;
  if (!b.ts_in_update && (e = launch_time_step(d_sl, b, st)) != cudaSuccess) return e;
  if ((e = launch_bc(d_sl, b, 1, st, begin_in_bc ? 1 : 0)) != cudaSuccess) return e;
  if ((e = launch_residual(d_sl, b, viscous, st, side ? 0 : 1)) != cudaSuccess) return e;
  if (side) {
    if ((e = cudaEventRecord(br->resid, st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(br->st, br->resid, 0)) != cudaSuccess) return e;
    if ((e = launch_norm_final(d_sl, b, br->st)) != cudaSuccess) return e;
  }
  if ((e = launch_rbc(d_sl, b, st)) != cudaSuccess) return e;
  if (side) {
    if ((e = cudaEventRecord(br->rbc, st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(br->st, br->rbc, 0)) != cudaSuccess) return e;
    if ((e = launch_lusgs_prep(d_sl, b, 1, br->st, 1, 2)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(br->edges, br->st)) != cudaSuccess) return e;
  }
  // the pipelined solver starts the other half of its batch here (an
  // external event node of the captured graph)
  if (after_rbc && (e = cudaEventRecordWithFlags(after_rbc, st, cudaEventRecordExternal)) != cudaSuccess) return e;
  if (lhs == 1 && turb) {
    // The turbulence solve (step.f:184-190) reads q, mu_t and tscale, which
    // the LU-SGS sweeps do not write, and writes its own variables and mu_t,
    // which the sweeps do not read once the records are built: after the
    // record / edge kernels (mu_t read, FP64 q round trip done) it runs on
    // a second stream beside the sweeps, joined before the update.
    if ((e = launch_lusgs_prep(d_sl, b, 1, st, 1, side ? 1 : 3)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(br->fork, st)) != cudaSuccess) return e;
    if (side && (e = cudaStreamWaitEvent(st, br->edges, 0)) != cudaSuccess) return e;
    if ((e = launch_lusgs_sweeps(d_sl, b, st, 1)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(br->st, br->fork, 0)) != cudaSuccess) return e;
    if ((turb & 1) && (e = launch_sa(d_sl, b, br->st, 0)) != cudaSuccess) return e;
    if ((turb & 2) && (e = launch_sst(d_sl, b, br->st)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(br->join, br->st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(st, br->join, 0)) != cudaSuccess) return e;
    // SA's closing turbc writes nu_tilde and mu_t on the halo ring, which
    // the state update does not touch (it reads and writes the interior
    // flow variables, and its time step reads the halo's flow variables):
    // it runs beside the update and joins at the end of the iteration.
    if (turb & 1) {
      if ((e = launch_sa_final_bc(d_sl, b, br->st)) != cudaSuccess) return e;
      if ((e = cudaEventRecord(br->join_end, br->st)) != cudaSuccess) return e;
    }
    if ((e = launch_update(d_sl, b, st)) != cudaSuccess) return e;
    if ((turb & 1) && (e = cudaStreamWaitEvent(st, br->join_end, 0)) != cudaSuccess) return e;
    return cudaSuccess;
  } else {
    if ((lhs & 1) && (e = launch_lusgs(d_sl, b, 1, st, 1)) != cudaSuccess) return e;
    if ((lhs & 2) && (e = launch_adi(d_sl, b, 1, st, 1)) != cudaSuccess) return e;
    if ((turb & 1) && (e = launch_sa(d_sl, b, st)) != cudaSuccess) return e;
    if ((turb & 2) && (e = launch_sst(d_sl, b, st)) != cudaSuccess) return e;
  }
  if ((e = launch_update(d_sl, b, st)) != cudaSuccess) return e;
  return cudaSuccess;  // the monitor runs inside k_update and k_bc
}

#define OT2D_INSTANTIATE(R)                                                                              \
  template cudaError_t launch_iteration<R>(const Slice<R>*, const Batch&, int, int, int, cudaStream_t, cudaEvent_t); \
  template cudaError_t launch_time_step<R>(const Slice<R>*, const Batch&, cudaStream_t);                \
  template cudaError_t launch_iter_begin<R>(const Slice<R>*, const Batch&, cudaStream_t);               \
  template cudaError_t launch_pitch<R>(const Slice<R>*, const Batch&, cudaStream_t);                    \
  template cudaError_t launch_bc<R>(const Slice<R>*, const Batch&, int, cudaStream_t, int);             \
  template cudaError_t launch_residual<R>(const Slice<R>*, const Batch&, int, cudaStream_t, int);       \
  template cudaError_t launch_norm_final<R>(const Slice<R>*, const Batch&, cudaStream_t);               \
  template cudaError_t launch_rbc<R>(const Slice<R>*, const Batch&, cudaStream_t);                      \
  template cudaError_t launch_rhslom<R>(const Slice<R>*, const Batch&, cudaStream_t);                   \
  template cudaError_t launch_lusgs<R>(const Slice<R>*, const Batch&, int, cudaStream_t, int);          \
  template cudaError_t launch_faces<R>(const Slice<R>*, const Batch&, int, int, cudaStream_t);          \
  template cudaError_t launch_resid_tiles<R>(const Slice<R>*, const Batch&, int, cudaStream_t);         \
  template cudaError_t launch_assemble<R>(const Slice<R>*, const Batch&, int, cudaStream_t);            \
  template cudaError_t launch_sa<R>(const Slice<R>*, const Batch&, cudaStream_t, int);                  \
  template cudaError_t launch_sa_final_bc<R>(const Slice<R>*, const Batch&, cudaStream_t);              \
  template cudaError_t launch_sst<R>(const Slice<R>*, const Batch&, cudaStream_t);                      \
  template cudaError_t launch_adi<R>(const Slice<R>*, const Batch&, int, cudaStream_t, int);            \
  template cudaError_t launch_update<R>(const Slice<R>*, const Batch&, cudaStream_t);                   \
  template cudaError_t launch_monitor<R>(const Slice<R>*, const Batch&, cudaStream_t);                  \
  template cudaError_t launch_shadow<R>(const Slice<R>*, const Batch&, cudaStream_t);                   \
  template cudaError_t launch_forces<R>(const Slice<R>*, const Batch&, const double* const*,            \
                                        const double* const*, double*, cudaStream_t);

}  // namespace ot2d
