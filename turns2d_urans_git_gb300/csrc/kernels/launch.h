// launch.h -- host-side launchers of the batched kernels.  Each launcher
// covers every slice of a batch with one kernel launch on `st`.
#pragma once
#include <atomic>
#include <cstdint>
#include <mutex>
#include <cuda_runtime.h>

namespace ot2d {

template <class R> struct Slice;
struct NormPart;

constexpr int CELL_BS = 256;
// the LU-SGS record kernel: threads per block (LU_PREP_BS / 32 chunks each)
constexpr int LU_PREP_BS = 512;
// threads of the one-CTA-per-slice boundary kernels (their loops run along
// the boundary rows; more threads, fewer serial passes per row)
constexpr int BC_BS = 512;
// threads of a CTA of one BC entry (several CTAs per slice)
constexpr int BCE_BS = 128;
// residual tile shapes (interior cells per CTA): 0 16x16, 1 32x8, 2 8x32
constexpr int RT_NSHAPE = 4;
inline void rt_shape_dims(int shape, int& tj, int& tk) {
  tj = shape == 1 || shape == 3 ? 32 : (shape == 2 ? 8 : 16);
  tk = shape == 1 ? 8 : (shape == 2 ? 32 : 16);
}
// scratch arrays per slice of the k-omega SST solve (k_sst.cuh: SSTw)
constexpr int SST_NSCRATCH = 27;
// scratch arrays per slice of the ADI operator (k_adi.cuh: ADIw)
constexpr int ADI_NSCRATCH = 25;

// One-time set-up of a launch site per device (kernel attributes such as
// the dynamic shared-memory limit, which CUDA keeps per device): run(f)
// calls f once for the calling thread's current device and remembers its
// success; concurrent callers on one device wait for the first.  One process
// may drive several GPUs, so a single process-wide flag would leave the
// other devices without the attribute.
struct DeviceOnce {
  static constexpr int MAXDEV = 64;
  std::atomic<bool> done[MAXDEV] = {};
  int value[MAXDEV] = {};   // a per-device value the set-up may record (a stream priority)
  std::mutex mu;
  template <class F>
  cudaError_t run(F&& f, int* val = nullptr) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAXDEV) return cudaErrorInvalidDevice;
    if (!done[dev].load(std::memory_order_acquire)) {
      std::lock_guard<std::mutex> g(mu);
      if (!done[dev].load(std::memory_order_relaxed)) {
        int v = 0;
        if ((e = f(v)) != cudaSuccess) return e;
        value[dev] = v;
        done[dev].store(true, std::memory_order_release);
      }
    }
    if (val) *val = value[dev];
    return cudaSuccess;
  }
};

// Largest dynamic shared memory a CTA may opt in to on sm_103a (227 KB).
constexpr int SMEM_OPTIN_MAX = 227 * 1024;

struct Batch {
  int nslice = 0;          // slices in the batch
  int moving = 0;          // some slice is time accurate on a pitching grid
  int precon = 0;          // some slice runs with Turkel preconditioning (k_mp2 >= 0)
  // the solver's batches of steady requests with a first-order time step
  // factor: the local time step of the next iteration is computed by the
  // state update (k_update<R, true>), not by a kernel of its own
  int ts_in_update = 0;
  int lim_mask = 0;        // reconstruction families of the slices: 1 central, 2 MUSCL, 4 WENO, 8 quad
  int rt_shape = 0;        // residual tile shape of the tile table (rt_shape_dims)
  int cell_blocks = 0;     // blocks of the cell-parallel kernels
  int max_lu_warps = 1;    // warps per CTA of the LU-SGS kernel
  int max_wall = 1;        // most wall cells of one slice (force kernel smem); also max jd
  int max_kd = 1;          // largest kd of the batch
  int max_nbc = 0;         // most &bcinp entries of one slice
  int jlines = 0, klines = 0;  // total k-lines / j-lines (SA line solves)
  const int32_t* d_first = nullptr;   // [nslice+1] first cell block of each slice
  const int32_t* d_jfirst = nullptr;  // [nslice+1] first k-line (lsolvej) of each slice
  const int32_t* d_kfirst = nullptr;  // [nslice+1] first j-line (lsolvek) of each slice
  const int32_t* d_lfirst = nullptr;  // [nslice+1] first LU-SGS record block of each slice
  int lu_blocks = 0;                  // blocks of the LU-SGS record kernel
  const int32_t* d_gfirst = nullptr;  // [nslice+1] first 32-line group (lsolvej) of each slice
  int jgroups = 0;                    // 32-line groups over the batch
  const int32_t* d_tfirst = nullptr;  // [nslice+1] first residual tile of each slice
  int tile_blocks = 0;                // residual tiles over the batch
  NormPart* d_part = nullptr;         // [max(cell_blocks, tile_blocks)] norm partials
  uint32_t poll_limit = 1u << 22;     // polls of a LU-SGS sweep wait before it gives up
  int lu_lag = 0;                     // extra steps each LU-SGS band trails its neighbour (schedule)
  int lu_group = 0;                   // record chunks per bulk copy of the sweeps (0: largest that fits)
};

// One full iteration of step.f for every slice of the batch:
// time_step, bc, rhsup (+visrhs, +time-spectral), norms, rbc, ilu2d,
// vmu_sa (turb bit 1), komegasst (turb bit 2), update, monitor.  lhs bit 1:
// some slice uses LU-SGS (ilhs = 1), bit 2: some slice uses ADI (ilhs = 2, 3).
// after_rbc (or null): recorded on st, as an external event of a captured
// graph, once the residual and its boundary conditions are done.
template <class R>
cudaError_t launch_iteration(const Slice<R>* d_sl, const Batch& b, int viscous, int turb, int lhs, cudaStream_t st,
                             cudaEvent_t after_rbc = nullptr);

// The second stream of an iteration (one per device and host thread) and
// the events of its fork and join; created on first use.  Call it once
// before capturing an iteration into a graph.
struct Branch {
  cudaStream_t st = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr, join_end = nullptr;
  cudaEvent_t resid = nullptr, rbc = nullptr, edges = nullptr;   // side kernels of the mixed path
};
cudaError_t branch_of_device(Branch*& out);

// Individual phases (the drop-in routines call these on a batch of one).
// Start of an iteration: step counters and Newton iteration counter of every
// slice, then (moving slices starting a physical step) pitch, stqol, metrics,
// face speeds and wall distances.
template <class R> cudaError_t launch_iter_begin(const Slice<R>* d_sl, const Batch& b, cudaStream_t st);
template <class R> cudaError_t launch_time_step(const Slice<R>* d_sl, const Batch& b, cudaStream_t st);
// pitch alone (the drop-in ot2d_pitch): slices with xc set and ist[4] == 1
template <class R> cudaError_t launch_pitch(const Slice<R>* d_sl, const Batch& b, cudaStream_t st);
// stqol over n elements of each of nv variables (stride qs): q of the
// current step, the stored levels and the Newton target (time.f:110-175)
cudaError_t launch_stqol(const double* q, double* qtn, double* qtnm1, double* qnewt, int64_t qs, int nv, int ntac,
                         int istep, cudaStream_t st);
// begin = 1 (mixed path): each slice's boundary CTA first applies the
// iteration's start to its slice (k_iter_begin's work), for an iteration
// with nothing between the two
template <class R> cudaError_t launch_bc(const Slice<R>* d_sl, const Batch& b, int advance, cudaStream_t st,
                                         int begin = 0);
// norms = 0: without the per-slice norm reduction (launch_norm_final)
template <class R> cudaError_t launch_residual(const Slice<R>* d_sl, const Batch& b, int viscous, cudaStream_t st,
                                               int norms = 1);
template <class R> cudaError_t launch_norm_final(const Slice<R>* d_sl, const Batch& b, cudaStream_t st);
// the fused residual tiles of one tile shape (TJ x TK), every
// (preconditioning, reconstruction family) kind the batch holds; defined in
// k_resid_launch.cuh and instantiated in resid_*.cu
template <class R, int TJ, int TK>
cudaError_t launch_resid_shape(const Slice<R>* d_sl, const Batch& b, int flags, cudaStream_t st);
template <class R> cudaError_t launch_rbc(const Slice<R>* d_sl, const Batch& b, cudaStream_t st);
// rhslom alone (sources.f:97-148) on the interior cells of every slice
template <class R> cudaError_t launch_rhslom(const Slice<R>* d_sl, const Batch& b, cudaStream_t st);
// scale = 1: multiply s by tscale first (step.f:141-148); 0: s already scaled.
// only_lu = 1: skip slices whose ilhs is not 1 (mixed batches); 0: every slice
template <class R> cudaError_t launch_lusgs(const Slice<R>* d_sl, const Batch& b, int scale, cudaStream_t st,
                                            int only_lu);
// the tiled residual alone with assembly flags AS_* (no norms)
template <class R> cudaError_t launch_resid_tiles(const Slice<R>* d_sl, const Batch& b, int flags, cudaStream_t st);
template <class R> cudaError_t launch_faces(const Slice<R>* d_sl, const Batch& b, int inviscid, int viscous, cudaStream_t st);
// assembly flags: see AS_* in kernels.cuh
enum { AS_ACC = 1, AS_INV = 2, AS_VISC = 4, AS_TS = 8, AS_NORM = 16 };
template <class R> cudaError_t launch_assemble(const Slice<R>* d_sl, const Batch& b, int flags, cudaStream_t st);
// vmu_sa; final_bc = 0 leaves out its closing turbc + halo c_turm, which the
// caller then launches itself (launch_sa_final_bc)
template <class R> cudaError_t launch_sa(const Slice<R>* d_sl, const Batch& b, cudaStream_t st, int final_bc = 1);
template <class R> cudaError_t launch_sa_final_bc(const Slice<R>* d_sl, const Batch& b, cudaStream_t st);
template <class R> cudaError_t launch_sst(const Slice<R>* d_sl, const Batch& b, cudaStream_t st);
// arc2d (ilhs = 2 pentadiagonal, 3 upwind tridiagonal); scale = 1: preceded
// by s *= tscale on all cells (step.f:141-148).  only_adi = 1: skip slices
// whose ilhs is not 2 or 3
template <class R> cudaError_t launch_adi(const Slice<R>* d_sl, const Batch& b, int scale, cudaStream_t st,
                                          int only_adi);
template <class R> cudaError_t launch_update(const Slice<R>* d_sl, const Batch& b, cudaStream_t st);
template <class R> cudaError_t launch_monitor(const Slice<R>* d_sl, const Batch& b, cudaStream_t st);
// refresh the compute copy of q from q64 on every cell (mixed path)
template <class R> cudaError_t launch_shadow(const Slice<R>* d_sl, const Batch& b, cudaStream_t st);
template <class R>
cudaError_t launch_forces(const Slice<R>* d_sl, const Batch& b, const double* const* d_xv, const double* const* d_yv,
                          double* d_out, cudaStream_t st);

}  // namespace ot2d
