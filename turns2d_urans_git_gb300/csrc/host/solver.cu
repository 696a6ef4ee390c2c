// solver.cu -- batched, continuously-admitting solver over device-resident
// meshes (the ot2d_solver_* ABI).  The iteration is the reference's
// Turns_overset.f:360-505 loop (time_step, step, monitor) applied to every
// live request at once: one launch per kernel family per iteration, captured
// in a CUDA graph that is rebuilt only when the set of live requests changes.
// Convergence, blow-up and monitor flags are raised on the device; the host
// reads the small status table every `check_every` iterations and retires
// finished requests (forces in FP64, slot and memory freed).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "geom.h"
#include "io.h"
#include "runtime.h"

namespace ot2d {
namespace {

struct Rec {
  DevSolve d;
  int id = -1;
  std::vector<int> slots;
  double orders = 10.0;
  int max_iters = 0;        // iterations (steady) or physical time steps (time accurate)
  long launched = 0;        // iterations run since admission
  bool live = false;
  ot2d_result res{};
  std::vector<double> qkeep;
  // force-stability convergence (ot2d_solver_set_force_tol): CL, CD of
  // the last FORCE_WIN status checks
  double win_cl[8] = {0}, win_cd[8] = {0};
  int nwin = 0;
  long force_at = 0;       // iteration count of the last force sample
  std::string store_dir;   // ot2d_solver_store_on_retire: written when retired
  bool queued = false;     // submitted, waiting for device memory
  int half = -1;           // its half of the batch when the batch has halves
  int part = -1;           // its part of the batch in the host-buffer path
};
constexpr int FORCE_WIN = 8;

// State set-up of a solve right after its admission (initial state from the
// caller or from a restart file); returns an OT2D status.
using InitFn = std::function<int(ot2d_solver*, Rec&)>;

// A submitted solve waiting for device memory.
struct Pending {
  int id = -1;
  ot2d_params p{};
  std::vector<double> xv, yv;
  double orders = 10.0;
  int max_iters = 0;
  size_t bytes = 0;
  double t_submit = 0;
  InitFn init;
};

// iterations an instance runs before it retires: max_iters, or max_iters
// physical steps of itnmax Newton iterations each
long iter_cap(const Rec& r) {
  const int itn = r.d.P.itnmax > 1 ? r.d.P.itnmax : 1;
  return (long)r.max_iters * itn;
}

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace
}  // namespace ot2d

using namespace ot2d;

struct ot2d_solver {
  int device = 0, precision = OT2D_FP64;
  cudaStream_t st = nullptr;
  cudaStream_t st_d2h = nullptr;          // downloads of ot2d_solver_iterate_host
  std::vector<cudaEvent_t> ev_d2h;        // per instance: its download finished
  cudaEvent_t ev_step = nullptr;          // the iteration's kernels finished
  int cap = 0;
  double* d_red = nullptr; int32_t* d_ist = nullptr;
  double* h_red = nullptr; int32_t* h_ist = nullptr;
  std::vector<int> free_slots;
  std::map<int, Rec> recs;
  std::vector<int> live;
  std::deque<Pending> queue;             // submitted, waiting for device memory (FIFO)
  size_t budget_auto = 0;                // 90 % of the free memory at creation
  size_t budget_set = 0;                 // OT2D_OPT_BUDGET_MB (0: the automatic budget)
  size_t used = 0;                       // device bytes of the live instances
  DevBatch<double> b64;
  DevBatch<float> b32;
  bool dirty = true;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  // Pipelined iteration (OT2D_OPT_PIPELINE): a large batch runs as two
  // halves, one graph each on its own stream; each half starts an iteration
  // once the other half's residual of the same (or the previous) iteration
  // is done, so one half's residual fills the SMs the other half's LU-SGS
  // sweeps leave idle.
  int pipeline = 1;
  bool split = false;        // the device-resident iteration runs as the halves
  bool halves = false;       // the halves' graphs exist
  bool split4 = false;       // the device-resident iteration runs as the four parts (OT2D_OPT_PIPELINE 2)
  DevBatch<double> h64[2];
  DevBatch<float> h32[2];
  cudaGraph_t hgraph[2] = {nullptr, nullptr};
  cudaGraphExec_t hexec[2] = {nullptr, nullptr};
  cudaStream_t st2 = nullptr;
  cudaEvent_t ev_half[2] = {nullptr, nullptr};   // recorded in each half's graph after its rbc
  cudaEvent_t ev_join = nullptr;
  // Host-buffer path: the batch in HP parts of about equal cells, a graph
  // and a stream each, so that some parts' copies run while others iterate
  // (built once that path is used)
  static constexpr int HP = 4;
  bool want_parts = false;
  bool parts = false;
  DevBatch<double> p64[HP];
  DevBatch<float> p32[HP];
  cudaGraph_t pgraph[HP] = {};
  cudaGraphExec_t pexec[HP] = {};
  cudaStream_t pst[HP] = {};
  cudaEvent_t ev_pdone[HP] = {};
  int next_id = 0;
  double t0 = 0;
  int check_every = 25;
  double force_dcl = 0, force_dcd = 0;   // > 0: also converge on stable forces
  int force_every = 0;                   // iterations between force samples (0: every check)
  int force_decades = 1;                 // norm drop below the peak the force rule needs
  uint32_t poll_limit = 1u << 22;        // polls of a sweep wait (OT2D_OPT_POLL_LIMIT)
  int lu_lag = 0, lu_group = 0;          // LU-SGS schedule (OT2D_OPT_LU_LAG, OT2D_OPT_LU_GROUP)
  int rt_shape = 0;                      // residual tile shape (OT2D_OPT_RT_SHAPE)
  std::vector<ot2d_tuning> tuning;       // per size class (ot2d_solver_set_tuning)
  ot2d_tuning applied{};                 // the choice of the current batch
  int keep_q = 0;
  int since_check = 0;
  bool any_viscous = false;
  int turb_bits = 0;   // 1: some SA instance, 2: some SST instance
  int lhs_bits = 0;    // 1: some LU-SGS instance, 2: some ADI instance
  double* d_forces = nullptr; size_t forces_cap = 0;
  DevBatch<double> f64;
  DevBatch<float> f32;
  const double** d_xy = nullptr; size_t xy_cap = 0;
  int last_err = 0;
  FILE* log = nullptr;                   // ot2d_solver_set_log: one JSON line per retired request
};

namespace {

int grow_slots(ot2d_solver* s, int need) {
  if ((int)s->free_slots.size() >= need) return OT2D_OK;
  int ncap = std::max(2 * s->cap, s->cap + need + 64);
  double* nr = nullptr; int32_t* ni = nullptr; double* hr = nullptr; int32_t* hi = nullptr;
  if (cudaMalloc(&nr, sizeof(double) * RED_N * ncap) != cudaSuccess) return OT2D_ERR_NOMEM;
  if (cudaMalloc(&ni, sizeof(int32_t) * IST_N * ncap) != cudaSuccess) { cudaFree(nr); return OT2D_ERR_NOMEM; }
  cudaMallocHost(&hr, sizeof(double) * RED_N * ncap);
  cudaMallocHost(&hi, sizeof(int32_t) * IST_N * ncap);
  cudaMemsetAsync(nr, 0, sizeof(double) * RED_N * ncap, s->st);
  cudaMemsetAsync(ni, 0, sizeof(int32_t) * IST_N * ncap, s->st);
  if (s->cap) {
    cudaMemcpyAsync(nr, s->d_red, sizeof(double) * RED_N * s->cap, cudaMemcpyDeviceToDevice, s->st);
    cudaMemcpyAsync(ni, s->d_ist, sizeof(int32_t) * IST_N * s->cap, cudaMemcpyDeviceToDevice, s->st);
  }
  cudaStreamSynchronize(s->st);
  if (s->d_red) cudaFree(s->d_red);
  if (s->d_ist) cudaFree(s->d_ist);
  if (s->h_red) cudaFreeHost(s->h_red);
  if (s->h_ist) cudaFreeHost(s->h_ist);
  s->d_red = nr; s->d_ist = ni; s->h_red = hr; s->h_ist = hi;
  for (int i = ncap - 1; i >= s->cap; --i) s->free_slots.push_back(i);
  s->cap = ncap;
  s->dirty = true;  // slot pointers moved
  return OT2D_OK;
}

template <class R>
void slices_of(ot2d_solver* s, const Rec& r, std::vector<Slice<R>>& out) {
  for (int nsp = 1; nsp <= r.d.nspec; ++nsp) {
    int sl = r.slots[nsp - 1];
    out.push_back(make_slice<R>(r.d, nsp, s->d_red + (size_t)RED_N * sl, s->d_ist + (size_t)IST_N * sl));
  }
}

void drop_graph(ot2d_solver* s) {
  if (s->gexec) cudaGraphExecDestroy(s->gexec);
  if (s->graph) cudaGraphDestroy(s->graph);
  s->gexec = nullptr; s->graph = nullptr;
  for (int h = 0; h < 2; ++h) {
    if (s->hexec[h]) cudaGraphExecDestroy(s->hexec[h]);
    if (s->hgraph[h]) cudaGraphDestroy(s->hgraph[h]);
    s->hexec[h] = nullptr; s->hgraph[h] = nullptr;
  }
  s->split = false;
  s->split4 = false;
  s->halves = false;
  for (int q = 0; q < ot2d_solver::HP; ++q) {
    if (s->pexec[q]) cudaGraphExecDestroy(s->pexec[q]);
    if (s->pgraph[q]) cudaGraphDestroy(s->pgraph[q]);
    s->pexec[q] = nullptr; s->pgraph[q] = nullptr;
  }
  s->parts = false;
}

// batches of at least this many slices run as two pipelined halves
constexpr int PIPE_MIN_SLICES = 16;

// one iteration of every live instance: the single graph, or the two halves
// with their cross waits
cudaError_t launch_graph_iteration(ot2d_solver* s) {
  if (s->split4) {
    // four independent parts, each on its own stream after what the solver
    // stream holds (uploads, a rebuild's time step)
    cudaError_t e = cudaEventRecord(s->ev_step, s->st);
    for (int q = 0; q < ot2d_solver::HP && e == cudaSuccess; ++q) {
      e = cudaStreamWaitEvent(s->pst[q], s->ev_step, 0);
      if (e == cudaSuccess) e = cudaGraphLaunch(s->pexec[q], s->pst[q]);
    }
    return e;
  }
  if (!s->split) return cudaGraphLaunch(s->gexec, s->st);
  cudaError_t e;
  // half 0 of iteration i after half 1's residual of iteration i-1
  if ((e = cudaStreamWaitEvent(s->st, s->ev_half[1], 0)) != cudaSuccess) return e;
  if ((e = cudaGraphLaunch(s->hexec[0], s->st)) != cudaSuccess) return e;
  // half 1 of iteration i after half 0's residual of iteration i
  if ((e = cudaStreamWaitEvent(s->st2, s->ev_half[0], 0)) != cudaSuccess) return e;
  return cudaGraphLaunch(s->hexec[1], s->st2);
}

// make the solver stream wait for the second half's work
cudaError_t join_halves(ot2d_solver* s) {
  if (s->split4) {
    cudaError_t e = cudaSuccess;
    for (int q = 0; q < ot2d_solver::HP && e == cudaSuccess; ++q) {
      e = cudaEventRecord(s->ev_pdone[q], s->pst[q]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s->st, s->ev_pdone[q], 0);
    }
    return e;
  }
  if (!s->split) return cudaSuccess;
  cudaError_t e = cudaEventRecord(s->ev_join, s->st2);
  return e == cudaSuccess ? cudaStreamWaitEvent(s->st, s->ev_join, 0) : e;
}

template <class R> DevBatch<R>* halves_of(ot2d_solver* s);
template <> DevBatch<double>* halves_of<double>(ot2d_solver* s) { return s->h64; }
template <> DevBatch<float>* halves_of<float>(ot2d_solver* s) { return s->h32; }
template <class R> DevBatch<R>* parts_of(ot2d_solver* s);
template <> DevBatch<double>* parts_of<double>(ot2d_solver* s) { return s->p64; }
template <> DevBatch<float>* parts_of<float>(ot2d_solver* s) { return s->p32; }

// The host-buffer path's parts: HP batches of about equal cells (a
// request's time instances in one part), each captured as its own graph
// on its own stream, with B's launch choices.
template <class R>
int build_parts(ot2d_solver* s, const DevBatch<R>& B, int visc) {
  constexpr int HP = ot2d_solver::HP;
  std::vector<int> ids = s->live;
  auto cells_of = [&](int id) { const ot2d_params& p = s->recs[id].d.P; return (size_t)p.jd * p.kd * p.nspec; };
  std::stable_sort(ids.begin(), ids.end(), [&](int a, int b) { return cells_of(a) > cells_of(b); });
  std::vector<Slice<R>> slp[HP];
  size_t load[HP] = {};
  for (int id : ids) {
    int q = 0;
    for (int i = 1; i < HP; ++i)
      if (load[i] < load[q]) q = i;
    load[q] += cells_of(id);
    slices_of<R>(s, s->recs[id], slp[q]);
    s->recs[id].part = q;
  }
  DevBatch<R>* P = parts_of<R>(s);
  for (int q = 0; q < HP; ++q) {
    if (!s->pst[q] && cudaStreamCreateWithFlags(&s->pst[q], cudaStreamNonBlocking) != cudaSuccess) return OT2D_ERR_CUDA;
    if (!s->ev_pdone[q] && cudaEventCreateWithFlags(&s->ev_pdone[q], cudaEventDisableTiming) != cudaSuccess)
      return OT2D_ERR_CUDA;
    P[q].rt_shape = B.rt_shape;
    int e = P[q].build(slp[q], s->st);
    if (e) return e;
    P[q].b.poll_limit = B.b.poll_limit;
    P[q].b.ts_in_update = B.b.ts_in_update;
    P[q].b.lu_lag = B.b.lu_lag;
    P[q].b.lu_group = B.b.lu_group;
    cudaStream_t cs = s->pst[q];
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return OT2D_ERR_CUDA;
    cudaError_t le = launch_iteration<R>(P[q].d_sl, P[q].b, visc, s->turb_bits, s->lhs_bits, cs);
    cudaError_t ce = cudaStreamEndCapture(cs, &s->pgraph[q]);
    if (le != cudaSuccess || ce != cudaSuccess) return OT2D_ERR_CUDA;
    if (cudaGraphInstantiate(&s->pexec[q], s->pgraph[q], 0) != cudaSuccess) return OT2D_ERR_CUDA;
  }
  s->parts = true;
  return OT2D_OK;
}

// With the time step folded into the state update, the first iteration of a
// new batch still needs it: computed now from the current state (for the
// requests already running, the values the last update computed).
template <class R>
int time_step_now(ot2d_solver* s, DevBatch<R>& B) {
  if (!B.b.ts_in_update) return OT2D_OK;
  return launch_time_step<R>(B.d_sl, B.b, s->st) == cudaSuccess ? OT2D_OK : OT2D_ERR_CUDA;
}

template <class R>
int rebuild_t(ot2d_solver* s, DevBatch<R>& B) {
  drop_graph(s);
  std::vector<Slice<R>> sl;
  s->any_viscous = false; s->turb_bits = 0; s->lhs_bits = 0;
  for (int id : s->live) {
    const Rec& r = s->recs[id];
    slices_of<R>(s, r, sl);
    if (!r.d.P.invisc) s->any_viscous = true;
    if (!r.d.P.lamin && r.d.P.iturb == 1) s->turb_bits |= 1;
    if (!r.d.P.lamin && r.d.P.iturb == 2) s->turb_bits |= 2;
    s->lhs_bits |= (r.d.P.ilhs == 1) ? 1 : 2;
  }
  s->dirty = false;
  if (sl.empty()) return OT2D_OK;
  // launch choices: the tuning entry of the batch's largest mesh, else the options
  ot2d_tuning ch{0, 0, s->rt_shape, s->lu_group, s->lu_lag, s->pipeline};
  {
    size_t best = 0;
    int kd = 0, jd = 0;
    for (int id : s->live) {
      const ot2d_params& p = s->recs[id].d.P;
      const size_t cells = (size_t)p.jd * p.kd * p.nspec;
      if (cells > best) { best = cells; kd = p.kd; jd = p.jd; }
    }
    for (const ot2d_tuning& t : s->tuning)
      if (kd <= t.kd_max && jd <= t.jd_max) { ch = t; break; }
  }
  s->applied = ch;
  B.rt_shape = ch.rt_shape;
  int e = B.build(sl, s->st);
  if (e) return e;
  B.b.poll_limit = s->poll_limit;
  // the next iteration's time step in the state update: every request
  // steady with a first-order time step factor (nothing between the update
  // and the next time step then changes what the time step reads)
  bool fuse_ts = true;
  for (int id : s->live) {
    const ot2d_params& pp = s->recs[id].d.P;
    if (pp.iunst != 0 || pp.ntac > 1 || pp.itnmax > 1) fuse_ts = false;
  }
  B.b.ts_in_update = fuse_ts ? 1 : 0;
  B.b.lu_lag = ch.lu_lag;
  B.b.lu_group = ch.lu_group;
  // The kernels branch on each slice's own params, so inviscid, laminar,
  // SA and SST requests can share one batch.
  Branch* br = nullptr;   // the turbulence branch's stream, created outside the capture
  if (branch_of_device(br) != cudaSuccess) return OT2D_ERR_CUDA;
  const int visc = s->any_viscous ? 1 : 0;
  const bool can_split = sl.size() >= (size_t)PIPE_MIN_SLICES && s->live.size() >= 2;
  const bool split = ch.pipeline == 1 && can_split;
  const bool can_parts = sl.size() >= (size_t)PIPE_MIN_SLICES && s->live.size() >= (size_t)ot2d_solver::HP;
  const bool split4 = ch.pipeline == 2 && can_parts;
  if (split4 && !s->ev_step && cudaEventCreateWithFlags(&s->ev_step, cudaEventDisableTiming) != cudaSuccess)
    return OT2D_ERR_CUDA;
  for (int id : s->live) { s->recs[id].half = -1; s->recs[id].part = -1; }
  // the parts: for the device-resident iteration (OT2D_OPT_PIPELINE 2) or
  // once the host-buffer path has been used
  const bool want_parts = (s->want_parts || ch.pipeline == 2) && sl.size() >= (size_t)PIPE_MIN_SLICES &&
                          s->live.size() >= (size_t)ot2d_solver::HP;
  if (!split) {
    if (cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return OT2D_ERR_CUDA;
    cudaError_t le = launch_iteration<R>(B.d_sl, B.b, visc, s->turb_bits, s->lhs_bits, s->st);
    cudaError_t ce = cudaStreamEndCapture(s->st, &s->graph);
    if (le != cudaSuccess || ce != cudaSuccess) return OT2D_ERR_CUDA;
    if (cudaGraphInstantiate(&s->gexec, s->graph, 0) != cudaSuccess) return OT2D_ERR_CUDA;
    if (want_parts && (e = build_parts<R>(s, B, visc))) return e;
    s->split4 = split4;
    return time_step_now<R>(s, B);
  }
  // two halves of about equal cells (a request's time instances stay in one
  // half: the time-spectral source couples them)
  std::vector<int> ids = s->live;
  auto cells_of = [&](int id) { const ot2d_params& p = s->recs[id].d.P; return (size_t)p.jd * p.kd * p.nspec; };
  std::stable_sort(ids.begin(), ids.end(), [&](int a, int b) { return cells_of(a) > cells_of(b); });
  std::vector<Slice<R>> slh[2];
  size_t load[2] = {0, 0};
  for (int id : ids) {
    const int h = load[0] <= load[1] ? 0 : 1;
    load[h] += cells_of(id);
    slices_of<R>(s, s->recs[id], slh[h]);
    s->recs[id].half = h;
  }
  if (!s->st2 && cudaStreamCreateWithFlags(&s->st2, cudaStreamNonBlocking) != cudaSuccess) return OT2D_ERR_CUDA;
  for (int h = 0; h < 2; ++h)
    if (!s->ev_half[h] && cudaEventCreateWithFlags(&s->ev_half[h], cudaEventDisableTiming) != cudaSuccess)
      return OT2D_ERR_CUDA;
  if (!s->ev_join && cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming) != cudaSuccess) return OT2D_ERR_CUDA;
  DevBatch<R>* H = halves_of<R>(s);
  for (int h = 0; h < 2; ++h) {
    H[h].rt_shape = ch.rt_shape;
    if ((e = H[h].build(slh[h], s->st))) return e;
    H[h].b.poll_limit = s->poll_limit;
    H[h].b.ts_in_update = B.b.ts_in_update;
    H[h].b.lu_lag = ch.lu_lag;
    H[h].b.lu_group = ch.lu_group;
    cudaStream_t cs = h == 0 ? s->st : s->st2;
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return OT2D_ERR_CUDA;
    cudaError_t le = launch_iteration<R>(H[h].d_sl, H[h].b, visc, s->turb_bits, s->lhs_bits, cs, s->ev_half[h]);
    cudaError_t ce = cudaStreamEndCapture(cs, &s->hgraph[h]);
    if (le != cudaSuccess || ce != cudaSuccess) return OT2D_ERR_CUDA;
    if (cudaGraphInstantiate(&s->hexec[h], s->hgraph[h], 0) != cudaSuccess) return OT2D_ERR_CUDA;
  }
  s->halves = true;
  s->split = split;
  if (want_parts && (e = build_parts<R>(s, B, visc))) return e;
  return time_step_now<R>(s, B);
}

int rebuild(ot2d_solver* s) {
  return s->precision == OT2D_FP64 ? rebuild_t<double>(s, s->b64) : rebuild_t<float>(s, s->b32);
}

template <class R>
int forces_t(ot2d_solver* s, const std::vector<int>& ids, DevBatch<R>& tmp) {
  std::vector<Slice<R>> sl;
  std::vector<const double*> xy;
  for (int id : ids) {
    const Rec& r = s->recs[id];
    slices_of<R>(s, r, sl);
  }
  for (int id : ids) {
    const Rec& r = s->recs[id];
    for (int nsp = 0; nsp < r.d.nspec; ++nsp) xy.push_back(r.d.xv + (size_t)nsp * r.d.nvert);
  }
  for (int id : ids) {
    const Rec& r = s->recs[id];
    for (int nsp = 0; nsp < r.d.nspec; ++nsp) xy.push_back(r.d.yv + (size_t)nsp * r.d.nvert);
  }
  const size_t n = sl.size();
  if (n == 0) return OT2D_OK;
  int e = tmp.build(sl, s->st);
  if (e) return e;
  if (s->forces_cap < n) {
    if (s->d_forces) cudaFree(s->d_forces);
    if (s->d_xy) cudaFree(s->d_xy);
    s->forces_cap = 2 * n;
    cudaMalloc(&s->d_forces, sizeof(double) * 4 * s->forces_cap);
    cudaMalloc(&s->d_xy, sizeof(double*) * 2 * s->forces_cap);
  }
  cudaMemcpyAsync(s->d_xy, xy.data(), sizeof(double*) * 2 * n, cudaMemcpyHostToDevice, s->st);
  if (launch_forces<R>(tmp.d_sl, tmp.b, s->d_xy, s->d_xy + n, s->d_forces, s->st) != cudaSuccess) return OT2D_ERR_CUDA;
  std::vector<double> f(4 * n);
  cudaMemcpyAsync(f.data(), s->d_forces, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, s->st);
  if (cudaStreamSynchronize(s->st) != cudaSuccess) return OT2D_ERR_CUDA;
  size_t i = 0;
  const double pi = 4.0 * std::atan(1.0);
  for (int id : ids) {
    Rec& r = s->recs[id];
    const ot2d_params& p = r.d.P;
    const double ca = std::cos(pi * p.alfa / 180.0), sa = std::sin(pi * p.alfa / 180.0);
    double cl = 0, cd = 0, cm = 0, cp = 0;
    for (int nsp = 0; nsp < r.d.nspec; ++nsp, ++i) {
      double cfx = f[4 * i], cfy = f[4 * i + 1], cm0 = f[4 * i + 2];
      cl = cl + (-cfx * sa + cfy * ca);
      cd = cd + (cfx * ca + cfy * sa);
      cm = cm + (cm0 - 0.00 * cfx + 0.25 * cfy);
      cp = cp + f[4 * i + 3];
    }
    r.res.cl = cl; r.res.cd = cd; r.res.cm = cm; r.res.cpower = cp;
  }
  return OT2D_OK;
}

// Phase timing of the iteration (events between the kernel families on the
// solver stream); advances the live requests by `iters` iterations.
template <class R>
int profile_t(ot2d_solver* s, DevBatch<R>& B, int iters, double* ms) {
  cudaEvent_t ev[OT2D_NPHASE + 1];
  for (auto& e : ev) cudaEventCreate(&e);
  for (int p = 0; p < OT2D_NPHASE; ++p) ms[p] = 0.0;
  const int visc = s->any_viscous ? 1 : 0, turb = s->turb_bits;
  // each phase on its own: the time step as a kernel of its own here
  Batch bp = B.b;
  bp.ts_in_update = 0;
  int err = OT2D_OK;
  for (int it = 0; it < iters && !err; ++it) {
    cudaError_t e = cudaSuccess;
    auto rec = [&](int i) { cudaEventRecord(ev[i], s->st); };
    rec(0);
    e = launch_iter_begin<R>(B.d_sl, bp, s->st);
    if (!e) e = launch_time_step<R>(B.d_sl, bp, s->st); rec(1);
    if (!e) e = launch_bc<R>(B.d_sl, bp, 1, s->st); rec(2);
    if (!e) e = launch_residual<R>(B.d_sl, bp, visc, s->st); rec(3);
    if (!e) e = launch_rbc<R>(B.d_sl, bp, s->st); rec(4);
    if (!e && (s->lhs_bits & 1)) e = launch_lusgs<R>(B.d_sl, bp, 1, s->st, 1);
    if (!e && (s->lhs_bits & 2)) e = launch_adi<R>(B.d_sl, bp, 1, s->st, 1);
    rec(5);
    if (!e && (turb & 1)) e = launch_sa<R>(B.d_sl, bp, s->st);
    if (!e && (turb & 2)) e = launch_sst<R>(B.d_sl, bp, s->st);
    rec(6);
    if (!e) e = launch_update<R>(B.d_sl, bp, s->st);
    rec(7);
    if (e != cudaSuccess || cudaEventSynchronize(ev[7]) != cudaSuccess) { err = OT2D_ERR_CUDA; break; }
    for (int p = 0; p < OT2D_NPHASE; ++p) {
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[p], ev[p + 1]);
      ms[p] += t;
    }
    ++s->since_check;
  }
  for (int p = 0; p < OT2D_NPHASE; ++p) ms[p] /= iters;
  for (auto& e : ev) cudaEventDestroy(e);
  return err;
}

// astore (io.f:2-170) of one live instance: the device pack converts and
// round-trips q; cell centres come from the device vertex grids through the
// set-up routine find_cellcenter; istep0 is the instance's step counter.
int store_rec(ot2d_solver* s, Rec& r, const std::string& dir) {
  const ot2d_params& p = r.d.P;
  const size_t n2 = r.d.n2, nv = r.d.nvert, ns = (size_t)p.nspec;
  int32_t ist[IST_N];
  std::vector<double> xv(nv * ns), yv(nv * ns), x(n2 * ns), y(n2 * ns);
  std::vector<int32_t> ib(n2 * ns);
  if (cudaMemcpyAsync(ist, s->d_ist + (size_t)IST_N * r.slots[0], sizeof(ist), cudaMemcpyDeviceToHost, s->st) !=
          cudaSuccess ||
      cudaMemcpyAsync(xv.data(), r.d.xv, xv.size() * 8, cudaMemcpyDeviceToHost, s->st) != cudaSuccess ||
      cudaMemcpyAsync(yv.data(), r.d.yv, yv.size() * 8, cudaMemcpyDeviceToHost, s->st) != cudaSuccess ||
      cudaMemcpyAsync(ib.data(), r.d.iblank, ib.size() * 4, cudaMemcpyDeviceToHost, s->st) != cudaSuccess ||
      cudaStreamSynchronize(s->st) != cudaSuccess)
    return OT2D_ERR_CUDA;
  for (size_t k = 0; k < ns; ++k)
    cell_centres(p, xv.data() + k * nv, yv.data() + k * nv, x.data() + k * n2, y.data() + k * n2);
  float* qc = s->precision == OT2D_FP32_MIXED ? (float*)r.d.q : nullptr;
  // totime as the driver keeps it: 0 at the start of the run, + dt per
  // physical step of a time-accurate run (Turns_overset.f:359, :365)
  ot2d_params pw = p;
  pw.totime = 0.0;
  if (p.iunst != 0)
    for (int i = 0; i < ist[1]; ++i) pw.totime = pw.totime + p.dt;
  return write_solution(dir, pw, r.d.q64, qc, x.data(), y.data(), ib.data(), ist[0], s->st);
}

size_t budget_of(const ot2d_solver* s) { return s->budget_set ? s->budget_set : s->budget_auto; }

// The launches of the batch a new mesh would join must still fit.
bool fits_with_live(ot2d_solver* s, const ot2d_params& p) {
  int kdm = p.kd, jdm = p.jd;
  bool pre = p.iprecon != 0;
  for (int id : s->live) {
    const ot2d_params& q = s->recs[id].d.P;
    kdm = std::max(kdm, (int)q.kd); jdm = std::max(jdm, (int)q.jd); pre = pre || q.iprecon;
  }
  return batch_fits(s->precision, pre, kdm, jdm);
}

// Create the device state of a submitted solve and make it live.
int admit(ot2d_solver* s, Pending& pd) {
  if (grow_slots(s, pd.p.nspec) != OT2D_OK) return OT2D_ERR_NOMEM;
  Rec r;
  int e = solve_create(r.d, pd.p, s->precision, pd.xv.data(), pd.yv.data(), s->st);
  if (e) return e;
  double orders = pd.orders;
  if (pd.p.iunst == 1) {
    // time accurate: max_iters physical steps, the pitch table for them,
    // no residual convergence test
    e = solve_motion_table(r.d, pd.max_iters, s->st);
    if (e) { solve_destroy(r.d); return e; }
    orders = 0.0;
  }
  r.id = pd.id;
  r.orders = orders; r.max_iters = pd.max_iters; r.live = true;
  r.res.id = r.id;
  r.res.t_submit = pd.t_submit;
  r.res.t_admit = now_s() - s->t0;
  std::vector<double> red(RED_N, 0.0);
  std::vector<int32_t> ist(IST_N, 0);
  red[7] = orders > 0 ? std::pow(10.0, -orders) : -1.0;
  ist[0] = pd.p.istep0; ist[1] = 0;
  for (int nsp = 0; nsp < pd.p.nspec; ++nsp) {
    int sl = s->free_slots.back(); s->free_slots.pop_back();
    r.slots.push_back(sl);
    cudaMemcpyAsync(s->d_red + (size_t)RED_N * sl, red.data(), sizeof(double) * RED_N, cudaMemcpyHostToDevice, s->st);
    cudaMemcpyAsync(s->d_ist + (size_t)IST_N * sl, ist.data(), sizeof(int32_t) * IST_N, cudaMemcpyHostToDevice, s->st);
  }
  if (cudaStreamSynchronize(s->st) != cudaSuccess) {
    for (int sl : r.slots) s->free_slots.push_back(sl);
    solve_destroy(r.d);
    return OT2D_ERR_CUDA;
  }
  const int id = r.id;
  {
    char m[96];
    std::snprintf(m, sizeof(m), "ot2d admit id=%d %dx%dx%d", id, (int)pd.p.jmax, (int)pd.p.kmax, (int)pd.p.nspec);
    nvtxMarkA(m);
  }
  s->used += r.d.bytes;
  auto prev = s->recs.find(id);
  if (prev != s->recs.end()) r.store_dir = prev->second.store_dir;   // set while it was queued
  s->recs[id] = std::move(r);
  s->live.push_back(id);
  s->dirty = true;
  if (pd.init) {
    Rec& rr = s->recs[id];
    e = pd.init(s, rr);
    if (e) {
      for (int sl : rr.slots) s->free_slots.push_back(sl);
      rr.slots.clear();
      s->used -= rr.d.bytes;
      solve_destroy(rr.d);
      rr.live = false;
      s->live.erase(std::remove(s->live.begin(), s->live.end(), id), s->live.end());
      return e;
    }
  }
  return OT2D_OK;
}

// Admit queued solves in submission order while they fit the budget and the
// batch launches; a failed admission retires that solve with its status.
void admit_queued(ot2d_solver* s) {
  while (!s->queue.empty()) {
    Pending& head = s->queue.front();
    if (s->used + head.bytes > budget_of(s) || !fits_with_live(s, head.p)) break;
    Pending pd = std::move(head);
    s->queue.pop_front();
    const int e = admit(s, pd);
    if (e) {
      Rec& r = s->recs[pd.id];
      r.live = false;
      r.queued = false;
      r.res.status = e;
      r.res.t_done = now_s() - s->t0;
    }
  }
}

// Submit a solve: admitted now when it fits (and nothing is queued ahead of
// it), queued otherwise.  Returns the id or -status.
int submit(ot2d_solver* s, const ot2d_params* p, const double* xv, const double* yv, double orders, int max_iters,
           InitFn init) {
  if (!s || !p || !xv || !yv || max_iters < 1) return -OT2D_ERR_ARG;
  cudaSetDevice(s->device);
  // a mesh that cannot launch even alone, or cannot fit the budget at all
  if (!batch_fits(s->precision, p->iprecon != 0, p->kd, p->jd)) return -OT2D_ERR_ARG;
  const size_t bytes = solve_bytes(*p, s->precision);
  if (bytes > budget_of(s)) return -OT2D_ERR_NOMEM;
  Pending pd;
  pd.id = s->next_id++;
  pd.p = *p;
  const size_t nv = (size_t)p->jmax * p->kmax;
  pd.xv.assign(xv, xv + nv);
  pd.yv.assign(yv, yv + nv);
  pd.orders = orders; pd.max_iters = max_iters; pd.bytes = bytes;
  pd.t_submit = now_s() - s->t0;
  pd.init = std::move(init);
  if (s->queue.empty() && s->used + bytes <= budget_of(s) && fits_with_live(s, *p)) {
    const int e = admit(s, pd);
    return e ? -e : pd.id;
  }
  Rec r;
  r.id = pd.id;
  r.res.id = pd.id;
  r.res.t_submit = pd.t_submit;
  r.res.t_admit = -1.0;
  r.max_iters = max_iters;
  r.queued = true;
  s->recs[pd.id] = std::move(r);
  const int id = pd.id;
  s->queue.push_back(std::move(pd));
  return id;
}

// One JSON line per retired request (ot2d_solver_set_log).
void log_retired(ot2d_solver* s, const Rec& r) {
  if (!s->log) return;
  const ot2d_params& p = r.d.P;
  std::fprintf(s->log,
               "{\"id\": %d, \"status\": %d, \"converged\": %d, \"iterations\": %d, \"precision\": \"%s\", "
               "\"jmax\": %d, \"kmax\": %d, \"nspec\": %d, \"fsmach\": %.17g, \"alfa\": %.17g, \"orders\": %.17g, "
               "\"rsum_first\": %.17g, \"rsum_last\": %.17g, \"cl\": %.17g, \"cd\": %.17g, \"cm\": %.17g, "
               "\"t_submit\": %.6f, \"t_admit\": %.6f, \"t_done\": %.6f}\n",
               r.id, r.res.status, r.res.converged, r.res.iterations, s->precision == OT2D_FP64 ? "fp64" : "fp32-mixed",
               (int)p.jmax, (int)p.kmax, (int)p.nspec, p.fsmach, p.alfa, r.orders, r.res.rsum_first, r.res.rsum_last,
               r.res.cl, r.res.cd, r.res.cm, r.res.t_submit, r.res.t_admit, r.res.t_done);
  std::fflush(s->log);
}

int check_inner(ot2d_solver* s);

int check(ot2d_solver* s) {
  nvtxRangePushA("ot2d status check");
  const int e = check_inner(s);
  nvtxRangePop();
  return e;
}

int check_inner(ot2d_solver* s) {
  s->since_check = 0;
  if (s->live.empty()) return OT2D_OK;
  cudaMemcpyAsync(s->h_red, s->d_red, sizeof(double) * RED_N * s->cap, cudaMemcpyDeviceToHost, s->st);
  cudaMemcpyAsync(s->h_ist, s->d_ist, sizeof(int32_t) * IST_N * s->cap, cudaMemcpyDeviceToHost, s->st);
  if (cudaStreamSynchronize(s->st) != cudaSuccess) return OT2D_ERR_CUDA;
  std::vector<int> done;
  for (int id : s->live) {
    Rec& r = s->recs[id];
    int status = 0, conv_it = 0, its = 0; bool conv = true;
    for (int sl : r.slots) {
      const int32_t* ist = s->h_ist + (size_t)IST_N * sl;
      if (ist[2] & 1) status = OT2D_ERR_NORM;
      else if ((ist[2] & 18) && !status) status = OT2D_ERR_MONITOR;   // bad state / folded cell
      else if ((ist[2] & 4) && !status) status = OT2D_ERR_TIMEOUT;    // a sweep wait gave up
      else if ((ist[2] & 8) && !status) status = OT2D_ERR_ARG;        // step beyond the motion table
      if (ist[3] == 0) conv = false;
      conv_it = std::max(conv_it, (int)ist[3]);
      its = ist[1];
    }
    const double* red = s->h_red + (size_t)RED_N * r.slots[0];
    r.res.rsum_first = red[4];
    r.res.rsum_last = red[5];
    r.res.iterations = conv ? conv_it : its;
    r.res.status = status;
    r.res.converged = (conv && !status) ? 1 : 0;
    if (status || conv || r.launched >= iter_cap(r)) done.push_back(id);
  }
  if (s->force_dcl > 0 || s->force_dcd > 0) {
    // forces of the instances still running; converged once CL and CD stayed
    // within the tolerances over the last FORCE_WIN checks and the L2 norm
    // is a decade below its peak
    std::vector<int> run;
    for (int id : s->live) {
      const Rec& r = s->recs[id];
      if (std::find(done.begin(), done.end(), id) != done.end()) continue;
      if (s->force_every > 0 && r.nwin > 0 && r.launched - r.force_at < s->force_every) continue;
      run.push_back(id);
    }
    if (!run.empty()) {
      int fe = (s->precision == OT2D_FP64) ? forces_t<double>(s, run, s->f64) : forces_t<float>(s, run, s->f32);
      if (fe) return fe;
      for (int id : run) {
        Rec& r = s->recs[id];
        const double* red = s->h_red + (size_t)RED_N * r.slots[0];
        r.win_cl[r.nwin % FORCE_WIN] = r.res.cl;
        r.win_cd[r.nwin % FORCE_WIN] = r.res.cd;
        ++r.nwin;
        r.force_at = r.launched;
        if (r.nwin < FORCE_WIN || !(red[5] <= std::pow(10.0, -s->force_decades) * red[6])) continue;
        double lo_l = r.win_cl[0], hi_l = lo_l, lo_d = r.win_cd[0], hi_d = lo_d;
        for (int i = 1; i < FORCE_WIN; ++i) {
          lo_l = std::min(lo_l, r.win_cl[i]); hi_l = std::max(hi_l, r.win_cl[i]);
          lo_d = std::min(lo_d, r.win_cd[i]); hi_d = std::max(hi_d, r.win_cd[i]);
        }
        if (hi_l - lo_l <= s->force_dcl && hi_d - lo_d <= s->force_dcd) { r.res.converged = 1; done.push_back(id); }
      }
    }
  }
  if (done.empty()) return OT2D_OK;
  int e = (s->precision == OT2D_FP64) ? forces_t<double>(s, done, s->f64) : forces_t<float>(s, done, s->f32);
  const double t = now_s() - s->t0;
  for (int id : done) {
    Rec& r = s->recs[id];
    r.res.t_done = t;
    {
      char m[80];
      std::snprintf(m, sizeof(m), "ot2d retire id=%d status=%d converged=%d", id, r.res.status, r.res.converged);
      nvtxMarkA(m);
    }
    log_retired(s, r);
    if (!r.store_dir.empty()) {
      const int se = store_rec(s, r, r.store_dir);
      if (se && !e) e = se;
    }
    if (s->keep_q) {
      r.qkeep.resize((size_t)r.d.n2 * r.d.nspec * r.d.P.nq);
      cudaMemcpy(r.qkeep.data(), r.d.q64, r.qkeep.size() * sizeof(double), cudaMemcpyDeviceToHost);
    }
    for (int sl : r.slots) s->free_slots.push_back(sl);
    r.slots.clear();
    s->used -= r.d.bytes;
    solve_destroy(r.d);
    r.live = false;
  }
  std::vector<int> nl;
  for (int id : s->live) if (s->recs[id].live) nl.push_back(id);
  s->live.swap(nl);
  s->dirty = true;
  // the memory just freed admits queued solves
  admit_queued(s);
  return e;
}

}  // namespace

extern "C" {

ot2d_solver* ot2d_solver_create(int32_t device, int32_t precision) {
  if (precision != OT2D_FP64 && precision != OT2D_FP32_MIXED) return nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return nullptr;
  ot2d_solver* s = new ot2d_solver();
  s->device = device; s->precision = precision;
  if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess) { delete s; return nullptr; }
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) s->budget_auto = fr / 10 * 9;
  s->t0 = now_s();
  return s;
}

void ot2d_solver_destroy(ot2d_solver* s) {
  if (!s) return;
  cudaStreamSynchronize(s->st);
  if (s->st2) cudaStreamSynchronize(s->st2);
  if (s->st_d2h) cudaStreamSynchronize(s->st_d2h);
  drop_graph(s);
  for (int h = 0; h < 2; ++h) {
    s->h64[h].release(); s->h32[h].release();
    if (s->ev_half[h]) cudaEventDestroy(s->ev_half[h]);
  }
  if (s->ev_join) cudaEventDestroy(s->ev_join);
  for (int q = 0; q < ot2d_solver::HP; ++q) {
    s->p64[q].release(); s->p32[q].release();
    if (s->ev_pdone[q]) cudaEventDestroy(s->ev_pdone[q]);
    if (s->pst[q]) { cudaStreamSynchronize(s->pst[q]); cudaStreamDestroy(s->pst[q]); }
  }
  if (s->st2) cudaStreamDestroy(s->st2);
  for (auto& kv : s->recs) solve_destroy(kv.second.d);
  for (cudaEvent_t e : s->ev_d2h) cudaEventDestroy(e);
  if (s->ev_step) cudaEventDestroy(s->ev_step);
  if (s->st_d2h) cudaStreamDestroy(s->st_d2h);
  s->b64.release(); s->b32.release(); s->f64.release(); s->f32.release();
  if (s->d_red) cudaFree(s->d_red);
  if (s->d_ist) cudaFree(s->d_ist);
  if (s->h_red) cudaFreeHost(s->h_red);
  if (s->h_ist) cudaFreeHost(s->h_ist);
  if (s->d_forces) cudaFree(s->d_forces);
  if (s->d_xy) cudaFree(s->d_xy);
  if (s->log) std::fclose(s->log);
  cudaStreamDestroy(s->st);
  delete s;
}

int ot2d_solver_set_option(ot2d_solver* s, int32_t key, int32_t value) {
  if (!s) return OT2D_ERR_ARG;
  if (key == OT2D_OPT_CHECK_EVERY && value >= 1) { s->check_every = value; return OT2D_OK; }
  if (key == OT2D_OPT_KEEP_Q) { s->keep_q = value ? 1 : 0; return OT2D_OK; }
  if (key == OT2D_OPT_FORCE_EVERY && value >= 0) { s->force_every = value; return OT2D_OK; }
  if (key == OT2D_OPT_FORCE_DECADES && value >= 0) { s->force_decades = value; return OT2D_OK; }
  if (key == OT2D_OPT_BUDGET_MB && value >= 0) { s->budget_set = (size_t)value << 20; return OT2D_OK; }
  if (key == OT2D_OPT_LU_LAG && value >= 0 && value <= 64) { s->lu_lag = value; s->dirty = true; return OT2D_OK; }
  if (key == OT2D_OPT_RT_SHAPE && value >= 0 && value < RT_NSHAPE) { s->rt_shape = value; s->dirty = true; return OT2D_OK; }
  if (key == OT2D_OPT_PIPELINE && value >= 0 && value <= 2) { s->pipeline = value; s->dirty = true; return OT2D_OK; }
  if (key == OT2D_OPT_LU_GROUP && (value == 0 || value == 1 || value == 2 || value == 4 || value == 8)) {
    s->lu_group = value;
    s->dirty = true;
    return OT2D_OK;
  }
  if (key == OT2D_OPT_POLL_LIMIT && value >= 1) {
    s->poll_limit = (uint32_t)value;
    s->dirty = true;   // the sweeps take the limit as a launch argument
    return OT2D_OK;
  }
  return OT2D_ERR_ARG;
}

int ot2d_solver_set_log(ot2d_solver* s, const char* path) {
  if (!s) return OT2D_ERR_ARG;
  if (s->log) { std::fclose(s->log); s->log = nullptr; }
  if (!path) return OT2D_OK;
  s->log = std::fopen(path, "a");
  return s->log ? OT2D_OK : OT2D_ERR_IO;
}

int ot2d_solver_set_tuning(ot2d_solver* s, const ot2d_tuning* t, int32_t n) {
  if (!s || n < 0 || (n && !t)) return OT2D_ERR_ARG;
  for (int i = 0; i < n; ++i) {
    const ot2d_tuning& e = t[i];
    const bool g = e.lu_group == 0 || e.lu_group == 1 || e.lu_group == 2 || e.lu_group == 4 || e.lu_group == 8;
    if (e.rt_shape < 0 || e.rt_shape >= RT_NSHAPE || !g || e.lu_lag < 0 || e.lu_lag > 64 ||
        e.pipeline < 0 || e.pipeline > 2)
      return OT2D_ERR_ARG;
  }
  s->tuning.assign(t, t + n);
  s->dirty = true;
  return OT2D_OK;
}

int ot2d_solver_set_force_tol(ot2d_solver* s, double dcl, double dcd) {
  if (!s || dcl < 0 || dcd < 0) return OT2D_ERR_ARG;
  s->force_dcl = dcl; s->force_dcd = dcd;
  return OT2D_OK;
}

int ot2d_solver_add(ot2d_solver* s, const ot2d_params* p, const double* xv, const double* yv, double orders,
                    int32_t max_iters) {
  return submit(s, p, xv, yv, orders, max_iters, InitFn());
}

int ot2d_solver_iterate(ot2d_solver* s, int32_t iters) {
  if (!s || iters < 0) return OT2D_ERR_ARG;
  cudaSetDevice(s->device);
  int done = 0;
  while (done < iters) {
    admit_queued(s);
    if (s->dirty) { int e = rebuild(s); if (e) return e; }
    if (s->live.empty()) break;
    int chunk = std::min(s->check_every - s->since_check, iters - done);
    // no instance runs past its cap: stop the chunk at the first cap
    long rem = chunk;
    for (int id : s->live) rem = std::min(rem, iter_cap(s->recs[id]) - s->recs[id].launched);
    chunk = (int)std::max(1L, rem);
    nvtxRangePushA("ot2d iterations");
    for (int i = 0; i < chunk; ++i)
      if (launch_graph_iteration(s) != cudaSuccess) { nvtxRangePop(); return OT2D_ERR_CUDA; }
    nvtxRangePop();
    if (join_halves(s) != cudaSuccess) return OT2D_ERR_CUDA;
    bool capped = false;
    for (int id : s->live) {
      Rec& r = s->recs[id];
      r.launched += chunk;
      if (r.launched >= iter_cap(r)) capped = true;
    }
    s->since_check += chunk;
    done += chunk;
    if (s->since_check >= s->check_every || capped) { int e = check(s); if (e) return e; }
  }
  return OT2D_OK;
}

int ot2d_solver_sync(ot2d_solver* s) {
  if (!s) return OT2D_ERR_ARG;
  return check(s);
}

int ot2d_solver_live(const ot2d_solver* s) { return s ? (int)(s->live.size() + s->queue.size()) : 0; }

int ot2d_solver_queued(const ot2d_solver* s) { return s ? (int)s->queue.size() : 0; }

int ot2d_solver_result(ot2d_solver* s, int32_t id, ot2d_result* out) {
  if (!s || !out) return OT2D_ERR_ARG;
  auto it = s->recs.find(id);
  if (it == s->recs.end()) return OT2D_ERR_ARG;
  *out = it->second.res;
  return OT2D_OK;
}

int ot2d_solver_get_q(ot2d_solver* s, int32_t id, double* q_out) {
  if (!s || !q_out) return OT2D_ERR_ARG;
  auto it = s->recs.find(id);
  if (it == s->recs.end()) return OT2D_ERR_ARG;
  Rec& r = it->second;
  if (r.live) {
    size_t n = r.d.n2 * r.d.nspec * r.d.P.nq;
    if (cudaMemcpyAsync(q_out, r.d.q64, n * sizeof(double), cudaMemcpyDeviceToHost, s->st) != cudaSuccess) return OT2D_ERR_CUDA;
    return cudaStreamSynchronize(s->st) == cudaSuccess ? OT2D_OK : OT2D_ERR_CUDA;
  }
  if (r.qkeep.empty()) return OT2D_ERR_ARG;
  std::memcpy(q_out, r.qkeep.data(), r.qkeep.size() * sizeof(double));
  return OT2D_OK;
}

size_t ot2d_solver_device_bytes(const ot2d_solver* s) {
  if (!s) return 0;
  size_t b = 0;
  for (auto& kv : s->recs) if (kv.second.live) b += kv.second.d.bytes;
  return b;
}

size_t ot2d_instance_bytes(const ot2d_params* p, int32_t precision) { return p ? solve_bytes(*p, precision) : 0; }

void* ot2d_solver_stream(ot2d_solver* s) { return s ? (void*)s->st : nullptr; }

int ot2d_solver_profile(ot2d_solver* s, int32_t iters, double* ms, int32_t nphase) {
  if (!s || !ms || iters < 1 || nphase < OT2D_NPHASE) return OT2D_ERR_ARG;
  cudaSetDevice(s->device);
  if (s->dirty) { int e = rebuild(s); if (e) return e; }
  if (s->live.empty()) return OT2D_ERR_ARG;
  return s->precision == OT2D_FP64 ? profile_t<double>(s, s->b64, iters, ms) : profile_t<float>(s, s->b32, iters, ms);
}

static int kernel_nodes(cudaGraph_t g) {
  size_t n = 0;
  if (!g || cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess) return -OT2D_ERR_CUDA;
  std::vector<cudaGraphNode_t> nodes(n);
  if (n && cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return -OT2D_ERR_CUDA;
  int k = 0;
  for (cudaGraphNode_t nd : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nd, &t) != cudaSuccess) return -OT2D_ERR_CUDA;
    if (t == cudaGraphNodeTypeKernel) ++k;
  }
  return k;
}

int ot2d_solver_graph_kernels(ot2d_solver* s) {
  if (!s) return -OT2D_ERR_ARG;
  cudaSetDevice(s->device);
  if (s->dirty) { int e = rebuild(s); if (e) return -e; }
  if (s->live.empty()) return 0;
  if (s->split4) {
    int k = 0;
    for (int q = 0; q < ot2d_solver::HP; ++q) {
      const int a = kernel_nodes(s->pgraph[q]);
      if (a < 0) return a;
      k += a;
    }
    return k;
  }
  if (!s->split) return kernel_nodes(s->graph);
  const int a = kernel_nodes(s->hgraph[0]), b = kernel_nodes(s->hgraph[1]);
  return a < 0 ? a : (b < 0 ? b : a + b);
}

// The time step of the whole batch (part < 0) or of one host-buffer part,
// when the batch folds it into the state update: after a host-buffer upload.
cudaError_t host_time_step(ot2d_solver* s, int part, cudaStream_t st) {
  if (s->precision == OT2D_FP32_MIXED) {
    DevBatch<float>& B = part < 0 ? s->b32 : s->p32[part];
    return B.b.ts_in_update ? launch_time_step<float>(B.d_sl, B.b, st) : cudaSuccess;
  }
  DevBatch<double>& B = part < 0 ? s->b64 : s->p64[part];
  return B.b.ts_in_update ? launch_time_step<double>(B.d_sl, B.b, st) : cudaSuccess;
}

// Host-buffer iterations over a batch in parts: per iteration, part q
// uploads its listed instances on its stream (each upload after that
// instance's previous download), makes its compute copy and time step, runs
// its graph and downloads its instances on the download stream.  Some
// parts' copies thus run while others iterate; every instance computes what
// it computes in the single graph.
int iterate_host_parts(ot2d_solver* s, int32_t n, std::vector<Rec*>& rs, double* const* q_host, int32_t iters,
                       int32_t& done) {
  constexpr int HP = ot2d_solver::HP;
  done = 0;
  int err = OT2D_OK;
  bool parts = true;
  for (int it = 0; it < iters && !err && parts; ++it) {
    done = it + 1;
    for (int q = 0; q < HP && !err; ++q) {
      cudaStream_t sq = s->pst[q];
      for (int i = 0; i < n && !err; ++i) {
        if (rs[i]->part != q) continue;
        const size_t bytes = rs[i]->d.n2 * rs[i]->d.nspec * rs[i]->d.P.nq * sizeof(double);
        if ((it > 0 && cudaStreamWaitEvent(sq, s->ev_d2h[i], 0) != cudaSuccess) ||
            cudaMemcpyAsync(rs[i]->d.q64, q_host[i], bytes, cudaMemcpyHostToDevice, sq) != cudaSuccess)
          err = OT2D_ERR_CUDA;
      }
      if (!err && s->precision == OT2D_FP32_MIXED &&
          launch_shadow<float>(s->p32[q].d_sl, s->p32[q].b, sq) != cudaSuccess)
        err = OT2D_ERR_CUDA;
      // the uploaded state may differ from the one the last update saw
      if (!err && host_time_step(s, q, sq) != cudaSuccess) err = OT2D_ERR_CUDA;
      if (!err && (cudaGraphLaunch(s->pexec[q], sq) != cudaSuccess ||
                   cudaEventRecord(s->ev_pdone[q], sq) != cudaSuccess ||
                   cudaStreamWaitEvent(s->st_d2h, s->ev_pdone[q], 0) != cudaSuccess))
        err = OT2D_ERR_CUDA;
      for (int i = 0; i < n && !err; ++i) {
        if (rs[i]->part != q) continue;
        const size_t bytes = rs[i]->d.n2 * rs[i]->d.nspec * rs[i]->d.P.nq * sizeof(double);
        if (cudaMemcpyAsync(q_host[i], rs[i]->d.q64, bytes, cudaMemcpyDeviceToHost, s->st_d2h) != cudaSuccess ||
            cudaEventRecord(s->ev_d2h[i], s->st_d2h) != cudaSuccess)
          err = OT2D_ERR_CUDA;
      }
    }
    bool capped = false;
    for (int id : s->live) {
      Rec& r = s->recs[id];
      if (++r.launched >= iter_cap(r)) capped = true;
    }
    if (!err && (++s->since_check >= s->check_every || capped)) {
      // the status read sees every part done and no upload in flight
      for (int q = 0; q < HP && !err; ++q)
        if (cudaStreamWaitEvent(s->st, s->ev_pdone[q], 0) != cudaSuccess) err = OT2D_ERR_CUDA;
      if (!err && cudaStreamSynchronize(s->st_d2h) != cudaSuccess) err = OT2D_ERR_CUDA;
      if (!err) err = check(s);
      if (!err && s->dirty) {
        for (int i = 0; i < n; ++i)
          if (!rs[i]->live) { err = OT2D_ERR_ARG; break; }
        if (!err) err = rebuild(s);
        parts = s->parts;   // retirements took the batch below the parts' size
      }
    }
  }
  if (cudaStreamSynchronize(s->st_d2h) != cudaSuccess && !err) err = OT2D_ERR_CUDA;
  for (int q = 0; q < HP; ++q)
    if (cudaStreamSynchronize(s->pst[q]) != cudaSuccess && !err) err = OT2D_ERR_CUDA;
  if (cudaStreamSynchronize(s->st) != cudaSuccess && !err) err = OT2D_ERR_CUDA;
  return err;
}

int ot2d_solver_iterate_host(ot2d_solver* s, int32_t n, const int32_t* ids, double* const* q_host, int32_t iters) {
  if (!s || n < 0 || (n && (!ids || !q_host)) || iters < 0) return OT2D_ERR_ARG;
  cudaSetDevice(s->device);
  if (s->dirty) { int e = rebuild(s); if (e) return e; }
  std::vector<Rec*> rs;
  for (int i = 0; i < n; ++i) {
    auto it = s->recs.find(ids[i]);
    if (it == s->recs.end() || !it->second.live) return OT2D_ERR_ARG;
    rs.push_back(&it->second);
  }
  // Downloads run on their own stream: instance i's upload for the next
  // iteration waits only for its own download, so the uploads of early
  // instances overlap the downloads of later ones (both copy directions).
  if (!s->st_d2h && cudaStreamCreateWithFlags(&s->st_d2h, cudaStreamNonBlocking) != cudaSuccess) return OT2D_ERR_CUDA;
  if (!s->ev_step && cudaEventCreateWithFlags(&s->ev_step, cudaEventDisableTiming) != cudaSuccess) return OT2D_ERR_CUDA;
  while ((int)s->ev_d2h.size() < n) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return OT2D_ERR_CUDA;
    s->ev_d2h.push_back(e);
  }
  // A batch large enough for parts overlaps some parts' copies with the
  // others' iterations.
  if (!s->parts && !s->want_parts && s->live.size() >= (size_t)ot2d_solver::HP) {
    s->want_parts = true;
    s->dirty = true;
    int e = rebuild(s);
    if (e) return e;
  }
  int err = OT2D_OK;
  int32_t done = 0;
  if (s->parts) {
    // the rest (if retirements took the batch below the parts' size) in
    // the single graph below
    if ((err = iterate_host_parts(s, n, rs, q_host, iters, done)) != OT2D_OK || done == iters) return err;
  }
  for (int it = done; it < iters && !err; ++it) {
    for (int i = 0; i < n && !err; ++i) {
      const size_t bytes = rs[i]->d.n2 * rs[i]->d.nspec * rs[i]->d.P.nq * sizeof(double);
      if ((it > 0 && cudaStreamWaitEvent(s->st, s->ev_d2h[i], 0) != cudaSuccess) ||
          cudaMemcpyAsync(rs[i]->d.q64, q_host[i], bytes, cudaMemcpyHostToDevice, s->st) != cudaSuccess)
        err = OT2D_ERR_CUDA;
    }
    if (!err && s->precision == OT2D_FP32_MIXED && launch_shadow<float>(s->b32.d_sl, s->b32.b, s->st) != cudaSuccess)
      err = OT2D_ERR_CUDA;
    // the uploaded state may differ from the one the last update saw
    if (!err && host_time_step(s, -1, s->st) != cudaSuccess) err = OT2D_ERR_CUDA;
    if (!err && (launch_graph_iteration(s) != cudaSuccess || join_halves(s) != cudaSuccess)) err = OT2D_ERR_CUDA;
    if (!err && (cudaEventRecord(s->ev_step, s->st) != cudaSuccess ||
                 cudaStreamWaitEvent(s->st_d2h, s->ev_step, 0) != cudaSuccess))
      err = OT2D_ERR_CUDA;
    for (int i = 0; i < n && !err; ++i) {
      const size_t bytes = rs[i]->d.n2 * rs[i]->d.nspec * rs[i]->d.P.nq * sizeof(double);
      if (cudaMemcpyAsync(q_host[i], rs[i]->d.q64, bytes, cudaMemcpyDeviceToHost, s->st_d2h) != cudaSuccess ||
          cudaEventRecord(s->ev_d2h[i], s->st_d2h) != cudaSuccess)
        err = OT2D_ERR_CUDA;
    }
    bool capped = false;
    for (int id : s->live) {
      Rec& r = s->recs[id];
      if (++r.launched >= iter_cap(r)) capped = true;
    }
    if (!err && (++s->since_check >= s->check_every || capped)) {
      // the status read must not see the next iteration's uploads in flight
      if (cudaStreamSynchronize(s->st_d2h) != cudaSuccess) err = OT2D_ERR_CUDA;
      else err = check(s);
      if (!err && s->dirty) {
        // instances retired: the caller's list no longer matches the batch
        for (int i = 0; i < n; ++i)
          if (!rs[i]->live) { err = OT2D_ERR_ARG; break; }
        if (!err) err = rebuild(s);
      }
    }
  }
  // every download has landed in the caller's buffers
  if (cudaStreamSynchronize(s->st_d2h) != cudaSuccess && !err) err = OT2D_ERR_CUDA;
  if (cudaStreamSynchronize(s->st) != cudaSuccess && !err) err = OT2D_ERR_CUDA;
  return err;
}

int ot2d_solver_store(ot2d_solver* s, int32_t id, const char* dir) {
  if (!s || !dir) return OT2D_ERR_ARG;
  auto it = s->recs.find(id);
  if (it == s->recs.end() || !it->second.live) return OT2D_ERR_ARG;
  cudaSetDevice(s->device);
  return store_rec(s, it->second, dir);
}

int ot2d_solver_store_on_retire(ot2d_solver* s, int32_t id, const char* dir) {
  if (!s) return OT2D_ERR_ARG;
  auto it = s->recs.find(id);
  if (it == s->recs.end() || !(it->second.live || it->second.queued)) return OT2D_ERR_ARG;
  it->second.store_dir = dir ? dir : "";
  return OT2D_OK;
}

int ot2d_solver_add_restart(ot2d_solver* s, const ot2d_params* p, const double* xv, const double* yv,
                            const char* dir, double orders, int32_t max_iters) {
  if (!s || !p || !dir) return -OT2D_ERR_ARG;
  const std::string d = dir;
  return submit(s, p, xv, yv, orders, max_iters, [d](ot2d_solver* s, Rec& r) -> int {
    double totime = 0.0;
    int istep0 = 0;
    float* qc = s->precision == OT2D_FP32_MIXED ? (float*)r.d.q : nullptr;
    int e = read_restart(d, r.d.P, r.d.q64, qc, &totime, &istep0, s->st);
    if (e) return e;
    // init.f:165 (istep0) of the restart file; the instance runs as a
    // reference restart does, with iread = 1 (the wall start-up ramps of
    // bc.f / komegasst.f are then off).  The file's totime is not kept: the
    // driver restarts it at 0 (Turns_overset.f:359).
    (void)totime;
    if (r.d.P.iread < 1) r.d.P.iread = 1;
    const int32_t i0 = istep0;
    if (cudaMemcpyAsync((char*)r.d.dP + offsetof(ot2d_params, iread), &r.d.P.iread, sizeof(int32_t),
                        cudaMemcpyHostToDevice, s->st) != cudaSuccess)
      return OT2D_ERR_CUDA;
    for (int sl : r.slots)
      if (cudaMemcpyAsync(s->d_ist + (size_t)IST_N * sl, &i0, sizeof(i0), cudaMemcpyHostToDevice, s->st) !=
          cudaSuccess)
        return OT2D_ERR_CUDA;
    return cudaStreamSynchronize(s->st) == cudaSuccess ? OT2D_OK : OT2D_ERR_CUDA;
  });
}

int ot2d_solver_add_state(ot2d_solver* s, const ot2d_params* p, const double* xv, const double* yv,
                          const double* q, double orders, int32_t max_iters) {
  if (!s || !p || !q) return -OT2D_ERR_ARG;
  const size_t n2 = (size_t)p->jd * p->kd, ns = (size_t)p->nspec, nv = (size_t)p->nv;
  // reference layout (n, s, cell) -> the unpack's record layout (s, n, cell)
  std::vector<double> rec(ns * nv * n2);
  for (size_t sp = 0; sp < ns; ++sp)
    for (size_t n = 0; n < nv; ++n)
      std::memcpy(rec.data() + (sp * nv + n) * n2, q + (n * ns + sp) * n2, n2 * sizeof(double));
  return submit(s, p, xv, yv, orders, max_iters, [rec = std::move(rec)](ot2d_solver* s, Rec& r) -> int {
    double* tmp = nullptr;
    int e = OT2D_OK;
    if (cudaMalloc(&tmp, rec.size() * sizeof(double)) != cudaSuccess) return OT2D_ERR_NOMEM;
    float* qc = s->precision == OT2D_FP32_MIXED ? (float*)r.d.q : nullptr;
    if (cudaMemcpyAsync(tmp, rec.data(), rec.size() * sizeof(double), cudaMemcpyHostToDevice, s->st) !=
            cudaSuccess ||
        io_unpack(tmp, r.d.q64, qc, r.d.n2, r.d.nspec, r.d.P.nq, r.d.P.nv, 0, s->st) != cudaSuccess ||
        cudaStreamSynchronize(s->st) != cudaSuccess)
      e = OT2D_ERR_CUDA;
    cudaFree(tmp);
    return e;
  });
}

}  // extern "C"
