// dropin.cu -- the Fortran-shaped drop-in routines (ot2d_rhsup, ...).
// Each call runs the same kernels as the batched solver on a batch of one
// slice built from the caller's arrays.  Argument pointers are resolved as
//   device / managed memory      -> used in place;
//   host memory in the registry  -> its device mirror (ot2d_register);
//   other host memory            -> copied to a staging buffer and back.
// The module state of the reference (params_global) is the calling thread's
// ot2d_set_params() value.  FP64 only: the drop-in path is the parity path.
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "geom.h"
#include "io.h"
#include "runtime.h"

namespace ot2d {
namespace {

struct Reg { size_t bytes; void* dev; };
std::mutex g_reg_mu;
std::map<uintptr_t, Reg> g_reg;

struct Staged { void* host; void* dev; size_t bytes; bool out; };

// scratch arrays per slice of a drop-in call (the k-omega SST solve is the
// largest user: SST_NSCRATCH)
constexpr size_t DW_SLOTS = SST_NSCRATCH + 1;

struct Ctx {
  ot2d_params P{};
  bool has = false;
  int err = 0;
  cudaStream_t st = nullptr;
  ot2d_params* dP = nullptr;
  double* dwork = nullptr; size_t wcap = 0;      // scratch arrays of one slice (or nspec slices)
  double* dred = nullptr; int32_t* dist = nullptr;
  int nslice = 1;
  DevBatch<double> batch;
  std::vector<Staged> staged;
  std::vector<void*> pool;                         // staging buffers of this call
  std::vector<double> norms;
  ~Ctx() {}
};
thread_local Ctx g_ctx;

int fail(int e) { if (e) g_ctx.err = e; return e; }

int ensure_stream() {
  if (!g_ctx.st) {
    if (cudaStreamCreateWithFlags(&g_ctx.st, cudaStreamNonBlocking) != cudaSuccess) return OT2D_ERR_CUDA;
    if (cudaMalloc(&g_ctx.dP, sizeof(ot2d_params)) != cudaSuccess) return OT2D_ERR_NOMEM;
    if (cudaMalloc(&g_ctx.dred, sizeof(double) * RED_N * 64) != cudaSuccess) return OT2D_ERR_NOMEM;
    if (cudaMalloc(&g_ctx.dist, sizeof(int32_t) * IST_N * 64) != cudaSuccess) return OT2D_ERR_NOMEM;
  }
  return OT2D_OK;
}

// Resolve one argument.  `in`: the routine reads it; `out`: it writes it.
void* resolve(void* p, size_t bytes, bool in, bool out, int& err) {
  if (!p || err) return p;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) == cudaSuccess &&
      (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged))
    return p;
  cudaGetLastError();
  {
    std::lock_guard<std::mutex> lk(g_reg_mu);
    auto it = g_reg.upper_bound((uintptr_t)p);
    if (it != g_reg.begin()) {
      --it;
      uintptr_t base = it->first;
      if ((uintptr_t)p + bytes <= base + it->second.bytes) return (char*)it->second.dev + ((uintptr_t)p - base);
    }
  }
  void* d = nullptr;
  if (cudaMalloc(&d, bytes) != cudaSuccess) { err = OT2D_ERR_NOMEM; return nullptr; }
  g_ctx.pool.push_back(d);
  if (in) {
    if (cudaMemcpyAsync(d, p, bytes, cudaMemcpyHostToDevice, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  } else if (cudaMemsetAsync(d, 0, bytes, g_ctx.st) != cudaSuccess) {
    err = OT2D_ERR_CUDA;
  }
  if (out) g_ctx.staged.push_back({p, d, bytes, true});
  return d;
}

// Copy outputs back, free the staging buffers, report errors.
int finish(int err) {
  if (!err) {
    for (auto& s : g_ctx.staged)
      if (cudaMemcpyAsync(s.host, s.dev, s.bytes, cudaMemcpyDeviceToHost, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  }
  if (cudaStreamSynchronize(g_ctx.st) != cudaSuccess && !err) err = OT2D_ERR_CUDA;
  for (void* d : g_ctx.pool) cudaFree(d);
  g_ctx.pool.clear();
  g_ctx.staged.clear();
  return fail(err);
}

// Host copy of an argument that may be device memory (geometry set-up).
std::vector<double> host_copy(const double* p, size_t n) {
  std::vector<double> v(n);
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) == cudaSuccess && (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged))
    cudaMemcpy(v.data(), p, n * sizeof(double), cudaMemcpyDeviceToHost);
  else {
    cudaGetLastError();
    std::memcpy(v.data(), p, n * sizeof(double));
  }
  return v;
}
void host_store(double* p, const double* v, size_t n) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) == cudaSuccess && (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged))
    cudaMemcpy(p, v, n * sizeof(double), cudaMemcpyHostToDevice);
  else {
    cudaGetLastError();
    std::memcpy(p, v, n * sizeof(double));
  }
}

// Scratch arrays for nslice slices; upload params.
int prepare(int nslice, int& err) {
  if ((err = ensure_stream())) return err;
  if (!g_ctx.has) return err = OT2D_ERR_NOPARAMS;
  const size_t n2 = (size_t)g_ctx.P.jd * g_ctx.P.kd, ws = (n2 + 63) / 64 * 64;
  const size_t rec = (size_t)lu_rec_elems(g_ctx.P.jd, g_ctx.P.kd, 8);
  const size_t quad = rt_lim_class(g_ctx.P.ilim) == 2 ? (size_t)quad_elems(g_ctx.P.jd, g_ctx.P.kd) : 0;
  const size_t need = ws * DW_SLOTS * nslice + 8 * ws + rec * nslice + quad * nslice;
  g_ctx.nslice = nslice;
  if (need > g_ctx.wcap) {
    if (g_ctx.dwork) cudaFree(g_ctx.dwork);
    if (cudaMalloc(&g_ctx.dwork, need * sizeof(double)) != cudaSuccess) { g_ctx.dwork = nullptr; g_ctx.wcap = 0; return err = OT2D_ERR_NOMEM; }
    g_ctx.wcap = need;
  }
  if (cudaMemcpyAsync(g_ctx.dP, &g_ctx.P, sizeof(ot2d_params), cudaMemcpyHostToDevice, g_ctx.st) != cudaSuccess)
    return err = OT2D_ERR_CUDA;
  return err;
}

// A slice over caller arrays (one time instance, variable stride qs).
bool sst_params(const ot2d_params& p) { return !p.lamin && p.iturb == 2; }

// k-omega SST geometry of one instance: sn = 1e10 on meshes without a wall
// (kwdist runs only with one, komegasst.f:67), and the wall term dely2
// uploaded to d_wd2
void sst_geometry(const ot2d_params& p, const double* x, const double* y, const double* xv, const double* yv,
                  double* sn, double* d_wd2, int& err) {
  const size_t n2 = (size_t)p.jd * p.kd;
  bool body = false;
  for (int ib = 0; ib < p.nbc; ++ib) if (p.ibtyp[ib] == 5) body = true;
  if (!body) for (size_t i = 0; i < n2; ++i) sn[i] = 1.e10;
  std::vector<double> wd2(n2);
  sst_wall_d2(p, x, y, xv, yv, wd2.data());
  if (!err && cudaMemcpy(d_wd2, wd2.data(), n2 * 8, cudaMemcpyHostToDevice) != cudaSuccess) err = OT2D_ERR_CUDA;
}

Slice<double> base_slice(int nsp, int nspec, int64_t qs) {
  Slice<double> S{};
  const ot2d_params& p = g_ctx.P;
  S.P = g_ctx.dP;
  S.jd = p.jd; S.kd = p.kd; S.nsp = nsp; S.nspec = nspec; S.qs = qs;
  const size_t n2 = (size_t)p.jd * p.kd, ws = (n2 + 63) / 64 * 64;
  S.w = g_ctx.dwork + (size_t)(nsp - 1) * ws * DW_SLOTS;
  S.wstride = (int64_t)ws;
  S.lurec = g_ctx.dwork + ws * DW_SLOTS * (size_t)g_ctx.nslice + 8 * ws + (size_t)(nsp - 1) * (size_t)lu_rec_elems(p.jd, p.kd, 8);
  S.red = g_ctx.dred + (size_t)RED_N * (nsp - 1);
  S.ist = nullptr;
  if (rt_lim_class(p.ilim) == 2) {
    const size_t rec = (size_t)lu_rec_elems(p.jd, p.kd, 8), qe = (size_t)quad_elems(p.jd, p.kd);
    S.quad = g_ctx.dwork + ws * DW_SLOTS * (size_t)g_ctx.nslice + 8 * ws + rec * (size_t)g_ctx.nslice + (size_t)(nsp - 1) * qe;
  }
  slice_consts(S, p);
  return S;
}

int run_batch(const std::vector<Slice<double>>& sl, int& err) {
  if (err) return err;
  if ((err = g_ctx.batch.build(sl, g_ctx.st))) return err;
  return err;
}

bool dims_ok(const int32_t* jd, const int32_t* kd) {
  return jd && kd && *jd == g_ctx.P.jd && *kd == g_ctx.P.kd;
}

// face normals (and time-spectral face speeds) from the vertex grid
// (xold..yole: the previous vertex levels of a time-accurate moving grid,
// or null)
int faces_upload(double* dst4, double* dst2, const double* xv, const double* yv, const double* ugv, const double* vgv,
                 size_t ws, int& err, const double* xold = nullptr, const double* yold = nullptr,
                 const double* xole = nullptr, const double* yole = nullptr) {
  const ot2d_params& p = g_ctx.P;
  const size_t nv = (size_t)p.jmax * p.kmax, n2 = (size_t)p.jd * p.kd;
  std::vector<double> hx = host_copy(xv, nv), hy = host_copy(yv, nv), hu, hvv;
  std::vector<double> f(4 * n2), t(2 * n2, 0.0);
  const bool swept = p.iunst > 0 && xold && yold && xole && yole;
  const bool ts = !swept && p.timespectral && ugv && vgv;
  if (ts) { hu = host_copy(ugv, nv); hvv = host_copy(vgv, nv); }
  face_normals(p, hx.data(), hy.data(), ts ? hu.data() : nullptr, ts ? hvv.data() : nullptr, f.data(), f.data() + n2,
               f.data() + 2 * n2, f.data() + 3 * n2, ts ? t.data() : nullptr, ts ? t.data() + n2 : nullptr);
  if (swept) {
    std::vector<double> a = host_copy(xold, nv), b = host_copy(yold, nv), c = host_copy(xole, nv), d = host_copy(yole, nv);
    face_speeds_swept(p, hx.data(), hy.data(), a.data(), b.data(), c.data(), d.data(), t.data(), t.data() + n2);
  }
  for (int a = 0; a < 4; ++a)
    if (cudaMemcpyAsync(dst4 + a * ws, f.data() + a * n2, n2 * 8, cudaMemcpyHostToDevice, g_ctx.st) != cudaSuccess)
      err = OT2D_ERR_CUDA;
  if ((ts || swept) && dst2)
    for (int a = 0; a < 2; ++a)
      if (cudaMemcpyAsync(dst2 + a * ws, t.data() + a * n2, n2 * 8, cudaMemcpyHostToDevice, g_ctx.st) != cudaSuccess)
        err = OT2D_ERR_CUDA;
  cudaStreamSynchronize(g_ctx.st);  // host vectors go out of scope
  return err;
}


// Device view of an argument without staging: the pointer itself for device
// memory, the registered mirror for registered host memory, else nullptr.
void* device_view(const void* p, size_t bytes) {
  if (!p) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) == cudaSuccess &&
      (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged))
    return const_cast<void*>(p);
  cudaGetLastError();
  std::lock_guard<std::mutex> lk(g_reg_mu);
  auto it = g_reg.upper_bound((uintptr_t)p);
  if (it == g_reg.begin()) return nullptr;
  --it;
  const uintptr_t base = it->first;
  if ((uintptr_t)p + bytes <= base + it->second.bytes) return (char*)it->second.dev + ((uintptr_t)p - base);
  return nullptr;
}

// Read an argument as the library sees it (device data for device or
// registered memory, else the host array).
int fetch(const void* p, size_t bytes, void* dst) {
  if (!bytes) return OT2D_OK;
  if (void* d = device_view(p, bytes))
    return cudaMemcpy(dst, d, bytes, cudaMemcpyDeviceToHost) == cudaSuccess ? OT2D_OK : OT2D_ERR_CUDA;
  std::memcpy(dst, p, bytes);
  return OT2D_OK;
}

// Write into an argument: device memory in place; host memory and, when it is
// registered, its device mirror too.
int put(void* p, const void* src, size_t bytes) {
  if (!bytes) return OT2D_OK;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) == cudaSuccess &&
      (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged))
    return cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess ? OT2D_OK : OT2D_ERR_CUDA;
  cudaGetLastError();
  std::memcpy(p, src, bytes);
  if (void* d = device_view(p, bytes))
    return cudaMemcpy(d, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess ? OT2D_OK : OT2D_ERR_CUDA;
  return OT2D_OK;
}

// store, io.f:278-340, for one mesh: q(jd,kd,nspec,nq) goes through the
// device pack (Q = (Q/J)*J written, Q/J restored in place); lg / lq: nspec
// unformatted units; iblank is written to the grid file when num_grids > 1.
int store_impl(double* q, const double* x, const double* y, const int32_t* iblank, int jd, int kd,
               const int32_t* lg, const int32_t* lq, int num_grids) {
  int err = ensure_stream();
  if (err) return err;
  if (!g_ctx.has) return OT2D_ERR_NOPARAMS;
  const ot2d_params& p = g_ctx.P;
  if (jd < 1 || kd < 1 || !q || !x || !y || !lg || !lq || (num_grids > 1 && !iblank) || p.nv < 4) return OT2D_ERR_ARG;
  const size_t n2 = (size_t)jd * kd, ns = (size_t)p.nspec, nv = (size_t)p.nv;
  const bool turb = p.iturb == 1 || p.iturb == 2;
  double* dq = (double*)resolve(q, n2 * ns * p.nq * 8, true, true, err);
  double* rec = nullptr;
  if (!err && cudaMalloc(&rec, ns * nv * n2 * 8) != cudaSuccess) err = OT2D_ERR_NOMEM;
  if (rec) g_ctx.pool.push_back(rec);
  if (!err && io_pack(dq, nullptr, rec, nullptr, n2, p.nspec, p.nq, p.nv, IO_REC, g_ctx.st) != cudaSuccess)
    err = OT2D_ERR_CUDA;
  std::vector<double> h(ns * nv * n2);
  if (!err && cudaMemcpyAsync(h.data(), rec, h.size() * 8, cudaMemcpyDeviceToHost, g_ctx.st) != cudaSuccess)
    err = OT2D_ERR_CUDA;
  if ((err = finish(err))) return err;
  std::vector<double> hx(n2 * ns), hy(n2 * ns);
  std::vector<int32_t> hib(num_grids > 1 ? n2 * ns : 0);
  if ((err = fetch(x, hx.size() * 8, hx.data())) || (err = fetch(y, hy.size() * 8, hy.data())) ||
      (err = fetch(iblank, hib.size() * 4, hib.data())))
    return err;
  const double hdr[4] = {p.fsmach, p.alfa, p.rey * p.fsmach, p.totime};   // fstip, alfa, reypr, totime
  for (size_t s = 0; s < ns && !err; ++s) {
    FILE* fq = unit_file(lq[s], false, true);
    FILE* fg = unit_file(lg[s], false, true);
    if (!fq || !fg) return OT2D_ERR_IO;
    const double* r = h.data() + s * nv * n2;
    Seg sh{hdr, sizeof(hdr)}, sq{r, 4 * n2 * 8}, st{r + 4 * n2, (nv - 4) * n2 * 8};
    Seg sg[3] = {{hx.data() + s * n2, n2 * 8}, {hy.data() + s * n2, n2 * 8},
                 {hib.empty() ? nullptr : hib.data() + s * n2, hib.empty() ? 0 : n2 * 4}};
    err = rec_write(fq, &sh, 1);
    if (!err) err = rec_write(fq, &sq, 1);
    if (!err && turb) err = rec_write(fq, &st, 1);
    if (!err) err = rec_write(fg, sg, num_grids > 1 ? 3 : 2);
  }
  return err;
}

// storevnu (io.f:173-215) and storekomega (io.f:218-275) for one mesh
int storeturb_impl(const double* x, const double* y, const int32_t* iblank, double* q, int jd, int kd,
                   const int32_t* lq, const int32_t* ltur, bool sst) {
  int err = ensure_stream();
  if (err) return err;
  if (!g_ctx.has) return OT2D_ERR_NOPARAMS;
  const ot2d_params& p = g_ctx.P;
  if (jd < 1 || kd < 1 || !q || !x || !y || !iblank || !ltur || (sst && !lq) || p.itrans != 0 ||
      p.nv < (sst ? 6 : 5))
    return OT2D_ERR_ARG;
  const size_t n2 = (size_t)jd * kd, ns = (size_t)p.nspec, nv = (size_t)p.nv, qs = n2 * ns;
  std::vector<double> tec(sst ? ns * 2 * n2 : 0), turbv(ns * (nv - 4) * n2);
  if (sst) {
    // k = q(5)/rho, omega = q(6)/rho with rho = q(1)*J, on the device
    double* dq = (double*)resolve(q, qs * p.nq * 8, true, false, err);
    double* dt = nullptr;
    if (!err && cudaMalloc(&dt, tec.size() * 8) != cudaSuccess) err = OT2D_ERR_NOMEM;
    if (dt) g_ctx.pool.push_back(dt);
    if (!err && io_pack(dq, nullptr, nullptr, dt, n2, p.nspec, p.nq, p.nv, IO_TEC, g_ctx.st) != cudaSuccess)
      err = OT2D_ERR_CUDA;
    if (!err && cudaMemcpyAsync(tec.data(), dt, tec.size() * 8, cudaMemcpyDeviceToHost, g_ctx.st) != cudaSuccess)
      err = OT2D_ERR_CUDA;
    if ((err = finish(err))) return err;
  }
  for (size_t s = 0; s < ns && !err; ++s)
    for (size_t n = 4; n < nv && !err; ++n)
      err = fetch(q + n * qs + s * n2, n2 * 8, turbv.data() + (s * (nv - 4) + (n - 4)) * n2);
  std::vector<double> hx(n2 * ns), hy(n2 * ns);
  std::vector<int32_t> hib(n2 * ns);
  if (!err) err = fetch(x, hx.size() * 8, hx.data());
  if (!err) err = fetch(y, hy.size() * 8, hy.data());
  if (!err) err = fetch(iblank, hib.size() * 4, hib.data());
  for (size_t s = 0; s < ns && !err; ++s) {
    FILE* ft = unit_file(ltur[s], true, true);
    if (!ft) return OT2D_ERR_IO;
    const double* tv = turbv.data() + s * (nv - 4) * n2;
    if (sst) {
      Seg sg{tv, (nv - 4) * n2 * 8};
      err = rec_write(unit_file(lq[s], false, true), &sg, 1);
    }
    if (!err) err = tec_zone(ft, jd, kd);
    if (!err) err = tec_reals(ft, hx.data() + s * n2, n2);
    if (!err) err = tec_reals(ft, hy.data() + s * n2, n2);
    if (!err) err = tec_ints(ft, hib.data() + s * n2, n2);
    if (!err && !sst) err = tec_reals(ft, tv, n2);
    if (!err && sst) err = tec_reals(ft, tec.data() + s * 2 * n2, n2);
    if (!err && sst) err = tec_reals(ft, tec.data() + s * 2 * n2 + n2, n2);
  }
  return err;
}
// ilu2d (lhs.f:470-814) or, pre = true, preilu2d (lhs.f:2-467) on one time
// instance: the routine is chosen by the call, not by params iprecon, as the
// reference's step.f chooses it
int lusgs_dropin(double* q, double* s, int32_t* jd, int32_t* kd, int32_t* js, int32_t* je, int32_t* ks, int32_t* ke,
                 double* xx, double* xy, double* yx, double* yy, double* ug, double* vg, double* turmu, double* tscale,
                 double* bt, bool pre) {
  int err = 0;
  if (prepare(1, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || !js || !je || !ks || !ke || *js != p.jbeg || *je != p.jend || *ks != p.kbeg || *ke != p.kend)
    return fail(OT2D_ERR_ARG);
  if (!q || !s || !xx || !xy || !yx || !yy || !turmu || !tscale || p.iunst == 2 || (pre && !bt))
    return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd;
  Slice<double> S = base_slice(1, 1, (int64_t)n2);
  S.k_mp2 = pre ? p.Mp * p.Mp : -1.0;
  S.q = S.q64 = (double*)resolve(q, n2 * p.nq * 8, true, true, err);
  S.s = (double*)resolve(s, n2 * p.nv * 8, true, true, err);
  S.xx = (double*)resolve(xx, n2 * 8, true, false, err);
  S.xy = (double*)resolve(xy, n2 * 8, true, false, err);
  S.yx = (double*)resolve(yx, n2 * 8, true, false, err);
  S.yy = (double*)resolve(yy, n2 * 8, true, false, err);
  S.ug = (double*)resolve(ug, n2 * 8, true, false, err);
  S.vg = (double*)resolve(vg, n2 * 8, true, false, err);
  S.turmu = (double*)resolve(turmu, n2 * 8, true, false, err);
  S.tscale = (double*)resolve(tscale, n2 * 8, true, false, err);
  if (pre) S.bt = (double*)resolve(bt, n2 * 8, true, false, err);
  // status word for the sweeps' bounded waits (bit 4: a wait gave up)
  S.ist = g_ctx.dist;
  if (!err && cudaMemsetAsync(g_ctx.dist, 0, sizeof(int32_t) * IST_N, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  std::vector<Slice<double>> sl{S};
  run_batch(sl, err);
  if (!err && launch_lusgs<double>(g_ctx.batch.d_sl, g_ctx.batch.b, 0, g_ctx.st, 0) != cudaSuccess) err = OT2D_ERR_CUDA;
  int32_t ist[IST_N] = {0};
  if (!err && cudaMemcpyAsync(ist, g_ctx.dist, sizeof(ist), cudaMemcpyDeviceToHost, g_ctx.st) != cudaSuccess)
    err = OT2D_ERR_CUDA;
  err = finish(err);
  if (!err && (ist[2] & 4)) err = fail(OT2D_ERR_TIMEOUT);
  return err;
}
// arc2d (lhs.f:817-1057) or, pre = true, arc2d_precon (lhs.f:1060-1330) on
// one time instance; as for the LU-SGS pair the call chooses the routine
int adi_dropin(double* q, double* s, int32_t* jd, int32_t* kd, int32_t* js, int32_t* je, int32_t* ks, int32_t* ke,
               double* xx, double* xy, double* yx, double* yy, double* ug, double* vg, double* turmu, int32_t* iblank,
               double* tscale, double* bt, bool pre) {
  int err = 0;
  if (prepare(1, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || !js || !je || !ks || !ke || *js != p.jbeg || *je != p.jend || *ks != p.kbeg || *ke != p.kend)
    return fail(OT2D_ERR_ARG);
  if (!q || !s || !xx || !xy || !yx || !yy || !turmu || !tscale || !iblank || p.jd < 10 || p.kd < 10 || (pre && !bt))
    return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd;
  Slice<double> S = base_slice(1, 1, (int64_t)n2);
  S.k_mp2 = pre ? p.Mp * p.Mp : -1.0;
  S.q = S.q64 = (double*)resolve(q, n2 * p.nq * 8, true, true, err);
  S.s = (double*)resolve(s, n2 * p.nv * 8, true, true, err);
  S.xx = (double*)resolve(xx, n2 * 8, true, false, err);
  S.xy = (double*)resolve(xy, n2 * 8, true, false, err);
  S.yx = (double*)resolve(yx, n2 * 8, true, false, err);
  S.yy = (double*)resolve(yy, n2 * 8, true, false, err);
  S.ug = (double*)resolve(ug, n2 * 8, true, false, err);
  S.vg = (double*)resolve(vg, n2 * 8, true, false, err);
  S.turmu = (double*)resolve(turmu, n2 * 8, true, false, err);
  S.iblank = (int32_t*)resolve(iblank, n2 * 4, true, false, err);
  S.tscale = (double*)resolve(tscale, n2 * 8, true, false, err);
  S.bt = bt ? (double*)resolve(bt, n2 * 8, true, false, err) : nullptr;
  std::vector<Slice<double>> sl{S};
  run_batch(sl, err);
  if (!err && launch_adi<double>(g_ctx.batch.d_sl, g_ctx.batch.b, 0, g_ctx.st, 0) != cudaSuccess) err = OT2D_ERR_CUDA;
  return finish(err);
}
// ---- overset interpolation (connectivity.f:2-190) ---------------------------
// One donor: where its mesh's q block starts for its time instance, the
// distance between variables, the mesh's jd, the donor cell, its offsets
// and the qbc row it fills (qbc: per time instance a (bcdim, nv) block).
struct OvsDon { int64_t qbase, vstride, boff; int32_t jm, ii, jj, bcdim, row, pad; double f1, f2; };
// One fringe cell: the same addressing, the qbc row it takes.
struct OvsFr { int64_t qbase, vstride, boff; int32_t jm, ii, jj, bcdim, row, pad; };

// :69-128 -- 9-point quadratic Lagrange weights (exact power-of-two
// scalings, so their grouping does not change a bit) on q*J (mean flow) and
// q (turbulence variables)
__global__ void k_ovs_gather(const OvsDon* __restrict__ dn, int nd, const double* __restrict__ qg,
                             double* __restrict__ qbc, int nq, int nv, int nmv) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nd) return;
  const OvsDon d = dn[e];
  const double onefourth = 1. / 4;
  const double djm1 = 1. + d.f1, dkm1 = 1. + d.f2, dj0 = d.f1, dk0 = d.f2, djp1 = 1. - d.f1, dkp1 = 1. - d.f2;
  double w[9];
  w[0] = (dj0 * djp1 * dk0 * dkp1) * onefourth;
  w[1] = -(2 * (djm1 * djp1 * dk0 * dkp1) * onefourth);
  w[2] = -((djm1 * dj0 * dk0 * dkp1) * onefourth);
  w[3] = -(2 * (dj0 * djp1 * dkm1 * dkp1) * onefourth);
  w[4] = 4 * (djm1 * djp1 * dkm1 * dkp1) * onefourth;
  w[5] = 2 * (djm1 * dj0 * dkm1 * dkp1) * onefourth;
  w[6] = -((dj0 * djp1 * dkm1 * dk0) * onefourth);
  w[7] = 2 * (djm1 * djp1 * dkm1 * dk0) * onefourth;
  w[8] = (djm1 * dj0 * dkm1 * dk0) * onefourth;
  // stencil cells (ii-1..ii+1, jj-1..jj+1), j fastest, in the reference's term order
  int64_t c[9];
#pragma unroll
  for (int t = 0; t < 9; ++t) c[t] = d.qbase + (int64_t)(d.jj - 2 + t / 3) * d.jm + (d.ii - 2 + t % 3);
  const double* J = qg + (int64_t)(nq - 1) * d.vstride;
  for (int n = 1; n <= nv; ++n) {
    const double* qn = qg + (int64_t)(n - 1) * d.vstride;
    double a;
    if (n <= nmv) {
      a = w[0] * qn[c[0]] * J[c[0]];
#pragma unroll
      for (int t = 1; t < 9; ++t) a = a + w[t] * qn[c[t]] * J[c[t]];
    } else {
      a = w[0] * qn[c[0]];
#pragma unroll
      for (int t = 1; t < 9; ++t) a = a + w[t] * qn[c[t]];
    }
    qbc[d.boff + (int64_t)(n - 1) * d.bcdim + (d.row - 1)] = a;
  }
}

// :154-167 -- fringe cells from qbc (mean flow divided by J)
__global__ void k_ovs_scatter(const OvsFr* __restrict__ fr, int nf, double* __restrict__ qg,
                              const double* __restrict__ qbc, int nq, int nv, int nmv) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nf) return;
  const OvsFr f = fr[e];
  const int64_t o = f.qbase + (int64_t)(f.jj - 1) * f.jm + (f.ii - 1);
  const double J = qg[(int64_t)(nq - 1) * f.vstride + o];
  for (int n = 1; n <= nv; ++n) {
    const double v = qbc[f.boff + (int64_t)(n - 1) * f.bcdim + (f.row - 1)];
    qg[(int64_t)(n - 1) * f.vstride + o] = n <= nmv ? v / J : v;
  }
}
}  // namespace
}  // namespace ot2d

using namespace ot2d;

extern "C" {

int ot2d_set_params(const ot2d_params* p) {
  if (!p) return fail(OT2D_ERR_ARG);
  if (p->nhalo != 1 || p->jd != p->jmax + 1 || p->kd != p->kmax + 1) return fail(OT2D_ERR_ARG);
  if (!rt_lim_known(p->ilim)) return fail(OT2D_ERR_ARG);   // reconstructions of rhsup (eulerrhs.f:84-97)
  if (rt_lim_class(p->ilim) == 2 && (p->jd < 7 || p->kd < 7)) return fail(OT2D_ERR_ARG);   // quad's end stencils
  g_ctx.P = *p;
  g_ctx.has = true;
  return OT2D_OK;
}

int ot2d_set_precision(int32_t mode) { return mode == OT2D_FP64 ? OT2D_OK : fail(OT2D_ERR_ARG); }

int ot2d_last_error(void) { return g_ctx.err; }

int ot2d_register(void* h, size_t bytes) {
  if (!h || !bytes) return fail(OT2D_ERR_ARG);
  void* d = nullptr;
  if (cudaMalloc(&d, bytes) != cudaSuccess) return fail(OT2D_ERR_NOMEM);
  if (cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice) != cudaSuccess) { cudaFree(d); return fail(OT2D_ERR_CUDA); }
  std::lock_guard<std::mutex> lk(g_reg_mu);
  auto it = g_reg.find((uintptr_t)h);
  if (it != g_reg.end()) { cudaFree(it->second.dev); g_reg.erase(it); }
  g_reg[(uintptr_t)h] = Reg{bytes, d};
  return OT2D_OK;
}

int ot2d_unregister(void* h) {
  std::lock_guard<std::mutex> lk(g_reg_mu);
  auto it = g_reg.find((uintptr_t)h);
  if (it == g_reg.end()) return fail(OT2D_ERR_ARG);
  cudaFree(it->second.dev);
  g_reg.erase(it);
  return OT2D_OK;
}

int ot2d_sync_to_host(void* h) {
  std::lock_guard<std::mutex> lk(g_reg_mu);
  auto it = g_reg.find((uintptr_t)h);
  if (it == g_reg.end()) return fail(OT2D_ERR_ARG);
  if (g_ctx.st) cudaStreamSynchronize(g_ctx.st);
  return cudaMemcpy(h, it->second.dev, it->second.bytes, cudaMemcpyDeviceToHost) == cudaSuccess ? OT2D_OK : fail(OT2D_ERR_CUDA);
}

int ot2d_sync_to_device(void* h) {
  std::lock_guard<std::mutex> lk(g_reg_mu);
  auto it = g_reg.find((uintptr_t)h);
  if (it == g_reg.end()) return fail(OT2D_ERR_ARG);
  return cudaMemcpy(it->second.dev, h, it->second.bytes, cudaMemcpyHostToDevice) == cudaSuccess ? OT2D_OK : fail(OT2D_ERR_CUDA);
}

int ot2d_rhsup(double* q, double* s, double* xx, double* xy, double* yx, double* yy, double* x, double* y,
               double* xv, double* yv, double* xold, double* yold, double* xole, double* yole, int32_t* iblank,
               double* ugv, double* vgv, int32_t* jd, int32_t* kd, int32_t* nei, int32_t* im, double* bt) {
  (void)xx; (void)xy; (void)yx; (void)yy; (void)x; (void)y; (void)im; (void)bt;
  int err = 0;
  if (prepare(1, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  const bool swept = p.iunst == 1;   // time-accurate moving grid: face speeds from the swept areas
  if (!dims_ok(jd, kd) || !nei || *nei != 1 || (p.iunst != 0 && !swept) || !q || !s || !xv || !yv || !iblank ||
      (swept && (!xold || !yold || !xole || !yole)))
    return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd;
  Slice<double> S = base_slice(1, 1, (int64_t)n2);
  const size_t ws = (size_t)S.wstride;
  double* faces = g_ctx.dwork + ws * DW_SLOTS;           // 4 face-normal arrays
  double* tjs = faces + 4 * ws;                     // 2 face-speed arrays
  faces_upload(faces, tjs, xv, yv, ugv, vgv, ws, err, xold, yold, xole, yole);
  S.q = S.q64 = (double*)resolve(q, n2 * p.nq * 8, true, false, err);
  S.s = (double*)resolve(s, n2 * p.nv * 8, true, true, err);
  S.iblank = (int32_t*)resolve(iblank, n2 * 4, true, false, err);
  S.fxa = faces; S.fya = faces + ws; S.gxa = faces + 2 * ws; S.gya = faces + 3 * ws;
  if ((p.timespectral && ugv && vgv) || swept) { S.ftj = tjs; S.gtj = tjs + ws; }
  std::vector<Slice<double>> sl{S};
  run_batch(sl, err);
  if (!err && launch_faces<double>(g_ctx.batch.d_sl, g_ctx.batch.b, 1, 0, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  if (!err && launch_assemble<double>(g_ctx.batch.d_sl, g_ctx.batch.b, AS_ACC | AS_INV, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  return finish(err);
}

int ot2d_visrhs(double* turmu, double* q, double* s, double* xx, double* xy, double* yx, double* yy, double* ug,
                double* vg, double* tscale, int32_t* iblank, int32_t* jd, int32_t* kd) {
  (void)ug; (void)vg; (void)tscale;
  int err = 0;
  if (prepare(1, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || !q || !s || !turmu || !xx || !xy || !yx || !yy || !iblank) return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd;
  Slice<double> S = base_slice(1, 1, (int64_t)n2);
  S.q = S.q64 = (double*)resolve(q, n2 * p.nq * 8, true, false, err);
  S.s = (double*)resolve(s, n2 * p.nv * 8, true, true, err);
  S.turmu = (double*)resolve(turmu, n2 * 8, true, false, err);
  S.xx = (double*)resolve(xx, n2 * 8, true, false, err);
  S.xy = (double*)resolve(xy, n2 * 8, true, false, err);
  S.yx = (double*)resolve(yx, n2 * 8, true, false, err);
  S.yy = (double*)resolve(yy, n2 * 8, true, false, err);
  S.iblank = (int32_t*)resolve(iblank, n2 * 4, true, false, err);
  std::vector<Slice<double>> sl{S};
  run_batch(sl, err);
  if (!err && p.invisc == 0) {
    if (launch_faces<double>(g_ctx.batch.d_sl, g_ctx.batch.b, 0, 1, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
    if (!err && launch_assemble<double>(g_ctx.batch.d_sl, g_ctx.batch.b, AS_ACC | AS_VISC, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  }
  return finish(err);
}

int ot2d_bc(double* q, double* x, double* y, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg,
            int32_t* im, int32_t* jd, int32_t* kd, double* bt) {
  (void)x; (void)y; (void)im;
  int err = 0;
  if (prepare(1, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || !q || !xx || !xy || !yx || !yy) return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd;
  Slice<double> S = base_slice(1, 1, (int64_t)n2);
  S.q = S.q64 = (double*)resolve(q, n2 * p.nq * 8, true, true, err);
  S.xx = S.xx64 = (double*)resolve(xx, n2 * 8, true, false, err);
  S.xy = S.xy64 = (double*)resolve(xy, n2 * 8, true, false, err);
  S.yx = S.yx64 = (double*)resolve(yx, n2 * 8, true, false, err);
  S.yy = S.yy64 = (double*)resolve(yy, n2 * 8, true, false, err);
  S.ug = S.ug64 = (double*)resolve(ug, n2 * 8, true, false, err);
  S.vg = S.vg64 = (double*)resolve(vg, n2 * 8, true, false, err);
  // bt of time_step enters the Turkel-form far field (bc.f:712-835); 1 when not given
  S.bt = bt ? (double*)resolve(bt, n2 * 8, true, false, err) : nullptr;
  std::vector<Slice<double>> sl{S};
  run_batch(sl, err);
  if (!err && launch_bc<double>(g_ctx.batch.d_sl, g_ctx.batch.b, 0, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  return finish(err);
}

int ot2d_rbc(double* q, double* s, double* x, double* y, double* xx, double* xy, double* yx, double* yy, double* ug,
             double* vg, int32_t* im, int32_t* jd, int32_t* kd, double* bt) {
  (void)x; (void)y; (void)xx; (void)xy; (void)yx; (void)yy; (void)ug; (void)vg; (void)im; (void)bt;
  int err = 0;
  if (prepare(1, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || !q || !s) return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd;
  Slice<double> S = base_slice(1, 1, (int64_t)n2);
  S.q = S.q64 = (double*)resolve(q, n2 * p.nq * 8, true, false, err);
  S.s = (double*)resolve(s, n2 * p.nv * 8, true, true, err);
  std::vector<Slice<double>> sl{S};
  run_batch(sl, err);
  if (!err && launch_rbc<double>(g_ctx.batch.d_sl, g_ctx.batch.b, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  return finish(err);
}

int ot2d_time_step(double* q, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg,
                   double* tscale, double* bt, int32_t* iblank, int32_t* jd, int32_t* kd) {
  int err = 0;
  if (prepare(1, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || !q || !xx || !xy || !yx || !yy || !tscale || !bt || !iblank) return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd;
  Slice<double> S = base_slice(1, 1, (int64_t)n2);
  S.q = S.q64 = (double*)resolve(q, n2 * p.nq * 8, true, false, err);
  S.xx = (double*)resolve(xx, n2 * 8, true, false, err);
  S.xy = (double*)resolve(xy, n2 * 8, true, false, err);
  S.yx = (double*)resolve(yx, n2 * 8, true, false, err);
  S.yy = (double*)resolve(yy, n2 * 8, true, false, err);
  S.ug = (double*)resolve(ug, n2 * 8, true, false, err);
  S.vg = (double*)resolve(vg, n2 * 8, true, false, err);
  S.tscale = (double*)resolve(tscale, n2 * 8, false, true, err);
  S.bt = (double*)resolve(bt, n2 * 8, false, true, err);
  S.iblank = (int32_t*)resolve(iblank, n2 * 4, true, false, err);
  std::vector<Slice<double>> sl{S};
  run_batch(sl, err);
  if (!err && launch_time_step<double>(g_ctx.batch.d_sl, g_ctx.batch.b, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  return finish(err);
}

int ot2d_ilu2d(double* q, double* s, int32_t* jd, int32_t* kd, int32_t* js, int32_t* je, int32_t* ks, int32_t* ke,
               double* xx, double* xy, double* yx, double* yy, double* ug, double* vg, double* turmu,
               double* tscale) {
  return lusgs_dropin(q, s, jd, kd, js, je, ks, ke, xx, xy, yx, yy, ug, vg, turmu, tscale, nullptr, false);
}

int ot2d_preilu2d(double* q, double* s, int32_t* jd, int32_t* kd, int32_t* js, int32_t* je, int32_t* ks, int32_t* ke,
                  double* xx, double* xy, double* yx, double* yy, double* ug, double* vg, double* turmu,
                  double* tscale, double* bt) {
  return lusgs_dropin(q, s, jd, kd, js, je, ks, ke, xx, xy, yx, yy, ug, vg, turmu, tscale, bt, true);
}

int ot2d_rhslom(double* q, double* s, int32_t* jd, int32_t* kd, int32_t* js, int32_t* je, int32_t* ks, int32_t* ke,
                double* bt) {
  int err = 0;
  if (prepare(1, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || !js || !je || !ks || !ke || *js != p.jbeg || *je != p.jend || *ks != p.kbeg || *ke != p.kend)
    return fail(OT2D_ERR_ARG);
  if (!q || !s || !bt) return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd;
  Slice<double> S = base_slice(1, 1, (int64_t)n2);
  S.k_mp2 = p.Mp * p.Mp;   // rhslom reads Mp whatever iprecon says
  S.q = S.q64 = (double*)resolve(q, n2 * p.nq * 8, true, false, err);
  S.s = (double*)resolve(s, n2 * p.nv * 8, true, true, err);
  S.bt = (double*)resolve(bt, n2 * 8, true, false, err);
  std::vector<Slice<double>> sl{S};
  run_batch(sl, err);
  if (!err && launch_rhslom<double>(g_ctx.batch.d_sl, g_ctx.batch.b, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  return finish(err);
}

int ot2d_arc2d(double* q, double* s, int32_t* jd, int32_t* kd, int32_t* js, int32_t* je, int32_t* ks, int32_t* ke,
               double* xx, double* xy, double* yx, double* yy, double* ug, double* vg, double* turmu, int32_t* iblank,
               double* tscale, double* bt) {
  return adi_dropin(q, s, jd, kd, js, je, ks, ke, xx, xy, yx, yy, ug, vg, turmu, iblank, tscale, bt, false);
}

int ot2d_arc2d_precon(double* q, double* s, int32_t* jd, int32_t* kd, int32_t* js, int32_t* je, int32_t* ks,
                      int32_t* ke, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg,
                      double* turmu, int32_t* iblank, double* tscale, double* bt) {
  return adi_dropin(q, s, jd, kd, js, je, ks, ke, xx, xy, yx, yy, ug, vg, turmu, iblank, tscale, bt, true);
}

int ot2d_vmu_sa(double* q, double* s, double* turmu, double* x, double* y, double* xv, double* yv, double* xx,
                double* xy, double* yx, double* yy, double* ug, double* vg, int32_t* jd, int32_t* kd,
                double* tscale, int32_t* iblank, int32_t* im, int32_t* nsp) {
  (void)im; (void)nsp;
  int err = 0;
  if (prepare(1, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || p.iturb != 1 || p.lamin || !q || !s || !turmu || !x || !y || !xv || !yv || !tscale || !iblank)
    return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd, nv = (size_t)p.jmax * p.kmax;
  Slice<double> S = base_slice(1, 1, (int64_t)n2);
  const size_t ws = (size_t)S.wstride;
  double* dsn = g_ctx.dwork + ws * DW_SLOTS;
  {
    std::vector<double> hx = host_copy(x, n2), hy = host_copy(y, n2), hxv = host_copy(xv, nv), hyv = host_copy(yv, nv);
    std::vector<double> sn(n2);
    wall_distance(p, hx.data(), hy.data(), hxv.data(), hyv.data(), sn.data());
    if (cudaMemcpy(dsn, sn.data(), n2 * 8, cudaMemcpyHostToDevice) != cudaSuccess) err = OT2D_ERR_CUDA;
  }
  S.q = S.q64 = (double*)resolve(q, n2 * p.nq * 8, true, true, err);
  S.s = (double*)resolve(s, n2 * p.nv * 8, true, false, err);
  S.turmu = (double*)resolve(turmu, n2 * 8, true, true, err);
  S.xx = S.xx64 = (double*)resolve(xx, n2 * 8, true, false, err);
  S.xy = S.xy64 = (double*)resolve(xy, n2 * 8, true, false, err);
  S.yx = S.yx64 = (double*)resolve(yx, n2 * 8, true, false, err);
  S.yy = S.yy64 = (double*)resolve(yy, n2 * 8, true, false, err);
  S.ug = S.ug64 = (double*)resolve(ug, n2 * 8, true, false, err);
  S.vg = S.vg64 = (double*)resolve(vg, n2 * 8, true, false, err);
  S.tscale = (double*)resolve(tscale, n2 * 8, true, false, err);
  S.iblank = (int32_t*)resolve(iblank, n2 * 4, true, false, err);
  S.sn = dsn;
  std::vector<Slice<double>> sl{S};
  run_batch(sl, err);
  if (!err && launch_sa<double>(g_ctx.batch.d_sl, g_ctx.batch.b, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  return finish(err);
}

int ot2d_komegasst(double* q, double* s, double* turmu, double* x, double* y, double* xv, double* yv, double* xx,
                   double* xy, double* yx, double* yy, double* ug, double* vg, int32_t* jd, int32_t* kd,
                   double* tscale, int32_t* iblank, int32_t* im) {
  (void)im;
  int err = 0;
  if (prepare(1, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || !sst_params(p) || p.itrans != 0 || !q || !s || !turmu || !x || !y || !xv || !yv || !tscale ||
      !iblank)
    return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd, nv = (size_t)p.jmax * p.kmax;
  Slice<double> S = base_slice(1, 1, (int64_t)n2);
  const size_t ws = (size_t)S.wstride;
  double* dsn = g_ctx.dwork + ws * DW_SLOTS;
  double* dwd2 = dsn + ws;
  {
    std::vector<double> hx = host_copy(x, n2), hy = host_copy(y, n2), hxv = host_copy(xv, nv), hyv = host_copy(yv, nv);
    std::vector<double> sn(n2);
    wall_distance(p, hx.data(), hy.data(), hxv.data(), hyv.data(), sn.data());
    sst_geometry(p, hx.data(), hy.data(), hxv.data(), hyv.data(), sn.data(), dwd2, err);
    if (!err && cudaMemcpy(dsn, sn.data(), n2 * 8, cudaMemcpyHostToDevice) != cudaSuccess) err = OT2D_ERR_CUDA;
  }
  S.q = S.q64 = (double*)resolve(q, n2 * p.nq * 8, true, true, err);
  S.s = (double*)resolve(s, n2 * p.nv * 8, true, true, err);
  S.turmu = (double*)resolve(turmu, n2 * 8, true, true, err);
  S.xx = S.xx64 = (double*)resolve(xx, n2 * 8, true, false, err);
  S.xy = S.xy64 = (double*)resolve(xy, n2 * 8, true, false, err);
  S.yx = S.yx64 = (double*)resolve(yx, n2 * 8, true, false, err);
  S.yy = S.yy64 = (double*)resolve(yy, n2 * 8, true, false, err);
  S.ug = S.ug64 = (double*)resolve(ug, n2 * 8, true, false, err);
  S.vg = S.vg64 = (double*)resolve(vg, n2 * 8, true, false, err);
  S.tscale = (double*)resolve(tscale, n2 * 8, true, false, err);
  S.iblank = (int32_t*)resolve(iblank, n2 * 4, true, false, err);
  S.sn = dsn;
  S.wd2 = dwd2;
  std::vector<Slice<double>> sl{S};
  run_batch(sl, err);
  if (!err && launch_sst<double>(g_ctx.batch.d_sl, g_ctx.batch.b, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  return finish(err);
}

int ot2d_timespectralrhs(double* q, double* s, double* Ds, int32_t* jd, int32_t* kd, int32_t* nsp) {
  int err = 0;
  if (prepare(1, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || !nsp || *nsp < 1 || *nsp > p.nspec || !q || !s || !Ds) return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd, ns = (size_t)p.nspec;
  Slice<double> S = base_slice(1, p.nspec, (int64_t)(n2 * ns));
  S.nsp = *nsp;
  double* dq = (double*)resolve(q, n2 * ns * p.nq * 8, true, false, err);
  double* ds = (double*)resolve(s, n2 * ns * p.nv * 8, true, true, err);
  S.Ds = (double*)resolve(Ds, ns * ns * 8, true, false, err);
  if (!err) { S.q = S.q64 = dq + (size_t)(*nsp - 1) * n2; S.s = ds + (size_t)(*nsp - 1) * n2; }
  std::vector<Slice<double>> sl{S};
  run_batch(sl, err);
  if (!err && p.timespectral &&
      launch_assemble<double>(g_ctx.batch.d_sl, g_ctx.batch.b, AS_ACC | AS_TS, g_ctx.st) != cudaSuccess)
    err = OT2D_ERR_CUDA;
  return finish(err);
}

int ot2d_step(double* q, double* qtn, double* qtnm1, double* qnewt, double* s, double* x, double* y, double* xv,
              double* yv, int32_t* iblank, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg,
              double* ugv, double* vgv, double* xold, double* yold, double* xole, double* yole, double* turmu,
              double* tscale, double* bt, double* Ds, int32_t* im, int32_t* jd, int32_t* kd) {
  (void)qtn; (void)qtnm1; (void)im;
  const int nspec = g_ctx.has ? g_ctx.P.nspec : 1;
  int err = 0;
  if (prepare(nspec, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  const bool swept = p.iunst == 1, newton = p.itnmax > 1;
  if (!dims_ok(jd, kd) || p.ilhs < 1 || p.ilhs > 3 || (p.iunst != 0 && !swept) || (newton && p.timespectral && swept) ||
      (!p.lamin && p.iturb != 1 && p.iturb != 2) || p.itrans != 0)
    return fail(OT2D_ERR_ARG);
  // Turkel preconditioning: rhslom, preilu2d and arc2d_precon read bt
  if (p.iprecon && !bt) return fail(OT2D_ERR_ARG);
  if (!q || !s || !x || !y || !xv || !yv || !iblank || !xx || !xy || !yx || !yy || !turmu || !tscale) return fail(OT2D_ERR_ARG);
  if (p.timespectral && (!ugv || !vgv || !ug || !vg || !Ds)) return fail(OT2D_ERR_ARG);
  if (swept && (!xold || !yold || !xole || !yole || !ug || !vg)) return fail(OT2D_ERR_ARG);
  if (newton && !qnewt) return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd, ns = (size_t)nspec, nv = (size_t)p.jmax * p.kmax, qs = n2 * ns;
  double* dq = (double*)resolve(q, qs * p.nq * 8, true, true, err);
  double* ds = (double*)resolve(s, qs * p.nv * 8, false, true, err);
  int32_t* dib = (int32_t*)resolve(iblank, qs * 4, true, false, err);
  double* dxx = (double*)resolve(xx, qs * 8, true, false, err);
  double* dxy = (double*)resolve(xy, qs * 8, true, false, err);
  double* dyx = (double*)resolve(yx, qs * 8, true, false, err);
  double* dyy = (double*)resolve(yy, qs * 8, true, false, err);
  double* dug = (p.timespectral || swept) ? (double*)resolve(ug, qs * 8, true, false, err) : nullptr;
  double* dvg = (p.timespectral || swept) ? (double*)resolve(vg, qs * 8, true, false, err) : nullptr;
  double* dqn = newton ? (double*)resolve(qnewt, qs * p.nv * 8, true, false, err) : nullptr;
  // bt of time_step (far-field BC, preconditioner); 1 when not given
  double* dbt = bt ? (double*)resolve(bt, qs * 8, true, false, err) : nullptr;
  if (newton && !err) {
    // newton's 1/(oat*h) (time.f:195-200) for the residual kernel
    double oat = 1.0;
    if (p.ntac >= 2 && p.istep > 1) oat = 2. / 3.;
    if (p.ntac == 3 && p.istep > 2) oat = 6. / 11.;
    const double tac = 1. / (oat * p.h);
    for (int nsp = 0; nsp < nspec && !err; ++nsp)
      if (cudaMemcpyAsync(g_ctx.dred + (size_t)RED_N * nsp + 8, &tac, sizeof(double), cudaMemcpyHostToDevice,
                          g_ctx.st) != cudaSuccess)
        err = OT2D_ERR_CUDA;
    cudaStreamSynchronize(g_ctx.st);
  }
  double* dturmu = (double*)resolve(turmu, qs * 8, true, true, err);
  double* dts = (double*)resolve(tscale, qs * 8, true, false, err);
  double* dDs = p.timespectral ? (double*)resolve(Ds, ns * ns * 8, true, false, err) : nullptr;
  // per-instance face normals and wall distance from the host grid
  const size_t ws = (n2 + 63) / 64 * 64;
  double* extra = nullptr;
  if (!err && cudaMalloc(&extra, sizeof(double) * ws * 8 * ns) != cudaSuccess) err = OT2D_ERR_NOMEM;
  if (extra) g_ctx.pool.push_back(extra);
  std::vector<Slice<double>> sl;
  std::vector<double> hx = host_copy(x, qs), hy = host_copy(y, qs), hxv = host_copy(xv, nv * ns), hyv = host_copy(yv, nv * ns);
  for (int nsp = 1; nsp <= nspec && !err; ++nsp) {
    double* e = extra + (size_t)(nsp - 1) * ws * 8;
    faces_upload(e, e + 4 * ws, xv + (nsp - 1) * nv, yv + (nsp - 1) * nv, ugv ? ugv + (nsp - 1) * nv : nullptr,
                 vgv ? vgv + (nsp - 1) * nv : nullptr, ws, err, swept ? xold : nullptr, swept ? yold : nullptr,
                 swept ? xole : nullptr, swept ? yole : nullptr);
    std::vector<double> sn(n2);
    wall_distance(p, hx.data() + (nsp - 1) * n2, hy.data() + (nsp - 1) * n2, hxv.data() + (nsp - 1) * nv,
                  hyv.data() + (nsp - 1) * nv, sn.data());
    if (sst_params(p))
      sst_geometry(p, hx.data() + (nsp - 1) * n2, hy.data() + (nsp - 1) * n2, hxv.data() + (nsp - 1) * nv,
                   hyv.data() + (nsp - 1) * nv, sn.data(), e + 7 * ws, err);
    if (cudaMemcpy(e + 6 * ws, sn.data(), n2 * 8, cudaMemcpyHostToDevice) != cudaSuccess) err = OT2D_ERR_CUDA;
    Slice<double> S = base_slice(nsp, nspec, (int64_t)qs);
    const size_t o = (size_t)(nsp - 1) * n2;
    S.q = S.q64 = dq + o; S.s = ds + o; S.iblank = dib + o;
    S.xx = S.xx64 = dxx + o; S.xy = S.xy64 = dxy + o; S.yx = S.yx64 = dyx + o; S.yy = S.yy64 = dyy + o;
    S.ug = S.ug64 = dug ? dug + o : nullptr; S.vg = S.vg64 = dvg ? dvg + o : nullptr;
    S.turmu = dturmu + o; S.tscale = dts + o;
    S.bt = dbt ? dbt + o : nullptr;
    S.fxa = e; S.fya = e + ws; S.gxa = e + 2 * ws; S.gya = e + 3 * ws;
    S.ftj = (p.timespectral || swept) ? e + 4 * ws : nullptr; S.gtj = (p.timespectral || swept) ? e + 5 * ws : nullptr;
    S.qnewt = dqn ? dqn + o : nullptr;
    S.sn = e + 6 * ws;
    S.wd2 = sst_params(p) ? e + 7 * ws : nullptr;
    S.Ds = dDs;
    sl.push_back(S);
  }
  run_batch(sl, err);
  const auto& B = g_ctx.batch;
  const int visc = p.invisc ? 0 : 1, turb = (!p.lamin && p.iturb == 1) ? 1 : 0, sst = sst_params(p) ? 1 : 0;
  if (!err && launch_bc<double>(B.d_sl, B.b, 0, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  if (!err && launch_residual<double>(B.d_sl, B.b, visc, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  if (!err && launch_rbc<double>(B.d_sl, B.b, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  if (!err && p.ilhs == 1 && launch_lusgs<double>(B.d_sl, B.b, 1, g_ctx.st, 0) != cudaSuccess) err = OT2D_ERR_CUDA;
  if (!err && p.ilhs != 1 && launch_adi<double>(B.d_sl, B.b, 1, g_ctx.st, 0) != cudaSuccess) err = OT2D_ERR_CUDA;
  if (!err && turb && launch_sa<double>(B.d_sl, B.b, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  if (!err && sst && launch_sst<double>(B.d_sl, B.b, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  if (!err && launch_update<double>(B.d_sl, B.b, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  if (!err) {
    std::vector<double> red((size_t)RED_N * nspec);
    cudaMemcpyAsync(red.data(), g_ctx.dred, red.size() * 8, cudaMemcpyDeviceToHost, g_ctx.st);
    cudaStreamSynchronize(g_ctx.st);
    g_ctx.norms.assign(3 * nspec, 0.0);
    for (int i = 0; i < nspec; ++i)
      for (int c = 0; c < 3; ++c) g_ctx.norms[3 * i + c] = red[(size_t)RED_N * i + c];
    for (int i = 0; i < nspec; ++i) if (!(g_ctx.norms[3 * i] <= 1000.0)) err = OT2D_ERR_NORM;
  }
  int e2 = finish(err == OT2D_ERR_NORM ? 0 : err);
  return e2 ? e2 : fail(err);
}

int ot2d_last_norms(double* out, int32_t n) {
  if (!out || n < 0) return fail(OT2D_ERR_ARG);
  for (int i = 0; i < n && i < (int)g_ctx.norms.size(); ++i) out[i] = g_ctx.norms[i];
  return OT2D_OK;
}

int ot2d_monitor(int32_t* mstop, double* q, int32_t* jd, int32_t* kd) {
  int err = 0;
  if (prepare(1, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  if (!mstop || !dims_ok(jd, kd) || !q) return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd, ns = (size_t)p.nspec;
  double* dq = (double*)resolve(q, n2 * ns * p.nq * 8, true, false, err);
  std::vector<Slice<double>> sl;
  for (int nsp = 1; nsp <= p.nspec && !err; ++nsp) {
    Slice<double> S = base_slice(1, 1, (int64_t)(n2 * ns));
    S.q = S.q64 = dq + (size_t)(nsp - 1) * n2;
    S.ist = g_ctx.dist;
    sl.push_back(S);
  }
  if (!err) cudaMemsetAsync(g_ctx.dist, 0, sizeof(int32_t) * IST_N, g_ctx.st);
  run_batch(sl, err);
  if (!err && launch_monitor<double>(g_ctx.batch.d_sl, g_ctx.batch.b, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  int32_t ist[IST_N] = {0, 0, 0, 0};
  if (!err) cudaMemcpyAsync(ist, g_ctx.dist, sizeof(ist), cudaMemcpyDeviceToHost, g_ctx.st);
  err = finish(err);
  *mstop = (ist[2] & 2) ? 1 : 0;
  return err;
}

int ot2d_force2d(int32_t* jd, int32_t* kd, double* x, double* y, double* xv, double* yv, double* q, double* xx,
                 double* xy, double* yx, double* yy, double* cfx, double* cfy, double* cm0, double* cpower,
                 int32_t* nsp) {
  (void)x; (void)y; (void)nsp;
  int err = 0;
  if (prepare(1, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || !q || !xv || !yv || !xx || !xy || !yx || !yy || !cfx || !cfy || !cm0 || !cpower)
    return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd, nv = (size_t)p.jmax * p.kmax;
  Slice<double> S = base_slice(1, 1, (int64_t)n2);
  S.q = S.q64 = (double*)resolve(q, n2 * p.nq * 8, true, false, err);
  S.xx64 = (double*)resolve(xx, n2 * 8, true, false, err);
  S.xy64 = (double*)resolve(xy, n2 * 8, true, false, err);
  S.yx64 = (double*)resolve(yx, n2 * 8, true, false, err);
  S.yy64 = (double*)resolve(yy, n2 * 8, true, false, err);
  double* dxv = (double*)resolve(xv, nv * 8, true, false, err);
  double* dyv = (double*)resolve(yv, nv * 8, true, false, err);
  const double** ptrs = nullptr;
  double* out = nullptr;
  if (!err && cudaMalloc(&ptrs, 2 * sizeof(double*)) != cudaSuccess) err = OT2D_ERR_NOMEM;
  if (ptrs) g_ctx.pool.push_back((void*)ptrs);
  if (!err && cudaMalloc(&out, 4 * sizeof(double)) != cudaSuccess) err = OT2D_ERR_NOMEM;
  if (out) g_ctx.pool.push_back(out);
  const double* hp[2] = {dxv, dyv};
  if (!err) cudaMemcpyAsync(ptrs, hp, sizeof(hp), cudaMemcpyHostToDevice, g_ctx.st);
  std::vector<Slice<double>> sl{S};
  run_batch(sl, err);
  if (!err && launch_forces<double>(g_ctx.batch.d_sl, g_ctx.batch.b, ptrs, ptrs + 1, out, g_ctx.st) != cudaSuccess)
    err = OT2D_ERR_CUDA;
  double h[4] = {0, 0, 0, 0};
  if (!err) cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, g_ctx.st);
  err = finish(err);
  *cfx = h[0]; *cfy = h[1]; *cm0 = h[2]; *cpower = h[3];
  return err;
}

int ot2d_find_cellcenter(double* x, double* y, double* xv, double* yv, int32_t* jd, int32_t* kd, int32_t* im) {
  (void)im;
  if (!g_ctx.has) return fail(OT2D_ERR_NOPARAMS);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || !x || !y || !xv || !yv) return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd, nv = (size_t)p.jmax * p.kmax;
  std::vector<double> hxv = host_copy(xv, nv), hyv = host_copy(yv, nv), hx(n2), hy(n2);
  cell_centres(p, hxv.data(), hyv.data(), hx.data(), hy.data());
  host_store(x, hx.data(), n2);
  host_store(y, hy.data(), n2);
  return OT2D_OK;
}

int ot2d_metfv(double* q, double* x, double* y, double* xv, double* yv, double* xx, double* xy, double* yx,
               double* yy, int32_t* jd, int32_t* kd, int32_t* im) {
  (void)x; (void)y; (void)im;
  if (!g_ctx.has) return fail(OT2D_ERR_NOPARAMS);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || !q || !xv || !yv || !xx || !xy || !yx || !yy) return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd, nv = (size_t)p.jmax * p.kmax;
  std::vector<double> hxv = host_copy(xv, nv), hyv = host_copy(yv, nv);
  std::vector<double> J(n2), a(n2), b(n2), c(n2), d(n2);
  int nneg = metrics(p, hxv.data(), hyv.data(), J.data(), a.data(), b.data(), c.data(), d.data());
  host_store(q + (size_t)(p.nq - 1) * n2, J.data(), n2);
  host_store(xx, a.data(), n2); host_store(xy, b.data(), n2);
  host_store(yx, c.data(), n2); host_store(yy, d.data(), n2);
  return nneg ? fail(OT2D_ERR_ARG) : OT2D_OK;
}

int ot2d_store(double* q, double* x, double* y, int32_t* iblank, int32_t* jd, int32_t* kd, int32_t* lg,
               int32_t* lq) {
  if (!jd || !kd) return fail(OT2D_ERR_ARG);
  return fail(store_impl(q, x, y, iblank, *jd, *kd, lg, lq, 1));
}

int ot2d_storevnu(double* x, double* y, int32_t* iblank, double* q, int32_t* jd, int32_t* kd, int32_t* lq,
                  int32_t* ltur) {
  if (!jd || !kd) return fail(OT2D_ERR_ARG);
  return fail(storeturb_impl(x, y, iblank, q, *jd, *kd, lq, ltur, false));
}

int ot2d_storekomega(double* x, double* y, int32_t* iblank, double* q, int32_t* jd, int32_t* kd, int32_t* lq,
                     int32_t* ltur) {
  if (!jd || !kd) return fail(OT2D_ERR_ARG);
  return fail(storeturb_impl(x, y, iblank, q, *jd, *kd, lq, ltur, true));
}

int ot2d_astore(double* x, double* y, int32_t* iblank, double* q, int32_t* iturb, int32_t* itrans, int32_t* jgmx,
                int32_t* kgmx, int32_t* nmesh, int32_t* ipointer, int32_t* igrd, int32_t* iqdim, int32_t* jd,
                int32_t* kd, int32_t* istep0, int32_t* ts, int32_t* nspec) {
  if (!g_ctx.has) return fail(OT2D_ERR_NOPARAMS);
  const ot2d_params& p = g_ctx.P;
  if (!x || !y || !iblank || !q || !iturb || !itrans || !jgmx || !kgmx || !nmesh || !ipointer || !igrd || !iqdim ||
      !jd || !kd || !istep0 || !ts || !nspec)
    return fail(OT2D_ERR_ARG);
  const int nm = *nmesh, ns = *nspec, it = *iturb;
  if (nm < 1 || ns != p.nspec || *itrans != 0 || it != p.iturb) return fail(OT2D_ERR_ARG);
  const bool tsf = *ts != 0, turb = it == 1 || it == 2;
  // meshes must lie inside x / y / iblank (igrd) and q (iqdim)
  for (int im = 0; im < nm; ++im) {
    const int64_t n2 = (int64_t)jgmx[im] * kgmx[im];
    const int64_t ig = ipointer[im], igq = ipointer[nm + im];
    if (jgmx[im] < 1 || kgmx[im] < 1 || ig < 1 || igq < 1 || ig - 1 + n2 * ns > *igrd ||
        igq - 1 + n2 * ns * p.nq > *iqdim)
      return fail(OT2D_ERR_ARG);
  }
  std::vector<int32_t> lg(ns), lq(ns), lt(ns);
  std::vector<int32_t> dims(2 * (size_t)nm);
  for (int im = 0; im < nm; ++im) { dims[2 * im] = jgmx[im]; dims[2 * im + 1] = kgmx[im]; }
  int err = 0;
  // io.f:38-71: open the grid / solution files, mesh-count and size records
  for (int s = 0; s < ns && !err; ++s) {
    lg[s] = 1000 * (s + 1) + 9; lq[s] = 1000 * (s + 1) + 8; lt[s] = 1000 * (s + 1) + 10;
    err = unit_open(lg[s], sol_file("", tsf, s + 1, 'g', it).c_str(), false, true);
    if (!err) err = unit_open(lq[s], sol_file("", tsf, s + 1, 'q', it).c_str(), false, true);
    const int32_t n1 = nm;
    for (int32_t u : {lg[s], lq[s]}) {
      Seg sm{&n1, 4}, sd{dims.data(), dims.size() * 4};
      if (!err && nm > 1) err = rec_write(unit_file(u, false, true), &sm, 1);
      if (!err) err = rec_write(unit_file(u, false, true), &sd, 1);
    }
  }
  // io.f:75-80: store every mesh
  for (int im = 0; im < nm && !err; ++im) {
    *jd = jgmx[im]; *kd = kgmx[im];
    const int64_t ig = ipointer[im] - 1, igq = ipointer[nm + im] - 1;
    err = store_impl(q + igq, x + ig, y + ig, iblank + ig, *jd, *kd, lg.data(), lq.data(), nm);
  }
  // io.f:84-158: the turbulence files
  for (int s = 0; s < ns && !err && turb; ++s) {
    err = unit_open(lt[s], sol_file("", tsf, s + 1, 't', it).c_str(), true, true);
    if (!err) err = tec_title(unit_file(lt[s], true, true), it);
  }
  for (int im = 0; im < nm && !err && turb; ++im) {
    *jd = jgmx[im]; *kd = kgmx[im];
    const int64_t ig = ipointer[im] - 1, igq = ipointer[nm + im] - 1;
    err = storeturb_impl(x + ig, y + ig, iblank + ig, q + igq, *jd, *kd, lq.data(), lt.data(), it == 2);
  }
  // io.f:162-168: istep0 and close
  for (int s = 0; s < ns; ++s) {
    if (!err) {
      Seg si{istep0, 4};
      err = rec_write(unit_file(lq[s], false, true), &si, 1);
    }
    int e1 = unit_close(lg[s]), e2 = unit_close(lq[s]), e3 = turb ? unit_close(lt[s]) : 0;
    if (!err) err = e1 ? e1 : (e2 ? e2 : e3);
  }
  return fail(err);
}

int ot2d_grid(double* xv, double* yv, int32_t* iblank, int32_t* jd, int32_t* kd, int32_t* logg) {
  if (!g_ctx.has) return fail(OT2D_ERR_NOPARAMS);
  if (!xv || !yv || !iblank || !jd || !kd || !logg || *jd < 1 || *kd < 1) return fail(OT2D_ERR_ARG);
  const int jmax = *jd - g_ctx.P.nadd, kmax = *kd - g_ctx.P.nadd;
  if (jmax < 1 || kmax < 1) return fail(OT2D_ERR_ARG);
  const size_t nv = (size_t)jmax * kmax, n2 = (size_t)*jd * *kd;
  std::vector<double> h(2 * nv);
  int err = rec_read(unit_file(*logg, false, false), h.data(), h.size() * 8);
  if (!err) err = put(xv, h.data(), nv * 8);
  if (!err) err = put(yv, h.data() + nv, nv * 8);
  std::vector<int32_t> one(n2, 1);   // num_grids = 1
  if (!err) err = put(iblank, one.data(), n2 * 4);
  return fail(err);
}

int ot2d_restr2(double* q, int32_t* jd, int32_t* kd, int32_t* logq) {
  if (!g_ctx.has) return fail(OT2D_ERR_NOPARAMS);
  if (!q || !jd || !kd || !logq || *jd < 1 || *kd < 1) return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)*jd * *kd;
  FILE* f = unit_file(*logq, false, false);
  double hdr[4];
  std::vector<double> h(4 * n2);
  int err = rec_read(f, hdr, sizeof(hdr));   // fstip, alf, reypr, totime
  if (!err) err = rec_read(f, h.data(), h.size() * 8);
  if (!err) { g_ctx.P.totime = hdr[3]; err = put(q, h.data(), h.size() * 8); }
  return fail(err);
}

int ot2d_restr_turb(double* q, int32_t* jd, int32_t* kd, int32_t* logq) {
  if (!g_ctx.has) return fail(OT2D_ERR_NOPARAMS);
  if (!q || !jd || !kd || !logq || *jd < 1 || *kd < 1 || g_ctx.P.nv < 4) return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)*jd * *kd, nt = (size_t)g_ctx.P.nv - 4;
  std::vector<double> h(nt * n2);
  int err = rec_read(unit_file(*logq, false, false), h.data(), h.size() * 8);
  if (!err) err = put(q + 4 * n2, h.data(), h.size() * 8);
  return fail(err);
}

int ot2d_qdivj(double* q, int32_t* jd, int32_t* kd) {
  int err = ensure_stream();
  if (err) return fail(err);
  if (!g_ctx.has) return fail(OT2D_ERR_NOPARAMS);
  if (!q || !jd || !kd || *jd < 1 || *kd < 1) return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)*jd * *kd;
  double* dq = (double*)resolve(q, n2 * g_ctx.P.nq * 8, true, true, err);
  if (!err && io_unpack(dq, dq, nullptr, n2, 1, g_ctx.P.nq, 4, 1, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  return finish(err);
}

int ot2d_pitch(int32_t* init, double* x, double* y, double* xv, double* yv, double* xold, double* yold, double* xole,
               double* yole, double* ug, double* vg, int32_t* jd, int32_t* kd) {
  (void)init;
  int err = 0;
  if (prepare(1, err)) return fail(err);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || !x || !y || !xv || !yv || !xold || !yold || !xole || !yole || !ug || !vg ||
      p.ntac < 1 || p.ntac > 3 || !(p.dt > 0))
    return fail(OT2D_ERR_ARG);
  const size_t n2 = (size_t)p.jd * p.kd, nv = (size_t)p.jmax * p.kmax;
  Slice<double> S = base_slice(1, 1, (int64_t)n2);
  S.xc = (double*)resolve(x, n2 * 8, true, true, err);
  S.yc = (double*)resolve(y, n2 * 8, true, true, err);
  S.xv = (double*)resolve(xv, nv * 8, true, true, err);
  S.yv = (double*)resolve(yv, nv * 8, true, true, err);
  S.xold = (double*)resolve(xold, nv * 8, true, true, err);
  S.yold = (double*)resolve(yold, nv * 8, true, true, err);
  S.xole = (double*)resolve(xole, nv * 8, true, true, err);
  S.yole = (double*)resolve(yole, nv * 8, true, true, err);
  S.ug = S.ug64 = (double*)resolve(ug, n2 * 8, true, true, err);
  S.vg = S.vg64 = (double*)resolve(vg, n2 * 8, true, true, err);
  // the increment of step istep (motion.f:576-583) as a one-entry table, and
  // a status word that reads "first Newton iteration of step 1 of the table"
  const double pi = 4.0 * std::atan(1.0);
  const double dtheta = -(p.angmax * (std::cos(p.rotf * (double)p.istep * p.dt) -
                                      std::cos(p.rotf * (double)(p.istep - 1) * p.dt)));
  const double m[4] = {std::sin(dtheta * pi / 180.), std::cos(dtheta * pi / 180.), std::sin(-1. * dtheta * pi / 180.),
                       std::cos(-1. * dtheta * pi / 180.)};
  double* dm = nullptr;
  if (!err && cudaMalloc(&dm, sizeof(m)) != cudaSuccess) err = OT2D_ERR_NOMEM;
  if (dm) g_ctx.pool.push_back(dm);
  if (!err && cudaMemcpyAsync(dm, m, sizeof(m), cudaMemcpyHostToDevice, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  const int32_t ist[IST_N] = {0, 1, 0, 0, 1, 0};
  if (!err && cudaMemcpyAsync(g_ctx.dist, ist, sizeof(ist), cudaMemcpyHostToDevice, g_ctx.st) != cudaSuccess)
    err = OT2D_ERR_CUDA;
  S.motion = dm; S.nmotion = 1; S.ist = g_ctx.dist;
  std::vector<Slice<double>> sl{S};
  run_batch(sl, err);
  if (!err && launch_pitch<double>(g_ctx.batch.d_sl, g_ctx.batch.b, g_ctx.st) != cudaSuccess) err = OT2D_ERR_CUDA;
  return finish(err);
}

int ot2d_stqol(double* q, double* qtn, double* qtnm1, double* qnewt, int32_t* jd, int32_t* kd) {
  int err = 0;
  if ((err = ensure_stream())) return fail(err);
  if (!g_ctx.has) return fail(OT2D_ERR_NOPARAMS);
  const ot2d_params& p = g_ctx.P;
  if (!dims_ok(jd, kd) || !q || !qtn || !qtnm1 || !qnewt || p.nv < 4) return fail(OT2D_ERR_ARG);
  const size_t qs = (size_t)p.jd * p.kd * p.nspec;
  double* dq = (double*)resolve(q, qs * p.nq * 8, true, false, err);
  double* d1 = (double*)resolve(qtn, qs * p.nv * 8, true, true, err);
  double* d2 = (double*)resolve(qtnm1, qs * p.nv * 8, true, true, err);
  double* d3 = (double*)resolve(qnewt, qs * p.nv * 8, false, true, err);
  if (!err && launch_stqol(dq, d1, d2, d3, (int64_t)qs, p.nv, p.ntac, p.istep, g_ctx.st) != cudaSuccess)
    err = OT2D_ERR_CUDA;
  return finish(err);
}

int ot2d_do_interpolations(double* qg, int32_t* jmx, int32_t* kmx, int32_t* ibcg, int32_t* imeshg, int32_t* idonorg,
                           double* fracg, int32_t* nfringeg, int32_t* ndonorg, int32_t* iisptrg, int32_t* iieptrg,
                           int32_t* idsize, int32_t* qsize, int32_t* nmesh) {
  int err = ensure_stream();
  if (err) return fail(err);
  if (!g_ctx.has) return fail(OT2D_ERR_NOPARAMS);
  const ot2d_params& p = g_ctx.P;
  if (!qg || !jmx || !kmx || !ibcg || !imeshg || !idonorg || !fracg || !nfringeg || !ndonorg || !iisptrg || !iieptrg ||
      !idsize || !qsize || !nmesh || *nmesh < 1 || *idsize < 0 || *qsize < 0 || p.nspec < 1 || p.nv < p.nmv ||
      p.nq <= p.nv)
    return fail(OT2D_ERR_ARG);
  const int nm = *nmesh, ns = p.nspec, ids = *idsize;
  // the connectivity is read on the host (it is the caller's, possibly device memory)
  std::vector<int32_t> hj(nm), hk(nm), nfr((size_t)nm * ns), ndo((size_t)nm * ns), iis((size_t)nm * ns),
      iie((size_t)nm * ns);
  const size_t nid = (size_t)ids * 2 * nm * ns;
  std::vector<int32_t> hib((size_t)ids * nm * ns), hmesh(nid), hdon(nid);
  std::vector<double> hfr(nid);
  if ((err = fetch(jmx, nm * 4, hj.data())) || (err = fetch(kmx, nm * 4, hk.data())) ||
      (err = fetch(nfringeg, nfr.size() * 4, nfr.data())) || (err = fetch(ndonorg, ndo.size() * 4, ndo.data())) ||
      (err = fetch(iisptrg, iis.size() * 4, iis.data())) || (err = fetch(iieptrg, iie.size() * 4, iie.data())) ||
      (err = fetch(ibcg, hib.size() * 4, hib.data())) || (err = fetch(imeshg, nid * 4, hmesh.data())) ||
      (err = fetch(idonorg, nid * 4, hdon.data())) || (err = fetch(fracg, nid * 8, hfr.data())))
    return fail(err);
  // mesh blocks of qg (connectivity.f:57-65): q(jmx, kmx, nspec, nq) one after another
  std::vector<int64_t> qoff(nm + 1, 0);
  for (int im = 0; im < nm; ++im) {
    if (hj[im] < 3 || hk[im] < 3) return fail(OT2D_ERR_ARG);
    qoff[im + 1] = qoff[im] + (int64_t)hj[im] * hk[im] * ns * p.nq;
  }
  if (qoff[nm] > (int64_t)*qsize) return fail(OT2D_ERR_ARG);
  std::vector<int64_t> boff(ns + 1, 0);
  for (int s = 0; s < ns; ++s) {
    const int bcdim = iie[(size_t)s * nm + (nm - 1)];
    if (bcdim < 0) return fail(OT2D_ERR_ARG);
    boff[s + 1] = boff[s] + (int64_t)bcdim * p.nv;
  }
  // every index is checked here, so the kernels read and write in bounds
  std::vector<OvsDon> dons;
  std::vector<OvsFr> frs;
  std::map<int64_t, size_t> last;   // fringe cell -> its last entry (the reference's later write wins)
  for (int s = 0; s < ns; ++s) {
    const int bcdim = iie[(size_t)s * nm + (nm - 1)];
    for (int im = 0; im < nm; ++im) {
      const size_t mi = (size_t)s * nm + im;
      const int jm = hj[im], km = hk[im];
      const int64_t vstride = (int64_t)jm * km * ns, qbase = qoff[im] + (int64_t)jm * km * s;
      if (ndo[mi] < 0 || ndo[mi] > ids || nfr[mi] < 0 || nfr[mi] > ids) return fail(OT2D_ERR_ARG);
      for (int id = 0; id < ndo[mi]; ++id) {
        OvsDon d{};
        d.qbase = qbase; d.vstride = vstride; d.boff = boff[s]; d.jm = jm; d.bcdim = bcdim;
        d.ii = hdon[(mi * 2 + 0) * ids + id]; d.jj = hdon[(mi * 2 + 1) * ids + id];
        d.f1 = hfr[(mi * 2 + 0) * ids + id]; d.f2 = hfr[(mi * 2 + 1) * ids + id];
        d.row = iis[mi] + id;
        if (d.ii < 2 || d.ii > jm - 1 || d.jj < 2 || d.jj > km - 1 || d.row < 1 || d.row > bcdim)
          return fail(OT2D_ERR_ARG);
        dons.push_back(d);
      }
      for (int id = 0; id < nfr[mi]; ++id) {
        OvsFr f{};
        f.qbase = qbase; f.vstride = vstride; f.boff = boff[s]; f.jm = jm; f.bcdim = bcdim;
        f.row = hib[mi * ids + id];
        f.ii = hmesh[(mi * 2 + 0) * ids + id]; f.jj = hmesh[(mi * 2 + 1) * ids + id];
        if (f.ii < 1 || f.ii > jm || f.jj < 1 || f.jj > km || f.row < 1 || f.row > bcdim) return fail(OT2D_ERR_ARG);
        const int64_t cell = qbase + (int64_t)(f.jj - 1) * jm + (f.ii - 1);
        auto it = last.find(cell);
        if (it != last.end()) frs[it->second] = f;
        else { last[cell] = frs.size(); frs.push_back(f); }
      }
    }
  }
  double* dq = (double*)resolve(qg, (size_t)qoff[nm] * 8, true, true, err);
  OvsDon* ddn = dons.empty() ? nullptr : (OvsDon*)resolve(dons.data(), dons.size() * sizeof(OvsDon), true, false, err);
  OvsFr* dfr = frs.empty() ? nullptr : (OvsFr*)resolve(frs.data(), frs.size() * sizeof(OvsFr), true, false, err);
  double* dqbc = nullptr;
  if (!err && boff[ns] > 0) {
    if (cudaMalloc(&dqbc, (size_t)boff[ns] * 8) != cudaSuccess) err = OT2D_ERR_NOMEM;
    else g_ctx.pool.push_back(dqbc);
  }
  const int nd = (int)dons.size(), nf = (int)frs.size();
  if (!err && nd > 0) k_ovs_gather<<<(nd + 127) / 128, 128, 0, g_ctx.st>>>(ddn, nd, dq, dqbc, p.nq, p.nv, p.nmv);
  if (!err && nf > 0) k_ovs_scatter<<<(nf + 127) / 128, 128, 0, g_ctx.st>>>(dfr, nf, dq, dqbc, p.nq, p.nv, p.nmv);
  if (!err && cudaGetLastError() != cudaSuccess) err = OT2D_ERR_CUDA;
  return finish(err);
}

}  // extern "C"
