// runtime.cu -- device residency of one solve and batch construction.
// Layout in HBM keeps the reference's column-major arrays
// (q(jd,kd,nspec,nq), s(jd,kd,nspec,nv), metrics (jd,kd,nspec)) so that a
// solve's arrays can be exchanged with Fortran callers unchanged.
#include "runtime.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "geom.h"

namespace ot2d {

const char* cuda_err_name(cudaError_t e) { return cudaGetErrorName(e); }

namespace {
constexpr size_t ALIGN = 256;
inline size_t al(size_t b) { return (b + ALIGN - 1) / ALIGN * ALIGN; }
// scratch arrays per time instance: the SA bands (9) and the drop-in face
// fluxes (20) fit in 20; the k-omega SST fields and two-equation bands take 27
inline int nscratch(const ot2d_params& p) {
  return ((!p.lamin && p.iturb == 2) || p.ilhs != 1) ? (SST_NSCRATCH > ADI_NSCRATCH ? SST_NSCRATCH : ADI_NSCRATCH) + 1
                                                     : 20;
}
inline bool is_sst(const ot2d_params& p) { return !p.lamin && p.iturb == 2; }

struct Layout {
  size_t total = 0;
  size_t take(size_t bytes) { size_t o = total; total += al(bytes); return o; }
};

// Plan (and optionally carve) the allocation of one solve.
template <class F>
size_t plan(const ot2d_params& p, int precision, F&& assign) {
  const size_t nspec = (size_t)p.nspec, n2 = (size_t)p.jd * p.kd, nvert = (size_t)p.jmax * p.kmax;
  const size_t ws = (n2 + 63) / 64 * 64;
  const bool mixed = precision == OT2D_FP32_MIXED;
  const size_t rb = mixed ? sizeof(float) : sizeof(double);
  const bool ts = p.timespectral != 0;
  const bool mv = p.iunst == 1;          // time-accurate pitching grid
  const bool gs = ts || mv;              // grid speeds present
  Layout L;
  assign("P", L.take(sizeof(ot2d_params)));
  assign("q64", L.take(sizeof(double) * n2 * nspec * p.nq));
  assign("xx64", L.take(sizeof(double) * n2 * nspec));
  assign("xy64", L.take(sizeof(double) * n2 * nspec));
  assign("yx64", L.take(sizeof(double) * n2 * nspec));
  assign("yy64", L.take(sizeof(double) * n2 * nspec));
  if (gs) {
    assign("ug64", L.take(sizeof(double) * n2 * nspec));
    assign("vg64", L.take(sizeof(double) * n2 * nspec));
  }
  if (ts) assign("Ds", L.take(sizeof(double) * nspec * nspec));
  if (mv) {
    assign("xc", L.take(sizeof(double) * n2 * nspec));
    assign("yc", L.take(sizeof(double) * n2 * nspec));
    assign("xold", L.take(sizeof(double) * nvert * nspec));
    assign("yold", L.take(sizeof(double) * nvert * nspec));
    assign("xole", L.take(sizeof(double) * nvert * nspec));
    assign("yole", L.take(sizeof(double) * nvert * nspec));
    if (p.itnmax > 1) {
      assign("qtn", L.take(sizeof(double) * n2 * nspec * p.nv));
      assign("qtnm1", L.take(sizeof(double) * n2 * nspec * p.nv));
      assign("qnewt", L.take(sizeof(double) * n2 * nspec * p.nv));
    }
  }
  assign("xv", L.take(sizeof(double) * nvert * nspec));
  assign("yv", L.take(sizeof(double) * nvert * nspec));
  assign("iblank", L.take(sizeof(int32_t) * n2 * nspec));
  if (mixed) {
    assign("q", L.take(rb * n2 * nspec * p.nq));
    assign("xx", L.take(rb * n2 * nspec));
    assign("xy", L.take(rb * n2 * nspec));
    assign("yx", L.take(rb * n2 * nspec));
    assign("yy", L.take(rb * n2 * nspec));
    if (gs) { assign("ug", L.take(rb * n2 * nspec)); assign("vg", L.take(rb * n2 * nspec)); }
  }
  assign("s", L.take(rb * n2 * nspec * p.nv));
  assign("fxa", L.take(rb * n2 * nspec));
  assign("fya", L.take(rb * n2 * nspec));
  assign("gxa", L.take(rb * n2 * nspec));
  assign("gya", L.take(rb * n2 * nspec));
  if (gs) { assign("ftj", L.take(rb * n2 * nspec)); assign("gtj", L.take(rb * n2 * nspec)); }
  assign("tscale", L.take(rb * n2 * nspec));
  assign("bt", L.take(rb * n2 * nspec));
  assign("turmu", L.take(rb * n2 * nspec));
  assign("sn", L.take(rb * n2 * nspec));
  assign("w", L.take(rb * ws * nscratch(p) * nspec));
  if (is_sst(p)) assign("wd2", L.take(sizeof(double) * n2 * nspec));
  // the freestream correction belongs to a fixed grid
  if (mixed && !mv) assign("sinf", L.take(rb * n2 * nspec * 4));
  assign("lurec", L.take(rb * (size_t)lu_rec_elems(p.jd, p.kd, (int)rb) * nspec));
  if (rt_lim_class(p.ilim) == 2) assign("quad", L.take(rb * (size_t)quad_elems(p.jd, p.kd) * nspec));
  return L.total;
}

template <class T>
cudaError_t upload_as(void* dst, const double* src, size_t n, cudaStream_t st, std::vector<T>& tmp) {
  if (std::is_same<T, double>::value) return cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, st);
  tmp.resize(n);
  for (size_t i = 0; i < n; ++i) tmp[i] = (T)src[i];
  return cudaMemcpyAsync(dst, tmp.data(), n * sizeof(T), cudaMemcpyHostToDevice, st);
}
}  // namespace

size_t solve_bytes(const ot2d_params& p, int precision) {
  return plan(p, precision, [](const char*, size_t) {});
}

bool batch_fits(int precision, bool precon, int kd_max, int jd_max) {
  if (kd_max < 3 || jd_max < 3 || kd_max - 2 > 1024) return false;
  const int nw = lu_nband(kd_max);
  size_t lu;
  if (precision == OT2D_FP32_MIXED)
    lu = precon ? lu_smem_bytes<float, true>(nw, 1, jd_max) : lu_smem_bytes<float, false>(nw, 1, jd_max);
  else
    lu = precon ? lu_smem_bytes<double, true>(nw, 1, jd_max) : lu_smem_bytes<double, false>(nw, 1, jd_max);
  return lu <= (size_t)SMEM_OPTIN_MAX && sizeof(double) * 3 * (size_t)jd_max <= (size_t)SMEM_OPTIN_MAX;
}

void solve_destroy(DevSolve& d) {
  if (d.mem) cudaFree(d.mem);
  if (d.motion) cudaFree(d.motion);
  d = DevSolve{};
}

int solve_motion_table(DevSolve& d, int nsteps, cudaStream_t st) {
  if (d.P.iunst != 1 || nsteps < 1) return OT2D_OK;
  const ot2d_params& p = d.P;
  const double pi = 4.0 * std::atan(1.0);
  std::vector<double> t(4 * (size_t)nsteps);
  for (int istep = 1; istep <= nsteps; ++istep) {
    // motion.f:579-583
    const double dtheta = -(p.angmax * (std::cos(p.rotf * (double)istep * p.dt) -
                                        std::cos(p.rotf * (double)(istep - 1) * p.dt)));
    double* m = t.data() + 4 * (size_t)(istep - 1);
    m[0] = std::sin(dtheta * pi / 180.);
    m[1] = std::cos(dtheta * pi / 180.);
    m[2] = std::sin(-1. * dtheta * pi / 180.);
    m[3] = std::cos(-1. * dtheta * pi / 180.);
  }
  if (d.motion) cudaFree(d.motion);
  d.motion = nullptr; d.nmotion = 0;
  if (cudaMalloc(&d.motion, t.size() * sizeof(double)) != cudaSuccess) { d.motion = nullptr; return OT2D_ERR_NOMEM; }
  if (cudaMemcpyAsync(d.motion, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return OT2D_ERR_CUDA;
  d.nmotion = nsteps;
  return OT2D_OK;
}

// Mixed path: the f32 residual (inviscid + viscous, no BCs) of the uniform
// freestream state just uploaded, kept in d.sinf and subtracted by the
// residual kernel every iteration.  In real arithmetic it is 0.
int freestream_residual_f32(DevSolve& d, cudaStream_t st) {
  std::vector<Slice<float>> sl;
  for (int nsp = 1; nsp <= d.P.nspec; ++nsp) {
    Slice<float> S = make_slice<float>(d, nsp, nullptr, nullptr);
    S.sinf = nullptr;
    sl.push_back(S);
  }
  DevBatch<float> B;
  int e = B.build(sl, st);
  if (e) { B.release(); return e; }
  const int flags = AS_INV | (d.P.invisc ? 0 : AS_VISC);
  const size_t qs = d.n2 * (size_t)d.P.nspec;
  bool bad = launch_resid_tiles<float>(B.d_sl, B.b, flags, st) != cudaSuccess;
  if (!bad && cudaMemcpyAsync(d.sinf, d.s, qs * 4 * sizeof(float), cudaMemcpyDeviceToDevice, st) != cudaSuccess) bad = true;
  if (!bad && cudaMemsetAsync(d.s, 0, qs * (size_t)d.P.nv * sizeof(float), st) != cudaSuccess) bad = true;
  if (!bad && cudaStreamSynchronize(st) != cudaSuccess) bad = true;
  B.release();
  return bad ? OT2D_ERR_CUDA : OT2D_OK;
}

int solve_create(DevSolve& d, const ot2d_params& p, int precision, const double* xv1, const double* yv1,
                 cudaStream_t st) {
  if (!xv1 || !yv1 || p.nspec < 1 || p.nhalo != 1 || p.jd != p.jmax + 1 || p.kd != p.kmax + 1) return OT2D_ERR_ARG;
  if (precision != OT2D_FP64 && precision != OT2D_FP32_MIXED) return OT2D_ERR_ARG;
  if (p.ilhs < 1 || p.ilhs > 3) return OT2D_ERR_ARG;        // LU-SGS or ADI (pentadiagonal / upwind)
  if (p.ilhs != 1 && (p.jd < 10 || p.kd < 10)) return OT2D_ERR_ARG;  // ADI lines of >= 8 points
  // the sweep's CTA and shared memory, the force kernel's staging
  if (!batch_fits(precision, p.iprecon != 0, p.kd, p.jd)) return OT2D_ERR_ARG;
  if (!p.lamin && p.iturb != 1 && p.iturb != 2) return OT2D_ERR_ARG;  // SA or k-omega SST
  if (p.itrans != 0) return OT2D_ERR_ARG;                            // no transition model
  // reconstructions rhsup dispatches (eulerrhs.f:84-97): |ilim| 0 central,
  // 1 MUSCL, 2 PPM quadratic, ilim 4 WENO5; any other value reconstructs
  // nothing in the reference
  if (!rt_lim_known(p.ilim)) return OT2D_ERR_ARG;
  if (rt_lim_class(p.ilim) == 2 && (p.jd < 7 || p.kd < 7)) return OT2D_ERR_ARG;   // quad's end stencils
  // steady, or time accurate with the pitching grid (Turns_overset.f:372-403:
  // iunst 1, motiontype 1) at first to third order; Newton iterations only
  // in time-accurate runs; not together with the time-spectral form
  if (p.iunst != 0 && !(p.iunst == 1 && p.motiontype == 1 && !p.timespectral && p.ntac >= 1 && p.ntac <= 3 &&
                        p.dt > 0 && p.h > 0))
    return OT2D_ERR_ARG;
  if (p.itnmax < 1 || (p.itnmax > 1 && p.iunst != 1)) return OT2D_ERR_ARG;
  // Turkel preconditioning (preilu2d with LU-SGS, arc2d_precon with ADI)
  if (p.iprecon && !(p.Mp > 0)) return OT2D_ERR_ARG;
  d = DevSolve{};
  d.P = p; d.precision = precision; d.nspec = p.nspec;
  // time.f:30-35: with time-accurate low-Mach preconditioning the time step
  // switches the module to dual time stepping (idual, idual_turb = 1) the
  // first time it runs; every later routine sees the switched values
  if (d.P.iprecon && d.P.timeac == 1 && !d.P.timespectral) { d.P.idual = 1; d.P.idual_turb = 1; }
  // Turns_overset.f:481: without preconditioning Mp is 1 (the far-field BC
  // reads it)
  if (!d.P.iprecon) d.P.Mp = 1.0;
  d.n2 = (size_t)p.jd * p.kd; d.nvert = (size_t)p.jmax * p.kmax; d.wstride = (d.n2 + 63) / 64 * 64;
  std::vector<std::pair<const char*, size_t>> offs;
  d.bytes = plan(p, precision, [&](const char* n, size_t o) { offs.emplace_back(n, o); });
  if (cudaMalloc(&d.mem, d.bytes) != cudaSuccess) { d.mem = nullptr; return OT2D_ERR_NOMEM; }
  char* base = (char*)d.mem;
  for (auto& o : offs) {
    void* ptr = base + o.second;
    std::string n = o.first;
    if (n == "P") d.dP = (ot2d_params*)ptr;
    else if (n == "q64") d.q64 = (double*)ptr;
    else if (n == "xx64") d.xx64 = (double*)ptr;
    else if (n == "xy64") d.xy64 = (double*)ptr;
    else if (n == "yx64") d.yx64 = (double*)ptr;
    else if (n == "yy64") d.yy64 = (double*)ptr;
    else if (n == "ug64") d.ug64 = (double*)ptr;
    else if (n == "vg64") d.vg64 = (double*)ptr;
    else if (n == "Ds") d.Ds = (double*)ptr;
    else if (n == "xv") d.xv = (double*)ptr;
    else if (n == "yv") d.yv = (double*)ptr;
    else if (n == "iblank") d.iblank = (int32_t*)ptr;
    else if (n == "q") d.q = ptr;
    else if (n == "xx") d.xx = ptr;
    else if (n == "xy") d.xy = ptr;
    else if (n == "yx") d.yx = ptr;
    else if (n == "yy") d.yy = ptr;
    else if (n == "ug") d.ug = ptr;
    else if (n == "vg") d.vg = ptr;
    else if (n == "s") d.s = ptr;
    else if (n == "fxa") d.fxa = ptr;
    else if (n == "fya") d.fya = ptr;
    else if (n == "gxa") d.gxa = ptr;
    else if (n == "gya") d.gya = ptr;
    else if (n == "ftj") d.ftj = ptr;
    else if (n == "gtj") d.gtj = ptr;
    else if (n == "tscale") d.tscale = ptr;
    else if (n == "bt") d.bt = ptr;
    else if (n == "turmu") d.turmu = ptr;
    else if (n == "sn") d.sn = ptr;
    else if (n == "w") d.w = ptr;
    else if (n == "lurec") d.lurec = ptr;
    else if (n == "quad") d.quad = ptr;
    else if (n == "wd2") d.wd2 = (double*)ptr;
    else if (n == "xc") d.xc = (double*)ptr;
    else if (n == "yc") d.yc = (double*)ptr;
    else if (n == "xold") d.xold = (double*)ptr;
    else if (n == "yold") d.yold = (double*)ptr;
    else if (n == "xole") d.xole = (double*)ptr;
    else if (n == "yole") d.yole = (double*)ptr;
    else if (n == "qtn") d.qtn = (double*)ptr;
    else if (n == "qtnm1") d.qtnm1 = (double*)ptr;
    else if (n == "qnewt") d.qnewt = (double*)ptr;
    else if (n == "sinf") d.sinf = ptr;
  }
  const bool mixed = precision == OT2D_FP32_MIXED;
  if (!mixed) { d.q = d.q64; d.xx = d.xx64; d.xy = d.xy64; d.yx = d.yx64; d.yy = d.yy64; d.ug = d.ug64; d.vg = d.vg64; }
  // ---- host geometry, per time instance
  const size_t n2 = d.n2, nv = d.nvert, ns = (size_t)p.nspec;
  const size_t qs = n2 * ns;
  std::vector<double> q(qs * p.nq, 0.0), xx(qs), xy(qs), yx(qs), yy(qs), ug(qs, 0.0), vg(qs, 0.0);
  std::vector<double> xv(nv * ns), yv(nv * ns), ugv(nv * ns, 0.0), vgv(nv * ns, 0.0);
  std::vector<double> x(n2), y(n2), sn(qs), fxa(qs), fya(qs), gxa(qs), gya(qs), ftj(qs, 0.0), gtj(qs, 0.0);
  std::vector<double> Ds(ns * ns, 0.0), wd2(is_sst(p) ? qs : 0);
  d.nscratch = nscratch(p);
  bool body = false;
  for (int ib = 0; ib < p.nbc; ++ib) if (p.ibtyp[ib] == 5) body = true;
  const double pi = 4.0 * std::atan(1.0);
  if (p.timespectral) ts_operator(p.nspec, Ds.data());
  for (int nsp = 1; nsp <= p.nspec; ++nsp) {
    double* xvn = xv.data() + (nsp - 1) * nv;
    double* yvn = yv.data() + (nsp - 1) * nv;
    double tspec = 0.0;
    if (p.rf != 0) tspec = 2 * pi * (nsp - 1) / p.nspec / std::fabs(p.rf);
    if (nsp == 1) { std::memcpy(xvn, xv1, nv * sizeof(double)); std::memcpy(yvn, yv1, nv * sizeof(double)); }
    else ts_pitch_grid(p, xv1, yv1, tspec, xvn, yvn);
    const size_t o = (nsp - 1) * n2;
    cell_centres(p, xvn, yvn, x.data(), y.data());
    double* J = q.data() + (p.nq - 1) * qs + o;
    if (metrics(p, xvn, yvn, J, xx.data() + o, xy.data() + o, yx.data() + o, yy.data() + o) != 0) {
      solve_destroy(d);
      return OT2D_ERR_ARG;
    }
    if (p.timespectral)
      ts_grid_speed(p, x.data(), y.data(), xvn, yvn, tspec, ug.data() + o, vg.data() + o, ugv.data() + (nsp - 1) * nv,
                    vgv.data() + (nsp - 1) * nv);
    freestream(p, q.data() + o, qs);
    wall_distance(p, x.data(), y.data(), xvn, yvn, sn.data() + o);
    if (is_sst(p)) {
      // kwdist runs only for meshes with a wall (komegasst.f:67); 1e10 otherwise
      if (!body) for (size_t i = 0; i < n2; ++i) sn[o + i] = 1.e10;
      sst_wall_d2(p, x.data(), y.data(), xvn, yvn, wd2.data() + o);
    }
    face_normals(p, xvn, yvn, ugv.data() + (nsp - 1) * nv, vgv.data() + (nsp - 1) * nv, fxa.data() + o, fya.data() + o,
                 gxa.data() + o, gya.data() + o, p.timespectral ? ftj.data() + o : nullptr,
                 p.timespectral ? gtj.data() + o : nullptr);
  }
  bool bad = false;
  auto chk = [&](cudaError_t e) { if (e != cudaSuccess) bad = true; };
  chk(cudaMemcpyAsync(d.dP, &d.P, sizeof(d.P), cudaMemcpyHostToDevice, st));
  chk(cudaMemcpyAsync(d.q64, q.data(), q.size() * 8, cudaMemcpyHostToDevice, st));
  chk(cudaMemcpyAsync(d.xx64, xx.data(), qs * 8, cudaMemcpyHostToDevice, st));
  chk(cudaMemcpyAsync(d.xy64, xy.data(), qs * 8, cudaMemcpyHostToDevice, st));
  chk(cudaMemcpyAsync(d.yx64, yx.data(), qs * 8, cudaMemcpyHostToDevice, st));
  chk(cudaMemcpyAsync(d.yy64, yy.data(), qs * 8, cudaMemcpyHostToDevice, st));
  if (p.timespectral) {
    chk(cudaMemcpyAsync(d.ug64, ug.data(), qs * 8, cudaMemcpyHostToDevice, st));
    chk(cudaMemcpyAsync(d.vg64, vg.data(), qs * 8, cudaMemcpyHostToDevice, st));
    chk(cudaMemcpyAsync(d.Ds, Ds.data(), ns * ns * 8, cudaMemcpyHostToDevice, st));
  }
  if (d.wd2) chk(cudaMemcpyAsync(d.wd2, wd2.data(), qs * 8, cudaMemcpyHostToDevice, st));
  if (d.xc) {
    // time-accurate grid at rest before its first step (init.f:101-108):
    // centres of instance 1, both previous vertex levels = the grid, no
    // grid speed; face speeds and stqol levels are set by the first step
    chk(cudaMemcpyAsync(d.xc, x.data(), n2 * 8, cudaMemcpyHostToDevice, st));
    chk(cudaMemcpyAsync(d.yc, y.data(), n2 * 8, cudaMemcpyHostToDevice, st));
    for (double* dst : {d.xold, d.xole}) chk(cudaMemcpyAsync(dst, xv.data(), nv * 8, cudaMemcpyHostToDevice, st));
    for (double* dst : {d.yold, d.yole}) chk(cudaMemcpyAsync(dst, yv.data(), nv * 8, cudaMemcpyHostToDevice, st));
    chk(cudaMemsetAsync(d.ug64, 0, qs * 8, st));
    chk(cudaMemsetAsync(d.vg64, 0, qs * 8, st));
    const size_t rb = mixed ? sizeof(float) : sizeof(double);
    if (mixed) { chk(cudaMemsetAsync(d.ug, 0, qs * rb, st)); chk(cudaMemsetAsync(d.vg, 0, qs * rb, st)); }
    chk(cudaMemsetAsync(d.ftj, 0, qs * rb, st));
    chk(cudaMemsetAsync(d.gtj, 0, qs * rb, st));
    for (double* a : {d.qtn, d.qtnm1, d.qnewt})
      if (a) chk(cudaMemsetAsync(a, 0, qs * (size_t)p.nv * 8, st));
  }
  chk(cudaMemcpyAsync(d.xv, xv.data(), xv.size() * 8, cudaMemcpyHostToDevice, st));
  chk(cudaMemcpyAsync(d.yv, yv.data(), yv.size() * 8, cudaMemcpyHostToDevice, st));
  std::vector<int32_t> ib(qs, 1);
  chk(cudaMemcpyAsync(d.iblank, ib.data(), qs * 4, cudaMemcpyHostToDevice, st));
  if (mixed) {
    std::vector<float> t1, t2, t3, t4, t5, t6, t7, t8, t9, t10, t11, t12, t13, t14, t15;
    chk(upload_as<float>(d.q, q.data(), q.size(), st, t1));
    chk(upload_as<float>(d.xx, xx.data(), qs, st, t2));
    chk(upload_as<float>(d.xy, xy.data(), qs, st, t3));
    chk(upload_as<float>(d.yx, yx.data(), qs, st, t4));
    chk(upload_as<float>(d.yy, yy.data(), qs, st, t5));
    if (p.timespectral) { chk(upload_as<float>(d.ug, ug.data(), qs, st, t6)); chk(upload_as<float>(d.vg, vg.data(), qs, st, t7)); }
    chk(upload_as<float>(d.fxa, fxa.data(), qs, st, t8));
    chk(upload_as<float>(d.fya, fya.data(), qs, st, t9));
    chk(upload_as<float>(d.gxa, gxa.data(), qs, st, t10));
    chk(upload_as<float>(d.gya, gya.data(), qs, st, t11));
    if (p.timespectral) { chk(upload_as<float>(d.ftj, ftj.data(), qs, st, t12)); chk(upload_as<float>(d.gtj, gtj.data(), qs, st, t13)); }
    chk(upload_as<float>(d.sn, sn.data(), qs, st, t14));
    chk(cudaMemsetAsync(d.turmu, 0, qs * sizeof(float), st));
    chk(cudaStreamSynchronize(st));
    if (!bad && d.sinf && freestream_residual_f32(d, st) != OT2D_OK) bad = true;
  } else {
    chk(cudaMemcpyAsync(d.fxa, fxa.data(), qs * 8, cudaMemcpyHostToDevice, st));
    chk(cudaMemcpyAsync(d.fya, fya.data(), qs * 8, cudaMemcpyHostToDevice, st));
    chk(cudaMemcpyAsync(d.gxa, gxa.data(), qs * 8, cudaMemcpyHostToDevice, st));
    chk(cudaMemcpyAsync(d.gya, gya.data(), qs * 8, cudaMemcpyHostToDevice, st));
    if (p.timespectral) {
      chk(cudaMemcpyAsync(d.ftj, ftj.data(), qs * 8, cudaMemcpyHostToDevice, st));
      chk(cudaMemcpyAsync(d.gtj, gtj.data(), qs * 8, cudaMemcpyHostToDevice, st));
    }
    chk(cudaMemcpyAsync(d.sn, sn.data(), qs * 8, cudaMemcpyHostToDevice, st));
    chk(cudaMemsetAsync(d.turmu, 0, qs * sizeof(double), st));
    chk(cudaStreamSynchronize(st));
  }
  if (bad) { solve_destroy(d); return OT2D_ERR_CUDA; }
  return OT2D_OK;
}

template <class R>
Slice<R> make_slice(const DevSolve& d, int nsp, double* red, int32_t* ist) {
  Slice<R> S{};
  const ot2d_params& p = d.P;
  const size_t o = (size_t)(nsp - 1) * d.n2;
  auto R_ = [&](void* a) -> R* { return a ? (R*)a + o : nullptr; };
  auto D_ = [&](double* a) -> double* { return a ? a + o : nullptr; };
  S.P = d.dP;
  S.jd = p.jd; S.kd = p.kd; S.nsp = nsp; S.nspec = p.nspec;
  S.qs = (int64_t)d.n2 * p.nspec;
  S.q = R_(d.q); S.q64 = D_(d.q64); S.s = R_(d.s);
  S.xx = R_(d.xx); S.xy = R_(d.xy); S.yx = R_(d.yx); S.yy = R_(d.yy);
  S.fxa = R_(d.fxa); S.fya = R_(d.fya); S.gxa = R_(d.gxa); S.gya = R_(d.gya);
  const bool gs = p.timespectral || d.xc;
  S.ftj = gs ? R_(d.ftj) : nullptr; S.gtj = gs ? R_(d.gtj) : nullptr;
  S.ug = gs ? R_(d.ug) : nullptr; S.vg = gs ? R_(d.vg) : nullptr;
  S.tscale = R_(d.tscale); S.bt = R_(d.bt); S.turmu = R_(d.turmu);
  S.iblank = d.iblank + o;
  S.sn = R_(d.sn);
  S.w = (R*)d.w + (size_t)(nsp - 1) * d.wstride * d.nscratch;
  S.wd2 = D_(d.wd2);
  S.sinf = R_(d.sinf);
  slice_consts(S, p);
  S.wstride = (int64_t)d.wstride;
  S.lurec = (R*)d.lurec + (size_t)(nsp - 1) * (size_t)lu_rec_elems(p.jd, p.kd, (int)sizeof(R));
  S.quad = d.quad ? (R*)d.quad + (size_t)(nsp - 1) * (size_t)quad_elems(p.jd, p.kd) : nullptr;
  S.red = red; S.ist = ist;
  S.Ds = p.timespectral ? d.Ds : nullptr;
  S.xx64 = D_(d.xx64); S.xy64 = D_(d.xy64); S.yx64 = D_(d.yx64); S.yy64 = D_(d.yy64);
  S.ug64 = gs ? D_(d.ug64) : nullptr; S.vg64 = gs ? D_(d.vg64) : nullptr;
  const size_t ov = (size_t)(nsp - 1) * d.nvert;
  S.xv = d.xv + ov; S.yv = d.yv + ov;
  if (d.xc) {
    S.xc = D_(d.xc); S.yc = D_(d.yc);
    S.xold = d.xold + ov; S.yold = d.yold + ov; S.xole = d.xole + ov; S.yole = d.yole + ov;
    S.qtn = D_(d.qtn); S.qtnm1 = D_(d.qtnm1); S.qnewt = D_(d.qnewt);
    S.motion = d.motion; S.nmotion = d.nmotion;
  }
  return S;
}
template Slice<double> make_slice<double>(const DevSolve&, int, double*, int32_t*);
template Slice<float> make_slice<float>(const DevSolve&, int, double*, int32_t*);

template <class R>
int DevBatch<R>::build(const std::vector<Slice<R>>& sl, cudaStream_t st) {
  const int n = (int)sl.size();
  // six prefix tables of n+1 entries: cell blocks, k-lines, j-lines, LU
  // record blocks, 32-line groups, residual tiles
  std::vector<int32_t> idx(6 * (n + 1));
  int cells = 0, jl = 0, kl = 0, lub = 0, grp = 0, tiles = 0, maxw = 1, maxwall = 1, maxkd = 1, moving = 0, precon = 0;
  int maxnbc = 0, limmask = 0;
  int tj = 16, tk = 16;
  rt_shape_dims(rt_shape, tj, tk);
  for (int i = 0; i < n; ++i) {
    if (sl[i].xc) moving = 1;
    if (sl[i].k_mp2 >= (R)0) precon = 1;
    maxnbc = std::max(maxnbc, (int)sl[i].nbc);
    limmask |= sl[i].lim == 4 ? 4 : (sl[i].lim == 1 ? 2 : (sl[i].lim == 2 ? 8 : 1));
    idx[i] = cells; idx[(n + 1) + i] = jl; idx[2 * (n + 1) + i] = kl; idx[3 * (n + 1) + i] = lub;
    idx[4 * (n + 1) + i] = grp; idx[5 * (n + 1) + i] = tiles;
    const int jd = sl[i].jd, kd = sl[i].kd;
    cells += (jd * kd + CELL_BS - 1) / CELL_BS;
    jl += kd - 2;   // k-lines solved along j
    kl += jd - 2;   // j-lines solved along k
    lub += (lu_nband(kd) * lu_nstep(jd) * 32 + LU_PREP_BS - 1) / LU_PREP_BS;
    grp += lu_nband(kd);
    tiles += ((jd - 2 + tj - 1) / tj) * ((kd - 2 + tk - 1) / tk);
    maxw = std::max(maxw, lu_nband(kd));
    maxwall = std::max(maxwall, jd);
    maxkd = std::max(maxkd, kd);
  }
  // a combination of meshes that fit alone may not fit together
  if (n > 0 && !batch_fits(sizeof(R) == sizeof(float) ? OT2D_FP32_MIXED : OT2D_FP64, precon != 0, maxkd, maxwall))
    return OT2D_ERR_ARG;
  idx[n] = cells; idx[2 * (n + 1) - 1] = jl; idx[3 * (n + 1) - 1] = kl; idx[4 * (n + 1) - 1] = lub;
  idx[5 * (n + 1) - 1] = grp; idx[6 * (n + 1) - 1] = tiles;
  if ((size_t)n > cap_sl) {
    if (d_sl) cudaFree(d_sl);
    if (d_idx) cudaFree(d_idx);
    cap_sl = std::max((size_t)n, (size_t)2 * cap_sl);
    if (cudaMalloc(&d_sl, cap_sl * sizeof(Slice<R>)) != cudaSuccess) return OT2D_ERR_NOMEM;
    if (cudaMalloc(&d_idx, 6 * (cap_sl + 1) * sizeof(int32_t)) != cudaSuccess) return OT2D_ERR_NOMEM;
  }
  const size_t nparts = (size_t)std::max(cells, tiles);
  if (nparts > cap_part) {
    if (d_part) cudaFree(d_part);
    cap_part = std::max(nparts, (size_t)2 * cap_part);
    if (cudaMalloc(&d_part, cap_part * sizeof(NormPart)) != cudaSuccess) return OT2D_ERR_NOMEM;
  }
  if (cudaMemcpyAsync(d_sl, sl.data(), n * sizeof(Slice<R>), cudaMemcpyHostToDevice, st) != cudaSuccess) return OT2D_ERR_CUDA;
  if (cudaMemcpyAsync(d_idx, idx.data(), idx.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return OT2D_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return OT2D_ERR_CUDA;
  b.nslice = n;
  b.moving = moving;
  b.precon = precon;
  b.cell_blocks = cells;
  b.max_lu_warps = maxw;
  b.max_wall = maxwall;
  b.max_kd = maxkd;
  b.max_nbc = maxnbc;
  b.lim_mask = limmask;
  b.rt_shape = rt_shape;
  b.jlines = jl; b.klines = kl;
  b.lu_blocks = lub;
  b.jgroups = grp;
  b.d_gfirst = d_idx + 4 * (n + 1);
  b.d_tfirst = d_idx + 5 * (n + 1);
  b.tile_blocks = tiles;
  b.d_first = d_idx; b.d_jfirst = d_idx + (n + 1); b.d_kfirst = d_idx + 2 * (n + 1); b.d_lfirst = d_idx + 3 * (n + 1);
  b.d_part = d_part;
  return OT2D_OK;
}

template <class R>
void DevBatch<R>::release() {
  if (d_sl) cudaFree(d_sl);
  if (d_idx) cudaFree(d_idx);
  if (d_part) cudaFree(d_part);
  d_sl = nullptr; d_idx = nullptr; d_part = nullptr; cap_sl = cap_part = 0;
}

template struct DevBatch<double>;
template struct DevBatch<float>;

}  // namespace ot2d
