// io.cu -- solution / restart files in the reference's record layout
// (src/io.f, src/init.f:138-206).  The state conversions of the file format
// (Q = (Q/J)*J on the way out, Q/J on the way in) run on the device over the
// resident state; the host only frames records and formats text.
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>

#include "io.h"

namespace ot2d {

// ---------------------------------------------------------------- unit table

namespace {
struct Unit { FILE* f; bool formatted; bool write; };
std::mutex g_unit_mu;
std::map<int, Unit> g_units;
}  // namespace

int unit_open(int unit, const char* path, bool formatted, bool for_write) {
  if (!path || !*path) return OT2D_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_unit_mu);
  auto it = g_units.find(unit);
  if (it != g_units.end()) { std::fclose(it->second.f); g_units.erase(it); }   // re-open closes first
  FILE* f = std::fopen(path, for_write ? (formatted ? "w" : "wb") : (formatted ? "r" : "rb"));
  if (!f) return OT2D_ERR_IO;
  g_units[unit] = Unit{f, formatted, for_write};
  return OT2D_OK;
}

int unit_close(int unit) {
  std::lock_guard<std::mutex> lk(g_unit_mu);
  auto it = g_units.find(unit);
  if (it == g_units.end()) return OT2D_OK;   // closing an unconnected unit is allowed
  const int e = std::fclose(it->second.f) == 0 ? OT2D_OK : OT2D_ERR_IO;
  g_units.erase(it);
  return e;
}

FILE* unit_file(int unit, bool formatted, bool for_write) {
  std::lock_guard<std::mutex> lk(g_unit_mu);
  auto it = g_units.find(unit);
  if (it == g_units.end() || it->second.formatted != formatted || it->second.write != for_write) return nullptr;
  return it->second.f;
}

// ------------------------------------------------------------------- records

int rec_write(FILE* f, const Seg* segs, int nseg) {
  if (!f) return OT2D_ERR_IO;
  size_t total = 0;
  for (int i = 0; i < nseg; ++i) total += segs[i].n;
  // records of 2 GiB and more would need the compilers' sub-record chains
  if (total > (size_t)INT32_MAX) return OT2D_ERR_ARG;
  const int32_t m = (int32_t)total;
  if (std::fwrite(&m, 4, 1, f) != 1) return OT2D_ERR_IO;
  for (int i = 0; i < nseg; ++i)
    if (segs[i].n && std::fwrite(segs[i].p, 1, segs[i].n, f) != segs[i].n) return OT2D_ERR_IO;
  if (std::fwrite(&m, 4, 1, f) != 1) return OT2D_ERR_IO;
  return OT2D_OK;
}

int rec_read(FILE* f, void* dst, size_t bytes) {
  if (!f) return OT2D_ERR_IO;
  int32_t m = 0, m2 = 0;
  if (std::fread(&m, 4, 1, f) != 1 || m < 0 || (size_t)m < bytes) return OT2D_ERR_IO;
  if (bytes && std::fread(dst, 1, bytes, f) != bytes) return OT2D_ERR_IO;
  if ((size_t)m > bytes && std::fseek(f, (long)((size_t)m - bytes), SEEK_CUR) != 0) return OT2D_ERR_IO;
  if (std::fread(&m2, 4, 1, f) != 1 || m2 != m) return OT2D_ERR_IO;
  return OT2D_OK;
}

// --------------------------------------------------------- formatted output

namespace {
// one Fw.d field: the value with d decimals right-justified in w columns,
// w asterisks when it does not fit; IEEE specials as gfortran spells them
void fmt_f(char* out, double v, int w, int d) {
  char b[64];
  if (std::isnan(v)) std::snprintf(b, sizeof(b), "%*s", w, "NaN");
  else if (std::isinf(v)) std::snprintf(b, sizeof(b), "%*s", w, v > 0 ? "Infinity" : "-Infinity");
  else std::snprintf(b, sizeof(b), "%*.*f", w, d, v);
  if ((int)std::strlen(b) > w) { std::memset(out, '*', w); out[w] = 0; return; }
  std::memcpy(out, b, (size_t)w + 1);
}
}  // namespace

int tec_reals(FILE* f, const double* v, size_t n) {
  if (!f) return OT2D_ERR_IO;
  char line[3 * 22 + 2], fld[32];
  for (size_t i = 0; i < n; i += 3) {
    size_t c = 0;
    for (size_t t = i; t < n && t < i + 3; ++t) { fmt_f(fld, v[t], 22, 13); std::memcpy(line + c, fld, 22); c += 22; }
    line[c++] = '\n';
    if (std::fwrite(line, 1, c, f) != c) return OT2D_ERR_IO;
  }
  if (n == 0 && std::fputc('\n', f) == EOF) return OT2D_ERR_IO;   // an empty list still ends a record
  return OT2D_OK;
}

int tec_ints(FILE* f, const int32_t* v, size_t n) {
  if (!f) return OT2D_ERR_IO;
  for (size_t i = 0; i < n; i += 3) {
    for (size_t t = i; t < n && t < i + 3; ++t) {
      char b[32];
      std::snprintf(b, sizeof(b), "%10d", (int)v[t]);
      if (std::strlen(b) > 10) std::memset(b, '*', 10), b[10] = 0;
      if (std::fputs(b, f) == EOF) return OT2D_ERR_IO;
    }
    if (std::fputc('\n', f) == EOF) return OT2D_ERR_IO;
  }
  if (n == 0 && std::fputc('\n', f) == EOF) return OT2D_ERR_IO;
  return OT2D_OK;
}

// list-directed output: a leading blank, character items as they are,
// default integers right-justified in 12 columns
int tec_title(FILE* f, int iturb) {
  if (!f) return OT2D_ERR_IO;
  int r = std::fprintf(f, " TITLE = \"Turbulence Model solution File\"\n");
  if (r > 0) {
    if (iturb == 2) r = std::fprintf(f, " VARIABLES = \"X\" \"Y\" \"IBlank\" \"K\" \"Omega\"\n");
    else r = std::fprintf(f, " VARIABLES = \"X\" \"Y\" \"IBlank\" \"Vnu_t\"\n");
  }
  return r > 0 ? OT2D_OK : OT2D_ERR_IO;
}

int tec_zone(FILE* f, int jd, int kd) {
  if (!f) return OT2D_ERR_IO;
  const int r = std::fprintf(f, " ZONE\n I = %12d, J = %12d\n ZONETYPE = Ordered, DATAPACKING = BLOCK\n", jd, kd);
  return r > 0 ? OT2D_OK : OT2D_ERR_IO;
}

std::string sol_file(const std::string& dir, bool ts, int nsp, char kind, int iturb) {
  std::string pre = dir.empty() ? std::string() : (dir.back() == '/' ? dir : dir + "/");
  const std::string n = std::to_string(nsp);
  switch (kind) {
    case 'g': return pre + (ts ? "fort_TS" + n + ".9" : std::string("fort.9"));
    case 'q': return pre + (ts ? "fort_TS" + n + ".8" : std::string("fort.8"));
    case 'r': return pre + (ts ? "fort_TS" + n + ".3" : std::string("fort.3"));
    default: {
      const std::string base = iturb == 2 ? "komega" : "SA";
      return pre + (ts ? base + "_TS" + n : base) + ".dat";
    }
  }
}

// ------------------------------------------------------------------- kernels

namespace {

__global__ void k_io_pack(double* __restrict__ q, float* __restrict__ qc, double* __restrict__ rec,
                          double* __restrict__ tec, int64_t n2, int nspec, int nq, int nv, int mode) {
  const int64_t qs = n2 * nspec;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < qs; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = i / n2, c = i - s * n2;
    const double J = q[(int64_t)(nq - 1) * qs + i];
    double q1 = q[i];
    if (mode & IO_REC) {
      double* r = rec + s * (int64_t)nv * n2 + c;
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        const double Q = q[n * qs + i] * J;
        r[n * n2] = Q;
        const double b = Q / J;
        q[n * qs + i] = b;
        if (qc) qc[n * qs + i] = (float)b;
        if (n == 0) q1 = b;
      }
      for (int n = 4; n < nv; ++n) r[n * n2] = q[n * qs + i];
    }
    if (mode & IO_TEC) {
      const double rho = q1 * J;
      double* t = tec + s * 2 * n2 + c;
      t[0] = q[4 * qs + i] / rho;
      t[n2] = q[5 * qs + i] / rho;
    }
  }
}

// rec and q may alias (element i is read and written by the same thread)
__global__ void k_io_unpack(const double* rec, double* q, float* qc, int64_t n2, int nspec, int nq, int nvin,
                            int divj) {
  const int64_t qs = n2 * nspec;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < qs; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = i / n2, c = i - s * n2;
    const double* r = rec + s * (int64_t)nvin * n2 + c;
    const double J = q[(int64_t)(nq - 1) * qs + i];
    for (int n = 0; n < nvin; ++n) {
      double v = r[n * n2];
      if (divj && n < 4) v = v / J;
      q[n * qs + i] = v;
      if (qc) qc[n * qs + i] = (float)v;
    }
  }
}

int io_grid(size_t cells) {
  size_t b = (cells + 255) / 256;
  const size_t cap = 152 * 8;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

cudaError_t io_pack(double* q, float* qc, double* rec, double* tec, size_t n2, int nspec, int nq, int nv, int mode,
                    cudaStream_t st) {
  if (!n2 || nspec < 1) return cudaSuccess;
  if (((mode & IO_REC) && !rec) || ((mode & IO_TEC) && (!tec || nv < 6))) return cudaErrorInvalidValue;
  k_io_pack<<<io_grid(n2 * nspec), 256, 0, st>>>(q, qc, rec, tec, (int64_t)n2, nspec, nq, nv, mode);
  return cudaGetLastError();
}

cudaError_t io_unpack(const double* rec, double* q, float* qc, size_t n2, int nspec, int nq, int nvin, int divj,
                      cudaStream_t st) {
  if (!n2 || nspec < 1) return cudaSuccess;
  k_io_unpack<<<io_grid(n2 * nspec), 256, 0, st>>>(rec, q, qc, (int64_t)n2, nspec, nq, nvin, divj);
  return cudaGetLastError();
}

// ----------------------------------------------------- whole-solve store/read

namespace {
struct DevTmp {
  double* p = nullptr;
  ~DevTmp() { if (p) cudaFree(p); }
};
}  // namespace

int write_solution(const std::string& dir, const ot2d_params& p, double* dq, float* dqc, const double* x,
                   const double* y, const int32_t* iblank, int istep0, cudaStream_t st) {
  // iturb other than 1 (SA) and 2 (SST): no turbulence records or file
  if (p.itrans != 0 || p.nv < 4 || (p.iturb == 1 && p.nv < 5) || (p.iturb == 2 && p.nv < 6)) return OT2D_ERR_ARG;
  const size_t n2 = (size_t)p.jd * p.kd, ns = (size_t)p.nspec, nv = (size_t)p.nv;
  const bool sst = p.iturb == 2, turb = p.iturb == 1 || p.iturb == 2, ts = p.timespectral != 0;
  const size_t nrec = ns * nv * n2, ntec = sst ? ns * 2 * n2 : 0;
  DevTmp tmp;
  if (cudaMalloc(&tmp.p, (nrec + ntec) * sizeof(double)) != cudaSuccess) return OT2D_ERR_NOMEM;
  if (io_pack(dq, dqc, tmp.p, sst ? tmp.p + nrec : nullptr, n2, p.nspec, p.nq, p.nv, IO_REC | (sst ? IO_TEC : 0),
              st) != cudaSuccess)
    return OT2D_ERR_CUDA;
  std::vector<double> h(nrec + ntec);
  if (cudaMemcpyAsync(h.data(), tmp.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return OT2D_ERR_CUDA;
  const int32_t dims[2] = {p.jd, p.kd};
  const double hdr[4] = {p.fsmach, p.alfa, p.rey * p.fsmach, p.totime};   // fstip, alfa, reypr, totime
  const int32_t i0 = istep0;
  for (size_t s = 0; s < ns; ++s) {
    const int nsp = (int)s + 1;
    const double* r = h.data() + s * nv * n2;
    FILE* fg = std::fopen(sol_file(dir, ts, nsp, 'g', p.iturb).c_str(), "wb");
    FILE* fq = std::fopen(sol_file(dir, ts, nsp, 'q', p.iturb).c_str(), "wb");
    FILE* ft = turb ? std::fopen(sol_file(dir, ts, nsp, 't', p.iturb).c_str(), "w") : nullptr;
    int e = (fg && fq && (ft || !turb)) ? OT2D_OK : OT2D_ERR_IO;
    Seg sd{dims, sizeof(dims)};
    if (!e) e = rec_write(fg, &sd, 1);
    if (!e) e = rec_write(fq, &sd, 1);
    // store (io.f:314-329)
    Seg sh{hdr, sizeof(hdr)};
    if (!e) e = rec_write(fq, &sh, 1);
    Seg sqv{r, 4 * n2 * sizeof(double)};
    if (!e) e = rec_write(fq, &sqv, 1);
    Seg stv{r + 4 * n2, (nv - 4) * n2 * sizeof(double)};
    if (!e && turb) e = rec_write(fq, &stv, 1);
    Seg sg[2] = {{x + s * n2, n2 * sizeof(double)}, {y + s * n2, n2 * sizeof(double)}};
    if (!e) e = rec_write(fg, sg, 2);
    // storevnu / storekomega (io.f:173-275); storekomega writes the
    // turbulence record a second time (io.f:253)
    if (!e && sst) e = rec_write(fq, &stv, 1);
    if (!e && turb) e = tec_title(ft, p.iturb);
    if (!e && turb) e = tec_zone(ft, p.jd, p.kd);
    if (!e && turb) e = tec_reals(ft, x + s * n2, n2);
    if (!e && turb) e = tec_reals(ft, y + s * n2, n2);
    if (!e && turb) e = tec_ints(ft, iblank + s * n2, n2);
    if (!e && turb && !sst) e = tec_reals(ft, r + 4 * n2, n2);
    if (!e && sst) {
      const double* t = h.data() + nrec + s * 2 * n2;
      e = tec_reals(ft, t, n2);
      if (!e) e = tec_reals(ft, t + n2, n2);
    }
    Seg si{&i0, sizeof(i0)};
    if (!e) e = rec_write(fq, &si, 1);   // astore, io.f:160
    if (fg && std::fclose(fg) != 0 && !e) e = OT2D_ERR_IO;
    if (fq && std::fclose(fq) != 0 && !e) e = OT2D_ERR_IO;
    if (ft && std::fclose(ft) != 0 && !e) e = OT2D_ERR_IO;
    if (e) return e;
  }
  return OT2D_OK;
}

int read_restart(const std::string& dir, const ot2d_params& p, double* dq, float* dqc, double* totime,
                 int* istep0, cudaStream_t st) {
  if (p.itrans != 0 || p.nv < 4 || (p.iturb == 1 && p.nv < 5) || (p.iturb == 2 && p.nv < 6)) return OT2D_ERR_ARG;
  const size_t n2 = (size_t)p.jd * p.kd, ns = (size_t)p.nspec;
  const bool turb = p.iturb == 1 || p.iturb == 2, ts = p.timespectral != 0;
  const size_t nvin = turb ? (size_t)p.nv : 4;
  std::vector<double> h(ns * nvin * n2);
  double tt = 0.0;
  int32_t i0 = 0;
  for (size_t s = 0; s < ns; ++s) {
    FILE* f = std::fopen(sol_file(dir, ts, (int)s + 1, 'r', p.iturb).c_str(), "rb");
    if (!f) return OT2D_ERR_IO;
    int32_t dims[2] = {0, 0};
    double hdr[4] = {0, 0, 0, 0};
    double* r = h.data() + s * nvin * n2;
    // init.f:157-165: header, restr2 (io.f:400-401), restr_turb (io.f:422), istep0
    int e = rec_read(f, dims, sizeof(dims));
    if (!e && (dims[0] != p.jd || dims[1] != p.kd)) e = OT2D_ERR_IO;
    if (!e) e = rec_read(f, hdr, sizeof(hdr));
    if (!e) e = rec_read(f, r, 4 * n2 * sizeof(double));
    if (!e && turb) e = rec_read(f, r + 4 * n2, (nvin - 4) * n2 * sizeof(double));
    if (!e) e = rec_read(f, &i0, sizeof(i0));
    std::fclose(f);
    if (e) return e;
    tt = hdr[3];
  }
  DevTmp tmp;
  if (cudaMalloc(&tmp.p, h.size() * sizeof(double)) != cudaSuccess) return OT2D_ERR_NOMEM;
  if (cudaMemcpyAsync(tmp.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return OT2D_ERR_CUDA;
  if (io_unpack(tmp.p, dq, dqc, n2, p.nspec, p.nq, (int)nvin, 1, st) != cudaSuccess) return OT2D_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return OT2D_ERR_CUDA;
  if (totime) *totime = tt;
  if (istep0) *istep0 = i0;
  return OT2D_OK;
}

}  // namespace ot2d

using namespace ot2d;

extern "C" {

int ot2d_unit_open(int32_t unit, const char* path, int32_t formatted, int32_t for_write) {
  return unit_open(unit, path, formatted != 0, for_write != 0);
}

int ot2d_unit_close(int32_t unit) { return unit_close(unit); }

int ot2d_unit_write_ints(int32_t unit, const int32_t* v, int32_t n) {
  if (n < 0 || (n && !v)) return OT2D_ERR_ARG;
  Seg sg{v, (size_t)n * 4};
  return rec_write(unit_file(unit, false, true), &sg, 1);
}

int ot2d_unit_read_ints(int32_t unit, int32_t* v, int32_t n) {
  if (n < 0 || (n && !v)) return OT2D_ERR_ARG;
  return rec_read(unit_file(unit, false, false), v, (size_t)n * 4);
}

}  // extern "C"
