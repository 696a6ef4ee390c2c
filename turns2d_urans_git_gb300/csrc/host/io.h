// io.h -- solution / restart files in the record layout of the reference's
// src/io.f (astore, store, storevnu, storekomega, grid, restr2, restr_turb)
// and init.f (qdivj).
//
// Files are Fortran sequential unformatted files as gfortran and ifort write
// them for records below 2 GiB: every record is a 4-byte little-endian byte
// count, the payload, and the byte count again.  Reals are 8-byte (the
// reference is compiled with -r8), integers 4-byte.  Formatted (Tecplot)
// files follow the reference's edit descriptors: '(3F22.13)' for reals,
// '(3I10)' for iblank, list-directed lines as gfortran lays them out.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "ot2d.h"

namespace ot2d {

// ---- unit table (Fortran unit numbers -> open files) ------------------------
// open(unit=u, file=path, form=...) with status 'unknown' for writing (the
// file is created or truncated) and 'old' for reading.
int unit_open(int unit, const char* path, bool formatted, bool for_write);
int unit_close(int unit);
// the open file of `unit` with the given form and direction, or nullptr
FILE* unit_file(int unit, bool formatted, bool for_write);

// ---- records ----------------------------------------------------------------
struct Seg { const void* p; size_t n; };
// one unformatted record made of the segments in order
int rec_write(FILE* f, const Seg* segs, int nseg);
// read the first `bytes` bytes of the next record into dst and skip the rest
// of it (a Fortran READ of fewer items than the record holds).  OT2D_ERR_IO
// if the record is shorter than `bytes` or the file ends.
int rec_read(FILE* f, void* dst, size_t bytes);

// ---- formatted (Tecplot) lines ---------------------------------------------
// '(3F22.13)': three values per line, the last line with the remainder
int tec_reals(FILE* f, const double* v, size_t n);
// '(3I10)'
int tec_ints(FILE* f, const int32_t* v, size_t n);
// list-directed header lines of storevnu / storekomega (io.f:100-101,
// :136-138) and the zone lines (io.f:199-201)
int tec_title(FILE* f, int iturb);
int tec_zone(FILE* f, int jd, int kd);

// file names of astore (io.f:39-53, :87-95, :123-131) for time instance
// nsp (1-based) in directory dir ("" = current directory); kind 'g' grid
// (unit 9), 'q' solution (unit 8), 'r' restart input (unit 3), 't' turbulence
std::string sol_file(const std::string& dir, bool ts, int nsp, char kind, int iturb);

// ---- device snapshot / restore ---------------------------------------------
// For every cell of every time instance of q (jd*kd*nspec cells per
// variable, nq variables, J in variable nq):
//  mode IO_REC (store, io.f:296-301, :315-320, :332):
//   rec[s][n]   = q(n)*J        n = 1..4
//   rec[s][n]   = q(n)          n = 5..nv
//   q(n)        = rec[s][n]/J   n = 1..4      (the qdivj after the write)
//   qc(n)       = (float)q(n)   compute copy of the mixed path (nullable)
//  mode IO_TEC (storekomega, io.f:241-246, :261-262; nv >= 6):
//   tec[s][0,1] = q(5)/rho, q(6)/rho with rho = q(1)*J, q(1) taken after
//                 the round trip when IO_REC is set too
// rec is [nspec][nv][n2] doubles, tec [nspec][2][n2].
enum { IO_REC = 1, IO_TEC = 2 };
cudaError_t io_pack(double* q, float* qc, double* rec, double* tec, size_t n2, int nspec, int nq, int nv, int mode,
                    cudaStream_t st);
// the inverse: q(n) = rec[s][n] / J for n = 1..4 (divj) or as read (!divj),
// q(n) = rec[s][n] for n = 5..nvin; qc refreshed.  rec may alias q when
// nspec == 1 and nvin <= nq (the in-place qdivj of init.f:180-206).
cudaError_t io_unpack(const double* rec, double* q, float* qc, size_t n2, int nspec, int nq, int nvin, int divj,
                      cudaStream_t st);

// ---- the store / restore of a whole solve ------------------------------------
// Host side of astore for one mesh held on the device: writes the solution
// file (header, per-instance records, istep0), the grid file of cell centres
// and, for SA / SST, the Tecplot turbulence file, into `dir`.  `dq` and
// `dqc` are the device state (FP64 master and the nullable compute copy);
// x, y are host cell centres [nspec][n2], iblank host [nspec][n2].
int write_solution(const std::string& dir, const ot2d_params& p, double* dq, float* dqc, const double* x,
                   const double* y, const int32_t* iblank, int istep0, cudaStream_t st);
// init.f:138-170 for one mesh: reads <dir>/fort.3 (or fort_TS<n>.3), the
// mesh-size header, restr2 and (SA/SST) restr_turb records and istep0, and
// restores q on the device (Q/J).  totime and istep0 of the file are
// returned.
int read_restart(const std::string& dir, const ot2d_params& p, double* dq, float* dqc, double* totime,
                 int* istep0, cudaStream_t st);

}  // namespace ot2d
