/*
 * ot2d_params.h -- plain-old-data mirror of the OVERTURNS-2D module
 * `params_global` fields that the per-iteration hot path reads.
 *
 * Reference: src/modules.f:4-213 (module params_global), filled by
 * read_inputs (src/setup.f:876-1268) and set_pointers_globals
 * (src/setup.f:55-108).  Every hot-path routine of the reference reads these
 * module variables implicitly; the C-ABI takes them explicitly through
 * ot2d_set_params() (or per instance in the batched API).
 *
 * Index conventions are the reference's: 1-based Fortran indices, arrays are
 * column-major q(jd,kd,nspec,nq) with j fastest.  Boundary-condition tables
 * use the reference's `&bcinp` vertex-index convention (negative = counted
 * from the end, converted to halo-cell indices as in src/bc.f:20-33).
 */
#ifndef OT2D_PARAMS_H
#define OT2D_PARAMS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OT2D_MAXBC 25

typedef struct ot2d_params {
  /* ---- sizes (set_pointers_globals, setup.f:55-108) ---- */
  int32_t jmax, kmax;      /* vertex counts                               */
  int32_t jd, kd;          /* cell-array extents incl. halo = jmax+nadd   */
  int32_t nhalo, nadd;     /* nadd = 2*nhalo-1                            */
  int32_t jbeg, jend, kbeg, kend; /* interior cell range                 */
  int32_t jtail1, jtail2, jle, half;
  int32_t nq, nv, nmv, nturb, nspec;
  /* ---- scheme switches (namelist &inputs, modules.f:197-208) ---- */
  int32_t irhsy, ilim, ilhs, iconstant_cfl, idual, idual_turb;
  int32_t iunst, ntac, itnmax, iread;
  int32_t invisc, lamin, iturb, itrans, timespectral, iprecon;
  int32_t motiontype;
  /* ---- iteration counters (Turns_overset.f:360-366, :475) ---- */
  int32_t istep, istep0, itn, npnorm;
  /* ---- flow constants (read_inputs, setup.f:1160-1204) ---- */
  double gamma, gm1, ggm1, pr, rey, tinf, rmue;
  double fsmach, fmtip, alfa;
  double rinf, uinf, vinf, einf, pinf, htinf, ainf;
  double vnuinf, tkeinf, tomegainf;
  double epse, dt, h, timeac, dualtime, cfltur;
  double rotf, rf, angmax, xac, yac, Mp, totime, theta_col;
  /* ---- boundary-condition table (&bcinp, setup.f:899-931) ---- */
  int32_t nbc, pad0;
  int32_t ibtyp[OT2D_MAXBC], ibdir[OT2D_MAXBC];
  int32_t jbcs[OT2D_MAXBC], jbce[OT2D_MAXBC];
  int32_t kbcs[OT2D_MAXBC], kbce[OT2D_MAXBC];
} ot2d_params;

/* Namelist-level inputs from which the derived constants are computed.
 * Mirrors the subset of `&inputs` (modules.f:197-208) the hot path needs. */
typedef struct ot2d_inputs {
  int32_t jmax, kmax, nhalo, jtail1, half;
  int32_t invisc, lamin, iturb, itrans;
  int32_t irhsy, ilim, ilhs, iconstant_cfl, idual, idual_turb;
  int32_t iunst, ntac, itnmax, iread;
  int32_t timespectral, nspec, motiontype, npnorm;
  double fsmach, fmtip, alfa, rey, vnuinf, tuinf;
  double dt, timeac, epse, cfltur;
  double rf, angmax, xac, yac;
  /* boundary conditions */
  int32_t nbc, pad0;
  int32_t ibtyp[OT2D_MAXBC], ibdir[OT2D_MAXBC];
  int32_t jbcs[OT2D_MAXBC], jbce[OT2D_MAXBC];
  int32_t kbcs[OT2D_MAXBC], kbce[OT2D_MAXBC];
} ot2d_inputs;

#ifdef __cplusplus
}
#endif
#endif /* OT2D_PARAMS_H */
