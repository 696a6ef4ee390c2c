/*
 * oracle.h -- TEST INFRASTRUCTURE ONLY (see oracle_common.h).
 * Internal declarations of the FP64 restatement of the OVERTURNS-2D routines.
 * Each function cites the reference routine it restates.
 */
#ifndef OT2D_ORACLE_H
#define OT2D_ORACLE_H
#include "oracle_common.h"

namespace oro {

/* setup.f:876-1268 (derived constants) + setup.f:55-108 + init.f:59-66 */
void read_inputs(const ot2d_inputs& in, P& p);
/* setup.f:111-345 */
void find_cellcenter(const P& p, A2 x, A2 y, const double* xv, const double* yv);
/* setup.f:440-724; returns number of non-positive Jacobians */
int metfv(const P& p, A3 q, const double* xv, const double* yv, A2 xx, A2 xy, A2 yx, A2 yy);
/* init.f:209-277, init.f:180-206 */
void qzero(const P& p, A3 q);
void qdivj(const P& p, A3 q);
/* setup.f:838-873 */
void computeTScoefs(int N, double* Ds);
/* setup.f:396-438 and setup.f:789-835 (sine pitching form) */
void find_coord_TS_orig(const P& p, double* xv, double* yv, const double* xv1, const double* yv1, double tspec);
void find_timemetrics_TS_orig(const P& p, A2 x, A2 y, const double* xv, const double* yv, double tspec,
                              A2 ug, A2 vg, double* ugv, double* vgv);

/* bc.f:2-85 */
void bc(const P& p, A3 q, A2 x, A2 y, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 bt);
/* bc.f:88-177 */
void rbc(const P& p, A3 q, A3 s);

/* eulerrhs.f:2-280 (nei=1, iprecon=.false.); xold..yole: the vertices of
 * the two previous time levels, needed when iunst > 0 (face speeds from the
 * swept areas, eulerrhs.f:118-140, :224-246) */
void rhsup(const P& p, A3 q, A3 s, const double* xv, const double* yv, I2 iblank,
           const double* ugv, const double* vgv, const double* xold = nullptr, const double* yold = nullptr,
           const double* xole = nullptr, const double* yole = nullptr);
/* motion.f:546-632 (pitch, motiontype 1): rotates the cell centres and the
 * vertices by the step's pitch increment about (xac, yac), sets the cell
 * grid speeds, shifts the two previous vertex levels */
void pitch(const P& p, A2 x, A2 y, double* xv, double* yv, double* xold, double* yold, double* xole, double* yole,
           A2 ug, A2 vg);
/* time.f:110-175 (all nspec instances; qtn, qtnm1, qnewt: (jd,kd,nspec,nv)) */
void stqol(const P& p, const double* q, double* qtn, double* qtnm1, double* qnewt);
/* time.f:178-210 for one instance: s -= (q - qnewt)/(oat*h) on the interior */
void newton(const P& p, A3 q, const double* qnewt, A3 s);
void newtonTS(const P& p, A3 q, const double* qnewt, A3 ss, A2 tscale);
/* visrhs.f:2-287 */
void visrhs(const P& p, A2 turmu, A3 q, A3 s, A2 xx, A2 xy, A2 yx, A2 yy);
/* time.f:2-108 (one time instance) */
void time_step(const P& p, A3 q, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 tscale, A2 bt, I2 iblank);
/* lhs.f:470-814 */
void ilu2d(const P& p, A3 q, A3 s, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 turmu, A2 tscale);
/* lhs.f:2-467 (Turkel-preconditioned LU-SGS) and sources.f:97-148 */
void preilu2d(const P& p, A3 q, A3 s, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 turmu, A2 tscale, A2 bt);
void rhslom(const P& p, A3 q, A3 s, A2 bt);
/* lhs.f:817-1057 (ilhs = 2: lhsinv + pentadag) */
void arc2d(const P& p, A3 q, A3 s, A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 turmu, I2 iblank, A2 tscale, A2 bt,
           bool pre = false);
/* samodel2d.f:200-240 */
void lamvis(const P& p, A3 q, A2 vmul);
/* samodel2d.f:243-293 */
void dist(const P& p, A2 sn, A2 x, A2 y, const double* xv, const double* yv);
/* komegasst.f:2-187 (no transition model); res_out (optional) = {restke, restomega} */
void komegasst(const P& p, A3 q, A3 s, A2 turmu, A2 x, A2 y, const double* xv, const double* yv,
               A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 tscale, I2 iblank, double* res_out);
/* samodel2d.f:2-197 */
void vmu_sa(const P& p, A3 q, A3 s, A2 turmu, A2 x, A2 y, const double* xv, const double* yv,
            A2 xx, A2 xy, A2 yx, A2 yy, A2 ug, A2 vg, A2 tscale, I2 iblank, double* resl2_out);
/* sources.f:2-27 */
void timespectralrhs(const P& p, const double* q, double* s, const double* Ds, int nsp);
/* step.f:332-392 (one instance); returns number of bad cells */
int monitor(const P& p, A3 q);
/* forces.f:130-398; out = {cfx, cfy, cm0, cpower} */
void force2d(const P& p, A3 q, A2 x, A2 y, const double* xv, const double* yv,
             A2 xx, A2 xy, A2 yx, A2 yy, double* out);

}  // namespace oro
#endif
