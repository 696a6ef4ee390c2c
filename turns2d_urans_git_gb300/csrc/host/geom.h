// geom.h -- host-side FP64 geometry set-up (see geom.cpp for the reference
// routines each function restates).
#pragma once
#include <cstddef>
#include "ot2d_params.h"

namespace ot2d {

void bc_cells(const ot2d_params& p, int ib, int& js, int& je, int& ks, int& ke);
void cell_centres(const ot2d_params& p, const double* xv, const double* yv, double* x, double* y);
// returns the number of non-positive Jacobians
int metrics(const ot2d_params& p, const double* xv, const double* yv, double* J, double* xx, double* xy, double* yx,
            double* yy);
void wall_distance(const ot2d_params& p, const double* x, const double* y, const double* xv, const double* yv, double* sn);
// dely2 of komegabc_wall (komegasst.f:1000-1007, :1042-1049) on every wall
// halo cell (squared distance from the first interior cell centre to the
// wall face midpoint); 0 elsewhere
void sst_wall_d2(const ot2d_params& p, const double* x, const double* y, const double* xv, const double* yv,
                 double* wd2);
void face_normals(const ot2d_params& p, const double* xv, const double* yv, const double* ugv, const double* vgv,
                  double* fxa, double* fya, double* gxa, double* gya, double* ftj, double* gtj);
// time-accurate face speeds from the areas the faces sweep between the
// vertex levels (eulerrhs.f:118-139, :224-246; second order when ntac = 2
// and istep > 1); ftj / gtj on the xi / eta faces as face_normals indexes them
void face_speeds_swept(const ot2d_params& p, const double* xv, const double* yv, const double* xold,
                       const double* yold, const double* xole, const double* yole, double* ftj, double* gtj);
void ts_pitch_grid(const ot2d_params& p, const double* xv1, const double* yv1, double tspec, double* xv, double* yv);
void ts_grid_speed(const ot2d_params& p, const double* x, const double* y, const double* xv, const double* yv,
                   double tspec, double* ug, double* vg, double* ugv, double* vgv);
void ts_operator(int n, double* Ds);
// freestream Q/J of one time instance; q(:,:,n) at q + (n-1)*qs, J already in q(:,:,nq)
void freestream(const ot2d_params& p, double* q, size_t qs);

}  // namespace ot2d
