/* CPU FP64 oracle (test infrastructure only): the overset interpolation
 * do_interpolations of src/connectivity.f:2-190, restated loop by loop.
 *
 * Donor values: for donor id of mesh im, the 9-point quadratic Lagrange
 * stencil around cell (ii,jj) with offsets fracg(id,1:2) (weights
 * connectivity.f:89-97) applied to q*J for the mean-flow variables and to q
 * for the turbulence variables (:101-125), gathered into qbc at row
 * iisptr-1+id.  Fringe cells: q(ii,jj,n) = qbc(ibcg(id),n)/J (mean flow) or
 * qbc (turbulence) (:154-167).  All donors are gathered before any fringe
 * cell is written (:43-130 then :134-185). */
#include <cstdint>
#include <vector>

#include "ot2d_params.h"

namespace {

using P = ot2d_params;

inline int64_t ix3(int64_t a, int64_t b, int64_t c, int64_t na, int64_t nb) { return a + na * (b + nb * c); }

}  // namespace

extern "C" {

/* Arguments as the reference's (connectivity.f:2-3), 1-based index values,
 * Fortran column-major arrays:
 *   imeshg, idonorg (idsize, 2, nmesh, nspec), ibcg (idsize, nmesh, nspec),
 *   fracg (idsize, 2, nmesh, nspec), nfringeg, ndonorg, iisptrg, iieptrg
 *   (nmesh, nspec), jmx, kmx (nmesh); params nspec, nq, nv, nmv. */
void oro_do_interpolations(const P* p, double* qg, const int32_t* jmx, const int32_t* kmx, const int32_t* ibcg,
                           const int32_t* imeshg, const int32_t* idonorg, const double* fracg,
                           const int32_t* nfringeg, const int32_t* ndonorg, const int32_t* iisptrg,
                           const int32_t* iieptrg, int32_t idsize, int64_t qsize, int32_t nmesh) {
  (void)qsize;
  const int nspec = p->nspec, nq = p->nq, nv = p->nv, nmv = p->nmv;
  const double onefourth = 1. / 4;
  for (int nsp = 1; nsp <= nspec; ++nsp) {
    const int bcdim = iieptrg[ix3(nmesh - 1, nsp - 1, 0, nmesh, nspec)];
    std::vector<double> qbc((size_t)bcdim * nv);
    auto QBC = [&](int row, int n) -> double& { return qbc[(size_t)(n - 1) * bcdim + (row - 1)]; };
    int64_t qptr = 1;
    for (int im = 1; im <= nmesh; ++im) {
      const int ndonor = ndonorg[(nsp - 1) * nmesh + (im - 1)];
      const int iisptr = iisptrg[(nsp - 1) * nmesh + (im - 1)];
      const int jm = jmx[im - 1], km = kmx[im - 1];
      auto q = [&](int j, int k, int n) -> double {
        return qg[qptr - 1 + (int64_t)jm * km * nspec * (n - 1) + (int64_t)jm * km * (nsp - 1) + (int64_t)jm * (k - 1) +
                  j - 1];
      };
      for (int id = 1; id <= ndonor; ++id) {
        auto dn = [&](int c) { return idonorg[(((int64_t)(nsp - 1) * nmesh + (im - 1)) * 2 + (c - 1)) * idsize + (id - 1)]; };
        auto fr = [&](int c) { return fracg[(((int64_t)(nsp - 1) * nmesh + (im - 1)) * 2 + (c - 1)) * idsize + (id - 1)]; };
        const int ii = dn(1), jj = dn(2);
        const int iim = ii - 1, jjm = jj - 1, iip = ii + 1, jjp = jj + 1;
        const double djm1 = 1. + fr(1), dkm1 = 1. + fr(2);
        const double dj0 = fr(1), dk0 = fr(2);
        const double djp1 = 1. - fr(1), dkp1 = 1. - fr(2);
        const double w1 = (dj0 * djp1 * dk0 * dkp1) * onefourth;
        const double w2 = -(2 * (djm1 * djp1 * dk0 * dkp1) * onefourth);
        const double w3 = -((djm1 * dj0 * dk0 * dkp1) * onefourth);
        const double w4 = -(2 * (dj0 * djp1 * dkm1 * dkp1) * onefourth);
        const double w5 = 4 * (djm1 * djp1 * dkm1 * dkp1) * onefourth;
        const double w6 = 2 * (djm1 * dj0 * dkm1 * dkp1) * onefourth;
        const double w7 = -((dj0 * djp1 * dkm1 * dk0) * onefourth);
        const double w8 = 2 * (djm1 * djp1 * dkm1 * dk0) * onefourth;
        const double w9 = (djm1 * dj0 * dkm1 * dk0) * onefourth;
        for (int n = 1; n <= nmv; ++n)
          QBC(iisptr - 1 + id, n) = w1 * q(iim, jjm, n) * q(iim, jjm, nq) + w2 * q(ii, jjm, n) * q(ii, jjm, nq) +
                                    w3 * q(iip, jjm, n) * q(iip, jjm, nq) + w4 * q(iim, jj, n) * q(iim, jj, nq) +
                                    w5 * q(ii, jj, n) * q(ii, jj, nq) + w6 * q(iip, jj, n) * q(iip, jj, nq) +
                                    w7 * q(iim, jjp, n) * q(iim, jjp, nq) + w8 * q(ii, jjp, n) * q(ii, jjp, nq) +
                                    w9 * q(iip, jjp, n) * q(iip, jjp, nq);
        for (int n = nmv + 1; n <= nv; ++n)
          QBC(iisptr - 1 + id, n) = w1 * q(iim, jjm, n) + w2 * q(ii, jjm, n) + w3 * q(iip, jjm, n) +
                                    w4 * q(iim, jj, n) + w5 * q(ii, jj, n) + w6 * q(iip, jj, n) +
                                    w7 * q(iim, jjp, n) + w8 * q(ii, jjp, n) + w9 * q(iip, jjp, n);
      }
      qptr += (int64_t)jm * km * nspec * nq;
    }
    qptr = 1;
    for (int im = 1; im <= nmesh; ++im) {
      const int nfringe = nfringeg[(nsp - 1) * nmesh + (im - 1)];
      const int jm = jmx[im - 1], km = kmx[im - 1];
      auto qa = [&](int j, int k, int n) -> double& {
        return qg[qptr - 1 + (int64_t)jm * km * nspec * (n - 1) + (int64_t)jm * km * (nsp - 1) + (int64_t)jm * (k - 1) +
                  j - 1];
      };
      for (int id = 1; id <= nfringe; ++id) {
        const int64_t base = ((int64_t)(nsp - 1) * nmesh + (im - 1));
        const int j = ibcg[base * idsize + (id - 1)];
        const int ii = imeshg[(base * 2 + 0) * idsize + (id - 1)];
        const int jj = imeshg[(base * 2 + 1) * idsize + (id - 1)];
        for (int n = 1; n <= nmv; ++n) qa(ii, jj, n) = QBC(j, n) / qa(ii, jj, nq);
        for (int n = nmv + 1; n <= nv; ++n) qa(ii, jj, n) = QBC(j, n);
      }
      qptr += (int64_t)jm * km * nspec * nq;
    }
  }
}

}  /* extern "C" */
