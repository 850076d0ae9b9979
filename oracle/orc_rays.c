/* orc_rays.c -- oracle (test infrastructure): column densities and the UV
 * field along the rays, restating CALC_UVFIELD (3DPDR.F90:1636-1701) and
 * calc_columndens (3DPDR.F90:1789-1844) for a list of cells.
 *
 * The evaluation points of cell c's ray j are offset[c*nrays+j] + i,
 * i = 0..epray[c*nrays+j], with coordinates xyz[3*point] and the projected
 * grid point gp[point] (pdr%epoint and pdr%projected; point 0 is the cell).
 * Expressions keep the Fortran evaluation order; PC is healpix_types.F90:98,
 * AV_fac and UV_fac the default-REAL literals of input_parameters.F90:57-58. */
#include <math.h>

#include "pdr_oracle.h"

static const double PC_ = 3.08568025e+18;

static double step_length(const double *xyz, long long p) {
  const double dx = xyz[3 * (p - 1)] - xyz[3 * p];
  const double dy = xyz[3 * (p - 1) + 1] - xyz[3 * p + 1];
  const double dz = xyz[3 * (p - 1) + 2] - xyz[3 * p + 2];
  return sqrt(dx * dx + dy * dy + dz * dz);
}

void orc_uvfield(int ncell, int nrays, const int *epray, const long long *offset, const double *xyz, const int *gp,
                 const double *rho, int field, const double *G, const double *vectors, double metallicity,
                 double *colden, double *AV, double *rad, double *uv) {
  const double av_fac = (double)6.289e-22f * metallicity, uv_fac = (double)3.02f;
  /* UNI: the ray with the largest -G.v, last one on ties (3DPDR.F90:1672-1683) */
  int jj_min = -1;
  double maxdot = 0.0;
  if (field == 1)
    for (int jj = 0; jj < nrays; jj++) {
      const double aux = -(G[0] * vectors[3 * jj] + G[1] * vectors[3 * jj + 1] + G[2] * vectors[3 * jj + 2]);
      if (aux >= maxdot) { maxdot = aux; jj_min = jj; }
    }
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ncell; c++) {
    for (int j = 0; j < nrays; j++) {
      const long long cj = (long long)c * nrays + j;
      double col = 0.0;
      if (epray[cj] > 0)
        for (int i = 1; i <= epray[cj]; i++) {
          const long long p = offset[cj] + i;
          const double step = step_length(xyz, p);
          col = col + ((rho[gp[p - 1]] + rho[gp[p]]) / 2.) * step * PC_;
        }
      colden[cj] = col;
      AV[cj] = col * av_fac;
      rad[cj] = 0.0;
      if (field == 0) rad[cj] = G[0] / (double)nrays;
      if (field == 1 && j == jj_min) rad[cj] = -(G[0] * vectors[3 * j] + G[1] * vectors[3 * j + 1] + G[2] * vectors[3 * j + 2]);
    }
    double u = 0.0;
    for (int j = 0; j < nrays; j++) {
      const long long cj = (long long)c * nrays + j;
      u = u + rad[cj] * exp(-AV[cj] * uv_fac);
      if (u < 1.0e-50) u = 0.0;
    }
    uv[c] = u;
  }
}

void orc_columns(int ncell, int nrays, const int *epray, const long long *offset, const double *xyz, const int *gp,
                 const double *rho, const double *ab, int nspec, const int *species, int nsel, double *out) {
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ncell; c++)
    for (int j = 0; j < nrays; j++) {
      const long long cj = (long long)c * nrays + j;
      double *o = out + cj * nsel;
      for (int s = 0; s < nsel; s++) o[s] = 0.0;
      if (epray[cj] == 0) continue;
      for (int i = 1; i <= epray[cj]; i++) {
        const long long p = offset[cj] + i;
        const double step = step_length(xyz, p);
        const int a = gp[p - 1], b = gp[p];
        for (int s = 0; s < nsel; s++) {
          const int k = species ? species[s] : s;
          o[s] = o[s] + step * PC_ * (rho[a] * ab[(long long)a * nspec + k] + rho[b] * ab[(long long)b * nspec + k]) / 2.;
        }
      }
    }
}
