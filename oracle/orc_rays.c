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

/* escape_probability.F90:57-106: the optical depth of every radiative line of
 * a coolant along every ray, from the populations pop[gridpoint*nlev + level]
 * of the grid points at the evaluation points; tau[(c*nlin + l)*nrays + j]. */
void orc_tau(const orc_coolant *cl, int ncell, int nrays, const int *epray, const long long *offset, const double *xyz,
             const int *gp, const double *pop, const double *T, double v_turb, double *tau) {
  const double KB = 1.38065040e-16, MP = 1.67262164e-24, C = 2.99792458e+10;
  const double PI = 3.141592653589793238462643383279502884197;
  const int nlev = cl->nlev;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ncell; c++) {
    const double frac2 = 1.0 / sqrt(8.0 * KB * T[c] / PI / MP + v_turb * v_turb);
    for (int l = 0; l < cl->nlin; l++) {
      const int il = cl->line_up[l], jl = cl->line_lo[l];
      const double f = cl->freq[il * nlev + jl];
      const double frac1 = (cl->A[il * nlev + jl] * (C * C * C)) / (8.0 * PI * (f * f * f));
      const double wi = cl->weights[il], wj = cl->weights[jl];
      for (int j = 0; j < nrays; j++) {
        const long long cj = (long long)c * nrays + j;
        double t = 0.0;
        for (int i = 1; i <= epray[cj]; i++) {
          const long long p = offset[cj] + i;
          const double *pa = pop + (long long)gp[p - 1] * nlev, *pb = pop + (long long)gp[p] * nlev;
          const double frac3 = ((pa[jl] * wi - pa[il] * wj) + (pb[jl] * wi - pb[il] * wj)) / 2. / wj;
          const double rhs2 = step_length(xyz, p);
          t = t + frac1 * frac2 * frac3 * rhs2 * PC_;
        }
        tau[((long long)c * cl->nlin + l) * nrays + j] = t;
      }
    }
  }
}
