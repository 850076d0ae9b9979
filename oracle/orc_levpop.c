/*
 * orc_levpop.c -- oracle: LAMDA coolant reader and the per-cell statistical
 * equilibrium step.  TEST INFRASTRUCTURE ONLY (see pdr_oracle.h).
 *
 * Restates read_input.F90:6-258 (record sequence, unit conversions, Einstein
 * B coefficients, detailed-balance reverse collision rates at the table
 * temperatures), find_Ccoeff.F90:1-150, escape_probability.F90:51-167 (the
 * part after the optical depths are known), solvlevpop.F90:1-174 (matrix
 * build with the 1e-8 conservation row and Numerical-Recipes Gauss-Jordan
 * elimination with full pivoting) and the LTE helpers 3DPDR.F90:1848-1898.
 */
#include "pdr_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const double KB_ = 1.38065040e-16, C_ = 2.99792458e+10, HP_ = 6.62606896e-27;
static const double PI_ = 3.141592653589793238462643383279502884197;

static int next_line(FILE *f, char *buf, int n) { return fgets(buf, n, f) != NULL; }

orc_coolant *orc_coolant_load(const char *path, int nlev, int ntemp, char *err, int errlen) {
  FILE *f = fopen(path, "r");
  if (!f) { snprintf(err, errlen, "cannot open %s", path); return NULL; }
  char line[8192];
  orc_coolant *c = (orc_coolant *)calloc(1, sizeof(orc_coolant));
  c->nlev = nlev;
  c->ntemp = ntemp;
  c->energies = calloc(nlev, sizeof(double));
  c->weights = calloc(nlev, sizeof(double));
  c->A = calloc((size_t)nlev * nlev, sizeof(double));
  c->B = calloc((size_t)nlev * nlev, sizeof(double));
  c->freq = calloc((size_t)nlev * nlev, sizeof(double));
  c->temps = calloc((size_t)7 * ntemp, sizeof(double));
  c->col = calloc((size_t)7 * nlev * nlev * ntemp, sizeof(double));
  for (int k = 0; k < 5; k++) next_line(f, line, sizeof line);   /* READ(8,'(////)') */
  next_line(f, line, sizeof line);
  int n = atoi(line);
  if (n != nlev) { snprintf(err, errlen, "incorrect number of energy levels"); goto fail; }
  next_line(f, line, sizeof line);
  n = 0;
  while (n < nlev) {
    if (!next_line(f, line, sizeof line)) goto eof;
    double e, w;
    if (sscanf(line, "%d %lf %lf", &n, &e, &w) != 3) goto eof;
    c->energies[n - 1] = e * C_ * HP_;
    c->weights[n - 1] = w;
  }
  next_line(f, line, sizeof line);
  next_line(f, line, sizeof line);
  c->nlin = atoi(line);
  c->line_up = calloc(c->nlin, sizeof(int));
  c->line_lo = calloc(c->nlin, sizeof(int));
  next_line(f, line, sizeof line);
  n = 0;
  int li = 0;
  while (n < c->nlin) {
    if (!next_line(f, line, sizeof line)) goto eof;
    int i, j;
    double a, fr;
    if (sscanf(line, "%d %d %d %lf %lf", &n, &i, &j, &a, &fr) != 5) goto eof;
    i--; j--;
    c->freq[i * nlev + j] = fr * 1.0e9;
    c->freq[j * nlev + i] = c->freq[i * nlev + j];
    c->A[i * nlev + j] = a;
    const double f3 = c->freq[i * nlev + j];
    c->B[i * nlev + j] = c->A[i * nlev + j] / (2.0 * HP_ * (f3 * f3 * f3) / (C_ * C_));
    c->B[j * nlev + i] = c->B[i * nlev + j] * (c->weights[i] / c->weights[j]);
    c->line_up[li] = i;
    c->line_lo[li] = j;
    li++;
  }
  for (int i = 0; i < nlev; i++)
    for (int j = 0; j < nlev; j++) {
      const double fq = fabs(c->energies[i] - c->energies[j]) / HP_;
      if (c->freq[i * nlev + j] != 0.0) {
        if (fabs(fq - c->freq[i * nlev + j]) / c->freq[i * nlev + j] > 1.0e-2) {
          snprintf(err, errlen, "calculated frequency differs by >1%%");
          goto fail;
        }
      } else {
        c->freq[i * nlev + j] = fq;
      }
    }
  next_line(f, line, sizeof line);
  next_line(f, line, sizeof line);
  const int npart = atoi(line);
  for (int l = 0; l < npart; l++) {
    next_line(f, line, sizeof line);
    next_line(f, line, sizeof line);
    const int p = atoi(line);
    next_line(f, line, sizeof line);
    next_line(f, line, sizeof line);
    const int ncol = atoi(line);
    next_line(f, line, sizeof line);
    next_line(f, line, sizeof line);
    const int m = atoi(line);
    if (m > ntemp) { snprintf(err, errlen, "too many temperature values"); goto fail; }
    if (p < 1 || p > 7) { snprintf(err, errlen, "unrecognized collision partner %d", p); goto fail; }
    next_line(f, line, sizeof line);
    /* temperatures may wrap over several records in list-directed input */
    int got = 0;
    while (got < m) {
      if (!next_line(f, line, sizeof line)) goto eof;
      char *s = line, *e;
      for (;;) {
        double v = strtod(s, &e);
        if (e == s) break;
        if (got < m) c->temps[(p - 1) * ntemp + got++] = v;
        s = e;
      }
    }
    next_line(f, line, sizeof line);
    double *col = c->col + (size_t)(p - 1) * nlev * nlev * ntemp;
    n = 0;
    while (n < ncol) {
      if (!next_line(f, line, sizeof line)) goto eof;
      char *s = line, *e;
      n = (int)strtol(s, &e, 10); s = e;
      int i = (int)strtol(s, &e, 10) - 1; s = e;
      int j = (int)strtol(s, &e, 10) - 1; s = e;
      for (int k = 0; k < m; k++) {
        double v = strtod(s, &e);
        s = e;
        col[((size_t)i * nlev + j) * ntemp + k] = v;
        /* detailed balance Cji = Cij gi/gj exp(-(Ei-Ej)/kT) (read_input.F90:123-126) */
        if (v != 0.0 && col[((size_t)j * nlev + i) * ntemp + k] == 0.0)
          col[((size_t)j * nlev + i) * ntemp + k] =
              v * (c->weights[i] / c->weights[j]) *
              exp(-(c->energies[i] - c->energies[j]) / (KB_ * c->temps[(p - 1) * ntemp + k]));
      }
    }
  }
  fclose(f);
  return c;
eof:
  snprintf(err, errlen, "unexpected end of %s", path);
fail:
  fclose(f);
  orc_coolant_free(c);
  return NULL;
}

void orc_coolant_free(orc_coolant *c) {
  if (!c) return;
  free(c->energies); free(c->weights); free(c->A); free(c->B); free(c->freq);
  free(c->temps); free(c->col); free(c->line_up); free(c->line_lo);
  free(c);
}

/* partner order in the LAMDA ids: 1 H2, 2 p-H2, 3 o-H2, 4 e, 5 H, 6 He, 7 H+ */
void orc_find_ccoeff(const orc_coolant *c, double T, const double *partner, double *C) {
  const int nlev = c->nlev, ntemp = c->ntemp;
  const double n_H = partner[0], n_Hp = partner[1], n_e = partner[2], n_He = partner[3], n_H2 = partner[4];
  for (int i = 0; i < nlev * nlev; i++) C[i] = 0.0;
  double fpara = 0.0, fortho = 0.0;
  if (n_H2 > 0.0) {
    fpara = 1.0 / (1.0 + 9.0 * exp(-170.5 / T));
    fortho = 1.0 - fpara;
  }
  for (int p = 0; p < 7; p++) {
    const double *tp = c->temps + (size_t)p * ntemp;
    if (tp[0] == 0.0) continue;
    int klo = 0, khi = 0; /* 1-based as in find_Ccoeff.F90:49-70 */
    for (int k = 1; k <= ntemp; k++) {
      if (tp[k - 1] > T) { klo = k - 1; khi = k; break; }
      else if (tp[k - 1] == 0.0) { klo = k - 1; khi = k - 1; break; }
    }
    if (khi == 0) { klo = ntemp; khi = ntemp; }
    else if (khi == 1) { klo = 1; khi = 1; }
    const double step = (klo == khi) ? 0.0 : (T - tp[klo - 1]) / (tp[khi - 1] - tp[klo - 1]);
    double w;
    switch (p) {
      case 0: w = n_H2; break;
      case 1: w = n_H2 * fpara; break;
      case 2: w = n_H2 * fortho; break;
      case 3: w = n_e; break;
      case 4: w = n_H; break;
      case 5: w = n_He; break;
      default: w = n_Hp; break;
    }
    const double *col = c->col + (size_t)p * nlev * nlev * ntemp;
    for (int i = 0; i < nlev; i++)
      for (int j = 0; j < nlev; j++) {
        const double lo = col[((size_t)i * nlev + j) * ntemp + klo - 1];
        const double hi = col[((size_t)i * nlev + j) * ntemp + khi - 1];
        const double tmp = lo + (hi - lo) * step;
        if (p == 1) C[i * nlev + j] = C[i * nlev + j] + tmp * n_H2 * fpara;
        else if (p == 2) C[i * nlev + j] = C[i * nlev + j] + tmp * n_H2 * fortho;
        else C[i * nlev + j] = C[i * nlev + j] + tmp * w;
      }
  }
}

void orc_escape_probability(const orc_coolant *c, const double *C, const double *s_pop,
                            const double *tau, int nrays, int pseudo1d, double Tdust,
                            double density, double metallicity, double g2d, double *transition,
                            double *line, double *cooling) {
  const int nlev = c->nlev;
  double field[64 * 64];
  for (int i = 0; i < nlev * nlev; i++) { field[i] = 0.0; line[i] = 0.0; }
  double cool = 0.0;
  /* optical depth of each pair per ray: input for radiative lines, 0 otherwise */
  for (int i = 0; i < nlev; i++) {
    for (int j = 0; j < i; j++) {
      const double f = c->freq[i * nlev + j], A = c->A[i * nlev + j];
      const double tmp2 = 2.0 * HP_ * (f * f * f) / (C_ * C_);
      double bb = tmp2 * (1.0 / (exp(HP_ * f / KB_ / 2.7) - 1.0));
      const double ngrain = 2.0e-12 * density * metallicity * 100. / g2d;
      const double emissivity = (2.0 * ngrain) * ((double)0.01f * ((double)1.3f * f / 3.0e11));
      const double bb_dust = tmp2 * (1.0 / (exp(HP_ * f / KB_ / Tdust) - 1.0) * emissivity);
      bb = bb + bb_dust;
      double S, beta;
      if (s_pop[i] == 0.0) {
        S = 0.0;
        beta = 1.0;
        goto no_line;
      }
      {
        const double tpop = (s_pop[j] * c->weights[i]) / (s_pop[i] * c->weights[j]) - 1.0;
        if (fabs(tpop) < 1.0e-50) {
          S = HP_ * f * s_pop[i] * A / 4. / PI_;
          beta = 1.0;
        } else {
          S = tmp2 / tpop;
          int li = -1;
          for (int q = 0; q < c->nlin; q++)
            if (c->line_up[q] == i && c->line_lo[q] == j) li = q;
          double bsum = 0.0;
          for (int r = 0; r < nrays; r++) {
            double t;
            if (pseudo1d && r != 6) t = 1.0e50;
            else t = (li >= 0) ? tau[li * nrays + r] : 0.0;
            double br;
            if (t < -5.0) br = (1.0 - exp(5.0)) / (-5.0);
            else if (fabs(t) < 1.0e-8) br = 1.0;
            else br = (1.0 - exp(-t)) / t;
            bsum += br;
          }
          beta = pseudo1d ? bsum : bsum / (double)nrays;
        }
      }
      line[i * nlev + j] = A * HP_ * f * s_pop[i] * beta * (S - bb) / S;
      cool = cool + line[i * nlev + j];
    no_line:
      field[i * nlev + j] = (1.0 - beta) * S + beta * bb;
      field[j * nlev + i] = field[i * nlev + j];
    }
  }
  for (int i = 0; i < nlev; i++)
    for (int j = 0; j < nlev; j++) {
      double t = c->A[i * nlev + j] + c->B[i * nlev + j] * field[i * nlev + j] + C[i * nlev + j];
      if (fabs(t) < 1.0e-50) t = 0.0;
      transition[i * nlev + j] = t;
    }
  *cooling = cool;
}

/* Numerical Recipes gaussj with full pivoting, one right-hand side
 * (solvlevpop.F90:65-174).  Returns 0, or 1 on a singular matrix. */
int orc_gauss_jordan(double *a, int n, double *b) {
  int ipiv[128], indxr[128], indxc[128];
  int irow = 0, icol = 0;
  for (int j = 0; j < n; j++) ipiv[j] = 0;
  for (int i = 0; i < n; i++) {
    double big = 0.0;
    for (int j = 0; j < n; j++) {
      if (ipiv[j] != 1) {
        for (int k = 0; k < n; k++) {
          if (ipiv[k] == 0) {
            if (fabs(a[j * n + k]) >= big) { big = fabs(a[j * n + k]); irow = j; icol = k; }
          } else if (ipiv[k] > 1) {
            return 1;
          }
        }
      }
    }
    ipiv[icol]++;
    if (irow != icol) {
      for (int l = 0; l < n; l++) { double d = a[irow * n + l]; a[irow * n + l] = a[icol * n + l]; a[icol * n + l] = d; }
      double d = b[irow]; b[irow] = b[icol]; b[icol] = d;
    }
    indxr[i] = irow;
    indxc[i] = icol;
    if (a[icol * n + icol] == 0.0) return 1;
    const double pivinv = 1.0 / a[icol * n + icol];
    a[icol * n + icol] = 1.0;
    for (int l = 0; l < n; l++) a[icol * n + l] = a[icol * n + l] * pivinv;
    b[icol] = b[icol] * pivinv;
    for (int ll = 0; ll < n; ll++) {
      if (ll != icol) {
        const double dum = a[ll * n + icol];
        a[ll * n + icol] = 0.0;
        for (int l = 0; l < n; l++) a[ll * n + l] = a[ll * n + l] - a[icol * n + l] * dum;
        b[ll] = b[ll] - b[icol] * dum;
      }
    }
  }
  for (int l = n - 1; l >= 0; l--)
    if (indxr[l] != indxc[l])
      for (int k = 0; k < n; k++) {
        double d = a[k * n + indxr[l]]; a[k * n + indxr[l]] = a[k * n + indxc[l]]; a[k * n + indxc[l]] = d;
      }
  return 0;
}

int orc_solvlevpop(int nlev, const double *transition, double density, double *solution) {
  double a[128 * 128];
  for (int i = 0; i < nlev; i++) {
    double out = 0.0;
    for (int j = 0; j < nlev; j++) {
      out = out + transition[i * nlev + j];
      a[i * nlev + j] = transition[j * nlev + i];
    }
    a[i * nlev + i] = -out;
  }
  for (int i = 0; i < nlev; i++) {
    solution[i] = 0.0;
    a[(nlev - 1) * nlev + i] = 1.0e-8;
  }
  solution[nlev - 1] = density * 1.0e-8;
  int s = orc_gauss_jordan(a, nlev, solution);
  for (int i = 0; i < nlev; i++)
    if (solution[i] < 0.0) solution[i] = 0.0;
  return s;
}

void orc_lte(const orc_coolant *c, double T, double density, double *pop) {
  double z = 0.0;
  for (int i = 0; i < c->nlev; i++) z = z + c->weights[i] * exp(-c->energies[i] / KB_ / T);
  for (int i = 0; i < c->nlev; i++) pop[i] = density * c->weights[i] * exp(-c->energies[i] / KB_ / T) / z;
}

int orc_levpop_batched(const orc_coolant *c, int ncell, const double *density, const double *T,
                       const double *Tdust, const double *partner5, const double *coolant_density,
                       const double *s_pop, const double *tau, int nrays, int pseudo1d,
                       double metallicity, double g2d, double *pop_out, double *cooling_out,
                       double *line_out, int nthreads) {
  const int nlev = c->nlev, nl = c->nlin;
  int status = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#else
  (void)nthreads;
#endif
  for (int cell = 0; cell < ncell; cell++) {
    double C[64 * 64], R[64 * 64], L[64 * 64];
    orc_find_ccoeff(c, T[cell], partner5 + (size_t)cell * 5, C);
    orc_escape_probability(c, C, s_pop + (size_t)cell * nlev, tau + (size_t)cell * nl * nrays, nrays,
                           pseudo1d, Tdust[cell], density[cell], metallicity, g2d, R, L,
                           cooling_out + cell);
    int s = orc_solvlevpop(nlev, R, coolant_density[cell], pop_out + (size_t)cell * nlev);
    if (s) status = 1;
    if (line_out) memcpy(line_out + (size_t)cell * nlev * nlev, L, sizeof(double) * nlev * nlev);
  }
  return status;
}
