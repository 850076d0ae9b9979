/*
 * orc_rates.c -- oracle: reaction-rate coefficients and self-shielding.
 * TEST INFRASTRUCTURE ONLY (see pdr_oracle.h).
 *
 * Restates calc_reac_rates.F90:16-401 (branch order, duplicate-reaction
 * temperature ranges, clamps), shield.F90 (H2PDRATE :27, COPDRATE :83,
 * CIPDRATE :132, SIPDRATE :180, H2SHIELD1 :231, COSHIELD :375, SCATTER :449,
 * XLAMBDA :525, LBAR :570), spline.F90 (SPLIE2 :11, SPLINE :65, SPLIN2 :128,
 * SPLINT :182) and h2_form.F90:8-113.
 *
 * The shielding tables are the published data the reference embeds:
 * Savage & Mathis (1979) tau(lambda)/tau(V) (modules.F90:354-366) and the
 * van Dishoeck & Black (1988) 12CO shielding grid (modules.F90:346-351,
 * 3DPDR.F90:1532-1537).
 */
#include "pdr_oracle.h"

#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const double PI_ = 3.141592653589793238462643383279502884197;
static const double KB_ = 1.38065040e-16, AU_ = 1.66053878e-24;

/* --- Savage & Mathis (1979) extinction curve, 30 points --- */
static const double L_GRID[30] = {910.0, 950.0, 1000.0, 1050.0, 1110.0, 1180.0, 1250.0, 1390.0,
                                  1490.0, 1600.0, 1700.0, 1800.0, 1900.0, 2000.0, 2100.0, 2190.0,
                                  2300.0, 2400.0, 2500.0, 2740.0, 3440.0, 4000.0, 4400.0, 5500.0,
                                  7000.0, 9000.0, 12500.0, 22000.0, 34000.0, 1.0e9};
static const double X_GRID[30] = {5.76, 5.18, 4.65, 4.16, 3.73, 3.40, 3.11, 2.74, 2.63, 2.62,
                                  2.54, 2.50, 2.58, 2.78, 3.01, 3.12, 2.86, 2.58, 2.35, 2.00,
                                  1.58, 1.42, 1.32, 1.00, 0.75, 0.48, 0.28, 0.12, 0.05, 0.00};
/* --- van Dishoeck & Black (1988) log10 12CO shielding: [iNCO][iNH2] --- */
static const double NCO_GRID[8] = {12.0, 13.0, 14.0, 15.0, 16.0, 17.0, 18.0, 19.0};
static const double NH2_GRID[6] = {18.0, 19.0, 20.0, 21.0, 22.0, 23.0};
static const double SCO_COLS[6][8] = {
    {0.000e+00, -1.408e-02, -1.099e-01, -4.400e-01, -1.154e+00, -1.888e+00, -2.760e+00, -4.001e+00},
    {-8.539e-02, -1.015e-01, -2.104e-01, -5.608e-01, -1.272e+00, -1.973e+00, -2.818e+00, -4.055e+00},
    {-1.451e-01, -1.612e-01, -2.708e-01, -6.273e-01, -1.355e+00, -2.057e+00, -2.902e+00, -4.122e+00},
    {-4.559e-01, -4.666e-01, -5.432e-01, -8.665e-01, -1.602e+00, -2.303e+00, -3.146e+00, -4.421e+00},
    {-1.303e+00, -1.312e+00, -1.367e+00, -1.676e+00, -2.305e+00, -3.034e+00, -3.758e+00, -5.077e+00},
    {-3.883e+00, -3.888e+00, -3.936e+00, -4.197e+00, -4.739e+00, -5.165e+00, -5.441e+00, -6.446e+00}};

/* Numerical-Recipes cubic spline second derivatives (spline.F90:65-125) */
void orc_spline(const double *x, const double *y, int n, double yp1, double ypn, double *y2) {
  double u[64];
  if (yp1 >= 1.0e30) { y2[0] = 0.0; u[0] = 0.0; }
  else { y2[0] = -0.5; u[0] = (3.0 / (x[1] - x[0])) * ((y[1] - y[0]) / (x[1] - x[0]) - yp1); }
  for (int i = 1; i < n - 1; i++) {
    const double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    const double p = sig * y2[i - 1] + 2.0;
    y2[i] = (sig - 1.0) / p;
    u[i] = (6.0 * ((y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1])) /
                (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
  }
  double qn, un;
  if (ypn >= 1.0e30) { qn = 0.0; un = 0.0; }
  else { qn = 0.5; un = (3.0 / (x[n - 1] - x[n - 2])) * (ypn - (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2])); }
  y2[n - 1] = (un - qn * u[n - 2]) / (qn * y2[n - 2] + 1.0);
  for (int i = n - 2; i >= 0; i--) y2[i] = y2[i] * y2[i + 1] + u[i];
}

/* spline evaluation with the bisection bracket of spline.F90:182-277 */
double orc_splint(const double *xa, const double *ya, const double *y2a, int n, double x) {
  const int ascnd = xa[n - 1] > xa[0];
  int jlo = 0, jhi = n + 1; /* 1-based bracket */
  while (jhi - jlo != 1) {
    const int jmid = (jhi + jlo) / 2;
    if ((x > xa[jmid - 1]) == ascnd) jlo = jmid;
    else jhi = jmid;
  }
  if (jlo == 0) { jlo = 1; jhi = 2; }
  if (jlo == n) { jlo = n - 1; jhi = n; }
  const double h = xa[jhi - 1] - xa[jlo - 1];
  const double A = (xa[jhi - 1] - x) / h, B = (x - xa[jlo - 1]) / h;
  return A * ya[jlo - 1] + B * ya[jhi - 1] +
         ((A * A * A - A) * y2a[jlo - 1] + (B * B * B - B) * y2a[jhi - 1]) * (h * h) / 6.0;
}

static double X_DERIV[30], SCO_DERIV[8][6];
static int tables_ready = 0;

static void init_tables(void) {
  if (tables_ready) return;
  orc_spline(L_GRID, X_GRID, 30, 1.0e30, 1.0e30, X_DERIV);
  /* SPLIE2: natural splines of the rows SCO(iNCO, :) over the NH2 grid */
  for (int i = 0; i < 8; i++) {
    double row[6], y2[6];
    for (int j = 0; j < 6; j++) row[j] = SCO_COLS[j][i];
    orc_spline(NH2_GRID, row, 6, 1.0e30, 1.0e30, y2);
    for (int j = 0; j < 6; j++) SCO_DERIV[i][j] = y2[j];
  }
  tables_ready = 1;
}

double orc_xlambda(double lambda, int xlambda_linear) {
  init_tables();
  static const double zero[30] = {0};
  if (lambda < L_GRID[0]) lambda = L_GRID[0];
  if (lambda > L_GRID[29]) lambda = L_GRID[29];
  return orc_splint(L_GRID, X_GRID, xlambda_linear ? zero : X_DERIV, 30, lambda);
}

double orc_scatter(double av, double lambda, int xlambda_linear) {
  static const double A[6] = {1.000, 2.006, -1.438, 0.7364, -0.5076, -0.0592};
  static const double K[6] = {0.7514, 0.8490, 1.013, 1.282, 2.005, 5.832};
  const double tauv = av / 1.086;
  const double taul = tauv * orc_xlambda(lambda, xlambda_linear);
  double s = 0.0;
  if (taul < 1.0) {
    const double e = K[0] * taul;
    if (e < 100.0) s = A[0] * exp(-e);
  } else {
    for (int i = 1; i <= 5; i++) {
      const double e = K[i] * taul;
      if (e < 100.0) s = s + A[i] * exp(-e);
    }
  }
  return s;
}

double orc_h2shield1(double nh2, double dopw, double radw) {
  const double fpara = 0.5, fosc = 1.0e-2;
  const double taud = nh2 * fpara * (1.497358985e-2) * fosc / dopw;
  double jd, jr;
  if (taud == 0.0) jd = 1.0;
  else if (taud < 2.0) jd = exp(-(0.666666667 * taud));
  else if (taud < 10.0) jd = 0.638 * pow(taud, -1.25);
  else if (taud < 100.0) jd = 0.505 * pow(taud, -1.15);
  else jd = 0.344 * pow(taud, -1.0667);
  if (radw == 0.0) jr = 0.0;
  else {
    const double r = radw / (1.772453851 * dopw);
    const double t = 3.02 * pow(r * 1.0e3, -0.064);
    const double u = sqrt(taud * r) / t;
    jr = r / (t * sqrt(0.785398163 + u * u));
  }
  return jd + jr;
}

double orc_coshield(double nco, double nh2) {
  init_tables();
  double lognco = log10(nco + 1.0), lognh2 = log10(nh2 + 1.0);
  if (lognco < NCO_GRID[0]) lognco = NCO_GRID[0];
  if (lognh2 < NH2_GRID[0]) lognh2 = NH2_GRID[0];
  if (lognco > NCO_GRID[7]) lognco = NCO_GRID[7];
  if (lognh2 > NH2_GRID[5]) lognh2 = NH2_GRID[5];
  /* SPLIN2: row splines in NH2, then a column spline in NCO */
  double yy[8], yy2[8];
  for (int i = 0; i < 8; i++) {
    double row[6];
    for (int j = 0; j < 6; j++) row[j] = SCO_COLS[j][i];
    yy[i] = orc_splint(NH2_GRID, row, SCO_DERIV[i], 6, lognh2);
  }
  orc_spline(NCO_GRID, yy, 8, 1.0e30, 1.0e30, yy2);
  const double v = orc_splint(NCO_GRID, yy, yy2, 8, lognco);
  return pow(10.0, v);
}

double orc_lbar(double nco, double nh2) {
  const double u = log10(nco + 1.0), w = log10(nh2 + 1.0);
  double l = (5675.0 - 200.6 * w) - (571.6 - 24.09 * w) * u + (18.22 - 0.7664 * w) * (u * u);
  if (l < 913.6) l = 913.6;
  if (l > 1076.1) l = 1076.1;
  return l;
}

double orc_h2_formation_rate(double Tg, double Td, double metallicity, double g2d) {
  const double thermal_velocity = 1.45e5 * sqrt(Tg / 1.0e2);
  const double tt = Tg / 1.0e2;
  const double sticking = 1.0 / (1.0 + 0.04 * sqrt(Tg + Td) + 0.2 * tt + 0.08 * (tt * tt));
  const double flux = 1.0e-10;
  const double sil_cs = 8.473e-22, gra_cs = 7.908e-22;
  double eff[2];
  const double mu = 0.005, nu_h2 = 3.0e12, nu_hc = 1.3e13;
  const double es[2] = {110.0, 260.0}, eh2[2] = {320.0, 520.0}, ehp[2] = {450.0, 800.0}, ehc = 3.0e4;
  for (int g = 0; g < 2; g++) {
    const double f1 = mu * flux / (2 * nu_h2 * exp(-eh2[g] / Td));
    const double sq = 1.0 + sqrt((ehc - es[g]) / (ehp[g] - es[g]));
    const double f2 = 1.0 * (sq * sq) / 4.0 * exp(-es[g] / Td);
    const double eps = 1.0 / (1.0 + nu_hc / (2 * flux) * exp(-1.5 * ehc / Td) * (sq * sq));
    eff[g] = 1.0 / (1.0 + f1 + f2) * eps;
  }
  return 0.5 * thermal_velocity * (sil_cs * eff[0] + gra_cs * eff[1]) * sticking * metallicity * 100. / g2d;
}

static double arrhenius(const orc_net *net, int j, double T) {
  if (net->gamma[j] < -200.0 && T < net->rtmin[j]) return 0.0;
  return net->alpha[j] * pow(T / 300.0, net->beta[j]) * exp(-(net->gamma[j] / T));
}

/* duplicate-group selection shared by the thermal/photo/CR branches
 * (calc_reac_rates.F90:117-145): the first member whose RTMAX >= T, or the
 * last member, gets the rate; earlier members get 0. */
static int dup_pick(const orc_net *net, int i, double T, double *rate) {
  int j = i;
  for (;;) {
    if (T <= net->rtmax[j]) return j;
    if (j + 1 >= net->nreac || net->duplicate[j + 1] < net->duplicate[j]) return j;
    rate[j] = 0.0;
    j++;
  }
}

int orc_rates_cell(const orc_net *net, const orc_phys *ph, double T, double Td, int nrays,
                   const double *rad_surface, const double *AV, const double *col,
                   double *rate, int *nr) {
  const int nreac = net->nreac;
  int status = 0;
  for (int i = 0; i < nreac; i++) rate[i] = 0.0;
  for (int k = 0; k < 6; k++) nr[k] = 0;
  const double dopw = ph->v_turb / (1000.0 * 1.0e-8), radw = 8.0e7;
  for (int i = 0; i < nreac; i++) {
    const int kind = net->rate_kind[i];
    const double a = net->alpha[i], b = net->beta[i], g = net->gamma[i];
    switch (kind) {
      case ORC_K_H2FORM:
        rate[i] = ph->h2form ? orc_h2_formation_rate(T, Td, ph->metallicity, ph->g2d) : 3.0e-18 * sqrt(T);
        nr[0] = i + 1;
        break;
      case ORC_K_PAH:
        rate[i] = a * pow(T / 100.0, b) * 0.4;
        break;
      case ORC_K_THERMAL:
        if (net->duplicate[i] == 0) rate[i] = arrhenius(net, i, T);
        else if (net->duplicate[i] == 1) { int j = dup_pick(net, i, T, rate); rate[j] = arrhenius(net, j, T); }
        break;
      case ORC_K_PHOTO_H2:
        for (int k = 0; k < nrays; k++)
          rate[i] = rate[i] + a * rad_surface[k] * orc_h2shield1(col[k * 5 + 0], dopw, radw) *
                                  orc_scatter(AV[k], 1000.0, ph->xlambda_linear) / 2.0;
        if (!strcmp(net->prod[i][0], "H") && !strcmp(net->prod[i][1], "H")) nr[1] = i + 1;
        break;
      case ORC_K_PHOTO_HD:
        for (int k = 0; k < nrays; k++)
          rate[i] = rate[i] + a * rad_surface[k] * orc_h2shield1(col[k * 5 + 1], dopw, radw) *
                                  orc_scatter(AV[k], 1000.0, ph->xlambda_linear) / 2.0;
        {
          int anyH = 0, anyD = 0;
          for (int q = 0; q < 4; q++) { anyH |= !strcmp(net->prod[i][q], "H"); anyD |= !strcmp(net->prod[i][q], "D"); }
          if (anyH && anyD) nr[2] = i + 1;
        }
        break;
      case ORC_K_PHOTO_CO:
        for (int k = 0; k < nrays; k++) {
          const double nco = col[k * 5 + 2], nh2 = col[k * 5 + 0];
          const double lam = orc_lbar(nco, nh2);
          rate[i] = rate[i] + a * rad_surface[k] * orc_coshield(nco, nh2) * orc_scatter(AV[k], lam, ph->xlambda_linear) / 2.0;
        }
        nr[3] = i + 1;
        break;
      case ORC_K_PHOTO_CI:
        for (int k = 0; k < nrays; k++) {
          const double tauc = g * AV[k] + 1.1e-17 * col[k * 5 + 3] +
                              (0.9 * pow(T, 0.27) * pow(col[k * 5 + 0] / 1.59e21, 0.45));
          rate[i] = rate[i] + a * rad_surface[k] * exp(-tauc) / 2.0;
        }
        nr[4] = i + 1;
        break;
      case ORC_K_PHOTO_SI:
        for (int k = 0; k < nrays; k++) rate[i] = rate[i] + a * rad_surface[k] * exp(-(g * AV[k])) / 2.0;
        nr[5] = i + 1;
        break;
      case ORC_K_PHOTO:
        if (net->duplicate[i] == 0) {
          for (int k = 0; k < nrays; k++) rate[i] = rate[i] + a * rad_surface[k] * exp(-(g * AV[k])) / 2.0;
        } else if (net->duplicate[i] == 1) {
          int j = dup_pick(net, i, T, rate);
          for (int k = 0; k < nrays; k++)
            rate[j] = rate[j] + net->alpha[j] * rad_surface[k] * exp(-(net->gamma[j] * AV[k])) / 2.0;
        }
        break;
      case ORC_K_CRP:
        if (net->duplicate[i] == 0) rate[i] = a * ph->zeta;
        else if (net->duplicate[i] == 1) { int j = dup_pick(net, i, T, rate); rate[j] = net->alpha[j] * ph->zeta; }
        break;
      case ORC_K_CRPHOT:
        if (net->duplicate[i] == 0) rate[i] = a * ph->zeta * pow(T / 300.0, b) * g / (1.0 - ph->omega);
        else if (net->duplicate[i] == 1) {
          int j = dup_pick(net, i, T, rate);
          rate[j] = net->alpha[j] * ph->zeta * pow(T / 300.0, net->beta[j]) * net->gamma[j] / (1.0 - ph->omega);
        }
        break;
      case ORC_K_FREEZE:
      case ORC_K_ELFRZE: {
        double cion = (b == 0.0) ? 1.0 : (b == 1.0 ? 1.0 + 16.71e-4 / (ph->grain_radius * T) : 0.0);
        rate[i] = a * 4.57e4 * 2.4e-22 * sqrt(T / g) * cion * 0.3;
        break;
      }
      case ORC_K_CRH:
        rate[i] = 2.06e-3 * ph->zeta * 2.4e-22 * ((g <= 1210.0) ? 1.0e5 : 0.0);
        break;
      case ORC_K_PHOTD: {
        const double y = (T < 50.0) ? 3.5e-3 : (T < 85.0 ? 4.0e-3 : (T < 100.0 ? 5.5e-3 : 7.5e-3));
        for (int k = 0; k < nrays; k++) rate[i] = rate[i] + 1.7e8 * rad_surface[k] * exp(-(1.8 * AV[k])) * 2.4e-22 * y;
        break;
      }
      case ORC_K_THERM:
        rate[i] = sqrt(2.0 * 1.5e15 * KB_ / (PI_ * PI_ * AU_) * a / g) * exp(-(a / Td));
        break;
      case ORC_K_GRAIN:
        rate[i] = a;
        break;
      case ORC_K_XRAY:
        rate[i] = 0.0;
        break;
    }
    /* clamps, calc_reac_rates.F90:387-396 */
    if (rate[i] < 0.0) status = -(i + 1);
    if (rate[i] > 1.0 && net->reac[i][0][0] != 'G') rate[i] = 1.0;
    if (rate[i] < 1.0e-99) rate[i] = 0.0;
  }
  return status;
}

int orc_rates_batched(const orc_net *net, const orc_phys *ph, int ncell, int nrays, const double *T,
                      const double *Td, const double *rad_surface, const double *AV,
                      const double *column5, double *rate, int nthreads) {
  int status = 0;
  init_tables();
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#else
  (void)nthreads;
#endif
  for (int c = 0; c < ncell; c++) {
    int nr[6];
    int s = orc_rates_cell(net, ph, T[c], Td[c], nrays, rad_surface + (size_t)c * nrays,
                           AV + (size_t)c * nrays, column5 + (size_t)c * nrays * 5,
                           rate + (size_t)c * net->nreac, nr);
    if (s) status = s;
  }
  return status;
}
