/*
 * orc_heating.c -- oracle: gas heating rates, restating
 * sub_calculate_heating.F90:7-386 (CALC_HEATING and its F/FF helpers).
 * TEST INFRASTRUCTURE ONLY (see pdr_oracle.h).
 *
 * Several constants in the reference are Fortran default-REAL literals
 * (e.g. "0.4*EV", "T**0.068"); they are single-precision values promoted to
 * double, and are written here as (double)x.f so the products agree bit for bit.
 */
#include "pdr_oracle.h"

#include <math.h>

static const double KB_ = 1.38065040e-16, EV_ = 1.60217646e-12;
static const double PI_ = 3.141592653589793238462643383279502884197;
#define R4(x) ((double)(x##f))

void orc_heating(const orc_net *net, int network, const orc_phys *ph, double density, double Tg,
                 double Td, double uv_field, const double *ab, const double *rate, const int *nr,
                 double *out) {
  const double n = density, T = Tg;
  const double Z = ph->metallicity;
  const double xe = ab[net->ielect];
  const double habing = 1.68 * uv_field;
  /* dust photoelectric heating, Tielens & Hollenbach (1985) */
  const double deltad = 1.0, deltauv = 1.8, y = 0.1, hnud = 6.0, hnuh = 13.6;
  const double xk = KB_ * T / (hnuh * EV_);
  const double xd = hnud / hnuh;
  const double gam = 2.9e-4 * y * sqrt(T) * habing / (xe * n);
  double delta = xk - xd + gam;
  double x = 0.5, xx = x;
  for (int it = 1; it <= 100; it++) {
    const double F = (x * x * x) + delta * (x * x) - gam;
    const double FF = 3 * (x * x) + delta * (2 * x);
    xx = x - (F / FF);
    if (fabs(xx - x) < 1.0e-2) break;
    x = xx;
  }
  x = xx;
  const double photoelectric = 2.7e-25 * deltauv * deltad * n * y * habing *
                               (((1.0 - x) * (1.0 - x)) / x + xk * ((x * x) - 1.0) / (x * x)) * Z;
  /* PAH photoelectric heating, Bakes & Tielens (1994) with Wolfire et al. (2003) */
  const double phi_pah = 1.0, alpha = 0.944;
  const double beta = 0.735 / pow(T, R4(0.068));
  delta = habing * sqrt(T) / (xe * n * phi_pah);
  const double eps = 4.87e-2 / (1.0 + 4.0e-3 * pow(delta, R4(0.73))) +
                     3.65e-2 * pow(T / 1.0e4, R4(0.7)) / (1.0 + 2.0e-4 * delta);
  const double pah_heat = 1.30e-24 * eps * habing * n;
  const double pah_cool = 4.65e-30 * pow(T, alpha) * pow(delta, beta) * xe * n * phi_pah * n;
  const double pah = (pah_heat - pah_cool) * Z;
  /* Weingartner & Draine (2001) */
  const double C0 = 5.72e+0, C1 = 3.45e-2, C2 = 7.08e-3, C3 = 1.98e-2, C4 = 4.95e-1, C5 = 6.92e-1, C6 = 5.20e-1;
  const double wd_arg = habing * sqrt(T) / (xe * n);
  const double weingartner = Z * 1.0e-26 * (habing * n) * (C0 + C1 * pow(T, C4)) /
                             (1.0 + C2 * pow(wd_arg, C5) * (1.0 + C3 * pow(wd_arg, C6)));
  const double *R = rate - 1; /* 1-based rate indices below */
  const double cion = (1.0 * EV_) * R[nr[4]] * ab[net->iC] * n;
  const double h2form = (1.5 * EV_) * R[nr[0]] * n * ab[net->iH] * n;
  const double h2phot = (R4(0.4) * EV_) * R[nr[1]] * ab[net->iH2] * n;
  const double ncr = 1.0e6 / sqrt(T) /
                     (1.6 * ab[net->iH] * exp(-((400.0 / T) * (400.0 / T))) +
                      1.4 * ab[net->iH2] * exp(-(18100.0 / (T + 1200.0))));
  const double fuv = (R4(2.2) * EV_) * 9.0 * R[nr[1]] * ab[net->iH2] * n / (1.0 + ncr / n);
  const double cr = (R4(9.4) * EV_) * (1.3e-17 * ph->zeta) * n * ab[net->iH2];
  const double vt = ph->v_turb / 1.0e5;
  const double turb = 3.5e-28 * (vt * vt * vt) * (1.0 / 5.0) * n;
  double chem = 0.0;
  const double *A = ab;
  if (network == 0) {
    chem = A[net->iH2x] * n * xe * R[216] * R4(10.9) * EV_
         + A[net->iH2x] * n * A[net->iH] * R[155] * R4(0.94) * EV_
         + A[net->iHCOx] * n * xe * n * (R[240] * (R4(7.51) * EV_))
         + A[net->iH3x] * n * xe * n * (R[217] * (R4(4.76) * EV_) + R[218] * (R4(9.23) * EV_))
         + A[net->iH3Ox] * n * xe * n * (R[236] * (R4(1.16) * EV_) + R[237] * (R4(5.63) * EV_) + R[238] * (R4(6.27) * EV_))
         + A[net->iHEx] * n * A[net->iH2] * n * (R[50] * (R4(6.51) * EV_) + R[170] * (R4(6.51) * EV_))
         + A[net->iHEx] * n * A[net->iCO] * n * (R[89] * (R4(2.22) * EV_) + R[90] * (R4(2.22) * EV_) + R[91] * (R4(2.22) * EV_));
  } else if (network == 1) {
    chem = A[net->iHCOx] * n * xe * n * (R[730] * (R4(7.51) * EV_))
         + A[net->iH3x] * n * xe * n * (R[706] * (R4(4.76) * EV_) + R[705] * (R4(9.23) * EV_))
         + A[net->iH3Ox] * n * xe * n * (R[717] * (R4(1.16) * EV_) + R[716] * (R4(5.63) * EV_) + R[714] * (R4(6.27) * EV_))
         + A[net->iHEx] * n * A[net->iH2] * n * (R[1227] * (R4(6.51) * EV_) + R[265] * (R4(6.51) * EV_))
         + A[net->iHEx] * n * A[net->iCO] * n * (R[1541] * (R4(2.22) * EV_));
  } else {
    /* mynetwork: the reference STOPs here (sub_calculate_heating.F90:250-253) */
    chem = NAN;
  }
  const double acc = 0.35 * exp(-sqrt((Td + T) / 5.0e2)) + 0.1;
  const double ngrain = 1.998e-12 * n * Z * 100. / ph->g2d;
  const double cgrain = PI_ * (ph->grain_radius * ph->grain_radius);
  const double gasgrain = 4.003e-12 * n * ngrain * cgrain * acc * sqrt(T) * (Td - T);
  const double total = +pah + cion + h2form + h2phot + fuv + cr + turb + chem + gasgrain;
  out[0] = photoelectric; out[1] = pah; out[2] = weingartner; out[3] = cion; out[4] = h2form;
  out[5] = h2phot; out[6] = fuv; out[7] = cr; out[8] = turb; out[9] = chem; out[10] = gasgrain;
  out[11] = total;
}
