/* orc_thermal.c -- oracle (test infrastructure): the per-cell thermal-balance
 * update of 3DPDR.F90:928-1050 and the level-population convergence check of
 * 3DPDR.F90:1084-1229, for a list of cells.
 *
 * The state flags byte of a cell holds converged (1), dobinarychop (2),
 * doleveltmin (4), level_converged (8) and previouschange ("H" 16, "C" 32,
 * neither 0: the reference allocates previouschange without a value,
 * 3DPDR.F90:321).  The cooling total is the left-to-right sum of the
 * coolants' rates (3DPDR.F90:897); heating[cell*hstride] is HEATING_RATE(12). */
#include <math.h>

#include "pdr_oracle.h"

enum { CONV = 1, CHOP = 2, LTMIN = 4, LCONV = 8, HEAT = 16, COOL = 32 };

void orc_thermal_balance(int ncell, double Tmin, double Tmax, double Fcrit, double Tdiff, int temp_fix,
                         int level_conv, int first_time, const double *heating, int hstride, int ncool,
                         const double *const *cooling, double *T, double *Tprev, double *Tlow, double *Thigh,
                         double *Fmean, double *Fratio, double *total_cooling, unsigned char *flags,
                         long long *nconverged) {
  long long nconv = 0;
  for (int c = 0; c < ncell; c++) {
    double cool = 0.0;
    for (int k = 0; k < ncool; k++) cool = k ? cool + cooling[k][c] : cooling[k][c];
    if (total_cooling) total_cooling[c] = cool;
    unsigned f = flags[c];
    if (f & CONV) { nconv++; continue; }            /* :912-913 */
    const double heat = heating[(long long)c * hstride];
    const double fm = heat - cool;                   /* :931-932 */
    Fmean[c] = fm;
    Fratio[c] = 2.0 * fabs(fm) / fabs(heat + cool);
    const double fr = Fratio[c];
    double t = T[c];
    if (level_conv && first_time) {                  /* :936-953 */
      const double dummy = t;
      if (fm == 0) {
        Tlow[c] = t;
        Thigh[c] = t;
      } else if (fm > 0) {
        Tlow[c] = t;
        t = 1.3 * t;
        f = (f & ~(HEAT | COOL)) | HEAT;
      } else if (fm < 0) {
        Thigh[c] = t;
        t = 0.7 * t;
        if (t < Tmin) t = Tmin;
        f = (f & ~(HEAT | COOL)) | COOL;
      }
      Tprev[c] = dummy;
      if (Tprev[c] < Tmin) Tprev[c] = Tmin;
    } else if (level_conv) {                         /* :955-1049 */
      double dummy = t;
      if (fr <= Fcrit) f |= CONV;
      if (!(f & CHOP)) {
        if (fm > 0 && (f & HEAT)) {
          Tlow[c] = t;
          t = 1.3 * t;
          Thigh[c] = t;
        }
        if (fm < 0 && (f & COOL)) {
          Thigh[c] = t;
          t = 0.7 * t;
          Tlow[c] = t;
          if (t < Tmin) {
            t = Tmin;
            Tlow[c] = Tmin;
            Thigh[c] = Tmin;
          }
        }
        if (fm > 0 && (f & COOL)) {
          t = (Thigh[c] + Tlow[c]) / 2.0;
          f |= CHOP;
        }
        if (fm < 0 && (f & HEAT)) {
          t = (Thigh[c] + Tlow[c]) / 2.0;
          f |= CHOP;
        }
      } else {
        if (fm > 0) {
          Tlow[c] = t;
          t = (t + Thigh[c]) / 2.0;
        }
        if (fm < 0) {
          Thigh[c] = t;
          t = (t + Tlow[c]) / 2.0;
        }
      }
      if (temp_fix && fabs(t - Tprev[c]) <= Tdiff && fr > Fcrit) f |= CONV;   /* :1010-1012 */
      Tprev[c] = dummy;
      if (dummy < Tmin && fm < 0) f |= CONV;
      if (dummy > Tmax && fm > 0) f |= CONV;
      if (f & CONV) {
        if (dummy < Tmin) {
          Tprev[c] = Tmin;
          t = Tmin;
          if (!(f & LTMIN)) {
            f &= ~(CONV | LCONV);
            dummy = Tmin;
          }
          f |= LTMIN;
        }
        if (dummy > Tmax) {
          Tprev[c] = Tmax;
          t = Tmax;
        }
      }
    }
    T[c] = t;
    flags[c] = (unsigned char)f;
    if (f & CONV) nconv++;
  }
  if (nconverged) *nconverged = nconv;
}

void orc_level_convergence(int ncell, int ncool, const int *nlev, const double *const *solution,
                           double *const *pop, const double *abundance, int nspec, const int *species,
                           int thermal_balance, unsigned char *flags, unsigned char *coolant_conv,
                           long long *counts) {
  for (int k = 0; k <= ncool; k++) counts[k] = 0;
  for (int c = 0; c < ncell; c++) {
    unsigned conv = 0;
    for (int k = 0; k < ncool; k++) {
      const int n = nlev[k];
      const double *s = solution[k] + (long long)c * n;
      const double *p = pop[k] + (long long)c * n;
      const double floor = abundance[(long long)c * nspec + species[k]] * 1.0e-10;
      int ok = 1;
      for (int l = 0; l < n; l++) {
        if (s[l] >= floor) {                                         /* :1090 */
          double relch;
          if (s[l] == 0.0 && p[l] == 0.0)
            relch = 0.0;
          else
            relch = 2.0 * fabs((s[l] - p[l]) / (s[l] + p[l]));
          if (relch > 1.0e-2) ok = 0;
        }
      }
      if (ok) {
        conv |= 1u << k;
        counts[1 + k]++;
      }
    }
    unsigned f = flags[c] & ~LCONV;                                   /* :1085 */
    if (conv == (1u << ncool) - 1u) {
      f |= LCONV;
      counts[0]++;
    }
    flags[c] = (unsigned char)f;
    if (coolant_conv) coolant_conv[c] = (unsigned char)conv;
  }
  /* :1202-1206: with thermal balance every level_converged is reset once all cells converged */
  if (thermal_balance && counts[0] == ncell)
    for (int c = 0; c < ncell; c++) flags[c] &= (unsigned char)~LCONV;
  /* :1161-1172: without thermal balance, once every cell converged the
   * reference leaves the loop (goto 2) before the population update */
  if (!thermal_balance && counts[0] == ncell) return;
  for (int k = 0; k < ncool; k++)                                    /* :1212-1229 */
    for (long long e = 0; e < (long long)ncell * nlev[k]; e++) pop[k][e] = solution[k][e];
}
