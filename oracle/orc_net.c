/*
 * orc_net.c -- oracle: network loader, generated-RHS semantics, Jacobian.
 * TEST INFRASTRUCTURE ONLY (see pdr_oracle.h).
 *
 * Loader: read_species.F90:15-194 and read_rates.F90:9-95 (CSV, list-directed
 * null fields keep their blank/zero initial values, duplicate detection and
 * RTMIN(I)=RTMAX(I-1) adjustment at read_rates.F90:61-74).
 * RHS: the form/loss structure MakeRates writes into odes_<net>.c:26-149
 * (ode[i] = form + x[i]*loss, x_e = sum of charged species, odes_reduced.c:44).
 */
#include "pdr_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static void trim(char *s) {
  size_t n = strlen(s);
  while (n && (s[n - 1] == ' ' || s[n - 1] == '\r' || s[n - 1] == '\n' || s[n - 1] == '\t')) s[--n] = 0;
  size_t k = 0;
  while (s[k] == ' ' || s[k] == '\t') k++;
  if (k) memmove(s, s + k, n - k + 1);
}

/* split a CSV record into at most maxf fields (no quoting with commas in these files) */
static int split_csv(char *line, char **f, int maxf) {
  int nf = 0;
  char *p = line;
  while (nf < maxf) {
    f[nf++] = p;
    char *c = strchr(p, ',');
    if (!c) break;
    *c = 0;
    p = c + 1;
  }
  for (int i = 0; i < nf; i++) trim(f[i]);
  return nf;
}

static int count_charge(const char *name) {
  if (strcmp(name, "e-") == 0 || strcmp(name, "ELECTR") == 0) return -1;
  int q = 0;
  for (const char *p = name; *p; p++) {
    if (*p == '+') q++;
    else if (*p == '-') q--;
  }
  return q;
}

static int is_blank(const char *s) { return s[0] == 0; }

orc_net *orc_net_load(const char *species_path, const char *rates_path, char *err, int errlen) {
  FILE *fs = fopen(species_path, "r");
  if (!fs) { snprintf(err, errlen, "cannot open %s", species_path); return NULL; }
  char line[4096];
  int nspec = 0;
  while (fgets(line, sizeof line, fs)) { char t[4096]; strcpy(t, line); trim(t); if (t[0]) nspec++; }
  rewind(fs);
  orc_net *net = (orc_net *)calloc(1, sizeof(orc_net));
  net->nspec = nspec;
  net->neq = nspec - 1;
  net->spec = calloc(nspec, sizeof *net->spec);
  net->abund0 = calloc(nspec, sizeof(double));
  net->mass = calloc(nspec, sizeof(double));
  net->charge = calloc(nspec, sizeof(int));
  int i = 0;
  while (i < nspec && fgets(line, sizeof line, fs)) {
    char *f[8];
    char t[4096]; strcpy(t, line); trim(t);
    if (!t[0]) continue;
    int nf = split_csv(line, f, 8);
    if (nf < 4) { snprintf(err, errlen, "bad species record %d", i + 1); fclose(fs); orc_net_free(net); return NULL; }
    strncpy(net->spec[i], f[1], ORC_NAME - 1);
    net->abund0[i] = atof(f[2]);
    net->mass[i] = atof(f[3]);
    net->charge[i] = count_charge(f[1]);
    i++;
  }
  fclose(fs);

  /* species labels, read_species.F90:89-148 (upper-case aliases included) */
  int *labs[] = {&net->iH, &net->iH2, &net->iHD, &net->iCO, &net->iC, &net->iS, &net->iCx, &net->iO,
                 &net->iHe, &net->iHx, &net->iHEx, &net->iH2x, &net->iH3x, &net->iH3Ox, &net->iHCOx, &net->ielect};
  for (size_t k = 0; k < sizeof labs / sizeof labs[0]; k++) *labs[k] = -1;
  for (i = 0; i < nspec; i++) {
    const char *s = net->spec[i];
    if (!strcmp(s, "H")) net->iH = i;
    if (!strcmp(s, "H2")) net->iH2 = i;
    if (!strcmp(s, "HD")) net->iHD = i;
    if (!strcmp(s, "CO")) net->iCO = i;
    if (!strcmp(s, "C")) net->iC = i;
    if (!strcmp(s, "S")) net->iS = i;
    if (!strcmp(s, "C+")) net->iCx = i;
    if (!strcmp(s, "O")) net->iO = i;
    if (!strcmp(s, "He") || !strcmp(s, "HE")) net->iHe = i;
    if (!strcmp(s, "H+")) net->iHx = i;
    if (!strcmp(s, "He+") || !strcmp(s, "HE+")) net->iHEx = i;
    if (!strcmp(s, "H2+")) net->iH2x = i;
    if (!strcmp(s, "H3+")) net->iH3x = i;
    if (!strcmp(s, "H3O+")) net->iH3Ox = i;
    if (!strcmp(s, "HCO+")) net->iHCOx = i;
    if (!strcmp(s, "e-") || !strcmp(s, "ELECTR")) net->ielect = i;
  }
  if (net->ielect != nspec - 1) {
    snprintf(err, errlen, "electron must be the last species (calculate_abundances.c:67)");
    orc_net_free(net);
    return NULL;
  }

  FILE *fr = fopen(rates_path, "r");
  if (!fr) { snprintf(err, errlen, "cannot open %s", rates_path); orc_net_free(net); return NULL; }
  int nreac = 0;
  while (fgets(line, sizeof line, fr)) { char t[4096]; strcpy(t, line); trim(t); if (t[0]) nreac++; }
  rewind(fr);
  net->nreac = nreac;
  net->reac = calloc(nreac, sizeof *net->reac);
  net->prod = calloc(nreac, sizeof *net->prod);
  net->alpha = calloc(nreac, sizeof(double));
  net->beta = calloc(nreac, sizeof(double));
  net->gamma = calloc(nreac, sizeof(double));
  net->rtmin = calloc(nreac, sizeof(double));
  net->rtmax = calloc(nreac, sizeof(double));
  net->duplicate = calloc(nreac, sizeof(int));
  net->ode_kind = calloc(nreac, sizeof(int));
  net->rate_kind = calloc(nreac, sizeof(int));
  net->ri = calloc(nreac, sizeof *net->ri);
  net->pi = calloc(nreac, sizeof *net->pi);
  int r = 0;
  while (r < nreac && fgets(line, sizeof line, fr)) {
    char t[4096]; strcpy(t, line); trim(t);
    if (!t[0]) continue;
    char *f[32];
    int nf = split_csv(line, f, 32);
    if (nf < 14) { snprintf(err, errlen, "bad rate record %d", r + 1); fclose(fr); orc_net_free(net); return NULL; }
    for (int k = 0; k < 3; k++) strncpy(net->reac[r][k], f[1 + k], ORC_NAME - 1);
    for (int k = 0; k < 4; k++) strncpy(net->prod[r][k], f[4 + k], ORC_NAME - 1);
    net->alpha[r] = is_blank(f[8]) ? 0.0 : atof(f[8]);
    net->beta[r] = is_blank(f[9]) ? 0.0 : atof(f[9]);
    net->gamma[r] = is_blank(f[10]) ? 0.0 : atof(f[10]);
    net->rtmin[r] = is_blank(f[12]) ? 0.0 : atof(f[12]);
    net->rtmax[r] = is_blank(f[13]) ? 0.0 : atof(f[13]);
    /* read_rates.F90:61-74 */
    if (r > 0) {
      int same = 1;
      for (int k = 0; k < 3; k++) same &= !strcmp(net->reac[r][k], net->reac[r - 1][k]);
      for (int k = 0; k < 4; k++) same &= !strcmp(net->prod[r][k], net->prod[r - 1][k]);
      if (same) {
        if (net->duplicate[r - 1] == 0) net->duplicate[r - 1] = 1;
        net->duplicate[r] = net->duplicate[r - 1] + 1;
        net->rtmin[r] = net->rtmax[r - 1];
      } else {
        net->duplicate[r] = 0;
      }
    }
    r++;
  }
  fclose(fr);
  if (r != nreac) { snprintf(err, errlen, "rate count mismatch"); orc_net_free(net); return NULL; }

  /* classification for the ODE and the rate evaluator */
  for (r = 0; r < nreac; r++) {
    char (*R)[ORC_NAME] = net->reac[r];
    char (*P)[ORC_NAME] = net->prod[r];
    int idx[3] = {-1, -1, -1};
    for (int k = 0; k < 3; k++)
      for (i = 0; i < nspec; i++)
        if (!strcmp(R[k], net->spec[i])) { idx[k] = i; break; }
    for (int k = 0; k < 4; k++) {
      net->pi[r][k] = -1;
      for (i = 0; i < nspec; i++)
        if (!strcmp(P[k], net->spec[i])) { net->pi[r][k] = i; break; }
    }
    const char *r2 = R[1];
    int xray = !strcmp(r2, "XRAY") || !strcmp(r2, "XRSEC") || !strcmp(r2, "XRLYA") || !strcmp(r2, "XRPHOT");
    int uni = !strcmp(r2, "PHOTON") || !strcmp(r2, "CRP") || !strcmp(r2, "CRPHOT") || is_blank(r2) ||
              !strcmp(r2, "FREEZE") || !strcmp(r2, "ELFRZE") || !strcmp(r2, "CRH") ||
              !strcmp(r2, "PHOTD") || !strcmp(r2, "THERM") || r2[0] == '#';
    net->ri[r][0] = idx[0];
    net->ri[r][1] = -1;
    if (xray) net->ode_kind[r] = ORC_R_XRAY;
    else if (!strcmp(R[2], "#")) net->ode_kind[r] = ORC_R_GRAINH2;
    else if (uni) net->ode_kind[r] = ORC_R_UNI;
    else { net->ode_kind[r] = ORC_R_BI; net->ri[r][1] = idx[1]; }
    if (idx[0] < 0 || (net->ode_kind[r] == ORC_R_BI && idx[1] < 0)) {
      snprintf(err, errlen, "reaction %d: unknown reactant", r + 1);
      orc_net_free(net);
      return NULL;
    }

    /* calc_reac_rates.F90:53-66 dispatch, then the thermal/photo sub-cases */
    int k;
    if (!strcmp(r2, "PHOTON")) {
      if (!strcmp(R[0], "H2") && is_blank(R[2])) k = ORC_K_PHOTO_H2;
      else if (!strcmp(R[0], "HD") && is_blank(R[2])) k = ORC_K_PHOTO_HD;
      else {
        int anyC = 0, anyO = 0;
        for (int q = 0; q < 4; q++) { anyC |= !strcmp(P[q], "C"); anyO |= !strcmp(P[q], "O"); }
        if (!strcmp(R[0], "CO") && is_blank(R[2]) && anyC && anyO) k = ORC_K_PHOTO_CO;
        else if (!strcmp(R[0], "C") && is_blank(R[2]) &&
                 ((!strcmp(P[0], "C+") && !strcmp(P[1], "e-")) || (!strcmp(P[0], "e-") && !strcmp(P[1], "C+"))))
          k = ORC_K_PHOTO_CI;
        else if (!strcmp(R[0], "S") && is_blank(R[2]) &&
                 ((!strcmp(P[0], "S+") && !strcmp(P[1], "e-")) || (!strcmp(P[0], "e-") && !strcmp(P[1], "S+"))))
          k = ORC_K_PHOTO_SI;
        else k = ORC_K_PHOTO;
      }
    } else if (!strcmp(r2, "CRP")) k = ORC_K_CRP;
    else if (!strcmp(r2, "CRPHOT")) k = ORC_K_CRPHOT;
    else if (!strcmp(r2, "FREEZE")) k = ORC_K_FREEZE;
    else if (!strcmp(r2, "ELFRZE")) k = ORC_K_ELFRZE;
    else if (!strcmp(r2, "CRH")) k = ORC_K_CRH;
    else if (!strcmp(r2, "PHOTD")) k = ORC_K_PHOTD;
    else if (!strcmp(r2, "THERM")) k = ORC_K_THERM;
    else if (r2[0] == '#') k = ORC_K_GRAIN;
    else if (xray) k = ORC_K_XRAY;
    else {
      int h2f = !strcmp(R[0], "H") && !strcmp(R[1], "H") && (is_blank(R[2]) || !strcmp(R[2], "#")) &&
                !strcmp(P[0], "H2") && (is_blank(P[1]) || !strcmp(P[1], "#"));
      int pah = 0;
      for (int q = 0; q < 3; q++)
        pah |= !strcmp(R[q], "PAH") || !strcmp(R[q], "PAH0") || !strcmp(R[q], "PAH+") || !strcmp(R[q], "PAH-");
      k = h2f ? ORC_K_H2FORM : (pah ? ORC_K_PAH : ORC_K_THERMAL);
    }
    net->rate_kind[r] = k;
  }
  return net;
}

/* Slot layout of the reference's generated network code (data/layout_<net>.d,
 * records "slot,species_file_name,generated_code_name,xe_coefficient").  The
 * generated f() addresses species by slot and sums x_e over fixed slots
 * (odes_<net>.c:44); the Fortran caller fills the slots in species-file order.
 * Re-resolving the reaction participants through the generated-code names
 * makes the oracle integrate the same system the reference integrates.
 * Species labels (iH, iH2x, ...) keep their species-file meaning, as the
 * Fortran side (heating, level populations) indexes by file position. */
int orc_net_load_layout(orc_net *net, const char *path, char *err, int errlen) {
  FILE *f = fopen(path, "r");
  if (!f) { snprintf(err, errlen, "cannot open %s", path); return 1; }
  char (*gname)[ORC_NAME] = calloc(net->nspec, sizeof *gname);
  int *coef = calloc(net->nspec, sizeof(int));
  int nrec = 0;
  char line[512];
  while (fgets(line, sizeof line, f)) {
    char *fl[5];
    char t[512]; strcpy(t, line); trim(t);
    if (!t[0]) continue;
    if (split_csv(line, fl, 5) < 4) { snprintf(err, errlen, "bad layout record"); goto bad; }
    int s = atoi(fl[0]) - 1;
    if (s < 0 || s >= net->neq || strcmp(fl[1], net->spec[s])) {
      snprintf(err, errlen, "layout record %s does not match the species list", fl[0]);
      goto bad;
    }
    strncpy(gname[s], fl[2], ORC_NAME - 1);
    coef[s] = atoi(fl[3]);
    nrec++;
  }
  fclose(f);
  if (nrec != net->neq) { snprintf(err, errlen, "layout has %d slots, expected %d", nrec, net->neq); free(gname); free(coef); return 1; }
  strncpy(gname[net->neq], net->spec[net->neq], ORC_NAME - 1);
  for (int r = 0; r < net->nreac; r++) {
    for (int k = 0; k < 2; k++) {
      if (net->ri[r][k] < 0) continue;
      const char *nm = net->reac[r][k];
      for (int i = 0; i < net->nspec; i++) if (!strcmp(nm, gname[i])) { net->ri[r][k] = i; break; }
    }
    for (int k = 0; k < 4; k++) {
      if (net->pi[r][k] < 0) continue;
      const char *nm = net->prod[r][k];
      for (int i = 0; i < net->nspec; i++) if (!strcmp(nm, gname[i])) { net->pi[r][k] = i; break; }
    }
  }
  for (int i = 0; i < net->neq; i++) net->charge[i] = coef[i];
  free(gname);
  free(coef);
  return 0;
bad:
  fclose(f);
  free(gname);
  free(coef);
  return 1;
}

void orc_net_free(orc_net *net) {
  if (!net) return;
  free(net->spec); free(net->abund0); free(net->mass); free(net->charge);
  free(net->reac); free(net->prod); free(net->alpha); free(net->beta); free(net->gamma);
  free(net->rtmin); free(net->rtmax); free(net->duplicate); free(net->ode_kind);
  free(net->rate_kind); free(net->ri); free(net->pi);
  free(net);
}

/* electron abundance by charge conservation (odes_reduced.c:44, odes_full.c:44) */
static double xe_of(const orc_net *net, const double *x) {
  double xe = 0.0;
  for (int i = 0; i < net->neq; i++)
    if (net->charge[i]) xe += (double)net->charge[i] * x[i];
  return xe;
}

void orc_rhs(const orc_net *net, const double *rate, double n_H, const double *x, double *ode,
             double *x_e_out) {
  const int neq = net->neq;
  double form[1024], loss[1024];
  if (neq > 1024) return;
  double x_e = xe_of(net, x);
  for (int i = 0; i < neq; i++) form[i] = loss[i] = 0.0;
  for (int r = 0; r < net->nreac; r++) {
    const int kind = net->ode_kind[r];
    if (kind == ORC_R_XRAY) continue;
    const double k = rate[r];
    const int a = net->ri[r][0];
    double flux;
    if (kind == ORC_R_UNI) {
      flux = k * x[a];
      loss[a] -= k;
    } else if (kind == ORC_R_GRAINH2) {
      flux = k * x[a] * n_H;
      loss[a] -= 2.0 * k * n_H;
    } else {
      const int b = net->ri[r][1];
      const double xa = (a == neq) ? x_e : x[a];
      const double xb = (b == neq) ? x_e : x[b];
      flux = k * xa * xb * n_H;
      if (a == b) {
        if (a != neq) loss[a] -= 2.0 * k * xa * n_H;
      } else {
        if (a != neq) loss[a] -= k * xb * n_H;
        if (b != neq) loss[b] -= k * xa * n_H;
      }
    }
    /* products with multiplicity (MakeRates writes "m*rate[..]*...") */
    for (int q = 0; q < 4; q++) {
      const int p = net->pi[r][q];
      if (p < 0 || p == neq) continue;
      int seen = 0;
      for (int qq = 0; qq < q; qq++) seen |= (net->pi[r][qq] == p);
      if (seen) continue;
      int m = 0;
      for (int qq = q; qq < 4; qq++) m += (net->pi[r][qq] == p);
      form[p] += (m == 1) ? flux : (double)m * flux;
    }
  }
  for (int i = 0; i < neq; i++) ode[i] = form[i] + x[i] * loss[i];
  if (x_e_out) *x_e_out = x_e;
}

/* d(flux)/d(reactant slot) for one reaction; de = d flux / d x_e */
static void jac_reaction(const orc_net *net, int r, const double *rate, double n_H, const double *x,
                         double x_e, double *J, int chain) {
  const int neq = net->neq;
  const int kind = net->ode_kind[r];
  if (kind == ORC_R_XRAY) return;
  const double k = rate[r];
  const int a = net->ri[r][0];
  int sp[2] = {-1, -1};
  double d[2] = {0.0, 0.0};
  int ns = 0;
  if (kind == ORC_R_UNI) {
    sp[0] = a; d[0] = k; ns = 1;
  } else if (kind == ORC_R_GRAINH2) {
    sp[0] = a; d[0] = k * n_H; ns = 1;
  } else {
    const int b = net->ri[r][1];
    const double xa = (a == neq) ? x_e : x[a];
    const double xb = (b == neq) ? x_e : x[b];
    if (a == b) { sp[0] = a; d[0] = 2.0 * k * xa * n_H; ns = 1; }
    else { sp[0] = a; d[0] = k * xb * n_H; sp[1] = b; d[1] = k * xa * n_H; ns = 2; }
  }
  /* net stoichiometry per species touched by this reaction */
  int touched[8], nt = 0;
  double nu[8];
  for (int q = 0; q < 4; q++) {
    int p = net->pi[r][q];
    if (p < 0 || p == neq) continue;
    int f = -1;
    for (int t = 0; t < nt; t++) if (touched[t] == p) f = t;
    if (f < 0) { touched[nt] = p; nu[nt] = 0.0; f = nt++; }
    nu[f] += 1.0;
  }
  {
    int reacts[2] = {a, (kind == ORC_R_BI) ? net->ri[r][1] : (kind == ORC_R_GRAINH2 ? a : -1)};
    for (int q = 0; q < 2; q++) {
      int p = reacts[q];
      if (p < 0 || p == neq) continue;
      int f = -1;
      for (int t = 0; t < nt; t++) if (touched[t] == p) f = t;
      if (f < 0) { touched[nt] = p; nu[nt] = 0.0; f = nt++; }
      nu[f] -= 1.0;
    }
  }
  for (int s = 0; s < ns; s++) {
    if (sp[s] == neq) {
      if (!chain) continue;
      /* chain rule through x_e = sum_j charge_j x_j */
      for (int j = 0; j < neq; j++) {
        if (!net->charge[j]) continue;
        const double dj = d[s] * (double)net->charge[j];
        for (int t = 0; t < nt; t++) J[touched[t] * neq + j] += nu[t] * dj;
      }
    } else {
      for (int t = 0; t < nt; t++) J[touched[t] * neq + sp[s]] += nu[t] * d[s];
    }
  }
}

void orc_jac(const orc_net *net, const double *rate, double n_H, const double *x, double *J) {
  const int neq = net->neq;
  memset(J, 0, sizeof(double) * neq * neq);
  double x_e = xe_of(net, x);
  for (int r = 0; r < net->nreac; r++) jac_reaction(net, r, rate, n_H, x, x_e, J, 1);
}

void orc_jac_xe_const(const orc_net *net, const double *rate, double n_H, const double *x,
                      double x_e, double *J) {
  const int neq = net->neq;
  memset(J, 0, sizeof(double) * neq * neq);
  for (int r = 0; r < net->nreac; r++) jac_reaction(net, r, rate, n_H, x, x_e, J, 0);
}
