/*
 * pdr_oracle.h -- CPU FP64 restatement of the 3D-PDR per-cell physics.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle for the
 * GPU path: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it.  The product (lib3dpdr_gb300.so) never links or calls it.
 *
 * Parity status: the RHS and network semantics are pinned against the
 * reference's own generated network code (odes_<net>.c compiled from the
 * reference sources into oracle/_ref).  The BDF integrator restates the
 * published SUNDIALS CVODE 2.5.0 method (the reference's missing third-party
 * dependency, .MISSING_LARGE_BLOBS:1); parity against real CVODE is UNPINNED
 * (no CVODE source or binary exists here) and is instead cross-checked against
 * high-accuracy SciPy solves.
 *
 * Reference files restated (paths within the 3D-PDR project):
 *   read_species.F90:15-194, read_rates.F90:9-95      network loaders
 *   odes_<net>.c (generated f())                       RHS semantics
 *   calculate_abundances.c:64-354                      driver (tout ladder, clamps, x_e quirk)
 *   calc_reac_rates.F90:16-401, shield.F90, spline.F90, h2_form.F90   rates
 *   read_input.F90:6-258, find_Ccoeff.F90, escape_probability.F90,
 *   solvlevpop.F90, 3DPDR.F90:1848-1898                level populations
 *   sub_calculate_heating.F90:7-386                    heating
 */
#ifndef PDR_ORACLE_H
#define PDR_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_NAME 16
#define ORC_NRAYS_MAX 64

/* reaction kinds as they enter the ODE right-hand side */
enum { ORC_R_UNI = 0,      /* flux = k x_a                        */
       ORC_R_BI = 1,       /* flux = k x_a x_b n_H                */
       ORC_R_GRAINH2 = 2,  /* "H,H,#": flux = k x_H n_H, dH = -2  */
       ORC_R_XRAY = 3 };   /* rate forced to 0 by the rate evaluator; dropped */

/* rate-evaluator branches of calc_reac_rates.F90 */
enum { ORC_K_THERMAL = 0, ORC_K_H2FORM, ORC_K_PAH, ORC_K_PHOTO_H2, ORC_K_PHOTO_HD,
       ORC_K_PHOTO_CO, ORC_K_PHOTO_CI, ORC_K_PHOTO_SI, ORC_K_PHOTO, ORC_K_CRP,
       ORC_K_CRPHOT, ORC_K_FREEZE, ORC_K_ELFRZE, ORC_K_CRH, ORC_K_PHOTD, ORC_K_THERM,
       ORC_K_GRAIN, ORC_K_XRAY };

typedef struct {
  int nspec, nreac, neq;          /* neq = nspec-1 (electron excluded)      */
  char (*spec)[ORC_NAME];
  double *abund0, *mass;
  int *charge;                    /* coefficient of each species in the x_e sum (name-derived
                                     charges unless replaced by orc_net_load_layout) */
  char (*reac)[3][ORC_NAME];
  char (*prod)[4][ORC_NAME];
  double *alpha, *beta, *gamma, *rtmin, *rtmax;
  int *duplicate;
  int *ode_kind;                  /* ORC_R_*  */
  int *rate_kind;                 /* ORC_K_*  */
  int (*ri)[2];                   /* reactant species index, -1 none, neq = electron */
  int (*pi)[4];                   /* product species index, -1 none/non-species, neq = electron */
  /* species index labels (0-based, -1 if absent): read_species.F90:89-148 */
  int iH, iH2, iHD, iCO, iC, iS, iCx, iO, iHe, iHx, iHEx, iH2x, iH3x, iH3Ox, iHCOx, ielect;
} orc_net;

orc_net *orc_net_load(const char *species_path, const char *rates_path, char *err, int errlen);
void orc_net_free(orc_net *net);
/* apply the slot layout and electron sum of the reference's generated network
 * code (data/layout_<net>.d); returns 0 on success */
int orc_net_load_layout(orc_net *net, const char *path, char *err, int errlen);

/* RHS in the generated code's form: ode[i] = form_i + x_i * loss_i, x_e from charge balance */
void orc_rhs(const orc_net *net, const double *rate, double n_H, const double *x,
             double *ode, double *x_e_out);
/* analytic dense Jacobian df_i/dx_j (row-major neq x neq) including dx_e/dx_j */
void orc_jac(const orc_net *net, const double *rate, double n_H, const double *x, double *J);
/* Jacobian as the generated Jac() would give it: x_e held constant (jacobian_<net>.c:41) */
void orc_jac_xe_const(const orc_net *net, const double *rate, double n_H, const double *x,
                      double x_e, double *J);

/* ---------------- BDF integrator (CVODE method restated) ---------------- */
typedef void (*orc_rhs_fn)(void *ctx, double t, const double *y, double *ydot);
typedef void (*orc_jac_fn)(void *ctx, double t, const double *y, double *J);

typedef struct {
  double rtol, atol;
  long mxstep;          /* max internal steps per output interval (CVodeSetMaxNumSteps) */
  int maxord;           /* 5 */
} orc_bdf_opts;

typedef struct {
  long nst, nfe, nje, nsetups, nni, ncfn, netf;
  int qlast;
  double hlast, tcur;
} orc_bdf_stats;

/* status codes follow CVODE's flags: 0 ok, -1 too much work, -3 error test
 * failures, -4 convergence failures */
typedef struct orc_bdf orc_bdf;
orc_bdf *orc_bdf_create(int n, orc_rhs_fn f, orc_jac_fn jac, void *ctx, const orc_bdf_opts *opt);
void orc_bdf_free(orc_bdf *o);
void orc_bdf_init(orc_bdf *o, double t0, const double *y0);                 /* CVodeInit */
int orc_bdf_solve(orc_bdf *o, double tout, double *yout, double *tret);     /* CVode, CV_NORMAL */
void orc_bdf_get_stats(const orc_bdf *o, orc_bdf_stats *st);
int orc_bdf_integrate(int n, orc_rhs_fn f, orc_jac_fn jac, void *ctx, double t0,
                      const double *y0, const double *touts, int ntout,
                      const orc_bdf_opts *opt, double *yout, orc_bdf_stats *st);

/* drop-in restatement of calculate_abundances_ (calculate_abundances.c:64-354);
 * layout abundance[n*nspec+i], rate[n*nreac+r]; returns the reference's status.
 * nthreads<=0: all OpenMP threads.  stats may be NULL (else 8 longs per cell:
 * nst,nfe,nje,nsetups,nni,ncfn,netf,flag). */
int orc_calculate_abundances(const orc_net *net, double *abundance, const double *rate,
                             const double *density, const double *temperature, int npart,
                             double reltol, double abstol, double start_time_yr,
                             double end_time_yr, int nthreads, long *stats);

/* ---------------- reaction rates (calc_reac_rates.F90) ---------------- */
typedef struct {
  double zeta;          /* ZETA = zeta_in/1.3e-17 (input_parameters.F90:30-31) */
  double omega, grain_radius, metallicity, g2d, v_turb /* cm/s */;
  int h2form;           /* -DH2FORM (makefile H2FORM=1) */
  int xlambda_linear;   /* 1: XLAMBDA with zero second derivatives (START-flag variant) */
} orc_phys;

/* one cell: column[k*5+c], c = {H2, HD, CO, C, S} for ray k */
int orc_rates_cell(const orc_net *net, const orc_phys *ph, double T, double Td, int nrays,
                   const double *rad_surface, const double *AV, const double *column5,
                   double *rate, int *nr /* NRGR,NRH2,NRHD,NRCO,NRCI,NRSI (1-based) */);
int orc_rates_batched(const orc_net *net, const orc_phys *ph, int ncell, int nrays,
                      const double *T, const double *Td, const double *rad_surface,
                      const double *AV, const double *column5, double *rate, int nthreads);

/* shielding helpers (exposed for unit tests) */
double orc_h2shield1(double nh2, double dopw, double radw);
double orc_coshield(double nco, double nh2);
double orc_scatter(double av, double lambda, int xlambda_linear);
double orc_xlambda(double lambda, int xlambda_linear);
double orc_lbar(double nco, double nh2);
double orc_h2_formation_rate(double Tg, double Td, double metallicity, double g2d);
void orc_spline(const double *x, const double *y, int n, double yp1, double ypn, double *y2);
double orc_splint(const double *xa, const double *ya, const double *y2a, int n, double x);

/* ---------------- level populations ---------------- */
typedef struct {
  int nlev, ntemp, nlin;
  double *energies, *weights;     /* [nlev] (erg), g                     */
  double *A, *B, *freq;           /* [nlev*nlev], element (i,j) at i*nlev+j (0-based) */
  double *temps;                  /* [7*ntemp] partner-major          */
  double *col;                    /* [7][nlev][nlev][ntemp]            */
  int *line_up, *line_lo;         /* radiative lines in file order (0-based) */
} orc_coolant;

orc_coolant *orc_coolant_load(const char *path, int nlev, int ntemp, char *err, int errlen);
void orc_coolant_free(orc_coolant *c);

/* partner densities: n(H), n(H+), n(e), n(He), n(H2) (find_Ccoeff.F90 argument order) */
void orc_find_ccoeff(const orc_coolant *c, double T, const double *partner, double *C);
/* escape_probability.F90 after tau: tau[(line)*nrays+ray] for radiative lines;
 * pseudo1d=1 uses ray 6 only (PSEUDO_1D), else the 3D ray average. */
void orc_escape_probability(const orc_coolant *c, const double *C, const double *s_pop,
                            const double *tau, int nrays, int pseudo1d, double Tdust,
                            double density, double metallicity, double g2d,
                            double *transition, double *line, double *cooling);
int orc_solvlevpop(int nlev, const double *transition, double density, double *solution);
int orc_gauss_jordan(double *a, int n, double *b);
void orc_lte(const orc_coolant *c, double T, double density, double *pop);

/* orc_rays.c: CALC_UVFIELD and calc_columndens over flattened evaluation points */
void orc_uvfield(int ncell, int nrays, const int *epray, const long long *offset, const double *xyz, const int *gp,
                 const double *rho, int field, const double *G, const double *vectors, double metallicity,
                 double *colden, double *AV, double *rad, double *uv);
void orc_columns(int ncell, int nrays, const int *epray, const long long *offset, const double *xyz, const int *gp,
                 const double *rho, const double *ab, int nspec, const int *species, int nsel, double *out);
void orc_tau(const orc_coolant *cl, int ncell, int nrays, const int *epray, const long long *offset, const double *xyz,
             const int *gp, const double *pop, const double *T, double v_turb, double *tau);

/* whole per-cell level-population step for one coolant */
int orc_levpop_batched(const orc_coolant *c, int ncell, const double *density, const double *T,
                       const double *Tdust, const double *partner5, const double *coolant_density,
                       const double *s_pop, const double *tau, int nrays, int pseudo1d,
                       double metallicity, double g2d, double *pop_out, double *cooling_out,
                       double *line_out, int nthreads);

/* ---------------- heating (sub_calculate_heating.F90) ---------------- */
/* network: 0 reduced, 1 full, 2 mynetwork; rate/abundance 0-based arrays of
 * the network; nr = NRGR..NRSI (1-based as returned by orc_rates_cell) */
void orc_heating(const orc_net *net, int network, const orc_phys *ph, double density,
                 double Tg, double Td, double uv_field, const double *abundance,
                 const double *rate, const int *nr, double *heating12);

/* ---------------- thermal balance (3DPDR.F90:928-1050, 1084-1229) ---------------- */
void orc_thermal_balance(int ncell, double Tmin, double Tmax, double Fcrit, double Tdiff, int temp_fix,
                         int level_conv, int first_time, const double *heating, int hstride, int ncool,
                         const double *const *cooling, double *T, double *Tprev, double *Tlow, double *Thigh,
                         double *Fmean, double *Fratio, double *total_cooling, unsigned char *flags,
                         long long *nconverged);
void orc_level_convergence(int ncell, int ncool, const int *nlev, const double *const *solution,
                           double *const *pop, const double *abundance, int nspec, const int *species,
                           int thermal_balance, unsigned char *flags, unsigned char *coolant_conv,
                           long long *counts);

#ifdef __cplusplus
}
#endif
#endif
