/*
 * pdrgpu.h -- C ABI of lib3dpdr_gb300.so, a GB300 (sm_103a) drop-in for the
 * per-grid-point chemistry and level-population solves of 3D-PDR.
 *
 * Every entry point is plain C: pointers, sizes and a cudaStream_t passed as
 * void*.  "d_" arguments are device pointers, "h_" host pointers.  All
 * functions return 0 on success and a negative PDR_E_* code on an API error;
 * pdr_last_error() returns the message of the last error of the calling thread.
 * There is no CPU fallback: without a usable GPU every compute call fails with
 * PDR_E_CUDA.
 */
#ifndef PDRGPU_H
#define PDRGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define PDR_E_ARG -1001    /* invalid argument                         */
#define PDR_E_IO -1002     /* input file missing or malformed          */
#define PDR_E_CUDA -1003   /* CUDA runtime error (no device, launch)   */
#define PDR_E_NET -1004    /* network does not fit a kernel / no match */

/* per-cell integrator status, CVODE's flag values (calculate_abundances.c:221-299) */
#define PDR_OK 0
#define PDR_TOO_MUCH_WORK -1
#define PDR_ERR_FAILURE -3
#define PDR_CONV_FAILURE -4

#define PDR_FP64 0   /* FP64 Newton matrix, partial-pivot LU (CVDense semantics)     */
#define PDR_MIXED 1  /* FP32 weight-scaled LU of I-gamma*J, FP64 state/RHS/residual;
                        cells whose Newton iteration fails are re-solved in FP64     */

typedef struct pdr_net pdr_net;
typedef struct pdr_coolant pdr_coolant;

/* physics constants of params.dat (input_parameters.F90:19-54) */
typedef struct {
  double zeta;          /* ZETA = cosmic-ray rate / 1.3e-17 s^-1                      */
  double omega;         /* dust albedo                                                */
  double grain_radius;  /* grain radius as given in params.dat                        */
  double metallicity;
  double g2d;           /* gas-to-dust ratio                                          */
  double v_turb;        /* turbulent velocity, cm/s                                   */
  int h2form;           /* 1: Cazaux & Tielens H2 formation (-DH2FORM), 0: 3e-18 sqrt(T) */
  int xlambda_linear;   /* 1: tau(lambda)/tau(V) by linear interpolation (the reference's
                           START-flag variant, shield.F90:398-401,543); 0: natural spline */
} pdr_phys;

typedef struct {
  double reltol;        /* relative_abundance_tolerance (1e-8, 3DPDR.F90:462)        */
  double abstol;        /* absolute_abundance_tolerance (1e-30, 3DPDR.F90:463)       */
  double start_time_yr; /* start_time (3DPDR.F90:452)                                 */
  double end_time_yr;   /* end_time (params.dat), used when d_t_end_yr is NULL       */
  long mxstep;          /* max internal steps per output interval (1e7, calculate_abundances.c:111) */
  int precision;        /* PDR_FP64 or PDR_MIXED                                      */
  int warps_per_block;  /* warp integrator: warps (cells in flight) per block, 1..8; 0:
                           8 (4 for register variants 2 and 3)                        */
  int blocks_per_sm;    /* 0: as many as fit                                          */
  int reg_variant;      /* warp integrator register budget (-1, the default: 1 for the
                           mixed form, 2 for FP64): 0 as needed (8 warps/SM),
                           1 at most 128 per thread (16 warps/SM, Nordsieck rows in
                           shared memory), 2 at most 168 (12 warps/SM), 3 as 2 with
                           the Nordsieck rows in shared memory; 2 and 3 take at most
                           4 warps per block                                          */
  int refill;           /* 0: persistent grid, cells refill from an atomic work queue;
                           1: persistent grid, static split; 2: one warp (block) per
                           cell, no persistence (the block integrator needs the mixed
                           form for this)                                          */
  int integrator;       /* 0: automatic (one warp per cell for 32 ODE species, else
                           one block per cell), 1: warp per cell, 2: block per cell */
  int max_sms;          /* 0: the persistent grid spans every SM; n > 0: only n SMs'
                           worth of blocks, leaving the rest to concurrent solves */
} pdr_chem_opts;

void pdr_chem_opts_default(pdr_chem_opts *opts);
const char *pdr_last_error(void);
int pdr_device_info(int *sm_count, int *cc_major, int *cc_minor);

/* ---- networks (read_species.F90:15-194, read_rates.F90:9-95) ----
 * layout_path: optional slot layout of the reference's generated network code
 * (data/layout_<net>.d); NULL keeps species-file order and name charges. */
int pdr_net_load(const char *species_path, const char *rates_path, const char *layout_path,
                 pdr_net **out);
void pdr_net_free(pdr_net *net);
int pdr_net_info(const pdr_net *net, int *nspec, int *nreac, int *neq);
/* register a network for calculate_abundances_ (matched by nspec/nreac) */
int pdr_net_register(pdr_net *net);

/* ---- chemistry: batched drop-in for calculate_abundances_ ----
 * d_abundance[ncell*nspec] (column-major (nspec,ncell), updated in place, the
 * electron slot receives x_e of the last RHS call), d_rate[ncell*nreac],
 * d_density[ncell]; d_t_end_yr[ncell] or NULL; d_status[ncell] receives the
 * CVODE flag of each cell; d_stats[ncell*8] (or NULL) receives nst, nfe, nje,
 * nsetups, nni, ncfn, netf, fell_back_to_fp64.  Replaces
 * calculate_abundances.c:124-326 for all cells in one persistent launch. */
int pdr_chem_solve_batched(const pdr_net *net, int ncell, double *d_abundance,
                           const double *d_rate, const double *d_density,
                           const double *d_t_end_yr, const pdr_chem_opts *opts, int *d_status,
                           int *d_stats, void *stream);

/* A solver instance with its own device scratch, sized at creation for up to
 * max_cells cells (no counterpart in the reference: it is what a serving loop
 * or any caller that overlaps solves on several streams needs).  Runs take the
 * same arguments as pdr_chem_solve_batched with the instance's options,
 * allocate nothing, and instances on different streams may overlap; runs of
 * one instance must not overlap each other. */
typedef struct pdr_solver pdr_solver;
int pdr_solver_create(const pdr_net *net, int max_cells, const pdr_chem_opts *opts, pdr_solver **out);
int pdr_solver_run(pdr_solver *solver, int ncell, double *d_abundance, const double *d_rate,
                   const double *d_density, const double *d_t_end_yr, int *d_status, int *d_stats,
                   void *stream);
/* limit the persistent grid of later runs to max_sms SMs' worth of blocks (0: all) */
int pdr_solver_set_max_sms(pdr_solver *solver, int max_sms);
/* Shrink the run of this instance that is in flight (or the next one, if it
 * starts after the copy) to max_sms SMs' worth of blocks: the blocks beyond
 * that take no further cells once they finish their current one, and the
 * remaining cells go to the blocks that stay, so another instance launched on
 * another stream gets those SMs within one cell's integration time.  The value
 * is written by a 4-byte copy on control_stream, which must not be the run's
 * own stream (the copy would wait for the run).  Each pdr_solver_run starts
 * again with every SM of its grid.  Results do not depend on the allowance.
 * Work-queue mode (refill 0) only; no counterpart in the reference. */
int pdr_solver_limit_sms(pdr_solver *solver, int max_sms, void *control_stream);
void pdr_solver_free(pdr_solver *solver);

/* ---- serving (no counterpart in the reference) ----
 * A server owns one lane per network, and each lane slots_per_lane launch
 * slots: a worker thread, a stream, a solver instance, pinned staging and
 * device buffers for max_batch_cells cells, all allocated by
 * pdr_server_create (nothing is allocated while serving).  Requests are blocks
 * of cells given by their physical conditions and initial abundances.  A free
 * slot takes every queued request of its network that fits, in arrival order,
 * and runs them as one launch (reaction rates, then the batched solve with
 * per-cell end times), so requests that arrive while other launches are on
 * the GPU start at once on another slot.  With partition_sms the SMs are
 * shared: a new launch takes an equal share with the launches in flight, and
 * those shrink to that share at their next cell boundary
 * (pdr_solver_limit_sms), so no launch waits for another to drain.  Admission
 * is by device-memory footprint: a request whose cells (inputs, rate
 * constants, outputs) would take the bytes of the requests admitted and not
 * yet finished above hbm_budget_mb is refused with PDR_E_BUSY, to be retried.
 * The arrays of a request must stay valid until pdr_server_wait returns for
 * its ticket; abundance[ncell*nspec] is overwritten with the result and
 * status[ncell] (or NULL) receives the cells' CVODE flags.  Each cell is
 * integrated on its own, so a request's results do not depend on the others
 * in flight. */
#define PDR_E_BUSY -1005   /* server: the request would exceed the memory budget now */
typedef struct pdr_server pdr_server;
typedef struct {
  int max_batch_cells;  /* cells per launch, also the largest request (65536)         */
  int nrays;            /* rays per cell in the requests (12)                           */
  int precision;        /* PDR_MIXED (default) or PDR_FP64                              */
  int partition_sms;    /* 1 (default): launches in flight share the SMs equally (see
                           above); 0: every launch is sized for all SMs and the
                           hardware shares them                                        */
  int slots_per_lane;   /* launches in flight per network (4)                           */
  double hbm_budget_mb; /* device-memory footprint of the admitted, unfinished requests
                           (0: what the slots' buffers hold)                           */
} pdr_server_opts;
typedef struct {
  int network;          /* index into the server's network list                        */
  int ncell;
  double t_end_yr;
  const double *n_H, *T, *Tdust;                   /* [ncell]                          */
  const double *rad_surface, *AV;                  /* [ncell*nrays]                    */
  const double *column5;                           /* [ncell*nrays*5]: H2, HD, CO, C, S */
  double *abundance;                               /* [ncell*nspec] in/out             */
  int *status;                                     /* [ncell] or NULL                  */
} pdr_serve_request;
void pdr_server_opts_default(pdr_server_opts *opts);
int pdr_server_create(pdr_net *const *nets, int nnet, const pdr_phys *phys, const pdr_server_opts *opts,
                      pdr_server **out);
int pdr_server_submit(pdr_server *server, const pdr_serve_request *request, long long *ticket);
/* blocks until the request is done; returns 0, the last nonzero cell flag, or
 * a PDR_E_* code; latency_ms (or NULL) receives submit-to-completion time */
int pdr_server_wait(pdr_server *server, long long ticket, double *latency_ms);
int pdr_server_stats(pdr_server *server, int lane, long long *batches, long long *cells);
/* bytes of device memory a request of ncell cells of that network takes while admitted */
int pdr_server_footprint(pdr_server *server, int network, int ncell, double *bytes);
void pdr_server_free(pdr_server *server);

/* Allocation-free variant of pdr_chem_solve_batched, with no counterpart in
 * the reference.  For callers that cannot call cudaMalloc (device memory owned
 * and capped by another framework's pool; serving loops that must not
 * allocate, and so synchronise the device, once running): the solver's scratch
 * (work-queue cursors, FP64 re-solve list) lives in a static device array of
 * at most 262,144 cells, which every GPU that loads the library holds until
 * exit.  Larger calls fail with PDR_E_ARG.  All calls on a device share the
 * array: calls that overlap on the GPU race and must be serialised by the
 * caller.  The first call on a device looks the array up with
 * cudaGetSymbolAddress; make it before any stream capture. */
int pdr_chem_solve_batched_noalloc(const pdr_net *net, int ncell, double *d_abundance,
                                   const double *d_rate, const double *d_density,
                                   const double *d_t_end_yr, const pdr_chem_opts *opts,
                                   int *d_status, int *d_stats, void *stream);

/* Autotuner: times launch shapes (warps per block, register variant, refill
 * policy) on copies of the first ncell_sample cells of the given inputs (the
 * inputs are not modified; the best of two runs per shape) and writes the
 * fastest into opts, keeping its other fields.  Allocates temporary device
 * buffers; call it before stream capture. */
int pdr_chem_autotune(const pdr_net *net, int ncell_sample, const double *d_abundance,
                      const double *d_rate, const double *d_density, pdr_chem_opts *opts,
                      void *stream);

/* Legacy symbol with the reference's exact signature (calculate_abundances.c:64):
 * host arrays, all arguments by reference (gfortran implicit interface).
 * Tolerances, times and the electron index are read from the Fortran module
 * variables the reference binds to C (modules.F90:165-166,383,529-530):
 * chemistry_module_mp_relative_abundance_tolerance_, ..._absolute_..._,
 * maincode_module_mp_start_time_, maincode_module_mp_end_time_,
 * global_module_mp_nelect_.  The network is the registered one whose
 * (nspec, nreac) match, else species_<net>.d/rates_<net>.d found in
 * $PDR_NETWORK_DIR or the working directory.  Returns the reference's status
 * (0, or the last failing CVODE flag) or a PDR_E_* code. */
int calculate_abundances_(double *abundance, double *rate, double *density, double *temperature,
                          int *npart, int *nspec, int *nreac);
/* The same host-buffer call with explicit options instead of the Fortran module
 * variables; net NULL selects the network as calculate_abundances_ does.
 * Copies in, solves (pdr_chem_solve_batched), copies out, synchronises. */
int pdr_calculate_abundances(pdr_net *net, double *abundance, double *rate, double *density,
                             double *temperature, int npart, int nspec, int nreac,
                             const pdr_chem_opts *opts);

/* ---- reaction rates: batched CALCULATE_REACTION_RATES (calc_reac_rates.F90:16-401) ----
 * d_rad_surface, d_AV: [ncell*nrays]; d_column5: [ncell*nrays*5] column
 * densities of H2, HD, CO, C, S along each ray; d_rate[ncell*nreac] out;
 * d_status[ncell]: 0, or -(the lowest reaction number with a negative rate; the
 * reference STOPs there). */
int pdr_rates_batched(const pdr_net *net, const pdr_phys *phys, int ncell, int nrays,
                      const double *d_T, const double *d_Td, const double *d_rad_surface,
                      const double *d_AV, const double *d_column5, double *d_rate, int *d_status,
                      void *stream);
/* The cosmic-ray variant of the same call (3dpdr_cr.tgz: calc_reac_rates.F90:19,
 * 40,254-303,359-361 take zetacrlocal in place of ZETA): d_zeta[ncell] is each
 * cell's cosmic-ray rate in the units of pdr_phys.zeta (s^-1 / 1.3e-17), used by
 * the CRP, CRPHOT and cosmic-ray desorption branches; NULL takes phys->zeta. */
int pdr_rates_batched_cr(const pdr_net *net, const pdr_phys *phys, int ncell, int nrays,
                         const double *d_T, const double *d_Td, const double *d_rad_surface,
                         const double *d_AV, const double *d_column5, const double *d_zeta,
                         double *d_rate, int *d_status, void *stream);
/* special reaction numbers NRGR, NRH2, NRHD, NRCO, NRCI, NRSI (1-based, 0 = absent) */
int pdr_net_special_reactions(const pdr_net *net, int nr[6]);

/* ---- level populations: batched FIND_CCOEFF + escape_probability + solvlevpop ----
 * pdr_coolant_load reads a LAMDA file as read_input.F90:6-258 does (nlev and
 * the temperature capacity ntemp as in input_parameters.F90:120-127).
 * pdr_levpop_batched replaces, for one coolant and every cell, the calls of
 * 3DPDR.F90:756-843: d_partner5[ncell*5] = number densities of H, H+, e-, He,
 * H2 (find_Ccoeff.F90 argument order); d_coolant_density[ncell] = n(coolant)
 * (the density argument of solvlevpop.F90:1); d_spop[ncell*nlev] the current
 * populations (escape_probability's s_pop); d_tau[ncell*nlin*nrays] the
 * line-centre optical depth of every radiative line (file order) along every
 * ray, i.e. the ray sums of escape_probability.F90:97-106; pseudo1d uses ray 6
 * only as PSEUDO_1D does.  Outputs: d_pop[ncell*nlev] (negatives set to 0),
 * d_cooling[ncell] (the coolant's cooling_rate), d_line[ncell*nlev*nlev] or
 * NULL, d_status[ncell] (0 ok, 1 singular matrix, 2 mixed solve re-done in
 * FP64) or NULL.  precision PDR_FP64 solves with the reference's full-pivot
 * Gauss-Jordan; PDR_MIXED uses, for coolants of more than 8 levels, an FP32
 * Gauss-Jordan inverse (partial pivoting) of the row-equilibrated matrix plus
 * up to two refinement steps (FP64 residual, FP32 correction), accepted when
 * the next correction is below 1e-7
 * of every population above 1e-6 of the coolant density and below 1e-4 of
 * those above 1e-12, and shrinking; other cells are re-solved in FP64 (status
 * 2).  Coolants of up to 8 levels take the FP64 solve in both forms. */
int pdr_coolant_load(const char *path, int nlev, int ntemp, pdr_coolant **out);
void pdr_coolant_free(pdr_coolant *c);
int pdr_coolant_info(const pdr_coolant *c, int *nlev, int *nlin);
int pdr_levpop_batched(const pdr_coolant *c, int ncell, int nrays, const double *d_density,
                       const double *d_T, const double *d_Tdust, const double *d_partner5,
                       const double *d_coolant_density, const double *d_spop, const double *d_tau,
                       int pseudo1d, double metallicity, double g2d, int precision, double *d_pop,
                       double *d_cooling, double *d_line, int *d_status, void *stream);

/* LTE level populations (CALCULATE_PARTITION_FUNCTION + CALCULATE_LTE_POPULATIONS,
 * 3DPDR.F90:1847-1894): d_pop[ncell*nlev] = n g_i exp(-E_i/kT) / Z for every
 * cell; d_status[ncell] (or NULL) is 1 where the populations miss the density
 * by more than 1e-3 (where the reference STOPs), else 0. */
int pdr_lte_batched(const pdr_coolant *c, int ncell, const double *d_T, const double *d_density, double *d_pop,
                    int *d_status, void *stream);

/* ---- rays: column densities and the UV field (3DPDR.F90:1636-1844) ----
 * The evaluation points of every (cell, ray), as the ray tracing leaves them
 * (pdr%epray, pdr%epoint, pdr%projected; 3DPDR.F90:346-350), flattened: the
 * points i = 0..epray of cell c's ray j are d_offset[c*nrays+j] + i in d_xyz
 * (x, y, z per point) and d_gridpoint (index of the grid point projected there,
 * into the grid arrays d_rho and d_abundance); point 0 is the cell itself.
 * epray = 0 is a ray with no evaluation points.  ngrid bounds the grid
 * indices: a ray that refers to a grid point outside [0, ngrid) gets NaN
 * results instead of reading outside the grid arrays. */
typedef struct {
  int ncell, nrays, ngrid;
  long long npoint;           /* length of the point arrays; rays reaching past it give NaN */
  const int *d_epray;         /* [ncell*nrays] */
  const long long *d_offset;  /* [ncell*nrays] */
  const double *d_xyz;        /* [npoint*3] */
  const int *d_gridpoint;     /* [npoint] */
} pdr_rays;

/* CALC_UVFIELD (3DPDR.F90:1636-1701) for every cell: the total-H column along
 * each ray, sum over points of (rho_{i-1} + rho_i)/2 * |x_i - x_{i-1}| * pc
 * (d_columndensity[ncell*nrays]), A_V = column * 6.289e-22 * metallicity
 * (d_AV), the surface field per ray (d_rad_surface; field 0 "ISO": G0/nrays,
 * field 1 "UNI": -G.v on the ray most anti-parallel to G, vectors[3*nrays] the
 * ray directions, host memory) and the attenuated field sum_j rad_j
 * exp(-3.02 A_V,j) with the reference's clamp of values below 1e-50 to 0 after
 * each ray (d_uvfield[ncell]).  G[3] on the host: G0 for "ISO" is G[0]. */
int pdr_uvfield_batched(const pdr_rays *rays, const double *d_rho, int field, const double *G,
                        const double *vectors, double metallicity, double *d_columndensity, double *d_AV,
                        double *d_rad_surface, double *d_uvfield, void *stream);

/* calc_columndens (3DPDR.F90:1789-1844): d_columns[(c*nrays+j)*nsel+s] = sum over
 * the points of ray j of |x_i - x_{i-1}| * pc * (rho_{i-1} x_{i-1,k} + rho_i x_{i,k})/2
 * for the species k = species[s] (host array of nsel <= 256 indices; NULL: the
 * first nsel species in order), x from d_abundance[gridpoint*nspec+k].  The
 * rates need k = H2, HD, CO, C, S in that order (their column5 argument). */
int pdr_column_densities_batched(const pdr_rays *rays, const double *d_rho, const double *d_abundance,
                                 int nspec, const int *species, int nsel, double *d_columns, void *stream);

/* Optical depths of a coolant's radiative lines along the rays: the sums of
 * escape_probability.F90:86-106 from the level populations of the grid points
 * at the rays' evaluation points.  d_pop[ngrid*nlev] are the populations of
 * every grid point (the gathers of 3DPDR.F90:736-751 read them), d_T[ncell]
 * the cells' gas temperatures (Tguess), v_turb in cm/s.  Output
 * d_tau[(c*nlin + l)*nrays + j] for line l in file order -- the layout
 * pdr_levpop_batched takes.  A ray with a bad index gets NaN. */
int pdr_optical_depths_batched(const pdr_coolant *c, const pdr_rays *rays, const double *d_pop, const double *d_T,
                               double v_turb, double *d_tau, void *stream);

/* ---- heating: batched CALC_HEATING (sub_calculate_heating.F90:7-386) ----
 * network 0 = reduced, 1 = full (the reference's compile-time choice of the
 * chemical-heating reactions); d_abundance[ncell*nspec] and d_rate[ncell*nreac]
 * in the network's species-file and rate-file order, d_uv_field[ncell] in
 * Draine units; d_heating[ncell*12] receives HEATING_RATE(1:12) (photoelectric,
 * PAH, Weingartner-Draine, C ionisation, H2 formation, H2 photodissociation,
 * FUV pumping, cosmic rays, turbulence, chemical, gas-grain, total). */
int pdr_heating_batched(const pdr_net *net, int network, const pdr_phys *phys, int ncell,
                        const double *d_density, const double *d_Tgas, const double *d_Tdust,
                        const double *d_uv_field, const double *d_abundance, const double *d_rate,
                        double *d_heating, void *stream);
/* The cosmic-ray variant (3dpdr_cr.tgz sub_calculate_heating.F90:11,26,210): the
 * cosmic-ray heating term takes each cell's d_zeta[ncell] (units of
 * pdr_phys.zeta) in place of ZETA; NULL takes phys->zeta. */
int pdr_heating_batched_cr(const pdr_net *net, int network, const pdr_phys *phys, int ncell,
                           const double *d_density, const double *d_Tgas, const double *d_Tdust,
                           const double *d_uv_field, const double *d_abundance, const double *d_rate,
                           const double *d_zeta, double *d_heating, void *stream);

/* ---- outer-iteration controllers resident on the device ----
 * The per-cell state of the thermal-balance search (3DPDR.F90:928-1050) lives
 * in device memory between outer iterations.  d_flags bits: */
#define PDR_TB_CONVERGED 1       /* converged(pp) */
#define PDR_TB_BINARY_CHOP 2     /* dobinarychop(pp) */
#define PDR_TB_LEVEL_TMIN 4      /* doleveltmin(pp) */
#define PDR_TB_LEVEL_CONVERGED 8 /* level_converged(pp) */
#define PDR_TB_HEATED 16         /* previouschange(pp) == "H" */
#define PDR_TB_COOLED 32         /* previouschange(pp) == "C" (neither: not yet set) */
#define PDR_MAX_COOLANTS 8

typedef struct {
  double Tmin, Tmax, Fcrit, Tdiff; /* params.dat thermal-balance block (input_parameters.F90:48-51) */
  int temp_fix;                    /* the TEMP_FIX build option (on in the reference makefile) */
} pdr_thermal_params;

typedef struct {
  int ncell;
  double *d_T;     /* gastemperature, updated in place */
  double *d_Tprev; /* previousgastemperature */
  double *d_Tlow, *d_Thigh;
  double *d_Fmean, *d_Fratio; /* written for the cells not yet converged */
  unsigned char *d_flags;
} pdr_thermal_state;

/* One pass of the thermal-balance loop body (3DPDR.F90:928-1050) for every
 * cell not yet converged: Fmean = heating - cooling, Fratio = 2|Fmean|/|heating
 * + cooling|, then the first 30% bracket (level_conv && first_time), or the
 * 30% steps, binary chop, TEMP_FIX and Tmin/Tmax ends (level_conv && !first_time);
 * with level_conv == 0 only Fmean and Fratio are updated.  The heating of cell
 * c is d_heating_total[c*heating_stride] (pass d_heating + 11, stride 12, for
 * pdr_heating_batched's output); the cooling is the left-to-right sum of the
 * ncool (<= PDR_MAX_COOLANTS) coolant rates, host array of device pointers
 * d_cooling[k][ncell] (3DPDR.F90:897: CII, CI, OI, CO), stored in
 * d_total_cooling (or NULL).  *d_nconverged (or NULL) receives the number of
 * converged cells after the pass (3DPDR.F90:1067-1069). */
int pdr_thermal_balance_batched(const pdr_thermal_params *params, int level_conv, int first_time,
                                const double *d_heating_total, int heating_stride, int ncool,
                                const double *const *d_cooling, const pdr_thermal_state *state,
                                double *d_total_cooling, int *d_nconverged, void *stream);

/* The level-population convergence check and update of 3DPDR.F90:1084-1229
 * for ncool (<= PDR_MAX_COOLANTS) coolants: host arrays nlev[k], species[k]
 * (the coolant's species, NCx NC NO NCO; nlev <= 4096) and of device pointers
 * d_solution[k][ncell*nlev[k]] (the new populations) and d_pop[k] (the
 * current ones, overwritten with the new).  Both are indexed [cell][level]:
 * element (c, l) is at c*nlev[k] + l.  The reference's CII_SOLUTION(pp,ilevel)
 * is column-major, i.e. [level][cell] in memory, so a Fortran caller passes
 * arrays dimensioned (nlev, ncell) or transposes SOLUTION first.  The
 * populations are replaced by SOLUTION in every cell, except that without
 * thermal balance and with every cell converged they are kept, as the
 * reference leaves its loop before the update then (3DPDR.F90:1161-1172).
 * A level is checked when its new
 * population is >= 1e-10 * abundance(species); the coolant converged in a cell
 * when every checked level changed by a relative 2|s-p|/(s+p) <= 1e-2.  Sets
 * PDR_TB_LEVEL_CONVERGED in d_flags where all coolants converged; with
 * thermal_balance != 0 clears it everywhere once every cell converged
 * (3DPDR.F90:1202-1206).  d_coolant_conv[ncell] (or NULL): bit k = coolant k
 * converged.  d_counts[1+ncool]: level-converged cells before that reset, then
 * the converged cells of each coolant. */
int pdr_level_convergence_batched(int ncell, int ncool, const int *nlev, const double *const *d_solution,
                                  double *const *d_pop, const double *d_abundance, int nspec, const int *species,
                                  int thermal_balance, unsigned char *d_flags, unsigned char *d_coolant_conv,
                                  int *d_counts, void *stream);

/* ---- diagnostics (tests pin the device code against the reference with these) ----
 * The device network RHS, as the generated f() of odes_<net>.c:26-149 computes
 * it (mode 0: d_out[nstate*neq], x_e of each state in d_xe), or the analytic
 * Jacobian including dx_e/dx_j (mode 1: d_out[nstate*neq*neq], row-major
 * J[i][j] = df_i/dx_j; jacobian_<net>.c is the reference counterpart, without
 * the x_e chain rule).  d_x[nstate*neq], d_rate[nstate*nreac], d_density[nstate].
 * Modes 0 and 1 run the code of the integrator the network uses (one warp per
 * cell for 32 ODE species, else one block per cell); modes 2 and 3 are modes
 * 0 and 1 through the block integrator's code for any network.  Modes 2 and 3
 * allocate temporary scratch and synchronise the stream. */
int pdr_chem_eval_batched(const pdr_net *net, int nstate, const double *d_x, const double *d_rate,
                          const double *d_density, int mode, double *d_out, double *d_xe, void *stream);
/* second derivatives of the shielding splines: XLAMBDA's 30-point table
 * (shield.F90:543) and COSHIELD's 8x6 grid ([iNCO*6+iNH2], shield.F90:398-401) */
int pdr_shield_tables(double *xderiv30, double *scoderiv48);
/* FMA throughput of the current device in TFLOP/s (precision 64 or 32), the
 * FP64/FP32 roofline denominators reported beside the measured kernels */
int pdr_probe_fma_tflops(int precision, double *tflops, void *stream);

#ifdef __cplusplus
}
#endif
#endif
