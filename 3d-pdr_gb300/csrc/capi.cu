// capi.cu -- the C ABI of lib3dpdr_gb300.so (declared in include/pdrgpu.h).
//
// calculate_abundances_ keeps the reference's symbol, arguments and status
// semantics (calculate_abundances.c:64-354); the batched entry points take
// device arrays and a stream so a caller can keep state resident in HBM and
// capture the calls in a CUDA graph.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "pdr_internal.h"

extern "C" {
// Fortran module variables the reference binds to C (modules.F90:165-166,383,
// 529-530).  Declared weak so the library also loads in programs that are not
// the 3D-PDR driver; calculate_abundances_ then reports that they are missing.
extern double chemistry_module_mp_relative_abundance_tolerance_ __attribute__((weak));
extern double chemistry_module_mp_absolute_abundance_tolerance_ __attribute__((weak));
extern double maincode_module_mp_start_time_ __attribute__((weak));
extern double maincode_module_mp_end_time_ __attribute__((weak));
extern int global_module_mp_nelect_ __attribute__((weak));
}

namespace pdr {

size_t chem_warp_smem_per_warp(const WarpTables &T, bool mixed, bool zshared);
int launch_chem_warp(const pdr_net *net, int ncell, double *ab, const double *rate, const double *dens,
                     const double *tend, const pdr_chem_opts &o, int *status, int *stats, int *queue,
                     int *fb_list, int *fb_count, const int *cell_list, const int *total_ptr, bool mixed,
                     int sm_count, cudaStream_t st, const int *sm_limit = nullptr);
int launch_chem_cta(const pdr_net *net, int ncell, double *ab, const double *rate, const double *dens,
                    const double *tend, const pdr_chem_opts &o, int *status, int *stats, int *queue,
                    int *fb_list, int *fb_count, const int *cell_list, const int *total_ptr, bool mixed,
                    int grid, void *scratch, cudaStream_t st, const int *sm_limit = nullptr, int grid_sms = 1);
size_t chem_cta_global_bytes(const pdr_net *net, bool mixed, int grid);
size_t chem_cta_smem(const pdr_net *net, bool mixed, bool *mat_smem);
int chem_cta_blocks_per_sm(const pdr_net *net, bool mixed);
int launch_rates(const pdr_net *net, const pdr_phys &ph, int ncell, int nrays, const double *T,
                 const double *Td, const double *rad, const double *AV, const double *col5, const double *zeta,
                 double *rate, int *status, int sm_count, cudaStream_t st);
int launch_chem_eval(const pdr_net *net, int nstate, const double *x, const double *rate, const double *dens,
                     double *out, double *xe_out, int mode, cudaStream_t st);
int launch_chem_eval_cta(const pdr_net *net, int nstate, const double *x, const double *rate, const double *dens,
                         double *out, double *xe_out, int mode, cudaStream_t st);
int upload_shield_tables(int dev);
int build_coolant_tables(pdr_coolant *c);
int launch_levpop(const pdr_coolant *c, const LevArgsHost &h, bool mixed, int sm_count, cudaStream_t st);
int launch_tau(const pdr_coolant *cool, const pdr_rays &r, const double *pop, const double *T, double v_turb,
               double *tau, int sm_count, cudaStream_t st);
int launch_uvfield(const pdr_rays &r, const double *rho, int field, const double *G, const double *vectors,
                   double metallicity, double *colden, double *AV, double *rad, double *uv, int sm_count,
                   cudaStream_t st);
int launch_columns(const pdr_rays &r, const double *rho, const double *ab, int nspec, const int *species, int nsel,
                   double *out, int sm_count, cudaStream_t st);
int launch_lte(const pdr_coolant *c, int ncell, const double *T, const double *density, double *pop, int *status,
               int sm_count, cudaStream_t st);
int launch_heating(const pdr_net *net, int network, const pdr_phys &ph, int ncell, const double *dens,
                   const double *Tg, const double *Td, const double *uv, const double *ab, const double *rate,
                   const double *zeta, double *out, cudaStream_t st);
void shield_tables_host(double *xderiv30, double *scoderiv48);
int launch_thermal(const pdr_thermal_params &p, int level_conv, int first_time, const double *heat, int hstride,
                   int ncool, const double *const *cool, const pdr_thermal_state &s, double *total, int *nconv,
                   cudaStream_t st);
int launch_level_convergence(int ncell, int ncool, const int *nlev, const double *const *sol, double *const *pop,
                             const double *ab, int nspec, const int *species, int thermal_balance,
                             unsigned char *flags, unsigned char *cconv, int *counts, int sm_count,
                             cudaStream_t st);

static thread_local std::string g_err;

void set_error(const std::string &msg) { g_err = msg; }

int cuda_fail(cudaError_t e, const char *what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return PDR_E_CUDA;
}

static int current_device(int *dev, int *sms) {
  int d = 0;
  cudaError_t e = cudaGetDevice(&d);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  int n = 0;
  e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  *dev = d;
  *sms = n;
  return 0;
}

// Per-device scratch of the batched solver: the work-queue cursors, the
// FP64-redo list of the mixed form and its count.  Grown on demand, never
// shrunk; a call made during stream capture must not need to grow it.
struct Scratch {
  int *counters = nullptr;   // [0] queue, [1] redo queue, [2] redo count
  int *redo = nullptr;
  size_t redo_cap = 0;
  void *cta = nullptr;       // block integrator: per-block rate constants (and matrices)
  size_t cta_bytes = 0;
  int *sm_limit = nullptr;   // solver instances: SMs their running launch may keep (null: all)
};
static std::mutex g_mu;
static Scratch g_scratch[64];

static int scratch_for(int dev, size_t ncell, Scratch **out) {
  std::lock_guard<std::mutex> lk(g_mu);
  Scratch &s = g_scratch[dev & 63];
  if (!s.counters) {
    cudaError_t e = cudaMalloc(&s.counters, 4 * sizeof(int));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(scratch)");
  }
  if (s.redo_cap < ncell) {
    if (s.redo) cudaFree(s.redo);
    s.redo = nullptr;
    size_t cap = ncell < 1024 ? 1024 : ncell;
    cudaError_t e = cudaMalloc(&s.redo, cap * sizeof(int));
    if (e != cudaSuccess) { s.redo_cap = 0; return cuda_fail(e, "cudaMalloc(redo list)"); }
    s.redo_cap = cap;
  }
  *out = &s;
  return 0;
}

static int cta_scratch(Scratch *s, size_t bytes) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (s->cta_bytes >= bytes) return 0;
  if (s->cta) cudaFree(s->cta);
  s->cta = nullptr;
  s->cta_bytes = 0;
  cudaError_t e = cudaMalloc(&s->cta, bytes);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(block integrator scratch)");
  s->cta_bytes = bytes;
  return 0;
}

// blocks per SM of the block integrator, cached per network and precision
static int cta_per_sm(const pdr_net *net, bool mixed) {
  static std::mutex mu;
  static std::vector<std::pair<const pdr_net *, int>> cache[2];
  std::lock_guard<std::mutex> lk(mu);
  for (auto &c : cache[mixed])
    if (c.first == net) return c.second;
  const int v = chem_cta_blocks_per_sm(net, mixed);
  if (v > 0) cache[mixed].push_back({net, v});
  return v;
}


bool uses_warp_path(const pdr_net *net, const pdr_chem_opts &o) {
  return (o.integrator == 1) || (o.integrator == 0 && net->warp_ok && net->host.neq == 32);
}

int check_opts(const pdr_net *net, const pdr_chem_opts &o, const char *who) {
  if (!(o.reltol >= 0.0) || !(o.abstol > 0.0) || o.mxstep <= 0 ||
      (o.precision != PDR_FP64 && o.precision != PDR_MIXED) || o.integrator < 0 || o.integrator > 2) {
    set_error(std::string(who) + ": invalid options");
    return PDR_E_ARG;
  }
  const bool warp_ok = net->warp_ok && net->host.neq == 32;
  const bool warp_path = uses_warp_path(net, o);
  if ((warp_path && !warp_ok) || (!warp_path && !net->cta_ok)) {
    set_error(std::string(who) + (warp_path ? ": the warp integrator takes networks of 32 ODE species"
                                            : ": the network is too large for the integrator tables"));
    return PDR_E_NET;
  }
  return 0;
}

// SMs the persistent grid spans
int eff_sms(const pdr_chem_opts &o, int sms) { return (o.max_sms > 0 && o.max_sms < sms) ? o.max_sms : sms; }

// grid of the block integrator for one precision
static int cta_grid(const pdr_net *net, const pdr_chem_opts &o, bool mixed, int sms) {
  sms = eff_sms(o, sms);
  int per_sm = cta_per_sm(net, mixed);
  if (per_sm < 1) per_sm = 1;
  if (o.blocks_per_sm > 0 && o.blocks_per_sm < per_sm) per_sm = o.blocks_per_sm;
  return sms * per_sm;
}

// bytes of block-integrator scratch one solve needs (both passes of the mixed form)
static size_t cta_bytes_needed(const pdr_net *net, const pdr_chem_opts &o, int sms) {
  const bool mixed = (o.precision == PDR_MIXED);
  size_t bytes = chem_cta_global_bytes(net, mixed, cta_grid(net, o, mixed, sms));
  if (mixed) bytes = std::max(bytes, chem_cta_global_bytes(net, false, cta_grid(net, o, false, sms)));
  return bytes;
}

// One batched solve with the given scratch: the mixed pass (or the FP64 pass)
// over all cells, then, for the mixed form, the FP64 pass over the cells it
// queued.  grow = false: the scratch must already be large enough (no allocation).
static int solve_core(const pdr_net *net, int ncell, double *ab, const double *rate, const double *dens,
                      const double *tend, const pdr_chem_opts &o, int *status, int *stats, Scratch *s, bool grow,
                      int sms, cudaStream_t st) {
  if (s->redo_cap < (size_t)ncell) {
    set_error("pdr: solver scratch holds fewer cells than the call");
    return PDR_E_ARG;
  }
  cudaError_t e = cudaMemsetAsync(s->counters, 0, 4 * sizeof(int), st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(scratch)");
  const bool mixed = (o.precision == PDR_MIXED);
  int rc;
  if (uses_warp_path(net, o)) {
    const int sm_use = eff_sms(o, sms);
    rc = launch_chem_warp(net, ncell, ab, rate, dens, tend, o, status, stats, s->counters + 0, s->redo,
                          s->counters + 2, nullptr, nullptr, mixed, sm_use, st, s->sm_limit);
    if (rc || !mixed) return rc;
    // cells whose FP32 Newton iteration failed are re-solved in FP64
    return launch_chem_warp(net, ncell, ab, rate, dens, tend, o, status, stats, s->counters + 1, nullptr, nullptr,
                            s->redo, s->counters + 2, false, sm_use, st, s->sm_limit);
  }
  // one block per cell: persistent grid of SMs x resident blocks, or (refill
  // 2) one block per cell and no persistence, which needs the Newton matrix in
  // shared memory (the per-block global slots would scale with the cells)
  const bool one_per_cell = (o.refill == 2);
  if (one_per_cell) {
    bool ms = false;
    chem_cta_smem(net, mixed, &ms);
    if (!ms) {
      set_error("pdr: one block per cell (refill 2) needs the Newton matrix in shared memory: use the mixed form");
      return PDR_E_ARG;
    }
  }
  const int grid_main = one_per_cell ? ncell : cta_grid(net, o, mixed, sms);
  size_t bytes = std::max(cta_bytes_needed(net, o, sms), chem_cta_global_bytes(net, mixed, grid_main));
  if (grow) {
    rc = cta_scratch(s, bytes);
    if (rc) return rc;
  } else if (s->cta_bytes < bytes) {
    set_error("pdr: solver scratch is too small for the block integrator");
    return PDR_E_ARG;
  }
  rc = launch_chem_cta(net, ncell, ab, rate, dens, tend, o, status, stats, s->counters + 0, s->redo, s->counters + 2,
                       nullptr, nullptr, mixed, grid_main, s->cta, st, s->sm_limit, eff_sms(o, sms));
  if (rc || !mixed) return rc;
  return launch_chem_cta(net, ncell, ab, rate, dens, tend, o, status, stats, s->counters + 1, nullptr, nullptr,
                         s->redo, s->counters + 2, false, cta_grid(net, o, false, sms), s->cta, st, s->sm_limit,
                         eff_sms(o, sms));
}

}  // namespace pdr

// A solver instance: its own scratch, sized once, so that runs allocate
// nothing and instances on different streams can overlap.
struct pdr_solver {
  const pdr_net *net = nullptr;
  pdr_chem_opts opts;
  int max_cells = 0, sms = 0, dev = 0;
  pdr::Scratch s;
  int *h_words = nullptr;   // pinned: [0] "no limit" (a large SM count), [1] the latest limit
};

namespace pdr {
}  // namespace pdr

using namespace pdr;

extern "C" {

const char *pdr_last_error(void) { return g_err.c_str(); }

void pdr_chem_opts_default(pdr_chem_opts *o) {
  if (!o) return;
  o->reltol = 1.0e-8;
  o->abstol = 1.0e-30;
  o->start_time_yr = 0.0;
  o->end_time_yr = 1.0e7;
  o->mxstep = 10000000L;
  o->precision = PDR_FP64;
  o->warps_per_block = 0;
  o->blocks_per_sm = 0;
  o->reg_variant = -1;  // per precision: the fastest variant measured on GB300
  o->refill = 0;
  o->integrator = 0;
  o->max_sms = 0;
}

int pdr_device_info(int *sm_count, int *cc_major, int *cc_minor) {
  int dev = 0, sms = 0;
  int rc = current_device(&dev, &sms);
  if (rc) return rc;
  if (sm_count) *sm_count = sms;
  int a = 0, b = 0;
  cudaDeviceGetAttribute(&a, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&b, cudaDevAttrComputeCapabilityMinor, dev);
  if (cc_major) *cc_major = a;
  if (cc_minor) *cc_minor = b;
  return 0;
}

int pdr_net_load(const char *species_path, const char *rates_path, const char *layout_path, pdr_net **out) {
  if (!species_path || !rates_path || !out) { set_error("pdr_net_load: null argument"); return PDR_E_ARG; }
  pdr_net *net = new pdr_net();
  std::string err = load_network(species_path, rates_path, layout_path, net->host);
  if (!err.empty()) { set_error(err); delete net; return PDR_E_IO; }
  int dev = 0, sms = 0;
  int rc = current_device(&dev, &sms);
  if (rc == 0) rc = upload_shield_tables(dev);
  if (rc == 0) rc = build_device_tables(net);
  if (rc) { pdr_net_free(net); return rc; }
  net->device = dev;
  *out = net;
  return 0;
}

void pdr_net_free(pdr_net *net) {
  if (!net) return;
  for (void *p : net->allocations) cudaFree(p);
  delete net;
}

int pdr_net_info(const pdr_net *net, int *nspec, int *nreac, int *neq) {
  if (!net) { set_error("pdr_net_info: null network"); return PDR_E_ARG; }
  if (nspec) *nspec = net->host.nspec;
  if (nreac) *nreac = net->host.nreac;
  if (neq) *neq = net->host.neq;
  return 0;
}

int pdr_net_special_reactions(const pdr_net *net, int nr[6]) {
  if (!net || !nr) { set_error("pdr_net_special_reactions: null argument"); return PDR_E_ARG; }
  for (int k = 0; k < 6; k++) nr[k] = net->host.nr[k];
  return 0;
}

static std::vector<pdr_net *> g_registered;

int pdr_net_register(pdr_net *net) {
  if (!net) { set_error("pdr_net_register: null network"); return PDR_E_ARG; }
  std::lock_guard<std::mutex> lk(g_mu);
  g_registered.push_back(net);
  return 0;
}

int pdr_chem_solve_batched(const pdr_net *net, int ncell, double *d_abundance, const double *d_rate,
                           const double *d_density, const double *d_t_end_yr, const pdr_chem_opts *opts,
                           int *d_status, int *d_stats, void *stream) {
  if (!net || ncell < 0 || !d_abundance || !d_rate || !d_density || !d_status) {
    set_error("pdr_chem_solve_batched: invalid argument");
    return PDR_E_ARG;
  }
  if (ncell == 0) return 0;
  pdr_chem_opts o;
  pdr_chem_opts_default(&o);
  if (opts) o = *opts;
  int rc = check_opts(net, o, "pdr_chem_solve_batched");
  if (rc) return rc;
  int dev = 0, sms = 0;
  rc = current_device(&dev, &sms);
  if (rc) return rc;
  Scratch *s = nullptr;
  rc = scratch_for(dev, (size_t)ncell, &s);
  if (rc) return rc;
  return solve_core(net, ncell, d_abundance, d_rate, d_density, d_t_end_yr, o, d_status, d_stats, s, true, sms,
                    (cudaStream_t)stream);
}

int pdr_solver_create(const pdr_net *net, int max_cells, const pdr_chem_opts *opts, pdr_solver **out) {
  if (!net || max_cells <= 0 || !out) {
    set_error("pdr_solver_create: invalid argument");
    return PDR_E_ARG;
  }
  *out = nullptr;
  pdr_chem_opts o;
  pdr_chem_opts_default(&o);
  if (opts) o = *opts;
  int rc = check_opts(net, o, "pdr_solver_create");
  if (rc) return rc;
  pdr_solver *v = new pdr_solver();
  v->net = net;
  v->opts = o;
  v->max_cells = max_cells;
  rc = current_device(&v->dev, &v->sms);
  cudaError_t e = cudaSuccess;
  if (!rc && (e = cudaMalloc(&v->s.counters, 4 * sizeof(int))) != cudaSuccess) rc = cuda_fail(e, "cudaMalloc(solver)");
  if (!rc && (e = cudaMalloc(&v->s.redo, sizeof(int) * (size_t)max_cells)) != cudaSuccess)
    rc = cuda_fail(e, "cudaMalloc(solver)");
  if (!rc) v->s.redo_cap = (size_t)max_cells;
  if (!rc && (e = cudaMalloc(&v->s.sm_limit, sizeof(int))) != cudaSuccess) rc = cuda_fail(e, "cudaMalloc(solver)");
  if (!rc && (e = cudaHostAlloc(&v->h_words, 2 * sizeof(int), cudaHostAllocDefault)) != cudaSuccess)
    rc = cuda_fail(e, "cudaHostAlloc(solver)");
  if (!rc) {
    v->h_words[0] = 1 << 20;
    v->h_words[1] = 1 << 20;
    if ((e = cudaMemcpy(v->s.sm_limit, v->h_words, sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess)
      rc = cuda_fail(e, "cudaMemcpy(solver)");
  }
  // scratch for a grid over every SM, so that pdr_solver_set_max_sms may widen it later
  pdr_chem_opts all = o;
  all.max_sms = 0;
  if (!rc && !uses_warp_path(net, o)) rc = cta_scratch(&v->s, cta_bytes_needed(net, all, v->sms));
  if (rc) {
    pdr_solver_free(v);
    return rc;
  }
  *out = v;
  return 0;
}

int pdr_solver_run(pdr_solver *v, int ncell, double *d_abundance, const double *d_rate, const double *d_density,
                   const double *d_t_end_yr, int *d_status, int *d_stats, void *stream) {
  if (!v || ncell < 0 || ncell > v->max_cells || !d_abundance || !d_rate || !d_density || !d_status) {
    set_error("pdr_solver_run: invalid argument (ncell above the solver's max_cells?)");
    return PDR_E_ARG;
  }
  if (ncell == 0) return 0;
  // a new run keeps every SM of its grid until pdr_solver_limit_sms says otherwise
  cudaError_t e = cudaMemcpyAsync(v->s.sm_limit, v->h_words, sizeof(int), cudaMemcpyHostToDevice,
                                  (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "pdr_solver_run: SM allowance");
  return solve_core(v->net, ncell, d_abundance, d_rate, d_density, d_t_end_yr, v->opts, d_status, d_stats, &v->s,
                    false, v->sms, (cudaStream_t)stream);
}

int pdr_solver_limit_sms(pdr_solver *v, int max_sms, void *control_stream) {
  if (!v || max_sms < 1) {
    set_error("pdr_solver_limit_sms: invalid argument");
    return PDR_E_ARG;
  }
  v->h_words[1] = max_sms;
  cudaError_t e = cudaMemcpyAsync(v->s.sm_limit, v->h_words + 1, sizeof(int), cudaMemcpyHostToDevice,
                                  (cudaStream_t)control_stream);
  return e == cudaSuccess ? 0 : cuda_fail(e, "pdr_solver_limit_sms");
}

int pdr_solver_set_max_sms(pdr_solver *v, int max_sms) {
  if (!v || max_sms < 0) {
    set_error("pdr_solver_set_max_sms: invalid argument");
    return PDR_E_ARG;
  }
  v->opts.max_sms = max_sms;
  return 0;
}

void pdr_solver_free(pdr_solver *v) {
  if (!v) return;
  if (v->s.counters) cudaFree(v->s.counters);
  if (v->s.redo) cudaFree(v->s.redo);
  if (v->s.cta) cudaFree(v->s.cta);
  if (v->s.sm_limit) cudaFree(v->s.sm_limit);
  if (v->h_words) cudaFreeHost(v->h_words);
  delete v;
}

int pdr_chem_autotune(const pdr_net *net, int ncell_sample, const double *d_abundance, const double *d_rate,
                      const double *d_density, pdr_chem_opts *opts, void *stream) {
  if (!net || ncell_sample <= 0 || !d_abundance || !d_rate || !d_density || !opts) {
    set_error("pdr_chem_autotune: invalid argument");
    return PDR_E_ARG;
  }
  const int ns = net->host.nspec;
  cudaStream_t st = (cudaStream_t)stream;
  double *ab = nullptr;
  int *status = nullptr;
  cudaError_t e = cudaMalloc(&ab, sizeof(double) * (size_t)ncell_sample * ns);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(autotune)");
  e = cudaMalloc(&status, sizeof(int) * (size_t)ncell_sample);
  if (e != cudaSuccess) { cudaFree(ab); return cuda_fail(e, "cudaMalloc(autotune)"); }
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  struct Cand { int wpb, reg, refill; };
  const Cand warp_cands[] = {{4, 0, 0}, {2, 0, 0}, {4, 1, 0}, {8, 1, 0}, {4, 2, 0}, {2, 2, 0},
                             {4, 3, 0}, {4, 1, 1}};
  const Cand cta_cands[] = {{0, 0, 0}, {0, 0, 1}};   // block integrator: work queue or static refill
  const bool warp_path = (opts->integrator == 1) || (opts->integrator == 0 && net->warp_ok && net->host.neq == 32);
  const Cand *cands = warp_path ? warp_cands : cta_cands;
  const int ncand = warp_path ? 8 : 2;
  const bool log = getenv("PDR_AUTOTUNE_LOG") != nullptr;
  float best = 1e30f;
  pdr_chem_opts best_o = *opts;
  int rc = 0;
  for (int ci = 0; ci < ncand; ci++) {
    const Cand &c = cands[ci];
    pdr_chem_opts o = *opts;
    o.warps_per_block = c.wpb;
    o.reg_variant = c.reg;
    o.refill = c.refill;
    o.blocks_per_sm = 0;
    // the best of two timed runs: the first of a shape also pays its
    // one-time kernel-attribute and occupancy set-up
    float ms = 1e30f;
    for (int rep = 0; rep < 2 && rc == 0; rep++) {
      e = cudaMemcpyAsync(ab, d_abundance, sizeof(double) * (size_t)ncell_sample * ns, cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) { rc = cuda_fail(e, "autotune copy"); break; }
      cudaEventRecord(t0, st);
      rc = pdr_chem_solve_batched(net, ncell_sample, ab, d_rate, d_density, nullptr, &o, status, nullptr, st);
      if (rc) break;
      cudaEventRecord(t1, st);
      e = cudaEventSynchronize(t1);
      if (e != cudaSuccess) { rc = cuda_fail(e, "autotune run"); break; }
      float t = 0.f;
      cudaEventElapsedTime(&t, t0, t1);
      if (t < ms) ms = t;
    }
    if (rc) break;
    if (log)
      fprintf(stderr, "pdr_chem_autotune: warps_per_block %d reg_variant %d refill %d: %.3f ms\n", c.wpb, c.reg,
              c.refill, ms);
    if (ms < best) { best = ms; best_o = o; }
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(ab);
  cudaFree(status);
  if (rc == 0) *opts = best_o;
  return rc;
}

int pdr_rates_batched_cr(const pdr_net *net, const pdr_phys *phys, int ncell, int nrays, const double *d_T,
                         const double *d_Td, const double *d_rad_surface, const double *d_AV,
                         const double *d_column5, const double *d_zeta, double *d_rate, int *d_status,
                         void *stream) {
  if (!net || !phys || ncell < 0 || nrays <= 0 || !d_T || !d_Td || !d_rad_surface || !d_AV ||
      !d_column5 || !d_rate) {
    set_error("pdr_rates_batched: invalid argument");
    return PDR_E_ARG;
  }
  if (ncell == 0) return 0;
  int dev = 0, sms = 0;
  int rc = current_device(&dev, &sms);
  if (rc) return rc;
  rc = upload_shield_tables(dev);
  if (rc) return rc;
  return launch_rates(net, *phys, ncell, nrays, d_T, d_Td, d_rad_surface, d_AV, d_column5, d_zeta, d_rate,
                      d_status, sms, (cudaStream_t)stream);
}

int pdr_rates_batched(const pdr_net *net, const pdr_phys *phys, int ncell, int nrays, const double *d_T,
                      const double *d_Td, const double *d_rad_surface, const double *d_AV,
                      const double *d_column5, double *d_rate, int *d_status, void *stream) {
  return pdr_rates_batched_cr(net, phys, ncell, nrays, d_T, d_Td, d_rad_surface, d_AV, d_column5, nullptr, d_rate,
                              d_status, stream);
}

// Diagnostic: the device RHS f(x) (mode 0, d_out[nstate*neq], d_xe[nstate]) or the
// analytic Jacobian (mode 1, d_out[nstate*neq*neq] row-major) at given states,
// by the integrator the network runs on; modes 2 and 3 evaluate the same with
// the block integrator's code for any network.
int pdr_chem_eval_batched(const pdr_net *net, int nstate, const double *d_x, const double *d_rate,
                          const double *d_density, int mode, double *d_out, double *d_xe, void *stream) {
  if (!net || nstate < 0 || !d_x || !d_rate || !d_density || !d_out || mode < 0 || mode > 3) {
    set_error("pdr_chem_eval_batched: invalid argument");
    return PDR_E_ARG;
  }
  const bool block = (mode >= 2) || !(net->warp_ok && net->host.neq == 32);
  if (block && !net->cta_ok) {
    set_error("pdr_chem_eval_batched: the network is too large for the integrator tables");
    return PDR_E_NET;
  }
  if (nstate == 0) return 0;
  if (block)
    return launch_chem_eval_cta(net, nstate, d_x, d_rate, d_density, d_out, d_xe, mode & 1, (cudaStream_t)stream);
  return launch_chem_eval(net, nstate, d_x, d_rate, d_density, d_out, d_xe, mode, (cudaStream_t)stream);
}

int pdr_coolant_load(const char *path, int nlev, int ntemp, pdr_coolant **out) {
  if (!path || !out || nlev < 2 || nlev > 64 || ntemp < 1) {
    set_error("pdr_coolant_load: invalid argument (2 <= nlev <= 64)");
    return PDR_E_ARG;
  }
  pdr_coolant *c = new pdr_coolant();
  std::string err = load_coolant(path, nlev, ntemp, c->host);
  if (!err.empty()) { set_error(err); delete c; return PDR_E_IO; }
  int rc = build_coolant_tables(c);
  if (rc) { pdr_coolant_free(c); return rc; }
  *out = c;
  return 0;
}

void pdr_coolant_free(pdr_coolant *c) {
  if (!c) return;
  for (void *p : c->allocations) cudaFree(p);
  delete c;
}

int pdr_coolant_info(const pdr_coolant *c, int *nlev, int *nlin) {
  if (!c) { set_error("pdr_coolant_info: null coolant"); return PDR_E_ARG; }
  if (nlev) *nlev = c->host.nlev;
  if (nlin) *nlin = c->host.nlin;
  return 0;
}

int pdr_levpop_batched(const pdr_coolant *c, int ncell, int nrays, const double *d_density, const double *d_T,
                       const double *d_Tdust, const double *d_partner5, const double *d_coolant_density,
                       const double *d_spop, const double *d_tau, int pseudo1d, double metallicity, double g2d,
                       int precision, double *d_pop, double *d_cooling, double *d_line, int *d_status,
                       void *stream) {
  if (!c || ncell < 0 || nrays < 1 || (pseudo1d && nrays < 7) || !d_density || !d_T || !d_Tdust ||
      !d_partner5 || !d_coolant_density || !d_spop || !d_tau || !d_pop || !d_cooling ||
      (precision != PDR_FP64 && precision != PDR_MIXED)) {
    set_error("pdr_levpop_batched: invalid argument");
    return PDR_E_ARG;
  }
  if (ncell == 0) return 0;
  int dev = 0, sms = 0;
  int rc = current_device(&dev, &sms);
  if (rc) return rc;
  LevArgsHost h;
  h.ncell = ncell; h.nrays = nrays; h.pseudo1d = pseudo1d; h.metallicity = metallicity; h.g2d = g2d;
  h.density = d_density; h.T = d_T; h.Td = d_Tdust; h.partner5 = d_partner5; h.cdens = d_coolant_density;
  h.spop = d_spop; h.tau = d_tau; h.pop = d_pop; h.cooling = d_cooling; h.line = d_line; h.status = d_status;
  return launch_levpop(c, h, precision == PDR_MIXED, sms, (cudaStream_t)stream);
}

int pdr_lte_batched(const pdr_coolant *c, int ncell, const double *d_T, const double *d_density, double *d_pop,
                    int *d_status, void *stream) {
  if (!c || ncell < 0 || !d_T || !d_density || !d_pop) {
    set_error("pdr_lte_batched: invalid argument");
    return PDR_E_ARG;
  }
  if (ncell == 0) return 0;
  int dev = 0, sms = 0;
  int rc = current_device(&dev, &sms);
  if (rc) return rc;
  return launch_lte(c, ncell, d_T, d_density, d_pop, d_status, sms, (cudaStream_t)stream);
}

static bool rays_ok(const pdr_rays *r) {
  return r && r->ncell >= 0 && r->nrays > 0 && r->ngrid > 0 &&
         (r->ncell == 0 || (r->d_epray && r->d_offset && r->d_xyz && r->d_gridpoint));
}

int pdr_uvfield_batched(const pdr_rays *rays, const double *d_rho, int field, const double *G, const double *vectors,
                        double metallicity, double *d_columndensity, double *d_AV, double *d_rad_surface,
                        double *d_uvfield, void *stream) {
  if (!rays_ok(rays) || !d_rho || !G || (field != 0 && field != 1) || (field == 1 && !vectors) ||
      !d_columndensity || !d_AV || !d_rad_surface || !d_uvfield) {
    set_error("pdr_uvfield_batched: invalid argument");
    return PDR_E_ARG;
  }
  if (rays->ncell == 0) return 0;
  int dev = 0, sms = 0;
  int rc = current_device(&dev, &sms);
  if (rc) return rc;
  return launch_uvfield(*rays, d_rho, field, G, vectors, metallicity, d_columndensity, d_AV, d_rad_surface,
                        d_uvfield, sms, (cudaStream_t)stream);
}

int pdr_column_densities_batched(const pdr_rays *rays, const double *d_rho, const double *d_abundance, int nspec,
                                 const int *species, int nsel, double *d_columns, void *stream) {
  if (!rays_ok(rays) || !d_rho || !d_abundance || nspec <= 0 || nsel <= 0 || nsel > 256 ||
      (!species && nsel > nspec) || !d_columns) {
    set_error("pdr_column_densities_batched: invalid argument");
    return PDR_E_ARG;
  }
  if (rays->ncell == 0) return 0;
  int dev = 0, sms = 0;
  int rc = current_device(&dev, &sms);
  if (rc) return rc;
  return launch_columns(*rays, d_rho, d_abundance, nspec, species, nsel, d_columns, sms, (cudaStream_t)stream);
}

int pdr_optical_depths_batched(const pdr_coolant *c, const pdr_rays *rays, const double *d_pop, const double *d_T,
                               double v_turb, double *d_tau, void *stream) {
  if (!c || !rays_ok(rays) || !d_pop || !d_T || !d_tau || !(v_turb >= 0.0)) {
    set_error("pdr_optical_depths_batched: invalid argument");
    return PDR_E_ARG;
  }
  if (rays->ncell == 0 || c->dev.nlin == 0) return 0;
  int dev = 0, sms = 0;
  int rc = current_device(&dev, &sms);
  if (rc) return rc;
  return launch_tau(c, *rays, d_pop, d_T, v_turb, d_tau, sms, (cudaStream_t)stream);
}

int pdr_heating_batched(const pdr_net *net, int network, const pdr_phys *phys, int ncell, const double *d_density,
                        const double *d_Tgas, const double *d_Tdust, const double *d_uv_field,
                        const double *d_abundance, const double *d_rate, double *d_heating, void *stream) {
  return pdr_heating_batched_cr(net, network, phys, ncell, d_density, d_Tgas, d_Tdust, d_uv_field, d_abundance,
                                d_rate, nullptr, d_heating, stream);
}

int pdr_heating_batched_cr(const pdr_net *net, int network, const pdr_phys *phys, int ncell, const double *d_density,
                           const double *d_Tgas, const double *d_Tdust, const double *d_uv_field,
                           const double *d_abundance, const double *d_rate, const double *d_zeta, double *d_heating,
                           void *stream) {
  if (!net || !phys || ncell < 0 || !d_density || !d_Tgas || !d_Tdust || !d_uv_field || !d_abundance ||
      !d_rate || !d_heating) {
    set_error("pdr_heating_batched: invalid argument");
    return PDR_E_ARG;
  }
  if (network != 0 && network != 1) {
    set_error("pdr_heating_batched: chemical heating is defined for the reduced (0) and full (1) networks "
              "only (the reference STOPs for mynetwork, sub_calculate_heating.F90:250)");
    return PDR_E_NET;
  }
  if (ncell == 0) return 0;
  return launch_heating(net, network, *phys, ncell, d_density, d_Tgas, d_Tdust, d_uv_field, d_abundance, d_rate,
                        d_zeta, d_heating, (cudaStream_t)stream);
}

int pdr_thermal_balance_batched(const pdr_thermal_params *params, int level_conv, int first_time,
                                const double *d_heating_total, int heating_stride, int ncool,
                                const double *const *d_cooling, const pdr_thermal_state *state,
                                double *d_total_cooling, int *d_nconverged, void *stream) {
  bool ok = params && state && state->ncell >= 0 && heating_stride >= 1 && ncool >= 1 && ncool <= PDR_MAX_COOLANTS &&
            d_cooling;
  if (ok && state->ncell > 0) {
    ok = d_heating_total && state->d_T && state->d_Tprev && state->d_Tlow && state->d_Thigh && state->d_Fmean &&
         state->d_Fratio && state->d_flags;
    for (int k = 0; ok && k < ncool; k++) ok = d_cooling[k] != nullptr;
  }
  if (!ok) {
    set_error("pdr_thermal_balance_batched: invalid argument");
    return PDR_E_ARG;
  }
  if (state->ncell == 0) {
    if (d_nconverged) {
      cudaError_t e = cudaMemsetAsync(d_nconverged, 0, sizeof(int), (cudaStream_t)stream);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(converged count)");
    }
    return 0;
  }
  return launch_thermal(*params, level_conv, first_time, d_heating_total, heating_stride, ncool, d_cooling, *state,
                        d_total_cooling, d_nconverged, (cudaStream_t)stream);
}

int pdr_level_convergence_batched(int ncell, int ncool, const int *nlev, const double *const *d_solution,
                                  double *const *d_pop, const double *d_abundance, int nspec, const int *species,
                                  int thermal_balance, unsigned char *d_flags, unsigned char *d_coolant_conv,
                                  int *d_counts, void *stream) {
  bool ok = ncell >= 0 && ncool >= 1 && ncool <= PDR_MAX_COOLANTS && nlev && species && d_solution && d_pop &&
            nspec > 0 && d_counts;
  for (int k = 0; ok && k < ncool; k++)
    ok = nlev[k] >= 1 && nlev[k] <= 4096 && species[k] >= 0 && species[k] < nspec && (ncell == 0 || (d_solution[k] && d_pop[k]));
  if (ok && ncell > 0) ok = d_abundance && d_flags;
  if (!ok) {
    set_error("pdr_level_convergence_batched: invalid argument");
    return PDR_E_ARG;
  }
  if (ncell == 0) {
    cudaError_t e = cudaMemsetAsync(d_counts, 0, sizeof(int) * (1 + ncool), (cudaStream_t)stream);
    return e == cudaSuccess ? 0 : cuda_fail(e, "cudaMemsetAsync(level convergence counts)");
  }
  int dev = 0, sms = 0;
  int rc = current_device(&dev, &sms);
  if (rc) return rc;
  return launch_level_convergence(ncell, ncool, nlev, d_solution, d_pop, d_abundance, nspec, species,
                                  thermal_balance, d_flags, d_coolant_conv, d_counts, sms, (cudaStream_t)stream);
}

// diagnostic export of the shielding spline tables (tests compare them with the oracle)
int pdr_shield_tables(double *xderiv30, double *scoderiv48) {
  if (!xderiv30 || !scoderiv48) { set_error("pdr_shield_tables: null argument"); return PDR_E_ARG; }
  shield_tables_host(xderiv30, scoderiv48);
  return 0;
}

// ---------------- legacy calculate_abundances_ ----------------

static pdr_net *find_network(int nspec, int nreac) {
  {
    std::lock_guard<std::mutex> lk(g_mu);
    for (pdr_net *n : g_registered)
      if (n->host.nspec == nspec && n->host.nreac == nreac) return n;
  }
  const char *dir = std::getenv("PDR_NETWORK_DIR");
  std::string base = dir ? std::string(dir) : std::string(".");
  const char *names[3] = {"reduced", "full", "mynetwork"};
  for (const char *nm : names) {
    std::string sp = base + "/species_" + nm + ".d", rp = base + "/rates_" + nm + ".d";
    std::string lp = base + "/layout_" + nm + ".d";
    FILE *f = std::fopen(sp.c_str(), "r");
    if (!f) continue;
    std::fclose(f);
    FILE *fl = std::fopen(lp.c_str(), "r");
    if (fl) std::fclose(fl);
    pdr_net *n = nullptr;
    if (pdr_net_load(sp.c_str(), rp.c_str(), fl ? lp.c_str() : nullptr, &n) != 0) continue;
    if (n->host.nspec == nspec && n->host.nreac == nreac) {
      pdr_net_register(n);
      return n;
    }
    pdr_net_free(n);
  }
  return nullptr;
}

struct LegacyBuffers {
  double *ab = nullptr, *rate = nullptr, *dens = nullptr;
  int *status = nullptr;
  size_t ab_n = 0, rate_n = 0, dens_n = 0, status_n = 0;
};
static LegacyBuffers g_legacy[64];

static int grow(void **p, size_t &have, size_t need, size_t elem) {
  if (have >= need) return 0;
  if (*p) cudaFree(*p);
  *p = nullptr;
  cudaError_t e = cudaMalloc(p, need * elem);
  if (e != cudaSuccess) { have = 0; return cuda_fail(e, "cudaMalloc(calculate_abundances_ buffers)"); }
  have = need;
  return 0;
}

int pdr_calculate_abundances(pdr_net *net, double *abundance, double *rate, double *density,
                             double *temperature, int npart, int nspec, int nreac, const pdr_chem_opts *opts) {
  (void)temperature;
  if (!abundance || !rate || !density || npart < 0) {
    set_error("pdr_calculate_abundances: invalid argument");
    return PDR_E_ARG;
  }
  if (npart == 0) return 0;
  if (!net) net = find_network(nspec, nreac);
  if (!net || net->host.nspec != nspec || net->host.nreac != nreac) {
    set_error("pdr_calculate_abundances: no network with the call's nspec/nreac is registered or found");
    return PDR_E_NET;
  }
  const int n = npart, ns = nspec, nr = nreac;
  int dev = 0, sms = 0;
  int rc = current_device(&dev, &sms);
  if (rc) return rc;
  LegacyBuffers &b = g_legacy[dev & 63];
  if ((rc = grow((void **)&b.ab, b.ab_n, (size_t)n * ns, sizeof(double)))) return rc;
  if ((rc = grow((void **)&b.rate, b.rate_n, (size_t)n * nr, sizeof(double)))) return rc;
  if ((rc = grow((void **)&b.dens, b.dens_n, (size_t)n, sizeof(double)))) return rc;
  if ((rc = grow((void **)&b.status, b.status_n, (size_t)n, sizeof(int)))) return rc;
  cudaStream_t st = nullptr;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(b.ab, abundance, (size_t)n * ns * sizeof(double), cudaMemcpyHostToDevice, st)) ||
      (e = cudaMemcpyAsync(b.rate, rate, (size_t)n * nr * sizeof(double), cudaMemcpyHostToDevice, st)) ||
      (e = cudaMemcpyAsync(b.dens, density, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st)))
    return cuda_fail(e, "calculate_abundances: host-to-device copy");
  rc = pdr_chem_solve_batched(net, n, b.ab, b.rate, b.dens, nullptr, opts, b.status, nullptr, st);
  if (rc) return rc;
  std::vector<int> status(n);
  if ((e = cudaMemcpyAsync(abundance, b.ab, (size_t)n * ns * sizeof(double), cudaMemcpyDeviceToHost, st)) ||
      (e = cudaMemcpyAsync(status.data(), b.status, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, st)) ||
      (e = cudaStreamSynchronize(st)))
    return cuda_fail(e, "calculate_abundances: device-to-host copy");
  int result = 0;
  for (int i = 0; i < n; i++)
    if (status[i] != 0) result = status[i];
  return result;
}

int calculate_abundances_(double *abundance, double *rate, double *density, double *temperature, int *npart,
                          int *nspec, int *nreac) {
  if (!abundance || !rate || !density || !npart || !nspec || !nreac || *npart < 0) {
    set_error("calculate_abundances_: invalid argument");
    return PDR_E_ARG;
  }
  if (!&chemistry_module_mp_relative_abundance_tolerance_ || !&chemistry_module_mp_absolute_abundance_tolerance_ ||
      !&maincode_module_mp_start_time_ || !&maincode_module_mp_end_time_ || !&global_module_mp_nelect_) {
    set_error("calculate_abundances_: the Fortran module variables (chemistry_module_mp_*, "
              "maincode_module_mp_*, global_module_mp_nelect_) are not defined by the caller");
    return PDR_E_ARG;
  }
  if (global_module_mp_nelect_ != *nspec) {
    set_error("calculate_abundances_: the electron must be the last species");
    return PDR_E_NET;
  }
  pdr_chem_opts o;
  pdr_chem_opts_default(&o);
  o.reltol = chemistry_module_mp_relative_abundance_tolerance_;
  o.abstol = chemistry_module_mp_absolute_abundance_tolerance_;
  o.start_time_yr = maincode_module_mp_start_time_;
  o.end_time_yr = maincode_module_mp_end_time_;
  if (const char *p = std::getenv("PDR_PRECISION")) o.precision = (std::strcmp(p, "mixed") == 0) ? PDR_MIXED : PDR_FP64;
  return pdr_calculate_abundances(nullptr, abundance, rate, density, temperature, *npart, *nspec, *nreac, &o);
}

}  // extern "C"
