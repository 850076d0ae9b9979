// pdr_internal.h -- host-side network model and device table layouts shared by
// the CUDA translation units of lib3dpdr_gb300.so.
#pragma once

#include <array>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pdrgpu.h"

namespace pdr {

// ODE kinds of a reaction (how it enters the generated RHS, odes_<net>.c)
enum OdeKind { ODE_UNI = 0, ODE_BI = 1, ODE_GRAINH2 = 2, ODE_XRAY = 3 };

// rate-evaluator branches of calc_reac_rates.F90:53-378
enum RateKind {
  RK_THERMAL = 0, RK_H2FORM, RK_PAH, RK_PHOTO_H2, RK_PHOTO_HD, RK_PHOTO_CO, RK_PHOTO_CI,
  RK_PHOTO_SI, RK_PHOTO, RK_CRP, RK_CRPHOT, RK_FREEZE, RK_ELFRZE, RK_CRH, RK_PHOTD, RK_THERM,
  RK_GRAIN, RK_XRAY
};

constexpr int kWarp = 32;

// Device tables of one network for a group of `lanes` threads integrating one
// cell: the warp-per-cell integrator (lanes = 32, neq <= 32) and the
// CTA-per-cell integrator (lanes = 32*ceil(neq/32), at least 64; neq <= 252
// so that a slot fits the 8-bit field of the packed term tables).
// Slot convention: 0..neq-1 species, neq = electron (x_e), neq+1 = constant 1.
struct WarpTables {
  int neq = 0, nreac = 0;
  int lanes = 0;       // table stride: threads of the group
  int rhs_len = 0;     // RHS terms per lane (balanced chunks)
  int nparts = 0;      // partial-sum slots (slot nparts is a constant zero)
  int plist_len = 0;   // partial slots summed per species
  int jac_len = 0;     // Jacobian terms per species (padded)
  int2 *rab = nullptr;        // [nreac] reactant slots (a, b)
  double *nh_mask = nullptr;  // [nreac] 1 if the rate constant is multiplied by n_H
  // RHS f_i = sum over terms of (nu kn_r) * operand: operands are the slot
  // values (0..neq+1) and the products x_a x_b of the distinct two-body
  // reactant pairs (neq+2 ..); the rate constants kn[0..nkn) are the per-cell
  // kn_r followed by the extras: the coefficient sum_r nu_r kn_r of the terms
  // of one species that share an operand, or nu kn_r of a single term with
  // |nu| > 1; kn[nkn] is a constant zero for the padding terms
  int nkn = 0, nkext = 0, npairs = 0, nop = 0;
  int2 *rhs_t = nullptr;      // [rhs_len][lanes] (kn index | (partial slot written after the term + 1) << 16,
                              //  operand | sign of nu << 31)
  int2 *pairs = nullptr;      // [npairs] slots (a, b) of each reactant pair
  int *kext_ptr = nullptr;    // [nkext+1] extra rate constant e = sum over kext_rn[kext_ptr[e]..kext_ptr[e+1])
  int2 *kext_rn = nullptr;    //   of nu * kn_r, (reaction r, nu) in reaction order
  int *plist = nullptr;       // [plist_len][lanes] partial slots of species `lane`
  int *jac_rab = nullptr;     // [jac_len][lanes] reaction | slot a << 16 | slot b << 24
  double *jac_nu = nullptr;   // [jac_len][lanes]
  float *jac_nu_f = nullptr;  // [jac_len][lanes]
  double *xe_coef = nullptr;  // [lanes] electron-sum coefficient per slot
  float *xe_coef_f = nullptr; // the same in FP32 (the mixed forms' Newton matrix)
  // term-parallel Jacobian assembly (block integrator): the (row, column)
  // contributions nu * dphi_r/dx_col of every term, sorted by entry and cut
  // into `lanes` balanced chunks; a chunk sums each run of one entry in a
  // register and stores it (kind 1), or, for a run that crosses a chunk
  // boundary, leaves its partial in a boundary slot (kind 2) that a second
  // pass adds up in chunk order
  int hlen = 0, nbnd = 0;
  // [hlen][lanes] one 8-byte load per contribution:
  //   .x = reaction | Db? << 16 | kind << 17 (0 accumulate, 1 store, 2 slot) | nu << 19 (signed, 0 = padding)
  //   .y = row | column << 8 | slot << 16
  int2 *h_xy = nullptr;
  double *h_nu = nullptr;     // [hlen][lanes] nu as FP64 (the FP64 forms: no integer conversion on the FP64 pipe)
  int *bnd_t = nullptr;       // [nbnd] row | column << 8 | sparse location << 16 of a boundary entry
  int *bnd_s = nullptr;       // [nbnd] first slot | (last slot + 1) << 16
  // Sparse Newton matrix of the block integrator's mixed form (sp.ok): the
  // bordered system over the N = neq+1 unknowns (species, then x_e with the
  // row x_e - sum_j c_j x_j = 0) instead of the x_e chain rule, whose rank-one
  // term fills most of the matrix.  Unknowns in a minimum-degree elimination
  // order; the first `a` rows (the "leaf" rows: few dependencies) stored
  // packed by row and factorised in place without pivoting, one dependency
  // level at a time; the last m = N - a rows, nearly dense after fill, hold
  // their leaf-column part packed and their trailing m x m block dense
  // (column-major, stride ldb), factorised with partial pivoting.  For a
  // kind-1 term entry the high 16 bits of h_xy.y hold its location in the
  // storage, for a boundary entry those of bnd_t.
  struct Sparse {
    int ok = 0;
    int N = 0, a = 0, m = 0, ldb = 0;
    int off_ba = 0, off_d = 0, total = 0;   // storage offsets / size, in elements
    int nnz_b = 0;                          // trailing rows' leaf-column entries
    int nlev = 0, nul = 0;
    int *perm = nullptr;      // [N] unknown (elimination order) -> slot (species, neq = x_e)
    int *iperm = nullptr;     // [N] slot -> unknown
    int *a_ptr = nullptr;     // [a+1] leaf row r: storage [a_ptr[r], a_ptr[r+1])
    unsigned short *a_col = nullptr;   // column (unknown) of each leaf-row entry, ascending
    int *a_diag = nullptr;    // [a] storage position of the diagonal
    int *lev_ptr = nullptr;   // [nlev+1] leaf rows by L-dependency level (rows are in level order)
    int *ul_rows = nullptr;   // [a] leaf rows by U-dependency level
    int *ul_ptr = nullptr;    // [nul+1]
    int *b_ptr = nullptr;     // [m+1] trailing row t: leaf-column entries at off_ba + [b_ptr[t], b_ptr[t+1])
    unsigned short *b_col = nullptr;   // their columns, ascending
    int *diag_loc = nullptr;  // [N] storage location of each diagonal entry
    int *e_loc = nullptr;     // [neq] location of (x_e row, species j), -1 where c_j = 0
  } sp;
};

// Device tables for the rate evaluator.
struct RateTables {
  int nreac = 0;
  int *kind = nullptr;        // RateKind
  int *dup = nullptr;         // DUPLICATE
  int *dup_next = nullptr;    // DUPLICATE(I+1) or -1 past the end
  double *alpha = nullptr, *beta = nullptr, *gamma = nullptr, *rtmin = nullptr, *rtmax = nullptr;
  int *flags = nullptr;       // bit0: reactant-1 name starts with 'G'; bit1: H2 photo sets NRH2;
                              // bit2: HD photo sets NRHD
  // evaluation order: the reactions whose rate is a sum over the rays (the
  // photo-reactions and photodesorption), grouped by kind, then the others,
  // grouped by kind (lanes of a warp then mostly take the same branch)
  int nray = 0, nother = 0;
  int *ray_reac = nullptr;    // [nray]
  int *other_reac = nullptr;  // [nother]
};

struct HostNet {
  int nspec = 0, nreac = 0, neq = 0;
  std::vector<std::string> spec;     // species-file names
  std::vector<std::string> slot;     // species each ODE slot represents in the RHS
  std::vector<int> xe;               // electron-sum coefficient per slot
  std::vector<std::array<std::string, 3>> reac;
  std::vector<std::array<std::string, 4>> prod;
  std::vector<double> alpha, beta, gamma, rtmin, rtmax;
  std::vector<int> dup, ode_kind, rate_kind, ra, rb;
  std::vector<std::array<int, 4>> pidx;
  int nr[6] = {0, 0, 0, 0, 0, 0};    // NRGR, NRH2, NRHD, NRCO, NRCI, NRSI (1-based)
};

std::string load_network(const char *species, const char *rates, const char *layout, HostNet &net);

// A LAMDA coolant as read by read_input.F90 (element (i,j) at i*nlev+j, 0-based)
struct HostCoolant {
  int nlev = 0, ntemp = 0, nlin = 0;
  std::vector<double> energies, weights, A, B, freq, temps /*[7][ntemp]*/, col /*[7][nlev*nlev][ntemp]*/;
  std::vector<int> line_up, line_lo;
};
std::string load_coolant(const char *path, int nlev, int ntemp, HostCoolant &c);

// Device tables of one coolant for the level-population kernel
struct CoolantTables {
  int nlev = 0, ntemp = 0, nlin = 0, npart = 0;
  int part[7] = {0, 0, 0, 0, 0, 0, 0};   // LAMDA partner ids (0-based) with rates, ascending
  double *temps = nullptr;     // [npart][ntemp]
  double *col = nullptr;       // [npart][ntemp][nlev*nlev]
  double *A = nullptr, *B = nullptr, *freq = nullptr, *weights = nullptr;
  double *energies = nullptr;  // [nlev] level energies, erg
  int *line_of_pair = nullptr; // [nlev*nlev] radiative line of (i,j), i>j, else -1
  int nrad = 0;
  int *rad_pairs = nullptr;    // [nrad] pairs i*nlev+j, i>j, with A or B nonzero either way
  double *pair_tmp2 = nullptr; // [nrad] 2 h nu^3 / c^2
  double *pair_cmb = nullptr;  // [nrad] tmp2 / (exp(h nu / k 2.7 K) - 1)
  double *pair_emis = nullptr; // [nrad] 0.01 (1.3 nu / 3e11), the dust emissivity factor
  int *line_up = nullptr, *line_lo = nullptr;   // [nlin] levels of each radiative line
  double *line_frac1 = nullptr;                 // [nlin] A c^3 / (8 pi nu^3)
};

// host-side argument bundle of the level-population launch
struct LevArgsHost {
  int ncell = 0, nrays = 0, pseudo1d = 0;
  double metallicity = 1.0, g2d = 100.0;
  const double *density = nullptr, *T = nullptr, *Td = nullptr, *partner5 = nullptr, *cdens = nullptr,
               *spop = nullptr, *tau = nullptr;
  double *pop = nullptr, *cooling = nullptr, *line = nullptr;
  int *status = nullptr;
};

}  // namespace pdr

struct pdr_coolant {
  pdr::HostCoolant host;
  pdr::CoolantTables dev;
  std::vector<void *> allocations;
};

struct pdr_net {
  pdr::HostNet host;
  int device = -1;
  bool warp_ok = false, cta_ok = false;
  pdr::WarpTables warp;   // warp-per-cell tables (neq <= 32)
  pdr::WarpTables cta;    // CTA-per-cell tables (neq <= 252)
  pdr::RateTables rates;
  std::vector<void *> allocations;
};

namespace pdr {
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
int build_device_tables(pdr_net *net);
// option checks and launch shape shared by the chemistry entry points (capi.cu)
bool uses_warp_path(const pdr_net *net, const pdr_chem_opts &o);
int check_opts(const pdr_net *net, const pdr_chem_opts &o, const char *who);
int eff_sms(const pdr_chem_opts &o, int sms);   // SMs the persistent grid spans
}  // namespace pdr
