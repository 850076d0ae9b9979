// chem_warp.cu -- batched BDF chemistry integrator, one warp per cell.
//
// Replaces the per-cell CVODE solve of calculate_abundances.c:124-326 for
// networks with at most 32 ODE species (the reduced network has exactly 32):
// lane i owns species i -- its Nordsieck row z[0..5][i], error weight and
// correction -- and row i of the Newton matrix, held in registers.
//
// The integrator restates the published CVODE method step for step (the same
// algorithm as the CPU oracle; constants and formulas are listed there):
// fixed-leading-coefficient BDF of order 1..5 in Nordsieck form, Newton
// iteration with at most 3 corrections, WRMS local error test, CVODE's step
// and order heuristics, initial-step estimate, tout ladder of
// calculate_abundances.c:214,302-303 with its retry rules, clamping of
// outputs below abstol and the x_e of the last RHS call in the electron slot.
//
// Per cell, the warp also builds the RHS and the analytic Jacobian from the
// network tables (pdr_net.cpp):
//   RHS  f_i = sum_r nu_ir phi_r,  phi_r = kn_r x_a x_b  (kn = k or k n_H),
//        fluxes computed reaction-parallel, then the stoichiometric terms are
//        summed in 32 balanced chunks with deterministic partial sums;
//   Jac  J_ij = sum_r nu_ir dphi_r/dx_j plus the chain rule through
//        x_e = sum_j c_j x_j (the generated Jac() of the reference omits it).
//
// Precision modes:
//   PDR_FP64  : M = I - gamma J in FP64, partial-pivot LU (CVDense semantics).
//   PDR_MIXED : M is formed and factorised in FP32 after the similarity
//               scaling W M W^-1 with W = diag(1/(rtol|y|+atol)) taken at
//               setup; the state, RHS, Newton residual and error test stay
//               FP64.  A cell whose Newton iteration fails with a fresh FP32
//               matrix is queued and re-solved from its inputs in FP64.
#include <cstdint>
#include <mutex>
#include <type_traits>

#include "bdf_core.cuh"
#include "pdr_internal.h"

namespace pdr {

namespace {

using namespace bdf;
constexpr unsigned FULL = 0xffffffffu;

struct ChemArgs {
  WarpTables tab;
  int ncell, nspec, nreac;
  double *abundance;
  const double *rate;
  const double *density;
  const double *t_end_yr;
  double t_end_default_yr, start_time_yr, reltol, abstol;
  long long mxstep, max_total_steps;
  int *status;
  int *stats;
  const int *cell_list;     // optional indirection (FP64 redo pass)
  int *queue;               // work-queue cursor
  int *fallback_list;       // mixed mode: cells to redo in FP64
  int *fallback_count;
  int refill_static;        // 1: warp w takes cells w, w+W, ... ; 0: atomic work queue
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(FULL, v, o));
  return v;
}

template <class T>
__device__ __forceinline__ T bcast(T v, int src) { return __shfl_sync(FULL, v, src); }

// index of the lane with the largest candidate value (lowest lane on ties);
// returns -1 when every candidate is zero
__device__ __forceinline__ int argmax_lane(float v, bool cand) {
  unsigned bits = cand ? __float_as_uint(v) : 0u;
  unsigned mx = __reduce_max_sync(FULL, bits);
  unsigned b = __ballot_sync(FULL, cand && bits == mx);
  return (mx == 0u) ? -1 : __ffs(b) - 1;
}
__device__ __forceinline__ int argmax_lane(double v, bool cand) {
  unsigned long long u = cand ? (unsigned long long)__double_as_longlong(v) : 0ull;
  unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
  unsigned mh = __reduce_max_sync(FULL, hi);
  unsigned ml = __reduce_max_sync(FULL, (hi == mh) ? lo : 0u);
  unsigned b = __ballot_sync(FULL, cand && hi == mh && lo == ml);
  return (mh == 0u && ml == 0u) ? -1 : __ffs(b) - 1;
}

// LU with partial pivoting of the rows held in shared memory, lane i = row i
// at a + i*ld.  Rows stay in place: on exit row i holds its multipliers in
// the columns before the step at which it was the pivot (mystep) and its U
// row from there on; invd = 1/diagonal, perm[k] = pivot row of step k.  (A
// register-resident row would need the nest fully unrolled and kept the
// integrator's state out of registers.)
template <int N, class MT>
__device__ __forceinline__ bool lu_rows(MT *a, int ld, int lane, int &mystep, MT &invd, int *perm) {
  mystep = (lane < N) ? -1 : N;
  MT *row = a + lane * ld;
#pragma unroll 1
  for (int k = 0; k < N; k++) {
    const bool cand = (mystep < 0);
    const int p = argmax_lane(cand ? fabs(row[k]) : MT(0), cand);
    if (p < 0) return false;
    const MT *prow = a + p * ld;
    MT rinv;
    if constexpr (sizeof(MT) == 8) rinv = __drcp_rn(prow[k]);
    else rinv = __frcp_rn(prow[k]);
    if (lane == p) { mystep = k; invd = rinv; perm[k] = p; }
    if (mystep < 0) {
      const MT l = row[k] * rinv;
      row[k] = l;
      for (int j = k + 1; j < N; j++) row[j] = fma(-l, prow[j], row[j]);
    }
    __syncwarp();
  }
  return true;
}

// Solve with the row-distributed LU: b is this lane's right-hand-side entry
// (row `lane`), the solution component for column `lane` is returned.
template <int N, class MT>
__device__ __forceinline__ MT lu_solve_rows(const MT *a, int ld, int lane, int mystep, MT invd, MT b,
                                            const int *perm) {
  const MT *row = a + (lane < N ? lane : 0) * ld;
#pragma unroll 4
  for (int k = 0; k < N; k++) {
    const MT yk = bcast(b, perm[k]);
    if (mystep > k) b = fma(-row[k], yk, b);
  }
  MT x = MT(0);
#pragma unroll 4
  for (int k = N - 1; k >= 0; k--) {
    const MT xk = bcast(b * invd, perm[k]);
    if (lane == k) x = xk;
    if (mystep < k) b = fma(-row[k], xk, b);
  }
  return x;
}

// One cell integrated by one warp: lane = species = Newton-matrix row.
// ZSH: Nordsieck rows in shared memory instead of registers.
template <int NSP, bool MIXED, bool ZSH>
struct WarpCell : Core<WarpCell<NSP, MIXED, ZSH>, ZSH, MIXED> {
  using MT = typename std::conditional<MIXED, float, double>::type;
  const ChemArgs &A;
  const int lane;
  const bool owns;
  const double inv_n = 1.0 / NSP;
  // shared-memory views of this warp
  double *kn, *scr, *xs, *part;
  MT *jrow;       // [NSP][NSP+3] Newton matrix rows / their LU factors
  float *sig;     // [NSP+2] column scales (mixed)
  int *perm;      // [NSP] pivot lane of each elimination step
  double cx;      // electron-sum coefficient of species `lane`
  int mystep;
  MT invd;
  double wsc, ssc;   // setup-time weight and its inverse (mixed scaling)

  __device__ __forceinline__ WarpCell(const ChemArgs &a, int ln) : A(a), lane(ln), owns(ln < NSP) {}
  __device__ __forceinline__ bool leader() const { return lane == 0; }
  __device__ __forceinline__ void sync() const { __syncwarp(); }
  __device__ __forceinline__ double sum_all(double v) const { return warp_sum(v); }
  __device__ __forceinline__ float sum_all(float v) const { return warp_sum(v); }
  __device__ __forceinline__ double max_all(double v) const { return warp_max(v); }

  // f(y): returns f_lane, records x_e of this call
  __device__ __forceinline__ double rhs(double yv) {
    const WarpTables &T = A.tab;
    if (owns) xs[lane] = yv;
    const double xe = warp_sum(owns ? cx * yv : 0.0);
    if (lane == 0) xs[NSP] = xe;
    this->xe_last = xe;
    __syncwarp();
    for (int r = lane; r < T.nreac; r += kWarp) {
      const int2 ab = __ldg(&T.rab[r]);
      scr[r] = kn[r] * xs[ab.x] * xs[ab.y];
    }
    __syncwarp();
    double s = 0.0;
#pragma unroll 2
    for (int t = 0; t < T.rhs_len; t++) {
      const int rf = __ldg(&T.rhs_rf[t * kWarp + lane]);
      const double nu = __ldg(&T.rhs_nu[t * kWarp + lane]);
      s = fma(nu, scr[rf & 0xffff], s);
      const int fl = (rf >> 16) - 1;
      if (fl >= 0) { part[fl] = s; s = 0.0; }
    }
    __syncwarp();
    double f = 0.0;
    for (int k = 0; k < T.plist_len; k++) f += part[__ldg(&T.plist[k * kWarp + lane])];
    __syncwarp();
    this->nfe++;
    return owns ? f : 0.0;
  }

  // Jacobian rows at y, times rf, plus the identity when `identity`:
  // FP64 m = rf*J (+I); mixed m = rf * W J W^-1 (+I), W = diag(1/(rtol|y|+atol))
  __device__ __forceinline__ void assemble(double yv, double rf_d, bool identity) {
    const WarpTables &T = A.tab;
    if (owns) xs[lane] = yv;
    const double xe = warp_sum(owns ? cx * yv : 0.0);
    if (lane == 0) xs[NSP] = xe;
    if constexpr (MIXED) {
      // column scales 1/w_j = rtol|y_j|+atol, normalised by atol so they fit FP32
      ssc = this->rtol * fabs(yv) + this->atol;
      wsc = 1.0 / ssc;
      if (owns) sig[lane] = (float)(ssc / this->atol);
      if (lane == 0) { sig[NSP] = 1.0f; sig[NSP + 1] = 0.0f; }
    }
    __syncwarp();
    MT *Da = reinterpret_cast<MT *>(scr);
    MT *Db = Da + T.nreac;
    for (int r = lane; r < T.nreac; r += kWarp) {
      const int2 ab = __ldg(&T.rab[r]);
      const double k = kn[r];
      if constexpr (MIXED) {
        Da[r] = (float)(k * xs[ab.y]) * sig[ab.x];
        Db[r] = (float)(k * xs[ab.x]) * sig[ab.y];
      } else {
        Da[r] = k * xs[ab.y];
        Db[r] = (ab.y == NSP + 1) ? 0.0 : k * xs[ab.x];
      }
    }
    MT *row = jrow + lane * (NSP + 3);
    if (owns)
      for (int j = 0; j < NSP + 2; j++) row[j] = MT(0);
    __syncwarp();
    if (owns) {
      for (int t = 0; t < T.jac_len; t++) {
        MT nu;
        if constexpr (MIXED) nu = __ldg(&T.jac_nu_f[t * kWarp + lane]);
        else nu = __ldg(&T.jac_nu[t * kWarp + lane]);
        if (nu == MT(0)) break;
        const int rab = __ldg(&T.jac_rab[t * kWarp + lane]);
        const int r = rab & 0xffff, a = (rab >> 16) & 0xff, b = (rab >> 24) & 0xff;
        row[a] = fma(nu, Da[r], row[a]);
        row[b] = fma(nu, Db[r], row[b]);
      }
    }
    __syncwarp();
    const MT e = owns ? row[NSP] : MT(0);
    MT rf;
    if constexpr (MIXED) rf = (MT)(rf_d * (wsc * this->atol));   // row weight, normalised like the columns
    else rf = (MT)rf_d;
#pragma unroll 4
    for (int j = 0; j < NSP; j++) {
      const MT cj = (MT)__ldg(&T.xe_coef[j]);
      MT v = owns ? row[j] : MT(0);
      if constexpr (MIXED) v = fmaf(e * cj, sig[j], v);
      else v = fma(e, cj, v);
      if (owns) row[j] = rf * v + ((identity && lane == j) ? MT(1) : MT(0));
    }
    __syncwarp();
  }

  // Newton matrix at y: FP64 M = I - gamma J, or FP32 W M W^-1, factorised
  __device__ __forceinline__ bool setup(double yv) {
    assemble(yv, -this->gamma, true);
    __syncwarp();
    const bool ok = lu_rows<NSP, MT>(jrow, NSP + 3, lane, mystep, invd, perm);
    const MT *row = jrow + lane * (NSP + 3);
    bool finite = true;
    if (owns)
      for (int j = 0; j < NSP; j++) finite &= isfinite(row[j]);
    finite = __all_sync(FULL, finite);
    this->after_setup();
    return ok && finite;
  }

  __device__ __forceinline__ double solve(double b) {
    double x;
    if constexpr (MIXED) {
      const float xs_ = lu_solve_rows<NSP, float>(jrow, NSP + 3, lane, mystep, invd, (float)(b * wsc), perm);
      x = (double)xs_ * ssc;
    } else {
      x = lu_solve_rows<NSP, double>(jrow, NSP + 3, lane, mystep, invd, b, perm);
    }
    return owns ? x : 0.0;
  }

  // calculate_abundances.c:132-317 for one cell
  __device__ __forceinline__ void run(int cell) {
    const int nspec = A.nspec;
    double *ab = A.abundance + (size_t)cell * nspec;
    const double n_H = A.density[cell];
    this->rtol = A.reltol;
    this->atol = A.abstol;
    this->mxstep = A.mxstep;
    this->max_total_steps = A.max_total_steps;
    cx = owns ? __ldg(&A.tab.xe_coef[lane]) : 0.0;
    // per-cell rate constants, multiplied by n_H for two-body terms
    const double *rate = A.rate + (size_t)cell * A.nreac;
    for (int r = lane; r < A.nreac; r += kWarp) kn[r] = __ldg(&rate[r]) * (__ldg(&A.tab.nh_mask[r]) != 0.0 ? n_H : 1.0);
    if (lane == 0) {
      xs[NSP + 1] = 1.0;
      part[A.tab.nparts] = 0.0;
    }
#pragma unroll
    for (int j = 0; j <= QMAX; j++) this->z[j] = 0.0;
    this->z[0] = owns ? ab[lane] : 0.0;
    this->xe_last = ab[nspec - 1];
    const double tend_yr = A.t_end_yr ? A.t_end_yr[cell] : A.t_end_default_yr;
    double yv = 0.0;
    const int status = this->integrate(A.start_time_yr, tend_yr, MIXED, &yv);
    if (status == FELL_BACK) {
      if (lane == 0) {
        const int k = atomicAdd(A.fallback_count, 1);
        A.fallback_list[k] = cell;
        A.status[cell] = FELL_BACK;
      }
      return;
    }
    if (yv < this->atol) yv = 0.0;
    if (owns) ab[lane] = yv;
    if (lane == 0) {
      ab[nspec - 1] = this->xe_last;
      A.status[cell] = status;
      if (A.stats) {
        int *s = A.stats + (size_t)cell * 8;
        s[0] = this->nst; s[1] = this->nfe; s[2] = this->nje; s[3] = this->nsetups;
        s[4] = this->nni; s[5] = this->ncfn; s[6] = this->netf; s[7] = MIXED ? 0 : (A.cell_list ? 1 : 0);
      }
    }
  }
};

// Register variants (the autotuner picks): RV 0 lets the compiler use the
// registers it wants (about 230; 8 warps/SM); RV 1 caps them at 128 for 16
// warps/SM with the Nordsieck rows in shared memory; RV 2 and 3 cap them at
// 168 for 12 warps/SM (blocks of at most 4 warps), Nordsieck rows in
// registers (2) or shared memory (3).
template <int RV> struct RegVariant;
template <> struct RegVariant<0> { static constexpr int threads = 256, min_blocks = 1; static constexpr bool zsh = false; };
template <> struct RegVariant<1> { static constexpr int threads = 256, min_blocks = 2; static constexpr bool zsh = true; };
template <> struct RegVariant<2> { static constexpr int threads = 128, min_blocks = 3; static constexpr bool zsh = false; };
template <> struct RegVariant<3> { static constexpr int threads = 128, min_blocks = 3; static constexpr bool zsh = true; };

template <int NSP, bool MIXED, int RV>
__global__ void __launch_bounds__(RegVariant<RV>::threads, RegVariant<RV>::min_blocks)
    chem_warp_kernel(const __grid_constant__ ChemArgs A, int total_cells, const int *total_ptr) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using MT = typename std::conditional<MIXED, float, double>::type;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nreac = A.nreac;
  // per-warp shared layout
  // scr: the fluxes (FP64) or the two Jacobian scatter buffers (MT each)
  const size_t kn_b = (size_t)nreac * 8, scr_b = (size_t)nreac * (MIXED ? 8 : 16), xs_b = 8 * (NSP + 2);
  const size_t part_b = 8 * (A.tab.nparts + 1);
  constexpr bool ZSH = RegVariant<RV>::zsh;
  const size_t jrow_b = sizeof(MT) * NSP * (NSP + 3), sig_b = 4 * (NSP + 2) + 4 * NSP;
  const size_t ws_b = sizeof(CoefShared) + (ZSH ? 8 * (QMAX + 1) * kWarp : 0);
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  const size_t per_warp = al(kn_b) + al(scr_b) + al(xs_b) + al(part_b) + al(jrow_b) + al(sig_b) + al(ws_b);
  unsigned char *base = smem_raw + per_warp * warp;
  WarpCell<NSP, MIXED, ZSH> c(A, lane);
  c.kn = reinterpret_cast<double *>(base);
  c.scr = reinterpret_cast<double *>(base + al(kn_b));
  c.xs = reinterpret_cast<double *>(base + al(kn_b) + al(scr_b));
  c.part = reinterpret_cast<double *>(base + al(kn_b) + al(scr_b) + al(xs_b));
  c.jrow = reinterpret_cast<MT *>(base + al(kn_b) + al(scr_b) + al(xs_b) + al(part_b));
  c.sig = reinterpret_cast<float *>(base + al(kn_b) + al(scr_b) + al(xs_b) + al(part_b) + al(jrow_b));
  c.perm = reinterpret_cast<int *>(c.sig + NSP + 2);
  c.ws = reinterpret_cast<CoefShared *>(base + al(kn_b) + al(scr_b) + al(xs_b) + al(part_b) + al(jrow_b) + al(sig_b));
  if constexpr (ZSH) {
    c.z.p = reinterpret_cast<double *>(reinterpret_cast<unsigned char *>(c.ws) + sizeof(CoefShared)) + lane;
    c.z.s = kWarp;
  }
  c.build_uniform_table();
  if (total_ptr) total_cells = *total_ptr;
  const int gwarp = blockIdx.x * (blockDim.x >> 5) + warp, nwarps = gridDim.x * (blockDim.x >> 5);
  for (int k = 0;; k++) {
    int idx = 0;
    if (A.refill_static) {
      idx = gwarp + k * nwarps;
    } else {
      if (lane == 0) idx = atomicAdd(A.queue, 1);
      idx = __shfl_sync(FULL, idx, 0);
    }
    if (idx >= total_cells) break;
    const int cell = A.cell_list ? A.cell_list[idx] : idx;
    c.run(cell);
    __syncwarp();
  }
}

// Diagnostic evaluation of the device RHS (mode 0) or Jacobian (mode 1) on
// given states: one warp per state, the same code the integrator runs.
template <int NSP>
__global__ void __launch_bounds__(128) eval_kernel(const __grid_constant__ ChemArgs A, int nstate,
                                                   const double *x, double *out, double *xe_out, int mode) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nreac = A.nreac;
  auto al = [](size_t v) { return (v + 15) & ~size_t(15); };
  const size_t kn_b = (size_t)nreac * 8, scr_b = (size_t)nreac * 16, xs_b = 8 * (NSP + 2);
  const size_t part_b = 8 * (A.tab.nparts + 1), jrow_b = 8 * NSP * (NSP + 3), sig_b = 4 * (NSP + 2) + 4 * NSP;
  const size_t per_warp = al(kn_b) + al(scr_b) + al(xs_b) + al(part_b) + al(jrow_b) + al(sig_b) + al(sizeof(CoefShared));
  unsigned char *base = smem_raw + per_warp * warp;
  WarpCell<NSP, false, false> c(A, lane);
  c.kn = reinterpret_cast<double *>(base);
  c.scr = reinterpret_cast<double *>(base + al(kn_b));
  c.xs = reinterpret_cast<double *>(base + al(kn_b) + al(scr_b));
  c.part = reinterpret_cast<double *>(base + al(kn_b) + al(scr_b) + al(xs_b));
  c.jrow = reinterpret_cast<double *>(base + al(kn_b) + al(scr_b) + al(xs_b) + al(part_b));
  c.sig = reinterpret_cast<float *>(base + al(kn_b) + al(scr_b) + al(xs_b) + al(part_b) + al(jrow_b));
  c.perm = reinterpret_cast<int *>(c.sig + NSP + 2);
  c.ws = reinterpret_cast<CoefShared *>(base + al(kn_b) + al(scr_b) + al(xs_b) + al(part_b) + al(jrow_b) + al(sig_b));
  c.rtol = A.reltol;
  c.mxstep = A.mxstep;
  c.max_total_steps = A.max_total_steps;
  c.atol = A.abstol;
  c.cx = (lane < NSP) ? __ldg(&A.tab.xe_coef[lane]) : 0.0;
  for (int s = blockIdx.x * (blockDim.x >> 5) + warp; s < nstate; s += gridDim.x * (blockDim.x >> 5)) {
    const double n_H = A.density[s];
    for (int r = lane; r < nreac; r += kWarp) c.kn[r] = A.rate[(size_t)s * nreac + r] * (A.tab.nh_mask[r] != 0.0 ? n_H : 1.0);
    if (lane == 0) { c.xs[NSP + 1] = 1.0; c.part[A.tab.nparts] = 0.0; }
    __syncwarp();
    const double yv = (lane < NSP) ? x[(size_t)s * NSP + lane] : 0.0;
    if (mode == 0) {
      const double f = c.rhs(yv);
      if (lane < NSP) out[(size_t)s * NSP + lane] = f;
      if (lane == 0 && xe_out) xe_out[s] = c.xe_last;
    } else {
      c.assemble(yv, 1.0, false);
      if (lane < NSP)
#pragma unroll
        for (int j = 0; j < NSP; j++) out[((size_t)s * NSP + lane) * NSP + j] = c.jrow[lane * (NSP + 3) + j];
    }
    __syncwarp();
  }
}

}  // namespace

size_t chem_warp_smem_per_warp(int nsp, int nreac, int nparts, bool mixed, bool zshared) {
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  const size_t mt = mixed ? 4 : 8;
  return al((size_t)nreac * 8) + al((size_t)nreac * (mixed ? 8 : 16)) + al(8 * (nsp + 2)) + al(8 * (nparts + 1)) +
         al(mt * nsp * (nsp + 3)) + al(4 * (nsp + 2) + 4 * nsp) +
         al(sizeof(CoefShared) + (zshared ? 8 * (QMAX + 1) * kWarp : 0));
}

// Launch the persistent warp kernel over `ncell` cells (or the cells listed in
// cell_list).  Returns 0 or a PDR_E_* code.
int launch_chem_warp(const pdr_net *net, int ncell, double *ab, const double *rate, const double *dens,
                     const double *tend, const pdr_chem_opts &o, int *status, int *stats, int *queue,
                     int *fb_list, int *fb_count, const int *cell_list, const int *total_ptr, bool mixed,
                     int sm_count, cudaStream_t st) {
  const WarpTables &T = net->warp;
  if (T.neq != 32) return PDR_E_NET;
  ChemArgs A;
  A.tab = T;
  A.ncell = ncell;
  A.nspec = net->host.nspec;
  A.nreac = net->host.nreac;
  A.abundance = ab;
  A.rate = rate;
  A.density = dens;
  A.t_end_yr = tend;
  A.t_end_default_yr = o.end_time_yr;
  A.start_time_yr = o.start_time_yr;
  A.reltol = o.reltol;
  A.abstol = o.abstol;
  A.mxstep = o.mxstep;
  A.max_total_steps = 500000;
  A.status = status;
  A.stats = stats;
  A.cell_list = cell_list;
  A.queue = queue;
  A.fallback_list = fb_list;
  A.fallback_count = fb_count;
  // refill 2 (one warp per cell, no persistence) applies to the pass over
  // all cells; the FP64 pass over a device-side list keeps the work queue
  const bool one_per_cell = (o.refill == 2) && !cell_list;
  A.refill_static = (o.refill == 1 || one_per_cell) ? 1 : 0;
  // defaults, the fastest shapes measured on GB300: mixed 128 registers with
  // 8-warp blocks (16 warps/SM), FP64 168 registers with 4-warp blocks
  const int rv = (o.reg_variant >= 0 && o.reg_variant <= 3) ? o.reg_variant : (mixed ? 1 : 2);
  const int wpb = o.warps_per_block > 0 ? o.warps_per_block : ((rv >= 2) ? 4 : 8);
  if (wpb > 8) return PDR_E_ARG;
  if (rv >= 2 && wpb > 4) return PDR_E_ARG;   // those variants launch at most 128 threads per block
  const bool zsh = (rv == 1 || rv == 3);
  const size_t smem = chem_warp_smem_per_warp(32, A.nreac, T.nparts, mixed, zsh) * wpb;
  const int variant = (mixed ? 4 : 0) + rv;
  using KFn = void (*)(ChemArgs, int, const int *);
  static const KFn kernels[8] = {chem_warp_kernel<32, false, 0>, chem_warp_kernel<32, false, 1>,
                                 chem_warp_kernel<32, false, 2>, chem_warp_kernel<32, false, 3>,
                                 chem_warp_kernel<32, true, 0>,  chem_warp_kernel<32, true, 1>,
                                 chem_warp_kernel<32, true, 2>,  chem_warp_kernel<32, true, 3>};
  // The dynamic shared-memory limit is an attribute of the function on each
  // device: it only ever grows (to the largest block size used so far on that
  // device), so that a launch with fewer warps never lowers it below what
  // another block size needs.  The occupancy is cached per (device, variant,
  // block size); calls made while a stream is being captured then issue no
  // attribute changes.
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  dev &= 63;
  static std::mutex mu;
  static size_t attr_smem[64][8] = {};
  static int cached_per_sm[64][8][9] = {};
  static size_t cached_smem[64][8][9] = {};
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (smem > attr_smem[dev][variant]) {
      e = cudaFuncSetAttribute(kernels[variant], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
      attr_smem[dev][variant] = smem;
    }
    if (cached_smem[dev][variant][wpb] != smem) {
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cached_per_sm[dev][variant][wpb], kernels[variant], wpb * 32,
                                                        smem);
      if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
      cached_smem[dev][variant][wpb] = smem;
    }
    per_sm = cached_per_sm[dev][variant][wpb];
  }
  if (o.blocks_per_sm > 0 && o.blocks_per_sm < per_sm) per_sm = o.blocks_per_sm;
  if (per_sm < 1) per_sm = 1;
  const int grid = one_per_cell ? (ncell + wpb - 1) / wpb : sm_count * per_sm;
  kernels[variant]<<<grid, wpb * 32, smem, st>>>(A, ncell, total_ptr);
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "chem_warp_kernel launch");
}

}  // namespace pdr

namespace pdr {
int launch_chem_eval(const pdr_net *net, int nstate, const double *x, const double *rate, const double *dens,
                     double *out, double *xe_out, int mode, cudaStream_t st) {
  const WarpTables &T = net->warp;
  if (T.neq != 32) return PDR_E_NET;
  ChemArgs A{};
  A.tab = T;
  A.nspec = net->host.nspec;
  A.nreac = net->host.nreac;
  A.rate = rate;
  A.density = dens;
  A.reltol = 1e-8;
  A.abstol = 1e-30;
  const size_t smem = chem_warp_smem_per_warp(32, A.nreac, T.nparts, false, false) * 4;
  auto k = eval_kernel<32>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(eval)");
  k<<<(nstate + 3) / 4, 128, smem, st>>>(A, nstate, x, out, xe_out, mode);
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "eval_kernel launch");
}
}  // namespace pdr
