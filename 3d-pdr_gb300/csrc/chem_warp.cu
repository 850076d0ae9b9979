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
//               setup, and the Nordsieck columns z2..z5 are FP32; the state,
//               z1, RHS, Newton residual and error test stay FP64.  A cell
//               whose Newton iteration keeps failing with a fresh FP32 matrix
//               is queued and re-solved from its inputs in FP64.
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
  // work-queue mode: SMs the launch may keep (device word, read between
  // cells; null: all).  Blocks beyond limit * gridDim.x / grid_sms take no
  // further cells, so a later launch on another stream gets their SMs.
  const int *sm_limit;
  int grid_sms;             // SMs the grid was sized for
};

// true when this block is beyond the launch's current SM allowance
__device__ __forceinline__ bool over_sm_limit(const int *sm_limit, int grid_sms) {
  if (!sm_limit) return false;
  const int lim = *reinterpret_cast<const volatile int *>(sm_limit);
  return (long long)blockIdx.x * grid_sms >= (long long)lim * gridDim.x;
}

// byte offsets of one warp's shared arrays (host and device agree)
struct WarpLayout {
  size_t kn, scr, xs, part, jrow, sig, ws, total;
};

__host__ __device__ inline WarpLayout warp_layout(int nsp, const WarpTables &T, bool mixed, bool zsh) {
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  WarpLayout L;
  size_t o = 0;
  L.kn = o; o += al(8 * (size_t)(T.nkn + 1));   // rate constants, extras, a zero
  // scr: the RHS operands (FP64) or the two Jacobian scatter buffers (FP32 or FP64 each)
  size_t scr = (size_t)T.nreac * (mixed ? 8 : 16);
  if (8 * (size_t)T.nop > scr) scr = 8 * (size_t)T.nop;
  L.scr = o; o += al(scr);
  L.xs = o; o += al(8 * (size_t)(nsp + 2));
  L.part = o; o += al(8 * (size_t)(T.nparts + 1));
  L.jrow = o; o += al((mixed ? 4 : 8) * (size_t)nsp * (nsp + 1));
  L.sig = o; o += al(4 * (size_t)(nsp + 2) + 4 * (size_t)nsp + 4 * (size_t)(nsp + 2));   // sig, perm, xs32
  // the Nordsieck rows when they live in shared memory: six FP64 columns, or
  // in the mixed form two FP64 and four FP32 columns
  L.ws = o; o += al(sizeof(CoefShared) + (zsh ? (mixed ? 2 * 8 + 4 * 4 : 8 * (QMAX + 1)) * kWarp : 0));
  L.total = o;
  return L;
}

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
      // four columns at a time, every load before any store (the compiler
      // cannot tell the pivot row and this row apart)
      int j = k + 1;
      for (; j + 4 <= N; j += 4) {
        const MT p0 = prow[j], p1 = prow[j + 1], p2 = prow[j + 2], p3 = prow[j + 3];
        const MT r0 = row[j], r1 = row[j + 1], r2 = row[j + 2], r3 = row[j + 3];
        row[j] = fma(-l, p0, r0);
        row[j + 1] = fma(-l, p1, r1);
        row[j + 2] = fma(-l, p2, r2);
        row[j + 3] = fma(-l, p3, r3);
      }
      for (; j < N; j++) row[j] = fma(-l, prow[j], row[j]);
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
  // Newton-matrix row stride: the species columns and the x_e column (odd, so
  // the rows of a warp fall in distinct banks)
  static constexpr int LDJ = NSP + 1;
  const ChemArgs &A;
  const int lane;
  const bool owns;
  const double inv_n = 1.0 / NSP;
  // shared-memory views of this warp
  double *kn, *scr, *xs, *part;
  MT *jrow;       // [NSP][NSP+3] Newton matrix rows / their LU factors
  float *sig;     // [NSP+2] column scales (mixed)
  int *perm;      // [NSP] pivot lane of each elimination step
  float *xs32;    // [NSP+2] FP32 copy of the slot values at setup (mixed)
  double cx;      // electron-sum coefficient of species `lane`
  int cxi;        // the same as an integer
  bool cx_unit;   // every coefficient of the network is -1, 0 or 1 (warp-uniform)
  int mystep;
  MT invd;
  double wsc, ssc;      // FP64 form: setup-time weight and its inverse
  float wsc32, ssc32;   // mixed form: the same in FP32 (the scaling of the FP32 matrix)

  __device__ __forceinline__ WarpCell(const ChemArgs &a, int ln) : A(a), lane(ln), owns(ln < NSP) {}
  __device__ __forceinline__ bool leader() const { return lane == 0; }
  __device__ __forceinline__ void sync() const { __syncwarp(); }
  __device__ __forceinline__ double sum_all(double v) const { return warp_sum(v); }
  __device__ __forceinline__ float sum_all(float v) const { return warp_sum(v); }
  __device__ __forceinline__ double max_all(double v) const { return warp_max(v); }

  __device__ __forceinline__ void set_xe_coef() {
    cx = owns ? __ldg(&A.tab.xe_coef[lane]) : 0.0;
    cxi = (int)cx;
    cx_unit = __all_sync(FULL, cx == (double)cxi && cxi >= -1 && cxi <= 1);
  }
  // this lane's term c_i x_i of x_e: a sign select when the coefficients are
  // -1, 0 or 1 (every FP64 warp instruction costs an FP64 issue slot)
  __device__ __forceinline__ double xe_term(double yv) const {
    if (cx_unit) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(yv);
      return (!owns || cxi == 0) ? 0.0 : __longlong_as_double((long long)(cxi < 0 ? (b ^ 0x8000000000000000ull) : b));
    }
    return owns ? cx * yv : 0.0;
  }

  // point the warp's arrays into its shared-memory slice
  __device__ __forceinline__ void bind(unsigned char *base, const WarpLayout &L) {
    kn = reinterpret_cast<double *>(base + L.kn);
    scr = reinterpret_cast<double *>(base + L.scr);
    xs = reinterpret_cast<double *>(base + L.xs);
    part = reinterpret_cast<double *>(base + L.part);
    jrow = reinterpret_cast<MT *>(base + L.jrow);
    sig = reinterpret_cast<float *>(base + L.sig);
    perm = reinterpret_cast<int *>(sig + NSP + 2);
    xs32 = reinterpret_cast<float *>(perm + NSP);
    this->ws = reinterpret_cast<CoefShared *>(base + L.ws);
  }

  // per-cell rate constants kn_r = k_r (times n_H for the terms that carry
  // it), the extras |nu| kn_r of the RHS terms with |nu| > 1, a zero for the
  // padding terms, and the constants of the slot and partial-sum arrays
  __device__ __forceinline__ void load_rates(const double *rate, double n_H) {
    const WarpTables &T = A.tab;
    for (int r = lane; r < T.nreac; r += kWarp) kn[r] = __ldg(&rate[r]) * (__ldg(&T.nh_mask[r]) != 0.0 ? n_H : 1.0);
    if (lane == 0) {
      kn[T.nkn] = 0.0;
      xs[NSP + 1] = 1.0;
      part[T.nparts] = 0.0;
    }
    __syncwarp();
    for (int e = lane; e < T.nkext; e += kWarp) {
      double k = 0.0;
      for (int q = __ldg(&T.kext_ptr[e]); q < __ldg(&T.kext_ptr[e + 1]); q++) {
        const int2 rn = __ldg(&T.kext_rn[q]);
        k = fma((double)rn.y, kn[rn.x], k);
      }
      kn[T.nreac + e] = k;
    }
    __syncwarp();
  }

  // f(y): returns f_lane, records x_e of this call.  The operands are this
  // state's slot values and the products x_a x_b of the two-body reactant
  // pairs (one FP64 multiply per pair instead of two per reaction); every
  // stoichiometric term is then one FMA with the signed rate constant.
  __device__ __forceinline__ double rhs(double yv) {
    const WarpTables &T = A.tab;
    double *P = scr;
    if (owns) P[lane] = yv;
    const double xe = warp_sum(xe_term(yv));
    if (lane == 0) {
      P[NSP] = xe;
      P[NSP + 1] = 1.0;
    }
    this->xe_last = xe;
    __syncwarp();
    for (int p = lane; p < T.npairs; p += kWarp) {
      const int2 ab = __ldg(&T.pairs[p]);
      P[NSP + 2 + p] = P[ab.x] * P[ab.y];
    }
    __syncwarp();
    double s = 0.0;
#pragma unroll 2
    for (int t = 0; t < T.rhs_len; t++) {
      const int2 d = __ldg(&T.rhs_t[t * kWarp + lane]);
      const double k = kn[d.x & 0xffff];
      // nu kn_r with nu = +-1 (|nu| > 1 reads its extra constant): the sign
      // bit of kn_r flipped in the integer pipe
      const double ks = __hiloint2double(__double2hiint(k) ^ (d.y & (int)0x80000000u), __double2loint(k));
      s = fma(ks, P[d.y & 0x7fffffff], s);
      const int fl = (int)((unsigned)d.x >> 16) - 1;
      if (fl >= 0) { part[fl] = s; s = 0.0; }
    }
    __syncwarp();
    double f = part[__ldg(&T.plist[lane])];
    for (int k = 1; k < T.plist_len; k++) f += part[__ldg(&T.plist[k * kWarp + lane])];
    __syncwarp();
    this->nfe++;
    return owns ? f : 0.0;
  }

  // Jacobian rows at y, times rf, plus the identity when `identity`:
  // FP64 m = rf*J (+I); mixed m = rf * W J W^-1 (+I), W = diag(1/(rtol|y|+atol))
  __device__ __forceinline__ void assemble(double yv, double rf_d, bool identity) {
    const WarpTables &T = A.tab;
    if (owns) xs[lane] = yv;
    const double xe = warp_sum(xe_term(yv));
    if (lane == 0) xs[NSP] = xe;
    if constexpr (MIXED) {
      // column scales 1/w_j = rtol|y_j|+atol, normalised by atol so they fit
      // FP32, formed in FP32 (the matrix is FP32; y and x_e converted once)
      const float y32 = (float)yv;
      ssc32 = fmaf(this->rtol32, fabsf(y32), this->atol32);
      wsc32 = __frcp_rn(ssc32);
      if (owns) {
        sig[lane] = ssc32 * __frcp_rn(this->atol32);
        xs32[lane] = y32;
      }
      if (lane == 0) {
        sig[NSP] = 1.0f;
        sig[NSP + 1] = 0.0f;
        xs32[NSP] = (float)xe;
        xs32[NSP + 1] = 1.0f;
      }
    }
    __syncwarp();
    MT *Da = reinterpret_cast<MT *>(scr);
    MT *Db = Da + T.nreac;
    for (int r = lane; r < T.nreac; r += kWarp) {
      const int2 ab = __ldg(&T.rab[r]);
      if constexpr (MIXED) {
        // dphi_r/dx_a and dphi_r/dx_b, column-scaled, in FP32: one conversion
        // of the rate constant per reaction
        const float k32 = (float)kn[r];
        Da[r] = k32 * (xs32[ab.y] * sig[ab.x]);
        Db[r] = k32 * (xs32[ab.x] * sig[ab.y]);
      } else {
        const double k = kn[r];
        Da[r] = k * xs[ab.y];
        Db[r] = (ab.y == NSP + 1) ? 0.0 : k * xs[ab.x];
      }
    }
    MT *row = jrow + lane * (LDJ);
    if (owns)
      for (int j = 0; j < LDJ; j++) row[j] = MT(0);
    __syncwarp();
    // term-parallel: the (row, column) contributions nu * dphi_r/dx_col sorted
    // by entry and cut into 32 balanced chunks; a lane sums each run of one
    // entry in a register and stores it, and a run that crosses a chunk
    // boundary leaves partials in slots (the RHS partial-sum buffer, free
    // here) that a second pass adds in chunk order.  The rows of the electron
    // and hydrogen hold most contributions: walking one row per lane left the
    // warp waiting on those two lanes.
    {
      MT *slots = reinterpret_cast<MT *>(part);
      MT s = MT(0);
#pragma unroll 2
      for (int t = 0; t < T.hlen; t++) {
        const int2 xy = __ldg(&T.h_xy[t * kWarp + lane]);
        const int x = xy.x, y = xy.y;
        MT nu;
        if constexpr (MIXED) nu = (MT)(x >> 19);
        else nu = __ldg(&T.h_nu[t * kWarp + lane]);
        const int r = x & 0xffff;
        s = fma(nu, (x & 0x10000) ? Db[r] : Da[r], s);
        const int kind = (x >> 17) & 3;
        if (kind == 1) {
          jrow[(y & 0xff) * (LDJ) + ((y >> 8) & 0xff)] = s;
          s = MT(0);
        } else if (kind == 2) {
          slots[y >> 16] = s;
          s = MT(0);
        }
      }
      __syncwarp();
      for (int b = lane; b < T.nbnd; b += kWarp) {
        const int tt = __ldg(&T.bnd_t[b]), ss = __ldg(&T.bnd_s[b]);
        MT acc = MT(0);
        for (int q = ss & 0xffff; q < (ss >> 16); q++) acc += slots[q];
        jrow[(tt & 0xff) * (LDJ) + ((tt >> 8) & 0xff)] = acc;
      }
      __syncwarp();
    }
    const MT e = owns ? row[NSP] : MT(0);
    MT rf;
    if constexpr (MIXED) rf = (MT)rf_d * (wsc32 * this->atol32);   // row weight, normalised like the columns
    else rf = (MT)rf_d;
#pragma unroll 4
    for (int j = 0; j < NSP; j++) {
      MT cj;
      if constexpr (MIXED) cj = __ldg(&T.xe_coef_f[j]);
      else cj = __ldg(&T.xe_coef[j]);
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
    const bool ok = lu_rows<NSP, MT>(jrow, LDJ, lane, mystep, invd, perm);
    const MT *row = jrow + lane * (LDJ);
    bool finite = true;
    if (owns)
      for (int j = 0; j < NSP; j++) finite &= isfinite(row[j]);
    finite = __all_sync(FULL, finite);
    this->after_setup();
    return ok && finite;
  }

  __device__ __forceinline__ double solve(double b) {
    const double x = lu_solve_rows<NSP, double>(jrow, LDJ, lane, mystep, invd, b, perm);
    return owns ? x : 0.0;
  }

  // mixed form: the residual is converted once and scaled in FP32 (the
  // scaling of the FP32 matrix), the correction comes back times ssc*gscale,
  // in FP32 for the norm and in FP64 for the state
  __device__ __forceinline__ double solve32(double b, float gs, float &x32) {
    const float xv = lu_solve_rows<NSP, float>(jrow, LDJ, lane, mystep, invd, (float)b * wsc32, perm);
    x32 = owns ? xv * (ssc32 * gs) : 0.0f;
    return (double)x32;
  }

  // calculate_abundances.c:132-317 for one cell
  __device__ __forceinline__ void run(int cell) {
    const int nspec = A.nspec;
    double *ab = A.abundance + (size_t)cell * nspec;
    this->rtol = A.reltol;
    this->atol = A.abstol;
    this->mxstep = A.mxstep;
    this->max_total_steps = A.max_total_steps;
    set_xe_coef();
    load_rates(A.rate + (size_t)cell * A.nreac, A.density[cell]);
    this->clear_row(owns ? ab[lane] : 0.0);
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
  constexpr bool ZSH = RegVariant<RV>::zsh;
  const WarpLayout L = warp_layout(NSP, A.tab, MIXED, ZSH);
  WarpCell<NSP, MIXED, ZSH> c(A, lane);
  c.bind(smem_raw + L.total * warp, L);
  if constexpr (ZSH) c.z.bind(reinterpret_cast<unsigned char *>(c.ws) + sizeof(CoefShared), lane, kWarp);
  // the uniform-history coefficient table, one copy per block
  __shared__ CoefUniform uni;
  c.wu = &uni;
  if (warp == 0) c.build_uniform_table();
  __syncthreads();
  if (total_ptr) total_cells = *total_ptr;
  const int gwarp = blockIdx.x * (blockDim.x >> 5) + warp, nwarps = gridDim.x * (blockDim.x >> 5);
  for (int k = 0;; k++) {
    int idx = 0;
    if (A.refill_static) {
      idx = gwarp + k * nwarps;
    } else {
      if (lane == 0) idx = over_sm_limit(A.sm_limit, A.grid_sms) ? 0x7fffffff : atomicAdd(A.queue, 1);
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
  const WarpLayout L = warp_layout(NSP, A.tab, false, false);
  WarpCell<NSP, false, false> c(A, lane);
  c.bind(smem_raw + L.total * warp, L);
  c.rtol = A.reltol;
  c.mxstep = A.mxstep;
  c.max_total_steps = A.max_total_steps;
  c.atol = A.abstol;
  c.set_xe_coef();
  for (int s = blockIdx.x * (blockDim.x >> 5) + warp; s < nstate; s += gridDim.x * (blockDim.x >> 5)) {
    c.load_rates(A.rate + (size_t)s * A.nreac, A.density[s]);
    const double yv = (lane < NSP) ? x[(size_t)s * NSP + lane] : 0.0;
    if (mode == 0) {
      const double f = c.rhs(yv);
      if (lane < NSP) out[(size_t)s * NSP + lane] = f;
      if (lane == 0 && xe_out) xe_out[s] = c.xe_last;
    } else {
      c.assemble(yv, 1.0, false);
      if (lane < NSP)
#pragma unroll
        for (int j = 0; j < NSP; j++) out[((size_t)s * NSP + lane) * NSP + j] = c.jrow[lane * WarpCell<NSP, false, false>::LDJ + j];
    }
    __syncwarp();
  }
}

}  // namespace

size_t chem_warp_smem_per_warp(const WarpTables &T, bool mixed, bool zshared) {
  return warp_layout(T.neq, T, mixed, zshared).total;
}

// Launch the persistent warp kernel over `ncell` cells (or the cells listed in
// cell_list).  Returns 0 or a PDR_E_* code.
int launch_chem_warp(const pdr_net *net, int ncell, double *ab, const double *rate, const double *dens,
                     const double *tend, const pdr_chem_opts &o, int *status, int *stats, int *queue,
                     int *fb_list, int *fb_count, const int *cell_list, const int *total_ptr, bool mixed,
                     int sm_count, cudaStream_t st, const int *sm_limit) {
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
  A.sm_limit = sm_limit;
  A.grid_sms = sm_count;
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
  const size_t smem = chem_warp_smem_per_warp(T, mixed, zsh) * wpb;
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
  const size_t smem = chem_warp_smem_per_warp(T, false, false) * 4;
  auto k = eval_kernel<32>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(eval)");
  k<<<(nstate + 3) / 4, 128, smem, st>>>(A, nstate, x, out, xe_out, mode);
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "eval_kernel launch");
}
}  // namespace pdr
