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
#include <type_traits>

#include "pdr_internal.h"

namespace pdr {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int QMAX = 5;
constexpr int MXNCF = 10, MXNEF = 7, MXNEF1 = 3, SMALL_NEF = 2, LONG_WAIT = 10, SMALL_NST = 10;
constexpr int MAXCOR = 3, MSBP = 20;
constexpr double CRDOWN = 0.3, DGMAX = 0.3, RDIV = 2.0, NLSCOEF = 0.1;
constexpr double ETAMX1 = 10000.0, ETAMX2 = 10.0, ETAMX3 = 10.0, ETAMXF = 0.2, ETAMIN = 0.1;
constexpr double ETACF = 0.25, ADDON = 1e-6, BIAS1 = 6.0, BIAS2 = 6.0, BIAS3 = 10.0, THRESH = 1.5;
constexpr double YEAR = 3.1556926e7;
constexpr int FELL_BACK = 1;   // internal status: redo this cell in FP64

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
};

// per-warp shared memory header (arrays of the integrator that all lanes read)
struct WarpShared {
  double tau[QMAX + 2];
  double l[QMAX + 1];
  double tq[6];
  // coefficients of a uniform step history (xi_j = j), per order 1..5:
  // l[0..5], tq[1..5] (tq[1], tq[3] as computed when an order change is due)
  double ul[QMAX + 1][QMAX + 1];
  double utq[QMAX + 1][6];
};

// squared-norm form of the step-ratio formula eta = 1/((bias*e)^(1/k) + 1e-6)
// with e2 = e^2; evaluated in FP32 (a heuristic factor, clamped afterwards)
__device__ __forceinline__ double eta_of(double e2, float bias, int k) {
  const float v = powf(bias * bias * (float)e2, 0.5f / (float)k);
  return 1.0 / ((double)v + ADDON);
}

// 1/x to double precision: FP32 seed and two Newton steps
__device__ __forceinline__ double rcp_nr(double x) {
  double r = (double)__frcp_rn((float)x);
  r = r * fma(-x, r, 2.0);
  r = r * fma(-x, r, 2.0);
  return r;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
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

// In-register LU with partial pivoting, lane = row.  m[] holds row `lane`;
// on exit m[j<step] are the multipliers, m[j>=step] the U row, mystep the
// elimination step at which this row was the pivot, invd 1/diagonal.
template <int N, class MT>
__device__ __forceinline__ bool lu_rows(MT (&m)[N], int lane, int &mystep, MT &invd) {
  mystep = (lane < N) ? -1 : N;
#pragma unroll
  for (int k = 0; k < N; k++) {
    const bool cand = (mystep < 0);
    const int p = argmax_lane(cand ? fabs(m[k]) : MT(0), cand);
    if (p < 0) return false;
    const MT u = bcast(m[k], p);
    MT rinv;
    if constexpr (sizeof(MT) == 8) rinv = __drcp_rn(u);
    else rinv = __frcp_rn(u);
    if (lane == p) { mystep = k; invd = rinv; }
    const bool upd = (mystep < 0);
    const MT l = m[k] * rinv;
    if (upd) m[k] = l;
#pragma unroll
    for (int j = k + 1; j < N; j++) {
      const MT pv = bcast(m[j], p);
      if (upd) m[j] = fma(-l, pv, m[j]);
    }
  }
  return true;
}

// Solve with the row-distributed LU: b is this lane's right-hand-side entry
// (row `lane`), the solution component for column `lane` is returned.
template <int N, class MT>
__device__ __forceinline__ MT lu_solve_rows(const MT (&m)[N], int lane, int mystep, MT invd, MT b) {
  // forward: L y = P b
#pragma unroll
  for (int k = 0; k < N; k++) {
    const int p = __ffs(__ballot_sync(FULL, mystep == k)) - 1;
    const MT yk = bcast(b, p);
    if (mystep > k) b = fma(-m[k], yk, b);
  }
  // backward: U x = y
  MT x = MT(0);
#pragma unroll
  for (int k = N - 1; k >= 0; k--) {
    const int p = __ffs(__ballot_sync(FULL, mystep == k)) - 1;
    const MT xk = bcast(b * invd, p);
    if (lane == k) x = xk;
    if (mystep < k) b = fma(-m[k], xk, b);
  }
  return x;
}

template <int NSP, bool MIXED>
struct Cell {
  using MT = typename std::conditional<MIXED, float, double>::type;
  const ChemArgs &A;
  const int lane;
  // shared-memory views of this warp
  double *kn, *scr, *xs, *part;
  MT *jrow;       // [NSP][NSP+3]
  float *sig;     // [NSP+2] column scales (mixed)
  WarpShared *ws;
  // network constants of this lane
  double cx;      // electron-sum coefficient of species `lane`
  // Nordsieck state (row `lane`)
  double z[QMAX + 1];
  double ewt, acor, y, ftmp, tmp;
  // Newton matrix
  MT m[NSP];
  int mystep;
  MT invd;
  double wsc, ssc;   // setup-time weight and its inverse (mixed scaling)
  // uniform integrator scalars
  double tn, h, hscale, hprime, eta, etamax, saved_tq5, gamma, gammap, gamrat, gscale, rl1;
  double crate2, acnrm2;   // squared convergence rate and squared WRMS norm of the correction
  double xe_last, rtol, atol;
  int q, qprime, qwait, jcur;
  long long nst, nstlp, nfe, nje, nsetups, nni, ncfn, netf;
  bool fell_back;

  __device__ __forceinline__ Cell(const ChemArgs &a, int ln) : A(a), lane(ln) {}

  // squared WRMS norm (sum of squares / n); the tests compare squares, so no sqrt
  __device__ __forceinline__ double wrms2(double v) const {
    double t = (lane < NSP) ? v * ewt : 0.0;
    return warp_sum(t * t) * (1.0 / NSP);
  }

  __device__ __forceinline__ void set_ewt() { ewt = (lane < NSP) ? rcp_nr(rtol * fabs(z[0]) + atol) : 0.0; }

  // f(y): returns f_lane, records x_e of this call
  __device__ __forceinline__ double rhs(double yv) {
    const WarpTables &T = A.tab;
    if (lane < NSP) xs[lane] = yv;
    const double xe = warp_sum(lane < NSP ? cx * yv : 0.0);
    if (lane == 0) xs[NSP] = xe;
    xe_last = xe;
    __syncwarp();
    for (int r = lane; r < T.nreac; r += kWarp) {
      const int2 ab = __ldg(&T.rab[r]);
      scr[r] = kn[r] * xs[ab.x] * xs[ab.y];
    }
    __syncwarp();
    double s = 0.0;
    for (int t = 0; t < T.rhs_len; t++) {
      const int r = __ldg(&T.rhs_r[t * kWarp + lane]);
      const double nu = __ldg(&T.rhs_nu[t * kWarp + lane]);
      const int fl = __ldg(&T.rhs_flush[t * kWarp + lane]);
      s = fma(nu, scr[r], s);
      if (fl >= 0) { part[fl] = s; s = 0.0; }
    }
    __syncwarp();
    double f = 0.0;
    for (int k = 0; k < T.plist_len; k++) f += part[__ldg(&T.plist[k * kWarp + lane])];
    __syncwarp();
    nfe++;
    return (lane < NSP) ? f : 0.0;
  }

  // Jacobian rows at y, times rf, plus the identity when `identity`:
  // FP64 m = rf*J (+I); mixed m = rf * W J W^-1 (+I), W = diag(1/(rtol|y|+atol))
  __device__ __forceinline__ void assemble(double yv, double rf_d, bool identity) {
    const WarpTables &T = A.tab;
    if (lane < NSP) xs[lane] = yv;
    const double xe = warp_sum(lane < NSP ? cx * yv : 0.0);
    if (lane == 0) xs[NSP] = xe;
    if constexpr (MIXED) {
      // column scales 1/w_j = rtol|y_j|+atol, normalised by atol so they fit FP32
      ssc = rtol * fabs(yv) + atol;
      wsc = 1.0 / ssc;
      if (lane < NSP) sig[lane] = (float)(ssc / atol);
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
    if (lane < NSP)
      for (int j = 0; j < NSP + 2; j++) row[j] = MT(0);
    __syncwarp();
    if (lane < NSP) {
      for (int t = 0; t < T.jac_len; t++) {
        MT nu;
        if constexpr (MIXED) nu = __ldg(&T.jac_nu_f[t * kWarp + lane]);
        else nu = __ldg(&T.jac_nu[t * kWarp + lane]);
        if (nu == MT(0)) break;
        const int r = __ldg(&T.jac_r[t * kWarp + lane]);
        const int2 ab = __ldg(&T.rab[r]);
        row[ab.x] = fma(nu, Da[r], row[ab.x]);
        row[ab.y] = fma(nu, Db[r], row[ab.y]);
      }
    }
    __syncwarp();
    const MT e = (lane < NSP) ? row[NSP] : MT(0);
    MT rf;
    if constexpr (MIXED) rf = (MT)(rf_d * (wsc * atol));   // row weight, normalised like the columns
    else rf = (MT)rf_d;
#pragma unroll
    for (int j = 0; j < NSP; j++) {
      const MT cj = (MT)__ldg(&T.xe_coef[j]);
      MT v = (lane < NSP) ? row[j] : MT(0);
      if constexpr (MIXED) v = fmaf(e * cj, sig[j], v);
      else v = fma(e, cj, v);
      m[j] = rf * v + ((identity && lane == j) ? MT(1) : MT(0));
    }
    __syncwarp();
  }

  // Newton matrix at y: FP64 M = I - gamma J, or FP32 W M W^-1 (see header)
  __device__ __forceinline__ bool setup(double yv) {
    nje++;
    nsetups++;
    assemble(yv, -gamma, true);
    const bool ok = lu_rows<NSP, MT>(m, lane, mystep, invd);
    bool finite = true;
#pragma unroll
    for (int j = 0; j < NSP; j++) finite &= isfinite(m[j]);
    finite = __all_sync(FULL, finite);
    jcur = 1;
    crate2 = 1.0;
    gammap = gamma;
    gamrat = 1.0;
    gscale = 1.0;
    nstlp = nst;
    return ok && finite;
  }

  __device__ __forceinline__ double solve(double b) {
    double x;
    if constexpr (MIXED) {
      const float xs_ = lu_solve_rows<NSP, float>(m, lane, mystep, invd, (float)(b * wsc));
      x = (double)xs_ * ssc;
    } else {
      x = lu_solve_rows<NSP, double>(m, lane, mystep, invd, b);
    }
    x *= gscale;   // 2/(1+gamma/gamma_setup) for a stale gamma, else 1
    return (lane < NSP) ? x : 0.0;
  }

  // Pascal-triangle prediction z <- z P (and its inverse), q-specialised
  template <int Q, int SIGN>
  __device__ __forceinline__ void pascal() {
#pragma unroll
    for (int k = 1; k <= Q; k++)
#pragma unroll
      for (int j = Q; j >= k; j--) z[j - 1] = (SIGN > 0) ? z[j - 1] + z[j] : z[j - 1] - z[j];
  }
  template <int SIGN>
  __device__ __forceinline__ void pascal_q() {
    switch (q) {
      case 1: pascal<1, SIGN>(); break;
      case 2: pascal<2, SIGN>(); break;
      case 3: pascal<3, SIGN>(); break;
      case 4: pascal<4, SIGN>(); break;
      default: pascal<5, SIGN>(); break;
    }
  }
  __device__ __forceinline__ void predict() {
    tn += h;
    pascal_q<1>();
  }

  __device__ __forceinline__ void restore(double saved_t) {
    tn = saved_t;
    pascal_q<-1>();
  }

  __device__ __forceinline__ void rescale() {
    double fac = eta;
#pragma unroll
    for (int j = 1; j <= QMAX; j++)
      if (j <= q) { z[j] *= fac; fac *= eta; }
    h = hscale * eta;
    hscale = h;
  }

  // order q -> q-1 (see the oracle's decrease_order)
  __device__ __forceinline__ void decrease_order() {
    if (q <= 2) return;
    double d[QMAX + 2];
#pragma unroll
    for (int j = 0; j < QMAX + 2; j++) d[j] = 0.0;
    d[2] = 1.0;
    double hsum = 0.0;
#pragma unroll
    for (int k = 1; k <= QMAX - 2; k++) {
      if (k <= q - 2) {
        hsum += ws->tau[k];
        const double xi = hsum / hscale;
#pragma unroll
        for (int j = QMAX + 1; j >= 1; j--) d[j] = d[j - 1] + d[j] * xi;
        d[0] *= xi;
      }
    }
    double zq = 0.0;
#pragma unroll
    for (int j = 0; j <= QMAX; j++) if (j == q) zq = z[j];
#pragma unroll
    for (int j = 2; j < QMAX; j++)
      if (j < q) z[j] -= d[j] * zq;
  }

  // order q -> q+1 using the saved correction in z[QMAX]
  __device__ __forceinline__ void increase_order() {
    double d[QMAX + 2];
#pragma unroll
    for (int j = 0; j < QMAX + 2; j++) d[j] = 0.0;
    d[2] = 1.0;
    double hsum = hscale, sum_j = 1.0, sum_xi = 1.0, prod = 1.0, xi_prev = 1.0;
#pragma unroll
    for (int k = 2; k <= QMAX; k++) {
      if (k <= q) {
        hsum += ws->tau[k];
        const double xi = hsum / hscale;
        sum_j += 1.0 / k;
        sum_xi += 1.0 / xi;
        prod *= xi;
        // multiply the polynomial by (x + xi_{k-1})
#pragma unroll
        for (int j = QMAX + 1; j >= 1; j--) d[j] = d[j - 1] + d[j] * xi_prev;
        d[0] *= xi_prev;
        xi_prev = xi;
      }
    }
    const double c = (sum_j - sum_xi) / prod;
    const double zn1 = c * z[QMAX];
#pragma unroll
    for (int j = 2; j <= QMAX; j++)
      if (j <= q) z[j] += d[j] * zn1;
#pragma unroll
    for (int j = 2; j <= QMAX; j++)
      if (j == q + 1) z[j] = zn1;
  }

  // Fixed-leading-coefficient BDF coefficients l[0..q] and error constants
  // tq[1..5] for step h and history tau[1..q] (q+1 for tq[3]).
  __device__ __forceinline__ static void coeffs(int q, bool order_change_due, double h, const double *tau,
                                                double *l, double *tq) {
#pragma unroll
    for (int j = 0; j <= QMAX; j++) l[j] = 0.0;
    l[0] = l[1] = 1.0;
    double a0 = -1.0, a0hat = -1.0, xi_inv = 1.0, xistar_inv = 1.0, hsum = h;
    if (q > 1) {
#pragma unroll
      for (int j = 2; j < QMAX; j++) {
        if (j < q) {
          hsum += tau[j - 1];
          xi_inv = h / hsum;
          a0 -= 1.0 / j;
#pragma unroll
          for (int i = QMAX; i >= 1; i--)
            if (i <= j) l[i] += l[i - 1] * xi_inv;
        }
      }
      a0 -= 1.0 / q;
      xistar_inv = -l[1] - a0;
      hsum += tau[q - 1];
      xi_inv = h / hsum;
      a0hat = -l[1] - xi_inv;
#pragma unroll
      for (int i = QMAX; i >= 1; i--)
        if (i <= q) l[i] += l[i - 1] * xistar_inv;
    }
    double lq = 0.0;
#pragma unroll
    for (int j = 0; j <= QMAX; j++) if (j == q) lq = l[j];
    const double A1 = 1.0 - a0hat + a0, A2 = 1.0 + q * A1;
    tq[2] = fabs(A1 / (a0 * A2));
    tq[5] = fabs(A2 * xistar_inv / (lq * xi_inv));
    if (order_change_due) {
      if (q > 1) {
        const double C = xistar_inv / lq, A3 = a0 + 1.0 / q, A4 = a0hat + xi_inv;
        tq[1] = fabs(C * (1.0 - A4 + A3) / A3);
      } else {
        tq[1] = 1.0;
      }
      hsum += tau[q];
      xi_inv = h / hsum;
      const double A5 = a0 - 1.0 / (q + 1), A6 = a0hat - xi_inv;
      tq[3] = fabs(((1.0 - A6 + A5) / A2) / (xi_inv * (q + 2) * A5));
    }
    tq[4] = NLSCOEF / tq[2];
  }

  // the per-warp table of uniform-history coefficients (h = tau_j = 1)
  __device__ __forceinline__ void build_uniform_table() {
    double one[QMAX + 2];
#pragma unroll
    for (int j = 0; j < QMAX + 2; j++) one[j] = 1.0;
    for (int qq = 1; qq <= QMAX; qq++) {
      double l[QMAX + 1], tq[6];
      coeffs(qq, true, 1.0, one, l, tq);
      __syncwarp();
      if (lane == 0) {
        for (int j = 0; j <= QMAX; j++) ws->ul[qq][j] = l[j];
        for (int j = 1; j <= 5; j++) ws->utq[qq][j] = tq[j];
      }
    }
    __syncwarp();
  }

  __device__ __forceinline__ void set_coeffs() {
    // a history of equal steps gives xi_j = j exactly: take the tabulated values
    bool uniform = true;
#pragma unroll
    for (int j = 1; j <= QMAX; j++)
      if (j <= q && ws->tau[j] != h) uniform = false;
    __syncwarp();
    if (uniform) {
      if (lane == 0) {
#pragma unroll
        for (int j = 0; j <= QMAX; j++) ws->l[j] = ws->ul[q][j];
        ws->tq[2] = ws->utq[q][2];
        ws->tq[4] = ws->utq[q][4];
        ws->tq[5] = ws->utq[q][5];
        if (qwait == 1) { ws->tq[1] = ws->utq[q][1]; ws->tq[3] = ws->utq[q][3]; }
      }
    } else {
      double l[QMAX + 1], tq[6];
      tq[1] = ws->tq[1];
      tq[3] = ws->tq[3];
      coeffs(q, qwait == 1, h, ws->tau, l, tq);
      if (lane == 0) {
#pragma unroll
        for (int j = 0; j <= QMAX; j++) ws->l[j] = l[j];
        ws->tq[1] = tq[1]; ws->tq[2] = tq[2]; ws->tq[3] = tq[3]; ws->tq[4] = tq[4]; ws->tq[5] = tq[5];
      }
    }
    __syncwarp();
    rl1 = 1.0 / ws->l[1];
    gamma = h * rl1;
    if (nst == 0) gammap = gamma;
    gamrat = (nst > 0) ? gamma / gammap : 1.0;
    gscale = (gamrat != 1.0) ? 2.0 / (1.0 + gamrat) : 1.0;
  }

  // 0 solved, 1 convergence failure (recoverable), 2 convergence failure that
  // sends a mixed-precision cell to the FP64 pass.  Norms are kept squared:
  // the tests del*min(1,R) <= 0.1/C_err, del > 2 del_prev and R = max(0.3 R,
  // del/del_prev) are evaluated on squares.
  __device__ __forceinline__ int nls(bool prev_fail) {
    bool call_setup = prev_fail || (nst == 0) || (nst >= nstlp + MSBP) || (fabs(gamrat - 1.0) > DGMAX);
    const double tq4 = ws->tq[4];
    const double tq4sq = tq4 * tq4;
    for (int attempt = 0; attempt < 2; attempt++) {
      y = z[0];
      ftmp = rhs(y);
      if (call_setup) {
        if (!setup(y)) return MIXED ? 2 : 1;
        call_setup = false;
      }
      acor = 0.0;
      double delp2 = 0.0;
      int mcor = 0;
      bool conv = false;
      for (;;) {
        tmp = gamma * ftmp - (rl1 * z[1] + acor);
        tmp = solve(tmp);
        nni++;
        const double del2 = wrms2(tmp);
        acor += tmp;
        y = z[0] + acor;
        if (mcor > 0) crate2 = fmax(CRDOWN * CRDOWN * crate2, del2 / delp2);
        if (del2 * fmin(1.0, crate2) <= tq4sq) {
          acnrm2 = (mcor == 0) ? del2 : wrms2(acor);
          jcur = 0;
          conv = true;
          break;
        }
        mcor++;
        if (mcor == MAXCOR || (mcor >= 2 && del2 > RDIV * RDIV * delp2)) break;
        delp2 = del2;
        ftmp = rhs(y);
      }
      if (conv) return 0;
      if (!jcur) { call_setup = true; continue; }
      return MIXED ? 2 : 1;
    }
    return MIXED ? 2 : 1;
  }

  __device__ __forceinline__ void set_eta() {
    if (eta < THRESH) { eta = 1.0; hprime = h; }
    else { eta = fmin(eta, etamax); hprime = h * eta; }
  }

  // one internal step: 0 ok, CVODE flag (<0), or FELL_BACK
  __device__ __forceinline__ int step() {
    const double saved_t = tn;
    int ncf = 0, nef = 0;
    bool prev_fail = false;
    double dsm2 = 0.0;
    if (nst > 0 && hprime != h) {
      if (qprime != q) {
        if (qprime > q) increase_order();
        else decrease_order();
        q = qprime;
        qwait = q + 1;
      }
      rescale();
    }
    for (;;) {
      predict();
      set_coeffs();
      const int r = nls(prev_fail);
      if (r == 2) return FELL_BACK;
      if (r != 0) {
        ncfn++;
        restore(saved_t);
        ncf++;
        etamax = 1.0;
        if (ncf == MXNCF) return PDR_CONV_FAILURE;
        eta = ETACF;
        prev_fail = true;
        rescale();
        continue;
      }
      const double tq2 = ws->tq[2];
      dsm2 = acnrm2 * (tq2 * tq2);
      if (dsm2 <= 1.0) break;
      nef++;
      netf++;
      prev_fail = true;
      restore(saved_t);
      if (nef == MXNEF) return PDR_ERR_FAILURE;
      etamax = 1.0;
      const int L = q + 1;
      if (nef <= MXNEF1) {
        eta = eta_of(dsm2, (float)BIAS2, L);
        eta = fmax(ETAMIN, eta);
        if (nef >= SMALL_NEF) eta = fmin(eta, ETAMXF);
        rescale();
        continue;
      }
      if (q > 1) {
        eta = ETAMIN;
        decrease_order();
        q--;
        qwait = q + 1;
        rescale();
        continue;
      }
      eta = ETAMIN;
      h *= eta;
      hscale = h;
      qwait = LONG_WAIT;
      tmp = rhs(z[0]);
      z[1] = h * tmp;
    }
    // complete the step
    nst++;
    __syncwarp();
    if (lane == 0) {
#pragma unroll
      for (int i = QMAX; i >= 2; i--)
        if (i <= q) ws->tau[i] = ws->tau[i - 1];
      if (q == 1 && nst > 1) ws->tau[2] = ws->tau[1];
      ws->tau[1] = h;
    }
    __syncwarp();
    switch (q) {
#define PDR_CORRECT(Q) case Q: _Pragma("unroll") for (int j = 0; j <= Q; j++) z[j] = fma(ws->l[j], acor, z[j]); break;
      PDR_CORRECT(1) PDR_CORRECT(2) PDR_CORRECT(3) PDR_CORRECT(4) PDR_CORRECT(5)
#undef PDR_CORRECT
    }
    qwait--;
    if (qwait == 1 && q != QMAX) {
      z[QMAX] = acor;
      saved_tq5 = ws->tq[5];
    }
    if (etamax == 1.0) {
      if (qwait < 2) qwait = 2;
      qprime = q;
      hprime = h;
      eta = 1.0;
    } else {
      const int L = q + 1;
      const double etaq = eta_of(dsm2, (float)BIAS2, L);
      if (qwait != 0) {
        eta = etaq;
        qprime = q;
        set_eta();
      } else {
        qwait = 2;
        double etaqm1 = 0.0, etaqp1 = 0.0;
        if (q > 1) {
          double zq = 0.0;
#pragma unroll
          for (int j = 0; j <= QMAX; j++) if (j == q) zq = z[j];
          const double tq1 = ws->tq[1];
          etaqm1 = eta_of(wrms2(zq) * (tq1 * tq1), (float)BIAS1, q);
        }
        if (q != QMAX && saved_tq5 != 0.0) {
          const double ratio = h / ws->tau[2];
          double rp = ratio;
          for (int k = 1; k < L; k++) rp *= ratio;
          const double cquot = (ws->tq[5] / saved_tq5) * rp;
          const double tq3 = ws->tq[3];
          etaqp1 = eta_of(wrms2(acor - cquot * z[QMAX]) * (tq3 * tq3), (float)BIAS3, L + 1);
        }
        const double etam = fmax(etaqm1, fmax(etaq, etaqp1));
        if (etam < THRESH) { eta = 1.0; qprime = q; }
        else if (etam == etaq) { eta = etaq; qprime = q; }
        else if (etam == etaqm1) { eta = etaqm1; qprime = q - 1; }
        else { eta = etaqp1; qprime = q + 1; z[QMAX] = acor; }
        set_eta();
      }
    }
    etamax = (nst <= SMALL_NST) ? ETAMX2 : ETAMX3;
    return 0;
  }

  __device__ __forceinline__ double initial_step(double t0, double tout) {
    const double tdist = fabs(tout - t0);
    const double tround = 2.220446049250313e-16 * fmax(fabs(t0), fabs(tout));
    const double hlb = 100.0 * tround;
    double hub_inv = (lane < NSP) ? fabs(z[1]) / (0.1 * fabs(z[0]) + atol) : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) hub_inv = fmax(hub_inv, __shfl_xor_sync(FULL, hub_inv, o));
    double hub = 0.1 * tdist;
    if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
    double hg = sqrt(hlb * hub);
    if (hub < hlb) return hg;
    bool ok = false;
    double hnew = hg;
    for (int it = 1; it <= 4; it++) {
      tmp = rhs(z[0] + hg * z[1]);
      const double yddnrm = sqrt(wrms2((tmp - z[1]) / hg));
      if (ok || it == 4) { hnew = hg; break; }
      hnew = (yddnrm * hub * hub > 2.0) ? sqrt(2.0 / yddnrm) : sqrt(hg * hub);
      const double hrat = hnew / hg;
      if (hrat > 0.5 && hrat < 2.0) ok = true;
      if (it > 1 && hrat > 2.0) { hnew = hg; ok = true; }
      hg = hnew;
    }
    double h0 = 0.5 * hnew;
    if (h0 < hlb) h0 = hlb;
    if (h0 > hub) h0 = hub;
    return h0;
  }

  __device__ __forceinline__ double interpolate(double t) const {
    const double s = (t - tn) / hscale;
    double v = 0.0;
#pragma unroll
    for (int j = QMAX; j >= 0; j--)
      if (j <= q) v = (j == q) ? z[j] : fma(s, v, z[j]);
    return v;
  }

  // CVode(..., CV_NORMAL) from the current state to tout
  __device__ __forceinline__ int solve_to(double tout, bool first, double t0, long long &total) {
    if (first) {
      set_ewt();
      z[1] = rhs(z[0]);
      const double h0 = initial_step(t0, tout);
      z[1] *= h0;
      h = hscale = hprime = h0;
      q = qprime = 1;
      qwait = 2;
      etamax = ETAMX1;
      nst = 0;
    } else if ((tn - tout) * h >= 0.0) {
      return 0;
    }
    long long nstloc = 0;
    for (;;) {
      if (nst > 0) set_ewt();
      if (nstloc >= A.mxstep || total >= A.max_total_steps) return PDR_TOO_MUCH_WORK;
      const int kf = step();
      if (kf != 0) return kf;
      nstloc++;
      total++;
      if ((tn - tout) * h >= 0.0) return 0;
    }
  }

  // full calculate_abundances.c:132-317 for one cell
  __device__ __forceinline__ void run(int cell) {
    const int nspec = A.nspec;
    double *ab = A.abundance + (size_t)cell * nspec;
    const double n_H = A.density[cell];
    rtol = A.reltol;
    atol = A.abstol;
    cx = (lane < NSP) ? __ldg(&A.tab.xe_coef[lane]) : 0.0;
    // per-cell rate constants, multiplied by n_H for two-body terms
    const double *rate = A.rate + (size_t)cell * A.nreac;
    for (int r = lane; r < A.nreac; r += kWarp) kn[r] = __ldg(&rate[r]) * (__ldg(&A.tab.nh_mask[r]) != 0.0 ? n_H : 1.0);
    if (lane == 0) {
      xs[NSP + 1] = 1.0;
      part[A.tab.nparts] = 0.0;
#pragma unroll
      for (int j = 0; j < QMAX + 2; j++) ws->tau[j] = 0.0;
#pragma unroll
      for (int j = 0; j < 6; j++) ws->tq[j] = 0.0;
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j <= QMAX; j++) z[j] = 0.0;
    z[0] = (lane < NSP) ? ab[lane] : 0.0;
    xe_last = ab[nspec - 1];
    nfe = nje = nsetups = nni = ncfn = netf = 0;
    nst = nstlp = 0;
    saved_tq5 = 0.0;
    crate2 = 1.0;
    gammap = gamma = 1.0;
    gamrat = 1.0;
    gscale = 1.0;
    jcur = 0;
    acor = 0.0;
    const double t0 = A.start_time_yr * YEAR;
    const double tend = (A.t_end_yr ? A.t_end_yr[cell] : A.t_end_default_yr) * YEAR;
    tn = t0;
    double tout = 1.0e-4 * YEAR, t = t0;
    int nfails = 0, status = 0, lastflag = 0;
    long long total = 0;
    bool first = true;
    double tlast = tout;
    do {
      const int flag = solve_to(tout, first, t0, total);
      first = false;
      if (flag == FELL_BACK) {
        if (lane == 0) {
          const int k = atomicAdd(A.fallback_count, 1);
          A.fallback_list[k] = cell;
          A.status[cell] = FELL_BACK;
        }
        return;
      }
      lastflag = flag;
      tlast = tout;
      if (flag != 0) {
        nfails++;
        if (!((flag == PDR_TOO_MUCH_WORK || flag == PDR_CONV_FAILURE) && nfails < 5)) {
          status = flag;
          if (flag != PDR_TOO_MUCH_WORK && flag != PDR_CONV_FAILURE) nfails = 5;
        }
        if (total >= A.max_total_steps) { status = PDR_TOO_MUCH_WORK; nfails = 5; }
        t = tn;
      } else {
        t = tout;
      }
      tout = tout * 10.0;
      if (tout > tend) tout = tend;
    } while (t < tout && nfails < 5);
    double yv = (lastflag == 0) ? interpolate(tlast) : z[0];
    if (yv < atol) yv = 0.0;
    if (lane < NSP) ab[lane] = yv;
    if (lane == 0) {
      ab[nspec - 1] = xe_last;
      A.status[cell] = status;
      if (A.stats) {
        int *s = A.stats + (size_t)cell * 8;
        s[0] = (int)nst; s[1] = (int)nfe; s[2] = (int)nje; s[3] = (int)nsetups;
        s[4] = (int)nni; s[5] = (int)ncfn; s[6] = (int)netf; s[7] = MIXED ? 0 : (A.cell_list ? 1 : 0);
      }
    }
  }
};

template <int NSP, bool MIXED>
__global__ void __launch_bounds__(256, 1) chem_warp_kernel(const __grid_constant__ ChemArgs A, int total_cells, const int *total_ptr) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using MT = typename std::conditional<MIXED, float, double>::type;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nreac = A.nreac;
  // per-warp shared layout
  const size_t kn_b = (size_t)nreac * 8, scr_b = (size_t)nreac * 16, xs_b = 8 * (NSP + 2);
  const size_t part_b = 8 * (A.tab.nparts + 1);
  const size_t jrow_b = sizeof(MT) * NSP * (NSP + 3), sig_b = 4 * (NSP + 2);
  const size_t ws_b = sizeof(WarpShared);
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  const size_t per_warp = al(kn_b) + al(scr_b) + al(xs_b) + al(part_b) + al(jrow_b) + al(sig_b) + al(ws_b);
  unsigned char *base = smem_raw + per_warp * warp;
  Cell<NSP, MIXED> c(A, lane);
  c.kn = reinterpret_cast<double *>(base);
  c.scr = reinterpret_cast<double *>(base + al(kn_b));
  c.xs = reinterpret_cast<double *>(base + al(kn_b) + al(scr_b));
  c.part = reinterpret_cast<double *>(base + al(kn_b) + al(scr_b) + al(xs_b));
  c.jrow = reinterpret_cast<MT *>(base + al(kn_b) + al(scr_b) + al(xs_b) + al(part_b));
  c.sig = reinterpret_cast<float *>(base + al(kn_b) + al(scr_b) + al(xs_b) + al(part_b) + al(jrow_b));
  c.ws = reinterpret_cast<WarpShared *>(base + al(kn_b) + al(scr_b) + al(xs_b) + al(part_b) + al(jrow_b) + al(sig_b));
  c.build_uniform_table();
  if (total_ptr) total_cells = *total_ptr;
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(A.queue, 1);
    idx = __shfl_sync(FULL, idx, 0);
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
  const size_t part_b = 8 * (A.tab.nparts + 1), jrow_b = 8 * NSP * (NSP + 3), sig_b = 4 * (NSP + 2);
  const size_t per_warp = al(kn_b) + al(scr_b) + al(xs_b) + al(part_b) + al(jrow_b) + al(sig_b) + al(sizeof(WarpShared));
  unsigned char *base = smem_raw + per_warp * warp;
  Cell<NSP, false> c(A, lane);
  c.kn = reinterpret_cast<double *>(base);
  c.scr = reinterpret_cast<double *>(base + al(kn_b));
  c.xs = reinterpret_cast<double *>(base + al(kn_b) + al(scr_b));
  c.part = reinterpret_cast<double *>(base + al(kn_b) + al(scr_b) + al(xs_b));
  c.jrow = reinterpret_cast<double *>(base + al(kn_b) + al(scr_b) + al(xs_b) + al(part_b));
  c.sig = reinterpret_cast<float *>(base + al(kn_b) + al(scr_b) + al(xs_b) + al(part_b) + al(jrow_b));
  c.ws = reinterpret_cast<WarpShared *>(base + al(kn_b) + al(scr_b) + al(xs_b) + al(part_b) + al(jrow_b) + al(sig_b));
  c.rtol = A.reltol;
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
        for (int j = 0; j < NSP; j++) out[((size_t)s * NSP + lane) * NSP + j] = c.m[j];
    }
    __syncwarp();
  }
}

}  // namespace

size_t chem_warp_smem_per_warp(int nsp, int nreac, int nparts, bool mixed) {
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  const size_t mt = mixed ? 4 : 8;
  return al((size_t)nreac * 8) + al((size_t)nreac * 16) + al(8 * (nsp + 2)) + al(8 * (nparts + 1)) +
         al(mt * nsp * (nsp + 3)) + al(4 * (nsp + 2)) + al(sizeof(WarpShared));
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
  const int wpb = o.warps_per_block > 0 ? o.warps_per_block : 4;
  const size_t smem = chem_warp_smem_per_warp(32, A.nreac, T.nparts, mixed) * wpb;
  cudaError_t e;
  if (mixed) {
    auto k = chem_warp_kernel<32, true>;
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, wpb * 32, smem);
    if (o.blocks_per_sm > 0 && o.blocks_per_sm < per_sm) per_sm = o.blocks_per_sm;
    if (per_sm < 1) per_sm = 1;
    k<<<sm_count * per_sm, wpb * 32, smem, st>>>(A, ncell, total_ptr);
  } else {
    auto k = chem_warp_kernel<32, false>;
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, wpb * 32, smem);
    if (o.blocks_per_sm > 0 && o.blocks_per_sm < per_sm) per_sm = o.blocks_per_sm;
    if (per_sm < 1) per_sm = 1;
    k<<<sm_count * per_sm, wpb * 32, smem, st>>>(A, ncell, total_ptr);
  }
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
  const size_t smem = chem_warp_smem_per_warp(32, A.nreac, T.nparts, false) * 4;
  auto k = eval_kernel<32>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(eval)");
  k<<<(nstate + 3) / 4, 128, smem, st>>>(A, nstate, x, out, xe_out, mode);
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "eval_kernel launch");
}
}  // namespace pdr
