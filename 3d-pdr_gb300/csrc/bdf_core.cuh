// bdf_core.cuh -- the CVODE-method BDF control logic shared by the
// warp-per-cell (chem_warp.cu) and CTA-per-cell (chem_cta.cu) integrators.
//
// It restates the published SUNDIALS CVODE method step for step -- the same
// algorithm as the CPU oracle (oracle/orc_bdf.c, which lists the sources and
// constants): fixed-leading-coefficient BDF of order 1..5 in Nordsieck form,
// Newton iteration with at most 3 corrections and CVODE's convergence and
// divergence tests, the WRMS local error test, CVODE's step-size and order
// selection, error- and convergence-failure recovery, the initial-step
// estimate, and the tout ladder of calculate_abundances.c:214-305 with its
// retry rules.  Every thread of the group owns one species (or none); the
// group type D supplies the collectives and the linear algebra:
//   bool owns; bool leader();  void sync();
//   double sum_all(double); float sum_all(float); double max_all(double);
//   double rhs(double y_own);  bool setup(double y_own);  double solve(double b_own);
//   and, for the mixed form, double solve32(double b_own, float gscale, float &x32)
//   (the correction times gscale, in FP64 and in FP32);
// Norms are kept squared (the tests compare squares, no sqrt); the step-ratio
// heuristics eta = 1/((bias*e)^(1/k) + 1e-6) are evaluated in FP32.
#pragma once

#include <type_traits>

#include "pdr_internal.h"

namespace pdr {
namespace bdf {

constexpr int QMAX = 5;
constexpr int MXNCF = 10, MXNEF = 7, MXNEF1 = 3, SMALL_NEF = 2, LONG_WAIT = 10, SMALL_NST = 10;
constexpr int MAXCOR = 3, MSBP = 20;
constexpr double CRDOWN = 0.3, DGMAX = 0.3, RDIV = 2.0, NLSCOEF = 0.1;
constexpr double ETAMX1 = 10000.0, ETAMX2 = 10.0, ETAMX3 = 10.0, ETAMXF = 0.2, ETAMIN = 0.1;
constexpr double ETACF = 0.25, ADDON = 1e-6, BIAS1 = 6.0, BIAS2 = 6.0, BIAS3 = 10.0, THRESH = 1.5;
constexpr double YEAR = 3.1556926e7;
constexpr int FELL_BACK = 1;   // internal status: redo this cell in FP64
// mixed form: a Newton failure with a fresh FP32 matrix is first handled as a
// convergence failure (step size x 0.25, as CVODE does); the fifth such
// failure within one step sends the cell to the FP64 pass (on the full
// network, three retries sent 0.3 % of cells there, five send none)
constexpr int MIXED_RETRIES = 5;

// shared memory of one integrator: arrays every thread reads.  The error
// constants tq[1..5] are kept in the norm type (tqf in the mixed form, tqd in
// FP64), and the mixed form mirrors the step history in FP32 (tauf), so that
// its FP32 coefficient recurrence and threshold tests read them without
// conversions: on GB300 an F2F costs an FP64 issue slot like a DFMA.
struct CoefShared {
  double tau[QMAX + 2];
  double l[QMAX + 1];
  double rl1;     // 1/l[1]
  double tqd[6];
  float tqf[6], tauf[QMAX + 2];
  float lf[QMAX + 1];   // l in FP32 (the mixed form's FP32 Nordsieck columns)
};

// coefficients of a uniform step history (xi_j = j), per order 1..5: the
// same for every integrator, so one copy serves a whole block
struct CoefUniform {
  double ul[QMAX + 1][QMAX + 1];
  double url1[QMAX + 1];
  double utqd[QMAX + 1][6];
  float utqf[QMAX + 1][6];
  float ulf[QMAX + 1][QMAX + 1];
};

// Comparisons of uniform FP64 scalars in integer arithmetic: for operands
// whose sign bits are clear, the bit patterns order like the values, and NaN
// (any payload) compares false as in FP.  A set sign bit takes the FP compare.
__device__ __forceinline__ bool nan_bits(unsigned long long b) {
  return (b & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull;
}
__device__ __forceinline__ bool ge_u(double a, double b) {
  const unsigned long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  if ((x | y) >> 63) return a >= b;
  return x >= y && !nan_bits(x) && !nan_bits(y);
}
__device__ __forceinline__ bool lt_u(double a, double b) {
  const unsigned long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  if ((x | y) >> 63) return a < b;
  return x < y && !nan_bits(x) && !nan_bits(y);
}
__device__ __forceinline__ bool eq_u(double a, double b) {
  const unsigned long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  if ((x | y) >> 63) return a == b;
  return x == y && !nan_bits(x);
}

// squared-norm form of eta = 1/((bias*e)^(1/k) + 1e-6) with e2 = e^2 (FP32)
__device__ __forceinline__ double eta_of(float e2, float bias, int k) {
  const float v = powf(bias * bias * e2, 0.5f / (float)k);
  return (double)(1.0f / (v + (float)ADDON));
}
__device__ __forceinline__ double eta_of(double e2, float bias, int k) { return eta_of((float)e2, bias, k); }

// 1/x to double precision: FP32 seed and two Newton steps
__device__ __forceinline__ double rcp_nr(double x) {
  double r = (double)__frcp_rn((float)x);
  r = r * fma(-x, r, 2.0);
  r = r * fma(-x, r, 2.0);
  return r;
}

// Nordsieck row of one thread's species held in six registers behind an
// index operator: a constant index selects a register, a run-time index a
// select chain -- never an address, so the integrator object is not forced
// into local memory by an indexed array member.
struct ZRow {
  double v0, v1, v2, v3, v4, v5;
  __device__ __forceinline__ double get(int j) const {
    return j == 0 ? v0 : j == 1 ? v1 : j == 2 ? v2 : j == 3 ? v3 : j == 4 ? v4 : v5;
  }
  __device__ __forceinline__ void set(int j, double x) {
    if (j == 0) v0 = x; else if (j == 1) v1 = x; else if (j == 2) v2 = x;
    else if (j == 3) v3 = x; else if (j == 4) v4 = x; else v5 = x;
  }
  struct Ref {
    ZRow &r;
    int j;
    __device__ __forceinline__ operator double() const { return r.get(j); }
    __device__ __forceinline__ Ref &operator=(double x) { r.set(j, x); return *this; }
    __device__ __forceinline__ Ref &operator=(const Ref &o) { r.set(j, (double)o); return *this; }
    __device__ __forceinline__ Ref &operator+=(double x) { r.set(j, r.get(j) + x); return *this; }
    __device__ __forceinline__ Ref &operator-=(double x) { r.set(j, r.get(j) - x); return *this; }
    __device__ __forceinline__ Ref &operator*=(double x) { r.set(j, r.get(j) * x); return *this; }
  };
  __device__ __forceinline__ Ref operator[](int j) { return Ref{*this, j}; }
  __device__ __forceinline__ double operator[](int j) const { return get(j); }
};

// Nordsieck row in shared memory, z[j] at p[j * s] (frees 12 registers)
struct ZShared {
  double *p;
  int s;
  __device__ __forceinline__ double &operator[](int j) const { return p[j * s]; }
  __device__ __forceinline__ void bind(void *base, int lane, int stride) {
    p = reinterpret_cast<double *>(base) + lane;
    s = stride;
  }
};

// Mixed-form Nordsieck row: the value y = z0 and the scaled first derivative
// z1 = h y' in FP64 -- they enter the corrector equation directly -- and the
// higher columns z2..z5 = h^j y^(j)/j! in FP32.  Those enter a step only
// through the predicted z0 and z1, as terms of relative size (h/tau)^j for a
// solution that varies on the time scale tau (error control at rtol 1e-8
// holds h/tau near rtol^(1/(q+1)), so about 1e-3 of y and below at q >= 2):
// their FP32 rounding moves the corrector's history term by ~1e-10 of y, about
// 1 % of the local error the tolerance allows, while the corrector equation
// itself (state, RHS, residual) stays FP64; the order heuristics read them
// only through norms.  The prediction, correction and rescaling of z2..z5
// then run on the FP32 pipe instead of the FP64 one.
// Columns 0 and 1 are indexed by z[0], z[1]; columns 2..5 by getf/setf.
struct ZRowM {
  double v0, v1;
  float f2, f3, f4, f5;
  __device__ __forceinline__ double get(int j) const { return j == 0 ? v0 : v1; }
  __device__ __forceinline__ void set(int j, double x) { if (j == 0) v0 = x; else v1 = x; }
  __device__ __forceinline__ float getf(int j) const { return j == 2 ? f2 : j == 3 ? f3 : j == 4 ? f4 : f5; }
  __device__ __forceinline__ void setf(int j, float x) {
    if (j == 2) f2 = x; else if (j == 3) f3 = x; else if (j == 4) f4 = x; else f5 = x;
  }
  struct Ref {
    ZRowM &r;
    int j;
    __device__ __forceinline__ operator double() const { return r.get(j); }
    __device__ __forceinline__ Ref &operator=(double x) { r.set(j, x); return *this; }
    __device__ __forceinline__ Ref &operator=(const Ref &o) { r.set(j, (double)o); return *this; }
    __device__ __forceinline__ Ref &operator+=(double x) { r.set(j, r.get(j) + x); return *this; }
    __device__ __forceinline__ Ref &operator-=(double x) { r.set(j, r.get(j) - x); return *this; }
    __device__ __forceinline__ Ref &operator*=(double x) { r.set(j, r.get(j) * x); return *this; }
  };
  __device__ __forceinline__ Ref operator[](int j) { return Ref{*this, j}; }
  __device__ __forceinline__ double operator[](int j) const { return get(j); }
};

// the same row in shared memory: z0, z1 at p[0], p[s]; z_j (j >= 2) at pf[(j-2)*s]
struct ZSharedM {
  double *p;
  float *pf;
  int s;
  __device__ __forceinline__ double &operator[](int j) const { return p[j * s]; }
  __device__ __forceinline__ float getf(int j) const { return pf[(j - 2) * s]; }
  __device__ __forceinline__ void setf(int j, float x) const { pf[(j - 2) * s] = x; }
  // base holds 2*stride doubles, then 4*stride floats
  __device__ __forceinline__ void bind(void *base, int lane, int stride) {
    p = reinterpret_cast<double *>(base) + lane;
    pf = reinterpret_cast<float *>(reinterpret_cast<double *>(base) + 2 * stride) + lane;
    s = stride;
  }
};

// NORM32: the error weights, WRMS norms and the convergence-rate estimate in
// FP32 (the mixed form).  They only feed threshold tests and step-ratio
// heuristics, and on GB300 every FP64 warp instruction costs 1/60 of an FP32
// one; the state, corrections, residuals and Nordsieck updates stay FP64.
template <class D, bool ZSHARED = false, bool NORM32 = false>
struct Core {
  using NT = typename std::conditional<NORM32, float, double>::type;
  __device__ __forceinline__ D &self() { return *static_cast<D *>(this); }
  CoefShared *ws = nullptr;
  CoefUniform *wu = nullptr;   // the uniform-history table (may be shared by several integrators)
  // Nordsieck row of this thread's species, weight, correction, work values
  using ZT = typename std::conditional<NORM32, typename std::conditional<ZSHARED, ZSharedM, ZRowM>::type,
                                       typename std::conditional<ZSHARED, ZShared, ZRow>::type>::type;
  ZT z;
  NT ewt;
  double acor, y, ftmp, tmp;
  // uniform integrator scalars
  double tn, h, hscale, hprime, eta, etamax, gamma, gammap, rl1;
  NT inv_gammap, gamrat, gscale, saved_tq5;
  NT h_nt;   // h in the norm type, set with the coefficients
  NT crate2, acnrm2;
  double xe_last, rtol, atol;
  int q, qprime, qwait, jcur;
  int nst, nstlp, nfe, nje, nsetups, nni, ncfn, netf;
  long long mxstep, max_total_steps;

  // the error constants and step history in the norm type
  __device__ __forceinline__ NT *tqn() const {
    if constexpr (NORM32) return ws->tqf;
    else return ws->tqd;
  }
  __device__ __forceinline__ NT utqn(int qq, int j) const {
    if constexpr (NORM32) return wu->utqf[qq][j];
    else return wu->utqd[qq][j];
  }
  __device__ __forceinline__ const NT *taun() const {
    if constexpr (NORM32) return ws->tauf;
    else return ws->tau;
  }

  float inv_n32 = 0.0f;   // 1/n in FP32, set at the start of integrate()
  __device__ __forceinline__ NT wrms2(double v) {
    const NT t = self().owns ? (NT)v * ewt : NT(0);
    if constexpr (NORM32) return self().sum_all(t * t) * inv_n32;
    else return self().sum_all(t * t) * (NT)self().inv_n;
  }
  // the same norm of a value already held in FP32 (the mixed form's Newton
  // correction comes out of the FP32 solve): no conversion
  __device__ __forceinline__ float wrms2_32(float v) {
    const float t = self().owns ? v * ewt : 0.0f;
    return self().sum_all(t * t) * inv_n32;
  }

  // FP32 copies of the tolerances (mixed form), set at the start of integrate()
  float rtol32 = 0.0f, atol32 = 0.0f;

  __device__ __forceinline__ void set_ewt() {
    // mixed: the weight is FP32, so it is formed from the FP32 value of y (one
    // conversion instead of an FP64 FMA and a conversion)
    if constexpr (NORM32) ewt = self().owns ? __frcp_rn(fmaf(rtol32, fabsf((float)z[0]), atol32)) : 0.0f;
    else ewt = self().owns ? rcp_nr(rtol * fabs(z[0]) + atol) : 0.0;
  }

  // Pascal-triangle prediction z <- z P (and its inverse), q-specialised
  template <int Q, int SIGN>
  __device__ __forceinline__ void pascal() {
#pragma unroll
    for (int k = 1; k <= Q; k++)
#pragma unroll
      for (int j = Q; j >= 1; j--)
        if (j >= k) z[j - 1] = (SIGN > 0) ? z[j - 1] + z[j] : z[j - 1] - z[j];
  }
  // mixed form: the FP32 columns 2..Q take the Pascal triangle among
  // themselves (their new values read only higher columns); z1 and z0 take
  // S1 = sum j z_j and S0 = sum z_j over the FP32 columns -- of the columns
  // before the update for the prediction, after it for the inverse -- in one
  // FP64 add each: z0 <- z0 + z1 + S0, z1 <- z1 + S1, and back
  template <int Q, int SIGN>
  __device__ __forceinline__ void pascal_m() {
    if constexpr (Q == 1) {
      z[0] = (SIGN > 0) ? z[0] + z[1] : z[0] - z[1];
    } else {
      float s0 = 0.0f, s1 = 0.0f;
      if constexpr (SIGN > 0) {
#pragma unroll
        for (int j = 2; j <= Q; j++) { const float f = z.getf(j); s0 += f; s1 = fmaf((float)j, f, s1); }
      }
#pragma unroll
      for (int k = 1; k <= Q; k++)
#pragma unroll
        for (int j = Q; j >= 3; j--)
          if (j >= k) z.setf(j - 1, (SIGN > 0) ? z.getf(j - 1) + z.getf(j) : z.getf(j - 1) - z.getf(j));
      if constexpr (SIGN < 0) {
#pragma unroll
        for (int j = 2; j <= Q; j++) { const float f = z.getf(j); s0 += f; s1 = fmaf((float)j, f, s1); }
      }
      if constexpr (SIGN > 0) {
        z[0] = z[0] + (z[1] + (double)s0);
        z[1] = z[1] + (double)s1;
      } else {
        z[1] = z[1] - (double)s1;
        z[0] = z[0] - (z[1] + (double)s0);
      }
    }
  }
  // the same with a run-time order, rolled (rows in shared memory)
  template <int SIGN>
  __device__ __forceinline__ void pascal_m_rolled() {
    if (q == 1) {
      z[0] = (SIGN > 0) ? z[0] + z[1] : z[0] - z[1];
      return;
    }
    float s0 = 0.0f, s1 = 0.0f;
    if (SIGN > 0) {
#pragma unroll 1
      for (int j = 2; j <= q; j++) { const float f = z.getf(j); s0 += f; s1 = fmaf((float)j, f, s1); }
    }
#pragma unroll 1
    for (int k = 1; k <= q; k++)
#pragma unroll 1
      for (int j = q; j >= (k > 3 ? k : 3); j--)
        z.setf(j - 1, (SIGN > 0) ? z.getf(j - 1) + z.getf(j) : z.getf(j - 1) - z.getf(j));
    if (SIGN < 0) {
#pragma unroll 1
      for (int j = 2; j <= q; j++) { const float f = z.getf(j); s0 += f; s1 = fmaf((float)j, f, s1); }
    }
    if (SIGN > 0) {
      z[0] = z[0] + (z[1] + (double)s0);
      z[1] = z[1] + (double)s1;
    } else {
      z[1] = z[1] - (double)s1;
      z[0] = z[0] - (z[1] + (double)s0);
    }
  }
  template <int SIGN>
  __device__ __forceinline__ void pascal_q() {
    if constexpr (NORM32) {
      if constexpr (ZSHARED) {
        pascal_m_rolled<SIGN>();
      } else {
        switch (q) {
          case 1: pascal_m<1, SIGN>(); break;
          case 2: pascal_m<2, SIGN>(); break;
          case 3: pascal_m<3, SIGN>(); break;
          case 4: pascal_m<4, SIGN>(); break;
          default: pascal_m<5, SIGN>(); break;
        }
      }
      return;
    }
    if constexpr (ZSHARED) {
      // rows in shared memory: a rolled loop keeps the step's code small
#pragma unroll 1
      for (int k = 1; k <= q; k++)
#pragma unroll 1
        for (int j = q; j >= k; j--) z[j - 1] = (SIGN > 0) ? z[j - 1] + z[j] : z[j - 1] - z[j];
      return;
    }
    switch (q) {
      case 1: pascal<1, SIGN>(); break;
      case 2: pascal<2, SIGN>(); break;
      case 3: pascal<3, SIGN>(); break;
      case 4: pascal<4, SIGN>(); break;
      default: pascal<5, SIGN>(); break;
    }
  }
  __device__ __forceinline__ void predict() { tn += h; pascal_q<1>(); }
  __device__ __forceinline__ void restore(double saved_t) { tn = saved_t; pascal_q<-1>(); }

  __device__ __forceinline__ void rescale() {
    if constexpr (NORM32) {
      z[1] = z[1] * eta;
      const float ef = (float)eta;
      float fac = ef * ef;
#pragma unroll
      for (int j = 2; j <= QMAX; j++)
        if (j <= q) { z.setf(j, z.getf(j) * fac); fac *= ef; }
    } else {
      double fac = eta;
#pragma unroll
      for (int j = 1; j <= QMAX; j++)
        if (j <= q) { z[j] *= fac; fac *= eta; }
    }
    h = hscale * eta;
    hscale = h;
  }

  // a fresh row: y0 in column 0, zeros elsewhere
  __device__ __forceinline__ void clear_row(double y0) {
    z[0] = y0;
    z[1] = 0.0;
    if constexpr (NORM32) {
#pragma unroll
      for (int j = 2; j <= QMAX; j++) z.setf(j, 0.0f);
    } else {
#pragma unroll
      for (int j = 2; j <= QMAX; j++) z[j] = 0.0;
    }
  }

  // mixed form: the order changes below on the FP32 columns, with the
  // coefficients from the FP32 step history
  __device__ __forceinline__ void decrease_order_m() {
    if (q <= 2) return;
    float d[QMAX + 2];
#pragma unroll
    for (int j = 0; j < QMAX + 2; j++) d[j] = 0.0f;
    d[2] = 1.0f;
    const float hs = (float)hscale;
    float hsum = 0.0f;
#pragma unroll
    for (int k = 1; k <= QMAX - 2; k++) {
      if (k <= q - 2) {
        hsum += ws->tauf[k];
        const float xi = hsum / hs;
#pragma unroll
        for (int j = QMAX + 1; j >= 1; j--) d[j] = d[j - 1] + d[j] * xi;
        d[0] *= xi;
      }
    }
    float zq = 0.0f;
#pragma unroll
    for (int j = 2; j <= QMAX; j++) if (j == q) zq = z.getf(j);
#pragma unroll
    for (int j = 2; j < QMAX; j++)
      if (j < q) z.setf(j, z.getf(j) - d[j] * zq);
  }
  __device__ __forceinline__ void increase_order_m() {
    float d[QMAX + 2];
#pragma unroll
    for (int j = 0; j < QMAX + 2; j++) d[j] = 0.0f;
    d[2] = 1.0f;
    const float hs = (float)hscale;
    float hsum = hs, sum_j = 1.0f, sum_xi = 1.0f, prod = 1.0f, xi_prev = 1.0f;
#pragma unroll
    for (int k = 2; k <= QMAX; k++) {
      if (k <= q) {
        hsum += ws->tauf[k];
        const float xi = hsum / hs;
        sum_j += 1.0f / k;
        sum_xi += 1.0f / xi;
        prod *= xi;
#pragma unroll
        for (int j = QMAX + 1; j >= 1; j--) d[j] = d[j - 1] + d[j] * xi_prev;
        d[0] *= xi_prev;
        xi_prev = xi;
      }
    }
    const float c = (sum_j - sum_xi) / prod;
    const float zn1 = c * z.getf(QMAX);
#pragma unroll
    for (int j = 2; j <= QMAX; j++)
      if (j <= q) z.setf(j, z.getf(j) + d[j] * zn1);
#pragma unroll
    for (int j = 2; j <= QMAX; j++)
      if (j == q + 1) z.setf(j, zn1);
  }

  // order q -> q-1: remove the x^q term keeping the value and slope at t_n and
  // the values at t_{n-1}..t_{n-q+2}: z_j -= d_j z_q, d = x^2 prod_{k<=q-2}(x+xi_k)
  __device__ __forceinline__ void decrease_order() {
    if constexpr (NORM32) decrease_order_m();
    else decrease_order_d();
  }
  __device__ __forceinline__ void decrease_order_d() {
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

  // order q -> q+1: add c x^2 prod_{k<q}(x+xi_k) so the polynomial also passes
  // through y_{n-q}; c = (sum_{j<=q} 1/j - sum_{i<=q} 1/xi_i)/prod_{i=2}^q xi_i * Delta_n
  __device__ __forceinline__ void increase_order() {
    if constexpr (NORM32) increase_order_m();
    else increase_order_d();
  }
  __device__ __forceinline__ void increase_order_d() {
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
  // tq[1..5] for step h and step history tau[1..q] (q+1 for tq[3])
  // T = double, or float in the mixed form: the coefficients only scale the
  // Newton correction and the error-test thresholds, so FP32 perturbs the
  // solution by ~1e-7 of the correction (itself of the size of the local
  // error), and the ~10 divisions here cost FP32 instead of FP64 issue slots
  template <class T>
  __device__ __forceinline__ static void coeffs(int q, bool order_change_due, T h, const T *tau, T *l, T *tq) {
#pragma unroll
    for (int j = 0; j <= QMAX; j++) l[j] = T(0);
    l[0] = l[1] = T(1);
    T a0 = T(-1), a0hat = T(-1), xi_inv = T(1), xistar_inv = T(1), hsum = h;
    if (q > 1) {
#pragma unroll
      for (int j = 2; j < QMAX; j++) {
        if (j < q) {
          hsum += tau[j - 1];
          xi_inv = h / hsum;
          a0 -= T(1) / T(j);
#pragma unroll
          for (int i = QMAX; i >= 1; i--)
            if (i <= j) l[i] += l[i - 1] * xi_inv;
        }
      }
      a0 -= T(1) / T(q);
      xistar_inv = -l[1] - a0;
      hsum += tau[q - 1];
      xi_inv = h / hsum;
      a0hat = -l[1] - xi_inv;
#pragma unroll
      for (int i = QMAX; i >= 1; i--)
        if (i <= q) l[i] += l[i - 1] * xistar_inv;
    }
    T lq = T(0);
#pragma unroll
    for (int j = 0; j <= QMAX; j++) if (j == q) lq = l[j];
    const T A1 = T(1) - a0hat + a0, A2 = T(1) + T(q) * A1;
    tq[2] = fabs(A1 / (a0 * A2));
    tq[5] = fabs(A2 * xistar_inv / (lq * xi_inv));
    if (order_change_due) {
      if (q > 1) {
        const T C = xistar_inv / lq, A3 = a0 + T(1) / T(q), A4 = a0hat + xi_inv;
        tq[1] = fabs(C * (T(1) - A4 + A3) / A3);
      } else {
        tq[1] = T(1);
      }
      hsum += tau[q];
      xi_inv = h / hsum;
      const T A5 = a0 - T(1) / T(q + 1), A6 = a0hat - xi_inv;
      tq[3] = fabs(((T(1) - A6 + A5) / A2) / (xi_inv * T(q + 2) * A5));
    }
    tq[4] = T(NLSCOEF) / tq[2];
  }

  // the table of uniform-history coefficients (h = tau_j = 1)
  __device__ __forceinline__ void build_uniform_table() {
    double one[QMAX + 2];
#pragma unroll
    for (int j = 0; j < QMAX + 2; j++) one[j] = 1.0;
    for (int qq = 1; qq <= QMAX; qq++) {
      double l[QMAX + 1], tq[6];
      coeffs<double>(qq, true, 1.0, one, l, tq);
      self().sync();
      if (self().leader()) {
        for (int j = 0; j <= QMAX; j++) {
          wu->ul[qq][j] = l[j];
          wu->ulf[qq][j] = (float)l[j];
        }
        wu->url1[qq] = 1.0 / l[1];
        for (int j = 1; j <= 5; j++) {
          wu->utqd[qq][j] = tq[j];
          wu->utqf[qq][j] = (float)tq[j];
        }
      }
    }
    self().sync();
  }

  // store l[0..Q] of the FP32/FP64 recurrence as FP64 (only the used terms)
  template <int Q>
  __device__ __forceinline__ void store_l(const NT *l) {
#pragma unroll
    for (int j = 0; j <= Q; j++) {
      ws->l[j] = (double)l[j];
      ws->lf[j] = (float)l[j];
    }
  }

  __device__ __forceinline__ void set_coeffs() {
    // a history of equal steps gives xi_j = j exactly: take the tabulated values
    bool uniform = true;
    const unsigned long long hb = __double_as_longlong(h);
#pragma unroll
    for (int j = 1; j <= QMAX; j++)
      if (j <= q && (unsigned long long)__double_as_longlong(ws->tau[j]) != hb) uniform = false;
    self().sync();
    NT *tq = tqn();
    if (uniform) {
      // h equals tau[1] bit for bit, so its FP32 value is the mirror's
      if constexpr (NORM32) h_nt = ws->tauf[1];
      else h_nt = h;
      if (self().leader()) {
#pragma unroll
        for (int j = 0; j <= QMAX; j++) {
          ws->l[j] = wu->ul[q][j];
          ws->lf[j] = wu->ulf[q][j];
        }
        ws->rl1 = wu->url1[q];
        tq[2] = utqn(q, 2);
        tq[4] = utqn(q, 4);
        tq[5] = utqn(q, 5);
        if (qwait == 1) { tq[1] = utqn(q, 1); tq[3] = utqn(q, 3); }
      }
    } else {
      h_nt = (NT)h;
      NT l[QMAX + 1], tqv[6];
      tqv[1] = tq[1];
      tqv[3] = tq[3];
      coeffs<NT>(q, qwait == 1, h_nt, taun(), l, tqv);
      if (self().leader()) {
        switch (q) {
          case 1: store_l<1>(l); break;
          case 2: store_l<2>(l); break;
          case 3: store_l<3>(l); break;
          case 4: store_l<4>(l); break;
          default: store_l<5>(l); break;
        }
        ws->rl1 = (double)(NT(1) / l[1]);
        tq[1] = tqv[1]; tq[2] = tqv[2]; tq[3] = tqv[3]; tq[4] = tqv[4]; tq[5] = tqv[5];
      }
    }
    self().sync();
    rl1 = ws->rl1;
    gamma = h * rl1;
    if (nst == 0) { gammap = gamma; inv_gammap = NT(1) / (NT)gamma; }
    gamrat = (nst > 0) ? (NT)gamma * inv_gammap : NT(1);
    if constexpr (NORM32) gscale = (gamrat != 1.0f) ? 2.0f * __frcp_rn(1.0f + gamrat) : 1.0f;
    else gscale = (gamrat != 1.0) ? 2.0 * rcp_nr(1.0 + gamrat) : 1.0;
  }

  // called by D::setup after forming the matrix
  __device__ __forceinline__ void after_setup() {
    nje++;
    nsetups++;
    jcur = 1;
    crate2 = 1.0;
    gammap = gamma;
    inv_gammap = NT(1) / (NT)gamma;
    gamrat = NT(1);
    gscale = 1.0;
    nstlp = nst;
  }

  // 0 solved, 1 convergence failure, 2 failure that sends the cell to the FP64 pass
  __device__ __forceinline__ int nls(bool prev_fail, bool fallback_on_fail) {
    bool call_setup = prev_fail || (nst == 0) || (nst >= nstlp + MSBP) || (fabs(gamrat - NT(1)) > NT(DGMAX));
    const NT tq4 = tqn()[4];
    const NT tq4sq = tq4 * tq4;
    const int fail = fallback_on_fail ? 2 : 1;
    for (int attempt = 0; attempt < 2; attempt++) {
      y = z[0];
      ftmp = self().rhs(y);
      if (call_setup) {
        if (!self().setup(y)) return fail;
        call_setup = false;
      }
      acor = 0.0;
      NT delp2 = 0;
      int mcor = 0;
      bool conv = false;
      const double rz1 = rl1 * z[1];   // fixed during the iteration
      for (;;) {
        tmp = gamma * ftmp - (rz1 + acor);
        NT del2;
        if constexpr (NORM32) {
          // the FP32 solve returns the correction already scaled by gscale,
          // and its FP32 value feeds the norm
          float t32;
          tmp = self().solve32(tmp, gscale, t32);
          del2 = wrms2_32(t32);
        } else {
          tmp = self().solve(tmp);
          if (gscale != NT(1)) tmp *= (double)gscale;
          del2 = wrms2(tmp);
        }
        nni++;
        acor += tmp;
        y = z[0] + acor;
        if (mcor > 0) crate2 = fmax(NT(CRDOWN * CRDOWN) * crate2, del2 / delp2);
        if (del2 * fmin(NT(1), crate2) <= tq4sq) {
          acnrm2 = (mcor == 0) ? del2 : wrms2(acor);
          jcur = 0;
          conv = true;
          break;
        }
        mcor++;
        if (mcor == MAXCOR || (mcor >= 2 && del2 > NT(RDIV * RDIV) * delp2)) break;
        delp2 = del2;
        ftmp = self().rhs(y);
      }
      if (conv) return 0;
      if (!jcur) { call_setup = true; continue; }
      return fail;
    }
    return fail;
  }

  __device__ __forceinline__ void set_eta() {
    if (lt_u(eta, THRESH)) { eta = 1.0; hprime = h; }
    else { eta = fmin(eta, etamax); hprime = h * eta; }
  }

  // one internal step: 0 ok, CVODE flag (<0), or FELL_BACK
  __device__ __forceinline__ int step(bool fallback_on_fail) {
    const double saved_t = tn;
    int ncf = 0, nef = 0;
    bool prev_fail = false;
    NT dsm2 = 0;
    if (nst > 0 && !eq_u(hprime, h)) {
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
      const int r = nls(prev_fail, fallback_on_fail);
      if (r == 2 && ncf + 1 >= MIXED_RETRIES) return FELL_BACK;
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
      const NT tq2 = tqn()[2];
      dsm2 = acnrm2 * (tq2 * tq2);
      if (dsm2 <= NT(1)) break;
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
      tmp = self().rhs(z[0]);
      z[1] = h * tmp;
    }
    // complete the step
    nst++;
    self().sync();
    if (self().leader()) {
#pragma unroll
      for (int i = QMAX; i >= 2; i--)
        if (i <= q) ws->tau[i] = ws->tau[i - 1];
      if (q == 1 && nst > 1) ws->tau[2] = ws->tau[1];
      ws->tau[1] = h;
      if constexpr (NORM32) {
        // the FP32 mirror: h_nt is (float)h of the coefficients of this step
#pragma unroll
        for (int i = QMAX; i >= 2; i--)
          if (i <= q) ws->tauf[i] = ws->tauf[i - 1];
        if (q == 1 && nst > 1) ws->tauf[2] = ws->tauf[1];
        ws->tauf[1] = h_nt;
      }
    }
    self().sync();
    // mixed form: the FP32 value of the correction for the FP32 columns, the
    // order-raise save and the order heuristics
    float acor32 = 0.0f;
    if constexpr (NORM32) {
      z[0] = fma(ws->l[0], acor, z[0]);
      z[1] = fma(ws->l[1], acor, z[1]);
      acor32 = (float)acor;
      if constexpr (ZSHARED) {
#pragma unroll 1
        for (int j = 2; j <= q; j++) z.setf(j, fmaf(ws->lf[j], acor32, z.getf(j)));
      } else {
#pragma unroll
        for (int j = 2; j <= QMAX; j++)
          if (j <= q) z.setf(j, fmaf(ws->lf[j], acor32, z.getf(j)));
      }
    } else if constexpr (ZSHARED) {
#pragma unroll 1
      for (int j = 0; j <= q; j++) z[j] = fma(ws->l[j], acor, z[j]);
    } else switch (q) {
#define PDR_CORRECT(Q) case Q: _Pragma("unroll") for (int j = 0; j <= Q; j++) z[j] = fma(ws->l[j], acor, z[j]); break;
      PDR_CORRECT(1) PDR_CORRECT(2) PDR_CORRECT(3) PDR_CORRECT(4) PDR_CORRECT(5)
#undef PDR_CORRECT
    }
    qwait--;
    if (qwait == 1 && q != QMAX) {
      if constexpr (NORM32) z.setf(QMAX, acor32);
      else z[QMAX] = acor;
      saved_tq5 = tqn()[5];
    }
    if (eq_u(etamax, 1.0)) {
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
          const NT tq1 = tqn()[1];
          if constexpr (NORM32) {
            float zq = 0.0f;
#pragma unroll
            for (int j = 2; j <= QMAX; j++) if (j == q) zq = z.getf(j);
            etaqm1 = eta_of(wrms2_32(zq) * (tq1 * tq1), (float)BIAS1, q);
          } else {
            double zq = 0.0;
#pragma unroll
            for (int j = 0; j <= QMAX; j++) if (j == q) zq = z[j];
            etaqm1 = eta_of(wrms2(zq) * (tq1 * tq1), (float)BIAS1, q);
          }
        }
        if (q != QMAX && saved_tq5 != NT(0)) {
          // step-ratio factor of the order-raise estimate (heuristic, FP32)
          float ratio;
          if constexpr (NORM32) ratio = h_nt / ws->tauf[2];
          else ratio = (float)h / (float)ws->tau[2];
          float rp = ratio;
          for (int k = 1; k < L; k++) rp *= ratio;
          const float cquot = ((float)tqn()[5] / (float)saved_tq5) * rp;
          const NT tq3 = tqn()[3];
          if constexpr (NORM32)
            etaqp1 = eta_of(wrms2_32(fmaf(-cquot, z.getf(QMAX), acor32)) * (tq3 * tq3), (float)BIAS3, L + 1);
          else
            etaqp1 = eta_of(wrms2(acor - (double)cquot * z[QMAX]) * (tq3 * tq3), (float)BIAS3, L + 1);
        }
        // ties keep the current order, then prefer the lower one
        const double etam = fmax(etaqm1, fmax(etaq, etaqp1));
        if (etam < THRESH) { eta = 1.0; qprime = q; }
        else if (etam == etaq) { eta = etaq; qprime = q; }
        else if (etam == etaqm1) { eta = etaqm1; qprime = q - 1; }
        else {
          eta = etaqp1;
          qprime = q + 1;
          if constexpr (NORM32) z.setf(QMAX, acor32);
          else z[QMAX] = acor;
        }
        set_eta();
      }
    }
    etamax = (nst <= SMALL_NST) ? ETAMX2 : ETAMX3;
    return 0;
  }

  // initial step from an estimate of ||y''|| (h^2/2 ||y''|| = 1, safety 0.5)
  __device__ __forceinline__ double initial_step(double t0, double tout) {
    const double tdist = fabs(tout - t0);
    const double tround = 2.220446049250313e-16 * fmax(fabs(t0), fabs(tout));
    const double hlb = 100.0 * tround;
    const double hub_inv = self().max_all(self().owns ? fabs(z[1]) / (0.1 * fabs(z[0]) + atol) : 0.0);
    double hub = 0.1 * tdist;
    if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
    double hg = sqrt(hlb * hub);
    if (hub < hlb) return hg;
    bool ok = false;
    double hnew = hg;
    for (int it = 1; it <= 4; it++) {
      tmp = self().rhs(z[0] + hg * z[1]);
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
    if constexpr (NORM32) {
      // z0 + s (z1 + s (sum_{j>=2} s^(j-2) z_j)), the FP32 columns by Horner in FP32
      if (q == 1) return fma(s, z[1], z[0]);
      const float sf = (float)s;
      float vf = 0.0f;
#pragma unroll
      for (int j = QMAX; j >= 2; j--)
        if (j <= q) vf = (j == q) ? z.getf(j) : fmaf(sf, vf, z.getf(j));
      return fma(s, fma(s, (double)vf, z[1]), z[0]);
    } else {
      double v = 0.0;
#pragma unroll
      for (int j = QMAX; j >= 0; j--)
        if (j <= q) v = (j == q) ? z[j] : fma(s, v, z[j]);
      return v;
    }
  }

  // CVode(..., CV_NORMAL) from the current state to tout
  __device__ __forceinline__ int solve_to(double tout, bool first, double t0, long long &total, bool fb) {
    if (first) {
      set_ewt();
      z[1] = self().rhs(z[0]);
      const double h0 = initial_step(t0, tout);
      z[1] *= h0;
      h = hscale = hprime = h0;
      q = qprime = 1;
      qwait = 2;
      etamax = ETAMX1;
      nst = 0;
    } else if (ge_u(tn, tout)) {   // h > 0: the integration runs forward
      return 0;
    }
    long long nstloc = 0;
    for (;;) {
      if (nst > 0) set_ewt();
      if (nstloc >= mxstep || total >= max_total_steps) return PDR_TOO_MUCH_WORK;
      const int kf = step(fb);
      if (kf != 0) return kf;
      nstloc++;
      total++;
      if (ge_u(tn, tout)) return 0;
    }
  }

  // calculate_abundances.c:132-317 for one cell from z[0] = y0: returns the
  // cell's status (CVODE flag, or FELL_BACK) and the output value of this
  // thread's species in *yout (interpolated at the last tout, or z[0] after a
  // failing call), before the abstol clamp
  __device__ __forceinline__ int integrate(double t0_yr, double tend_yr, bool fb, double *yout) {
    if (self().leader()) {
#pragma unroll
      for (int j = 0; j < QMAX + 2; j++) { ws->tau[j] = 0.0; ws->tauf[j] = 0.0f; }
#pragma unroll
      for (int j = 0; j < 6; j++) { ws->tqd[j] = 0.0; ws->tqf[j] = 0.0f; }
    }
    self().sync();
    rtol32 = (float)rtol;
    atol32 = (float)atol;
    inv_n32 = (float)self().inv_n;
    nfe = nje = nsetups = nni = ncfn = netf = 0;
    nst = nstlp = 0;
    saved_tq5 = NT(0);
    crate2 = 1.0;
    gammap = gamma = 1.0;
    inv_gammap = 1.0;
    gamrat = 1.0;
    gscale = 1.0;
    jcur = 0;
    acor = 0.0;
    const double t0 = t0_yr * YEAR, tend = tend_yr * YEAR;
    tn = t0;
    double tout = 1.0e-4 * YEAR, t = t0;
    int nfails = 0, status = 0, lastflag = 0;
    long long total = 0;
    bool first = true;
    double tlast = tout;
    do {
      const int flag = solve_to(tout, first, t0, total, fb);
      first = false;
      if (flag == FELL_BACK) return FELL_BACK;
      lastflag = flag;
      tlast = tout;
      if (flag != 0) {
        nfails++;
        if (!((flag == PDR_TOO_MUCH_WORK || flag == PDR_CONV_FAILURE) && nfails < 5)) {
          status = flag;
          if (flag != PDR_TOO_MUCH_WORK && flag != PDR_CONV_FAILURE) nfails = 5;
        }
        if (total >= max_total_steps) { status = PDR_TOO_MUCH_WORK; nfails = 5; }
        t = tn;
      } else {
        t = tout;
      }
      tout = tout * 10.0;
      if (tout > tend) tout = tend;
    } while (t < tout && nfails < 5);
    *yout = (lastflag == 0) ? interpolate(tlast) : z[0];
    return status;
  }
};

}  // namespace bdf
}  // namespace pdr
