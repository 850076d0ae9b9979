// rates.cu -- batched reaction-rate evaluation with self-shielding
// (GPU form of CALCULATE_REACTION_RATES, calc_reac_rates.F90:16-401).
//
// One warp per cell, lanes over reactions; the reaction-parameter table is
// staged once per block in shared memory and reused for every cell the block
// visits.  Each reaction's branch, duplicate-group selection (the first member
// whose RTMAX >= T, else the last member, calc_reac_rates.F90:117-145) and the
// clamps of :387-396 are evaluated independently per lane.  The per-ray sums
// keep the reference's ray order.  Shielding follows shield.F90: Federman
// H2SHIELD1 (:231), the van Dishoeck & Black 2-D spline COSHIELD (:375, natural
// splines of spline.F90), SCATTER (:449) with XLAMBDA (:525) and LBAR (:570);
// H2 formation on grains follows h2_form.F90:8-113.
#include <cmath>
#include <vector>

#include <mutex>

#include "pdr_internal.h"

namespace pdr {

// Savage & Mathis (1979) tau(lambda)/tau(V) (the extinction table of the
// reference, modules.F90:354-366) and the van Dishoeck & Black (1988) log10
// 12CO shielding grid (modules.F90:346-351, values 3DPDR.F90:1532-1537).
static const double kLGrid[30] = {910.0, 950.0, 1000.0, 1050.0, 1110.0, 1180.0, 1250.0, 1390.0,
                                  1490.0, 1600.0, 1700.0, 1800.0, 1900.0, 2000.0, 2100.0, 2190.0,
                                  2300.0, 2400.0, 2500.0, 2740.0, 3440.0, 4000.0, 4400.0, 5500.0,
                                  7000.0, 9000.0, 12500.0, 22000.0, 34000.0, 1.0e9};
static const double kXGrid[30] = {5.76, 5.18, 4.65, 4.16, 3.73, 3.40, 3.11, 2.74, 2.63, 2.62,
                                  2.54, 2.50, 2.58, 2.78, 3.01, 3.12, 2.86, 2.58, 2.35, 2.00,
                                  1.58, 1.42, 1.32, 1.00, 0.75, 0.48, 0.28, 0.12, 0.05, 0.00};
static const double kNCOGrid[8] = {12.0, 13.0, 14.0, 15.0, 16.0, 17.0, 18.0, 19.0};
static const double kNH2Grid[6] = {18.0, 19.0, 20.0, 21.0, 22.0, 23.0};
// [iNH2][iNCO]
static const double kSCO[6][8] = {
    {0.000e+00, -1.408e-02, -1.099e-01, -4.400e-01, -1.154e+00, -1.888e+00, -2.760e+00, -4.001e+00},
    {-8.539e-02, -1.015e-01, -2.104e-01, -5.608e-01, -1.272e+00, -1.973e+00, -2.818e+00, -4.055e+00},
    {-1.451e-01, -1.612e-01, -2.708e-01, -6.273e-01, -1.355e+00, -2.057e+00, -2.902e+00, -4.122e+00},
    {-4.559e-01, -4.666e-01, -5.432e-01, -8.665e-01, -1.602e+00, -2.303e+00, -3.146e+00, -4.421e+00},
    {-1.303e+00, -1.312e+00, -1.367e+00, -1.676e+00, -2.305e+00, -3.034e+00, -3.758e+00, -5.077e+00},
    {-3.883e+00, -3.888e+00, -3.936e+00, -4.197e+00, -4.739e+00, -5.165e+00, -5.441e+00, -6.446e+00}};

struct ShieldTables {
  double lgrid[30], xgrid[30], xderiv[30];
  double nco[8], nh2[6], sco[8][6], scoderiv[8][6];
};
__constant__ ShieldTables c_shield;

// natural cubic spline second derivatives (the tridiagonal sweep of the
// Numerical-Recipes routine the reference uses, spline.F90:65-125)
template <class R>
__host__ __device__ void spline_natural(const R *x, const R *y, int n, R *y2, R *u) {
  y2[0] = 0.0;
  u[0] = 0.0;
  for (int i = 1; i < n - 1; i++) {
    const R sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    const R p = sig * y2[i - 1] + 2.0;
    y2[i] = (sig - 1.0) / p;
    u[i] = (6.0 * ((y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1])) /
                (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
  }
  y2[n - 1] = 0.0;
  for (int i = n - 2; i >= 0; i--) y2[i] = y2[i] * y2[i + 1] + u[i];
}

// cubic spline value with the bisection bracket of spline.F90:182-277
template <class R>
__host__ __device__ R splint(const R *xa, const R *ya, const R *y2a, int n, R x) {
  const bool asc = xa[n - 1] > xa[0];
  int lo = 0, hi = n + 1;
  while (hi - lo != 1) {
    const int mid = (hi + lo) / 2;
    if ((x > xa[mid - 1]) == asc) lo = mid;
    else hi = mid;
  }
  if (lo == 0) { lo = 1; hi = 2; }
  if (lo == n) { lo = n - 1; hi = n; }
  const R h = xa[hi - 1] - xa[lo - 1];
  const R A = (xa[hi - 1] - x) / h, B = (x - xa[lo - 1]) / h;
  return A * ya[lo - 1] + B * ya[hi - 1] +
         ((A * A * A - A) * y2a[lo - 1] + (B * B * B - B) * y2a[hi - 1]) * (h * h) / 6.0;
}

static bool g_shield_ready[64];

int upload_shield_tables(int dev) {
  if (dev >= 0 && dev < 64 && g_shield_ready[dev]) return 0;
  ShieldTables t;
  double u[64];
  for (int i = 0; i < 30; i++) { t.lgrid[i] = kLGrid[i]; t.xgrid[i] = kXGrid[i]; }
  spline_natural<double>(t.lgrid, t.xgrid, 30, t.xderiv, u);
  for (int i = 0; i < 8; i++) t.nco[i] = kNCOGrid[i];
  for (int j = 0; j < 6; j++) t.nh2[j] = kNH2Grid[j];
  for (int i = 0; i < 8; i++) {
    double row[6], y2[6];
    for (int j = 0; j < 6; j++) { row[j] = kSCO[j][i]; t.sco[i][j] = kSCO[j][i]; }
    spline_natural<double>(t.nh2, row, 6, y2, u);
    for (int j = 0; j < 6; j++) t.scoderiv[i][j] = y2[j];
  }
  cudaError_t e = cudaMemcpyToSymbol(c_shield, &t, sizeof t);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyToSymbol(shield tables)");
  if (dev >= 0 && dev < 64) g_shield_ready[dev] = true;
  return 0;
}

// host copies for the test/diagnostic export
void shield_tables_host(double *xderiv30, double *scoderiv48) {
  double lg[30], xg[30], u[64];
  for (int i = 0; i < 30; i++) { lg[i] = kLGrid[i]; xg[i] = kXGrid[i]; }
  spline_natural<double>(lg, xg, 30, xderiv30, u);
  double nh2[6];
  for (int j = 0; j < 6; j++) nh2[j] = kNH2Grid[j];
  for (int i = 0; i < 8; i++) {
    double row[6], y2[6];
    for (int j = 0; j < 6; j++) row[j] = kSCO[j][i];
    spline_natural<double>(nh2, row, 6, y2, u);
    for (int j = 0; j < 6; j++) scoderiv48[i * 6 + j] = y2[j];
  }
}

namespace {

constexpr double KB = 1.38065040e-16, AU = 1.66053878e-24;
constexpr double PI = 3.141592653589793238462643383279502884197;

__device__ double xlambda(double lambda, int linear) {
  const ShieldTables &t = c_shield;
  if (lambda < t.lgrid[0]) lambda = t.lgrid[0];
  if (lambda > t.lgrid[29]) lambda = t.lgrid[29];
  double zero[30];
  if (linear)
    for (int i = 0; i < 30; i++) zero[i] = 0.0;
  return splint<double>(t.lgrid, t.xgrid, linear ? zero : t.xderiv, 30, lambda);
}

__device__ double scatter(double av, double lambda, int linear) {
  const double A[6] = {1.000, 2.006, -1.438, 0.7364, -0.5076, -0.0592};
  const double K[6] = {0.7514, 0.8490, 1.013, 1.282, 2.005, 5.832};
  const double taul = (av / 1.086) * xlambda(lambda, linear);
  double s = 0.0;
  if (taul < 1.0) {
    const double e = K[0] * taul;
    if (e < 100.0) s = A[0] * exp(-e);
  } else {
    for (int i = 1; i <= 5; i++) {
      const double e = K[i] * taul;
      if (e < 100.0) s = s + A[i] * exp(-e);
    }
  }
  return s;
}

__device__ double h2shield1(double nh2, double dopw, double radw) {
  const double taud = nh2 * 0.5 * (1.497358985e-2) * 1.0e-2 / dopw;
  double jd, jr;
  if (taud == 0.0) jd = 1.0;
  else if (taud < 2.0) jd = exp(-(0.666666667 * taud));
  else if (taud < 10.0) jd = 0.638 * pow(taud, -1.25);
  else if (taud < 100.0) jd = 0.505 * pow(taud, -1.15);
  else jd = 0.344 * pow(taud, -1.0667);
  if (radw == 0.0) jr = 0.0;
  else {
    const double r = radw / (1.772453851 * dopw);
    const double t = 3.02 * pow(r * 1.0e3, -0.064);
    const double u = sqrt(taud * r) / t;
    jr = r / (t * sqrt(0.785398163 + u * u));
  }
  return jd + jr;
}

__device__ double coshield(double nco, double nh2) {
  const ShieldTables &t = c_shield;
  double lnco = log10(nco + 1.0), lnh2 = log10(nh2 + 1.0);
  if (lnco < t.nco[0]) lnco = t.nco[0];
  if (lnh2 < t.nh2[0]) lnh2 = t.nh2[0];
  if (lnco > t.nco[7]) lnco = t.nco[7];
  if (lnh2 > t.nh2[5]) lnh2 = t.nh2[5];
  double yy[8], yy2[8], u[8];
  for (int i = 0; i < 8; i++) yy[i] = splint<double>(t.nh2, t.sco[i], t.scoderiv[i], 6, lnh2);
  spline_natural<double>(t.nco, yy, 8, yy2, u);
  return pow(10.0, splint<double>(t.nco, yy, yy2, 8, lnco));
}

__device__ double lbar(double nco, double nh2) {
  const double u = log10(nco + 1.0), w = log10(nh2 + 1.0);
  double l = (5675.0 - 200.6 * w) - (571.6 - 24.09 * w) * u + (18.22 - 0.7664 * w) * (u * u);
  if (l < 913.6) l = 913.6;
  if (l > 1076.1) l = 1076.1;
  return l;
}

__device__ double h2_formation(double Tg, double Td, double Z, double g2d) {
  const double vth = 1.45e5 * sqrt(Tg / 1.0e2);
  const double tt = Tg / 1.0e2;
  const double stick = 1.0 / (1.0 + 0.04 * sqrt(Tg + Td) + 0.2 * tt + 0.08 * (tt * tt));
  const double flux = 1.0e-10, mu = 0.005, nu_h2 = 3.0e12, nu_hc = 1.3e13, ehc = 3.0e4;
  const double es[2] = {110.0, 260.0}, eh2[2] = {320.0, 520.0}, ehp[2] = {450.0, 800.0};
  double eff[2];
  for (int g = 0; g < 2; g++) {
    const double f1 = mu * flux / (2 * nu_h2 * exp(-eh2[g] / Td));
    const double sq = 1.0 + sqrt((ehc - es[g]) / (ehp[g] - es[g]));
    const double f2 = 1.0 * (sq * sq) / 4.0 * exp(-es[g] / Td);
    const double eps = 1.0 / (1.0 + nu_hc / (2 * flux) * exp(-1.5 * ehc / Td) * (sq * sq));
    eff[g] = 1.0 / (1.0 + f1 + f2) * eps;
  }
  return 0.5 * vth * (8.473e-22 * eff[0] + 7.908e-22 * eff[1]) * stick * Z * 100. / g2d;
}

struct RateRow {
  double alpha, beta, gamma, rtmin, rtmax;
  int kind, dup, tail, flags;
};

// only the selected member of a duplicate group gets a rate (the member whose
// temperature range holds T, else the group's last)
__device__ __forceinline__ bool dup_selected(const RateRow *tab, int r, double t) {
  const RateRow &w = tab[r];
  if (w.dup > 0 && (w.kind == RK_THERMAL || w.kind == RK_PHOTO || w.kind == RK_CRP || w.kind == RK_CRPHOT)) {
    int head = r;
    while (head > 0 && tab[head].dup > 1) head--;
    int sel = head;
    while (!(t <= tab[sel].rtmax || tab[sel].tail)) sel++;
    return sel == r;
  }
  return true;
}

// one ray's term of a ray-summed rate (the summand of calc_reac_rates.F90's
// loop over the rays, the same expression in the same order)
__device__ __forceinline__ double ray_term(const RateRow &w, double t, const double *rs, const double *av,
                                           const double *cc, int ray, double dopw, double radw, int linear) {
  const double a = w.alpha, g = w.gamma;
  switch (w.kind) {
    case RK_PHOTO_H2:
    case RK_PHOTO_HD: {
      const int c = (w.kind == RK_PHOTO_H2) ? 0 : 1;
      return a * rs[ray] * h2shield1(cc[ray * 5 + c], dopw, radw) * scatter(av[ray], 1000.0, linear) / 2.0;
    }
    case RK_PHOTO_CO: {
      const double nco = cc[ray * 5 + 2], nh2 = cc[ray * 5 + 0];
      return a * rs[ray] * coshield(nco, nh2) * scatter(av[ray], lbar(nco, nh2), linear) / 2.0;
    }
    case RK_PHOTO_CI: {
      const double tauc = g * av[ray] + 1.1e-17 * cc[ray * 5 + 3] +
                          (0.9 * pow(t, 0.27) * pow(cc[ray * 5 + 0] / 1.59e21, 0.45));
      return a * rs[ray] * exp(-tauc) / 2.0;
    }
    case RK_PHOTD: {
      const double y = (t < 50.0) ? 3.5e-3 : (t < 85.0 ? 4.0e-3 : (t < 100.0 ? 5.5e-3 : 7.5e-3));
      return 1.7e8 * rs[ray] * exp(-(1.8 * av[ray])) * 2.4e-22 * y;
    }
    default:   // RK_PHOTO, RK_PHOTO_SI
      return a * rs[ray] * exp(-(g * av[ray])) / 2.0;
  }
}

// calc_reac_rates.F90's clamps: a negative rate is reported, rates above 1
// are capped unless the first reactant is a grain, rates below 1e-99 are zero
__device__ __forceinline__ void store_rate(double k, const RateRow &w, int r, double *out, bool &neg, int &negr) {
  if (k < 0.0) { negr = neg ? min(negr, r + 1) : r + 1; neg = true; }
  if (k > 1.0 && !(w.flags & 1)) k = 1.0;
  if (k < 1.0e-99) k = 0.0;
  out[r] = k;
}

// One warp per cell.  The ray-summed reactions go first, one reaction per
// group of nrays lanes (a lane per ray: the shielding functions of a ray run
// in parallel, and the group's sum is taken in ray order); then the other
// reactions, a lane each, in the order of their kinds.
__global__ void __launch_bounds__(256) rates_kernel(const __grid_constant__ RateTables T, pdr_phys ph,
                                                    int ncell, int nrays, const double *__restrict__ Tg,
                                                    const double *__restrict__ Td,
                                                    const double *__restrict__ rad,
                                                    const double *__restrict__ AV,
                                                    const double *__restrict__ col5,
                                                    const double *__restrict__ zeta_cell,
                                                    double *__restrict__ rate, int *__restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem[];
  RateRow *tab = reinterpret_cast<RateRow *>(smem);
  const int nreac = T.nreac;
  for (int r = threadIdx.x; r < nreac; r += blockDim.x) {
    RateRow w;
    w.alpha = T.alpha[r]; w.beta = T.beta[r]; w.gamma = T.gamma[r];
    w.rtmin = T.rtmin[r]; w.rtmax = T.rtmax[r];
    w.kind = T.kind[r]; w.dup = T.dup[r];
    w.tail = (T.dup_next[r] < 0 || T.dup_next[r] < T.dup[r]) ? 1 : 0;
    w.flags = T.flags[r];
    tab[r] = w;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  const double dopw = ph.v_turb / (1000.0 * 1.0e-8), radw = 8.0e7;
  const int linear = ph.xlambda_linear;
  for (int cell = blockIdx.x * wpb + (threadIdx.x >> 5); cell < ncell; cell += gridDim.x * wpb) {
    const double t = Tg[cell], td = Td[cell];
    // ZETA, or the cell's own rate in the cosmic-ray variant (zetacrlocal)
    const double zeta = zeta_cell ? zeta_cell[cell] : ph.zeta;
    const double *rs = rad + (size_t)cell * nrays;
    const double *av = AV + (size_t)cell * nrays;
    const double *cc = col5 + (size_t)cell * nrays * 5;
    double *out = rate + (size_t)cell * nreac;
    bool neg = false;
    int negr = 0;
    if (nrays <= 32) {
      const int per = 32 / nrays;
      const int g = lane / nrays, ray = lane - g * nrays;
      for (int base = 0; base < T.nray; base += per) {
        const int j = base + g;
        const bool act = (g < per) && (j < T.nray);
        const int r = act ? __ldg(&T.ray_reac[j]) : 0;
        double term = 0.0;
        if (act && dup_selected(tab, r, t)) term = ray_term(tab[r], t, rs, av, cc, ray, dopw, radw, linear);
        double k = 0.0;
        for (int q = 0; q < nrays; q++) k = k + __shfl_sync(0xffffffffu, term, min(g * nrays + q, 31));
        if (act && ray == 0) store_rate(k, tab[r], r, out, neg, negr);
      }
    } else {
      for (int j = lane; j < T.nray; j += 32) {
        const int r = __ldg(&T.ray_reac[j]);
        double k = 0.0;
        if (dup_selected(tab, r, t))
          for (int ray = 0; ray < nrays; ray++) k = k + ray_term(tab[r], t, rs, av, cc, ray, dopw, radw, linear);
        store_rate(k, tab[r], r, out, neg, negr);
      }
    }
    for (int i = lane; i < T.nother; i += 32) {
      const int r = __ldg(&T.other_reac[i]);
      const RateRow &w = tab[r];
      double k = 0.0;
      if (dup_selected(tab, r, t)) {
        const double a = w.alpha, b = w.beta, g = w.gamma;
        switch (w.kind) {
          case RK_H2FORM: k = ph.h2form ? h2_formation(t, td, ph.metallicity, ph.g2d) : 3.0e-18 * sqrt(t); break;
          case RK_PAH: k = a * pow(t / 100.0, b) * 0.4; break;
          case RK_THERMAL:
            k = (g < -200.0 && t < w.rtmin) ? 0.0 : a * pow(t / 300.0, b) * exp(-(g / t));
            break;
          case RK_CRP: k = a * zeta; break;
          case RK_CRPHOT: k = a * zeta * pow(t / 300.0, b) * g / (1.0 - ph.omega); break;
          case RK_FREEZE:
          case RK_ELFRZE: {
            const double cion = (b == 0.0) ? 1.0 : (b == 1.0 ? 1.0 + 16.71e-4 / (ph.grain_radius * t) : 0.0);
            k = a * 4.57e4 * 2.4e-22 * sqrt(t / g) * cion * 0.3;
            break;
          }
          case RK_CRH: k = 2.06e-3 * zeta * 2.4e-22 * ((g <= 1210.0) ? 1.0e5 : 0.0); break;
          case RK_THERM: k = sqrt(2.0 * 1.5e15 * KB / (PI * PI * AU) * a / g) * exp(-(a / td)); break;
          case RK_GRAIN: k = a; break;
          default: k = 0.0; break;
        }
      }
      store_rate(k, w, r, out, neg, negr);
    }
    // the lowest-numbered negative rate of the cell, as a negative status
    const unsigned anyneg = __ballot_sync(0xffffffffu, neg);
    if (status) {
      int rr = neg ? negr : 0x7fffffff;
      for (int o = 16; o > 0; o >>= 1) rr = min(rr, __shfl_xor_sync(0xffffffffu, rr, o));
      if (lane == 0) status[cell] = anyneg ? -rr : 0;
    }
  }
}

}  // namespace

int launch_rates(const pdr_net *net, const pdr_phys &ph, int ncell, int nrays, const double *T,
                 const double *Td, const double *rad, const double *AV, const double *col5, const double *zeta,
                 double *rate, int *status, int sm_count, cudaStream_t st) {
  const size_t smem = sizeof(RateRow) * (size_t)net->rates.nreac;
  if (smem > 200 * 1024) return PDR_E_NET;
  // the attribute only grows, so concurrent launches for networks of
  // different sizes (server lanes) never lower it under each other
  // (per device: the attribute is a property of the function on each device)
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  dev &= 63;
  {
    static std::mutex mu;
    static size_t attr[64] = {};
    std::lock_guard<std::mutex> lk(mu);
    if (smem > attr[dev]) {
      e = cudaFuncSetAttribute(rates_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(rates)");
      attr[dev] = smem;
    }
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rates_kernel, 256, smem);
  if (per_sm < 1) per_sm = 1;
  long long blocks = (ncell + 7) / 8;
  long long cap = (long long)sm_count * per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  rates_kernel<<<(int)blocks, 256, smem, st>>>(net->rates, ph, ncell, nrays, T, Td, rad, AV, col5, zeta, rate,
                                                status);
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "rates_kernel launch");
}

}  // namespace pdr
