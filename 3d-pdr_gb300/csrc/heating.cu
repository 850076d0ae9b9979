// heating.cu -- batched gas heating rates (GPU form of CALC_HEATING,
// sub_calculate_heating.F90:7-386), one thread per cell.
//
// The twelve terms and their total follow the reference term by term,
// including its Newton iteration for the grain-charge parameter X (:80-86),
// the network-specific chemical heating with the reference's hard-coded
// reaction numbers (reduced :228-238, full :240-247) and the Fortran
// default-REAL literals (e.g. 0.4*EV, T**0.068), which are single-precision
// constants promoted to double and are written here as (double)x.f.
#include "pdr_internal.h"

namespace pdr {
namespace {

constexpr double KB = 1.38065040e-16, EV = 1.60217646e-12;
constexpr double PI = 3.141592653589793238462643383279502884197;
#define R4(x) ((double)(x##f))

struct HeatArgs {
  int ncell, nspec, nreac, network;
  // species labels (0-based, species-file positions as the Fortran side uses them)
  int iE, iH, iH2, iC, iCO, iH2x, iH3x, iH3Ox, iHCOx, iHEx;
  int nr[6];   // NRGR..NRSI, 1-based
  pdr_phys ph;
  const double *zeta;   // per-cell ZETA (the cosmic-ray variant's zetacrlocal) or null
  const double *density, *Tg, *Td, *uv, *ab, *rate;
  double *out;
};

__global__ void __launch_bounds__(256) heating_kernel(const __grid_constant__ HeatArgs A) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= A.ncell) return;
  const double n = A.density[cell], T = A.Tg[cell], Td = A.Td[cell];
  const double *ab = A.ab + (size_t)cell * A.nspec;
  const double *R = A.rate + (size_t)cell * A.nreac - 1;   // 1-based reaction numbers
  const double Z = A.ph.metallicity;
  const double xe = ab[A.iE];
  const double habing = 1.68 * A.uv[cell];
  const double deltad = 1.0, deltauv = 1.8, y = 0.1, hnud = 6.0, hnuh = 13.6;
  const double xk = KB * T / (hnuh * EV), xd = hnud / hnuh;
  const double gam = 2.9e-4 * y * sqrt(T) * habing / (xe * n);
  double delta = xk - xd + gam;
  double x = 0.5, xx = x;
  for (int it = 1; it <= 100; it++) {
    const double F = (x * x * x) + delta * (x * x) - gam;
    const double FF = 3 * (x * x) + delta * (2 * x);
    xx = x - (F / FF);
    if (fabs(xx - x) < 1.0e-2) break;
    x = xx;
  }
  x = xx;
  const double pe = 2.7e-25 * deltauv * deltad * n * y * habing *
                    (((1.0 - x) * (1.0 - x)) / x + xk * ((x * x) - 1.0) / (x * x)) * Z;
  const double alpha = 0.944, beta = 0.735 / pow(T, R4(0.068));
  delta = habing * sqrt(T) / (xe * n * 1.0);
  const double eps = 4.87e-2 / (1.0 + 4.0e-3 * pow(delta, R4(0.73))) +
                     3.65e-2 * pow(T / 1.0e4, R4(0.7)) / (1.0 + 2.0e-4 * delta);
  const double pah = (1.30e-24 * eps * habing * n - 4.65e-30 * pow(T, alpha) * pow(delta, beta) * xe * n * 1.0 * n) * Z;
  const double C0 = 5.72e+0, C1 = 3.45e-2, C2 = 7.08e-3, C3 = 1.98e-2, C4 = 4.95e-1, C5 = 6.92e-1, C6 = 5.20e-1;
  const double wa = habing * sqrt(T) / (xe * n);
  const double wd = Z * 1.0e-26 * (habing * n) * (C0 + C1 * pow(T, C4)) /
                    (1.0 + C2 * pow(wa, C5) * (1.0 + C3 * pow(wa, C6)));
  const double cion = (1.0 * EV) * R[A.nr[4]] * ab[A.iC] * n;
  const double h2f = (1.5 * EV) * R[A.nr[0]] * n * ab[A.iH] * n;
  const double h2p = (R4(0.4) * EV) * R[A.nr[1]] * ab[A.iH2] * n;
  const double ncr = 1.0e6 / sqrt(T) /
                     (1.6 * ab[A.iH] * exp(-((400.0 / T) * (400.0 / T))) + 1.4 * ab[A.iH2] * exp(-(18100.0 / (T + 1200.0))));
  const double fuv = (R4(2.2) * EV) * 9.0 * R[A.nr[1]] * ab[A.iH2] * n / (1.0 + ncr / n);
  const double zeta = A.zeta ? A.zeta[cell] : A.ph.zeta;
  const double cr = (R4(9.4) * EV) * (1.3e-17 * zeta) * n * ab[A.iH2];
  const double vt = A.ph.v_turb / 1.0e5;
  const double turb = 3.5e-28 * (vt * vt * vt) * (1.0 / 5.0) * n;
  double chem;
  if (A.network == 0) {
    chem = ab[A.iH2x] * n * xe * R[216] * R4(10.9) * EV
         + ab[A.iH2x] * n * ab[A.iH] * R[155] * R4(0.94) * EV
         + ab[A.iHCOx] * n * xe * n * (R[240] * (R4(7.51) * EV))
         + ab[A.iH3x] * n * xe * n * (R[217] * (R4(4.76) * EV) + R[218] * (R4(9.23) * EV))
         + ab[A.iH3Ox] * n * xe * n * (R[236] * (R4(1.16) * EV) + R[237] * (R4(5.63) * EV) + R[238] * (R4(6.27) * EV))
         + ab[A.iHEx] * n * ab[A.iH2] * n * (R[50] * (R4(6.51) * EV) + R[170] * (R4(6.51) * EV))
         + ab[A.iHEx] * n * ab[A.iCO] * n * (R[89] * (R4(2.22) * EV) + R[90] * (R4(2.22) * EV) + R[91] * (R4(2.22) * EV));
  } else {
    chem = ab[A.iHCOx] * n * xe * n * (R[730] * (R4(7.51) * EV))
         + ab[A.iH3x] * n * xe * n * (R[706] * (R4(4.76) * EV) + R[705] * (R4(9.23) * EV))
         + ab[A.iH3Ox] * n * xe * n * (R[717] * (R4(1.16) * EV) + R[716] * (R4(5.63) * EV) + R[714] * (R4(6.27) * EV))
         + ab[A.iHEx] * n * ab[A.iH2] * n * (R[1227] * (R4(6.51) * EV) + R[265] * (R4(6.51) * EV))
         + ab[A.iHEx] * n * ab[A.iCO] * n * (R[1541] * (R4(2.22) * EV));
  }
  const double acc = 0.35 * exp(-sqrt((Td + T) / 5.0e2)) + 0.1;
  const double ngrain = 1.998e-12 * n * Z * 100. / A.ph.g2d;
  const double cgrain = PI * (A.ph.grain_radius * A.ph.grain_radius);
  const double gg = 4.003e-12 * n * ngrain * cgrain * acc * sqrt(T) * (Td - T);
  double *o = A.out + (size_t)cell * 12;
  o[0] = pe; o[1] = pah; o[2] = wd; o[3] = cion; o[4] = h2f; o[5] = h2p; o[6] = fuv; o[7] = cr;
  o[8] = turb; o[9] = chem; o[10] = gg;
  o[11] = +pah + cion + h2f + h2p + fuv + cr + turb + chem + gg;
}

}  // namespace

int launch_heating(const pdr_net *net, int network, const pdr_phys &ph, int ncell, const double *dens,
                   const double *Tg, const double *Td, const double *uv, const double *ab, const double *rate,
                   const double *zeta, double *out, cudaStream_t st) {
  const HostNet &h = net->host;
  auto idx = [&](const char *a, const char *b) {
    for (int i = 0; i < h.nspec; i++)
      if (h.spec[i] == a || (b && h.spec[i] == b)) return i;
    return -1;
  };
  HeatArgs A;
  A.ncell = ncell; A.nspec = h.nspec; A.nreac = h.nreac; A.network = network; A.ph = ph;
  A.iE = h.nspec - 1;
  A.iH = idx("H", nullptr); A.iH2 = idx("H2", nullptr); A.iC = idx("C", nullptr); A.iCO = idx("CO", nullptr);
  A.iH2x = idx("H2+", nullptr); A.iH3x = idx("H3+", nullptr); A.iH3Ox = idx("H3O+", nullptr);
  A.iHCOx = idx("HCO+", nullptr); A.iHEx = idx("He+", "HE+");
  for (int k = 0; k < 6; k++) A.nr[k] = h.nr[k];
  const int need[] = {A.iH, A.iH2, A.iC, A.iCO, A.iH2x, A.iH3x, A.iH3Ox, A.iHCOx, A.iHEx};
  for (int v : need)
    if (v < 0) { set_error("heating: the network lacks a species the heating terms use"); return PDR_E_NET; }
  if (A.nr[0] == 0 || A.nr[1] == 0 || A.nr[4] == 0) {
    set_error("heating: the network lacks the H2 formation, H2 or C photo-reactions");
    return PDR_E_NET;
  }
  const int maxr = network == 0 ? 240 : 1541;
  if (h.nreac < maxr) { set_error("heating: reaction numbers of the chemical heating exceed the network"); return PDR_E_NET; }
  A.density = dens; A.Tg = Tg; A.Td = Td; A.uv = uv; A.ab = ab; A.rate = rate; A.out = out; A.zeta = zeta;
  heating_kernel<<<(ncell + 255) / 256, 256, 0, st>>>(A);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "heating_kernel launch");
}

}  // namespace pdr
