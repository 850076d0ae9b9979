// rays.cu -- column densities and the attenuated UV field along the rays.
//
// CALC_UVFIELD (3DPDR.F90:1636-1701) and calc_columndens (3DPDR.F90:1789-1844)
// for all cells at once.  Both walk the evaluation points of every ray in
// order: each step between consecutive points has length |x_i - x_{i-1}| and
// contributes the trapezoid of the two points' densities (times an abundance
// for the species columns).  The sums keep the reference's order and its
// unfused products (explicit round-to-nearest intrinsics), so the columns
// agree with a serial evaluation bit for bit; only the UV field's exp differs
// from a CPU libm in the last place.
//
// The work is gathers: per point 3 coordinates, a grid index, the density of
// that grid point and, for the columns, its abundances.  Threads take one
// cell (UV field) or one (cell, ray, group of 8 species) (columns) and walk
// its points sequentially; consecutive threads take consecutive cells (rays),
// whose point lists are adjacent in memory.
#include <algorithm>

#include "pdr_internal.h"

namespace pdr {
namespace {

constexpr double PC = 3.08568025e+18;   // parsec in cm (healpix_types.F90:98)
constexpr int SG = 8;                     // species per thread in the columns kernel

// |x_i - x_{i-1}| as the reference writes it: sqrt((dx^2 + dy^2) + dz^2)
__device__ __forceinline__ double step_length(const double *xyz, long long p) {
  const double dx = __dsub_rn(xyz[3 * (p - 1)], xyz[3 * p]);
  const double dy = __dsub_rn(xyz[3 * (p - 1) + 1], xyz[3 * p + 1]);
  const double dz = __dsub_rn(xyz[3 * (p - 1) + 2], xyz[3 * p + 2]);
  return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

struct UvArgs {
  int ncell, nrays, ngrid, field, uni_ray;
  long long npoint;
  const int *epray;
  const long long *offset;
  const double *xyz;
  const int *gp;
  const double *rho;
  double g_iso, g_uni, av_fac, uv_fac;
  double *colden, *AV, *rad, *uv;
};

__global__ void uvfield_kernel(const __grid_constant__ UvArgs A) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < A.ncell; c += gridDim.x * blockDim.x) {
    double uv = 0.0;
    for (int j = 0; j < A.nrays; j++) {
      const size_t cj = (size_t)c * A.nrays + j;
      const int ne = A.epray[cj];
      double col = 0.0;
      const long long pstart = A.offset[cj];
      if (ne > 0 && (pstart < 0 || pstart + ne >= A.npoint)) col = nan("");
      else if (ne > 0) {
        const long long p0 = pstart;
        const int g0 = A.gp[p0];
        double rho_prev = (g0 >= 0 && g0 < A.ngrid) ? A.rho[g0] : nan("");
        for (int i = 1; i <= ne; i++) {
          const long long p = p0 + i;
          const int gi = A.gp[p];
          const double rho_i = (gi >= 0 && gi < A.ngrid) ? A.rho[gi] : nan("");
          const double step = step_length(A.xyz, p);
          col = __dadd_rn(col, __dmul_rn(__dmul_rn(__dadd_rn(rho_prev, rho_i) * 0.5, step), PC));
          rho_prev = rho_i;
        }
      }
      const double av = __dmul_rn(col, A.av_fac);
      double rad = 0.0;
      if (A.field == 0) rad = A.g_iso;
      else if (j == A.uni_ray) rad = A.g_uni;
      A.colden[cj] = col;
      A.AV[cj] = av;
      A.rad[cj] = rad;
      uv = __dadd_rn(uv, __dmul_rn(rad, exp(__dmul_rn(-av, A.uv_fac))));
      if (uv < 1.0e-50) uv = 0.0;
    }
    A.uv[c] = uv;
  }
}

constexpr int MAXSEL = 256;

struct ColArgs {
  int ncell, nrays, ngrid, nspec, nsel, ngroup;
  long long npoint;
  const int *epray;
  const long long *offset;
  const double *xyz;
  const int *gp;
  const double *rho, *ab;
  double *out;
  int species[MAXSEL];   // validated on the host
};

__global__ void columns_kernel(const __grid_constant__ ColArgs A) {
  const long long total = (long long)A.ncell * A.nrays * A.ngroup;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int g = (int)(t % A.ngroup);
    const long long cj = t / A.ngroup;
    const int s0 = g * SG, ns = min(SG, A.nsel - s0);
    int k[SG];
    double acc[SG];
#pragma unroll
    for (int u = 0; u < SG; u++) {
      k[u] = (u < ns) ? A.species[s0 + u] : 0;
      acc[u] = 0.0;
    }
    const int ne = A.epray[cj];
    const long long p0 = A.offset[cj];
    bool bad = (ne > 0) && (p0 < 0 || p0 + ne >= A.npoint);
    if (ne > 0 && !bad) {
      int gprev = A.gp[p0];
      if (gprev < 0 || gprev >= A.ngrid) { bad = true; gprev = 0; }
      double rprev = A.rho[gprev];
      for (int i = 1; i <= ne && !bad; i++) {
        const long long p = p0 + i;
        int gi = A.gp[p];
        if (gi < 0 || gi >= A.ngrid) { bad = true; break; }
        const double ri = A.rho[gi];
        const double sp = __dmul_rn(step_length(A.xyz, p), PC);
        const double *xa = A.ab + (size_t)gprev * A.nspec, *xb = A.ab + (size_t)gi * A.nspec;
#pragma unroll
        for (int u = 0; u < SG; u++)
          if (u < ns) {
            const double mid = __dadd_rn(__dmul_rn(rprev, xa[k[u]]), __dmul_rn(ri, xb[k[u]]));
            acc[u] = __dadd_rn(acc[u], __dmul_rn(sp, mid) * 0.5);
          }
        gprev = gi;
        rprev = ri;
      }
    }
    double *o = A.out + cj * A.nsel + s0;
#pragma unroll
    for (int u = 0; u < SG; u++)
      if (u < ns) o[u] = bad ? nan("") : acc[u];
  }
}

struct TauArgs {
  int ncell, nrays, ngrid, nlev, nlin;
  long long npoint;
  const int *epray;
  const long long *offset;
  const double *xyz;
  const int *gp;
  const double *pop, *T, *weights, *frac1;
  const int *up, *lo;
  double v2;
  double *tau;
};

// one warp per (cell, ray), lanes over the radiative lines
__global__ void tau_kernel(const __grid_constant__ TauArgs A) {
  constexpr double KB = 1.38065040e-16, MP = 1.67262164e-24, PI = 3.141592653589793238462643383279502884197;
  const int lane = threadIdx.x & 31;
  const long long nwarp = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long cj = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5);
       cj < (long long)A.ncell * A.nrays; cj += nwarp) {
    const int c = (int)(cj / A.nrays), j = (int)(cj % A.nrays);
    // FRAC2 of escape_probability.F90:57 for this cell's temperature
    const double frac2 = 1.0 / __dsqrt_rn(__dadd_rn(
        __ddiv_rn(__ddiv_rn(__dmul_rn(8.0 * KB, A.T[c]), PI), MP), A.v2));
    const int ne = A.epray[cj];
    const long long p0 = A.offset[cj];
    bool bad = (ne > 0) && (p0 < 0 || p0 + ne >= A.npoint);
    // lines in chunks of 64, two per lane, so that each point's step length is
    // computed once per chunk; a point's term g_u n_l - g_l n_u is shared by the
    // two steps it ends and starts
    for (int l0 = 0; l0 < A.nlin; l0 += 64) {
      int u[2], d[2];
      double gu[2], gd[2], f12[2], prev[2], tau[2];
      bool act[2];
#pragma unroll
      for (int s = 0; s < 2; s++) {
        const int l = l0 + 32 * s + lane;
        act[s] = l < A.nlin;
        u[s] = act[s] ? A.up[l] : 0;
        d[s] = act[s] ? A.lo[l] : 0;
        gu[s] = act[s] ? A.weights[u[s]] : 1.0;
        gd[s] = act[s] ? A.weights[d[s]] : 1.0;
        f12[s] = act[s] ? __dmul_rn(A.frac1[l], frac2) : 0.0;
        tau[s] = 0.0;
        prev[s] = 0.0;
      }
      bool badl = bad;
      if (ne > 0 && !bad) {
        const int ga = A.gp[p0];
        if (ga < 0 || ga >= A.ngrid) badl = true;
        else {
          const double *pa = A.pop + (size_t)ga * A.nlev;
#pragma unroll
          for (int s = 0; s < 2; s++)
            if (act[s]) prev[s] = __dsub_rn(__dmul_rn(pa[d[s]], gu[s]), __dmul_rn(pa[u[s]], gd[s]));
        }
        for (int i = 1; i <= ne && !badl; i++) {
          const long long p = p0 + i;
          const int gb = A.gp[p];
          if (gb < 0 || gb >= A.ngrid) { badl = true; break; }
          const double step = step_length(A.xyz, p);
          const double *pb = A.pop + (size_t)gb * A.nlev;
#pragma unroll
          for (int s = 0; s < 2; s++)
            if (act[s]) {
              const double cur = __dsub_rn(__dmul_rn(pb[d[s]], gu[s]), __dmul_rn(pb[u[s]], gd[s]));
              const double frac3 = __ddiv_rn(__dadd_rn(prev[s], cur) * 0.5, gd[s]);
              tau[s] = __dadd_rn(tau[s], __dmul_rn(__dmul_rn(__dmul_rn(f12[s], frac3), step), PC));
              prev[s] = cur;
            }
        }
      }
#pragma unroll
      for (int s = 0; s < 2; s++)
        if (act[s]) A.tau[((size_t)c * A.nlin + l0 + 32 * s + lane) * A.nrays + j] = badl ? nan("") : tau[s];
    }
  }
}

}  // namespace

int launch_tau(const pdr_coolant *cool, const pdr_rays &r, const double *pop, const double *T, double v_turb,
               double *tau, int sm_count, cudaStream_t st) {
  TauArgs A;
  A.ncell = r.ncell;
  A.nrays = r.nrays;
  A.ngrid = r.ngrid;
  A.npoint = r.npoint;
  A.nlev = cool->dev.nlev;
  A.nlin = cool->dev.nlin;
  A.epray = r.d_epray;
  A.offset = r.d_offset;
  A.xyz = r.d_xyz;
  A.gp = r.d_gridpoint;
  A.pop = pop;
  A.T = T;
  A.weights = cool->dev.weights;
  A.frac1 = cool->dev.line_frac1;
  A.up = cool->dev.line_up;
  A.lo = cool->dev.line_lo;
  A.v2 = v_turb * v_turb;
  A.tau = tau;
  const long long warps = (long long)r.ncell * r.nrays;
  const int blocks = (int)std::max(1ll, std::min((warps + 3) / 4, (long long)sm_count * 16));
  tau_kernel<<<blocks, 128, 0, st>>>(A);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "tau_kernel launch");
}

int launch_uvfield(const pdr_rays &r, const double *rho, int field, const double *G, const double *vectors,
                   double metallicity, double *colden, double *AV, double *rad, double *uv, int sm_count,
                   cudaStream_t st) {
  UvArgs A;
  A.ncell = r.ncell;
  A.nrays = r.nrays;
  A.ngrid = r.ngrid;
  A.npoint = r.npoint;
  A.field = field;
  A.epray = r.d_epray;
  A.offset = r.d_offset;
  A.xyz = r.d_xyz;
  A.gp = r.d_gridpoint;
  A.rho = rho;
  A.colden = colden;
  A.AV = AV;
  A.rad = rad;
  A.uv = uv;
  // Fortran default-REAL literals of input_parameters.F90:57-58
  A.av_fac = (double)6.289e-22f * metallicity;
  A.uv_fac = (double)3.02f;
  A.g_iso = G[0] / (double)r.nrays;
  A.g_uni = 0.0;
  A.uni_ray = -1;
  if (field == 1) {
    // the ray most anti-parallel to G (last one on ties, 3DPDR.F90:1672-1683)
    double best = 0.0;
    for (int j = 0; j < r.nrays; j++) {
      const double d = -(G[0] * vectors[3 * j] + G[1] * vectors[3 * j + 1] + G[2] * vectors[3 * j + 2]);
      if (d >= best) { best = d; A.uni_ray = j; }
    }
    if (A.uni_ray >= 0) A.g_uni = best;
  }
  const int blocks = std::max(1, std::min((r.ncell + 127) / 128, sm_count * 16));
  uvfield_kernel<<<blocks, 128, 0, st>>>(A);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "uvfield_kernel launch");
}

int launch_columns(const pdr_rays &r, const double *rho, const double *ab, int nspec, const int *species, int nsel,
                   double *out, int sm_count, cudaStream_t st) {
  ColArgs A;
  A.ncell = r.ncell;
  A.nrays = r.nrays;
  A.ngrid = r.ngrid;
  A.npoint = r.npoint;
  A.nspec = nspec;
  A.nsel = nsel;
  A.ngroup = (nsel + SG - 1) / SG;
  A.epray = r.d_epray;
  A.offset = r.d_offset;
  A.xyz = r.d_xyz;
  A.gp = r.d_gridpoint;
  A.rho = rho;
  A.ab = ab;
  A.out = out;
  if (nsel > MAXSEL) return PDR_E_ARG;
  for (int s = 0; s < nsel; s++) {
    A.species[s] = species ? species[s] : s;
    if (A.species[s] < 0 || A.species[s] >= nspec) {
      set_error("pdr_column_densities_batched: species index out of range");
      return PDR_E_ARG;
    }
  }
  const long long total = (long long)r.ncell * r.nrays * A.ngroup;
  const long long want = (total + 127) / 128;
  const int blocks = (int)std::max(1ll, std::min(want, (long long)sm_count * 16));
  columns_kernel<<<blocks, 128, 0, st>>>(A);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "columns_kernel launch");
}

}  // namespace pdr
