// thermal.cu -- the outer-iteration controllers resident on the device:
// the per-cell thermal-balance update (3DPDR.F90:928-1050) and the
// level-population convergence check with the population update
// (3DPDR.F90:1084-1229).
//
// Both keep their per-cell state in HBM between outer iterations; the host
// reads back only the counts it prints (converged cells, level-converged
// cells per coolant).  The arithmetic is the reference's: the cooling total is
// the left-to-right sum of the coolants (3DPDR.F90:897), the 30% brackets are
// 1.3D0*T and 0.7D0*T, the binary chop (a+b)/2.0D0 -- no products feed an add,
// so nothing is contracted and the results are bit-identical to the host's.
#include "pdr_internal.h"

namespace pdr {
namespace {

constexpr unsigned CONV = PDR_TB_CONVERGED, CHOP = PDR_TB_BINARY_CHOP, LTMIN = PDR_TB_LEVEL_TMIN,
                   LCONV = PDR_TB_LEVEL_CONVERGED, HEAT = PDR_TB_HEATED, COOL = PDR_TB_COOLED;

struct ThermArgs {
  int ncell, hstride, ncool, level_conv, first_time, temp_fix;
  double Tmin, Tmax, Fcrit, Tdiff;
  const double *heat;
  const double *cool[PDR_MAX_COOLANTS];
  double *T, *Tprev, *Tlow, *Thigh, *Fmean, *Fratio, *total;
  unsigned char *flags;
  int *nconv;
};

// Warp-aggregated count of the lanes with `pred` set.
__device__ __forceinline__ void count_add(int *counter, bool pred) {
  const unsigned b = __ballot_sync(0xffffffffu, pred);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(counter, __popc(b));
}

__global__ void __launch_bounds__(256) thermal_kernel(const __grid_constant__ ThermArgs A) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  bool conv_out = false;
  if (c < A.ncell) {
    double cool = A.cool[0][c];
    for (int k = 1; k < A.ncool; k++) cool = __dadd_rn(cool, A.cool[k][c]);
    if (A.total) A.total[c] = cool;
    unsigned f = A.flags[c];
    if (f & CONV) {
      conv_out = true;   // 3DPDR.F90:912-913: a converged cell keeps its state
    } else {
      const double heat = A.heat[(size_t)c * A.hstride];
      const double fm = __dsub_rn(heat, cool);
      const double fr = __ddiv_rn(__dmul_rn(2.0, fabs(fm)), fabs(__dadd_rn(heat, cool)));
      A.Fmean[c] = fm;
      A.Fratio[c] = fr;
      double t = A.T[c];
      if (A.level_conv && A.first_time) {
        // first bracket (3DPDR.F90:936-953)
        const double dummy = t;
        if (fm == 0.0) {
          A.Tlow[c] = t;
          A.Thigh[c] = t;
        } else if (fm > 0.0) {
          A.Tlow[c] = t;
          t = __dmul_rn(1.3, t);
          f = (f & ~(HEAT | COOL)) | HEAT;
        } else if (fm < 0.0) {
          A.Thigh[c] = t;
          t = __dmul_rn(0.7, t);
          if (t < A.Tmin) t = A.Tmin;
          f = (f & ~(HEAT | COOL)) | COOL;
        }
        A.Tprev[c] = dummy < A.Tmin ? A.Tmin : dummy;
      } else if (A.level_conv) {
        // 30% steps until the sign of the imbalance turns, then the binary
        // chop (3DPDR.F90:955-1003)
        double dummy = t;
        double tlow = A.Tlow[c], thigh = A.Thigh[c];
        if (fr <= A.Fcrit) f |= CONV;
        if (!(f & CHOP)) {
          if (fm > 0.0 && (f & HEAT)) {
            tlow = t;
            t = __dmul_rn(1.3, t);
            thigh = t;
          }
          if (fm < 0.0 && (f & COOL)) {
            thigh = t;
            t = __dmul_rn(0.7, t);
            tlow = t;
            if (t < A.Tmin) t = tlow = thigh = A.Tmin;
          }
          if (fm > 0.0 && (f & COOL)) {
            t = __ddiv_rn(__dadd_rn(thigh, tlow), 2.0);
            f |= CHOP;
          }
          if (fm < 0.0 && (f & HEAT)) {
            t = __ddiv_rn(__dadd_rn(thigh, tlow), 2.0);
            f |= CHOP;
          }
        } else {
          if (fm > 0.0) {
            tlow = t;
            t = __ddiv_rn(__dadd_rn(t, thigh), 2.0);
          }
          if (fm < 0.0) {
            thigh = t;
            t = __ddiv_rn(__dadd_rn(t, tlow), 2.0);
          }
        }
        // TEMP_FIX (3DPDR.F90:1007-1022), then the Tmin/Tmax ends (:1025-1048)
        if (A.temp_fix && fabs(__dsub_rn(t, A.Tprev[c])) <= A.Tdiff && fr > A.Fcrit) f |= CONV;
        double tprev = dummy;
        if (dummy < A.Tmin && fm < 0.0) f |= CONV;
        if (dummy > A.Tmax && fm > 0.0) f |= CONV;
        if (f & CONV) {
          if (dummy < A.Tmin) {
            tprev = t = A.Tmin;
            if (!(f & LTMIN)) {
              f &= ~(CONV | LCONV);
              dummy = A.Tmin;
            }
            f |= LTMIN;
          }
          if (dummy > A.Tmax) tprev = t = A.Tmax;
        }
        A.Tprev[c] = tprev;
        A.Tlow[c] = tlow;
        A.Thigh[c] = thigh;
      }
      A.T[c] = t;
      A.flags[c] = (unsigned char)f;
      conv_out = (f & CONV) != 0;
    }
  }
  if (A.nconv) count_add(A.nconv, conv_out);
}

struct LevConvArgs {
  int ncell, ncool, nspec;
  int nlev[PDR_MAX_COOLANTS], species[PDR_MAX_COOLANTS];
  const double *sol[PDR_MAX_COOLANTS];
  double *pop[PDR_MAX_COOLANTS];
  const double *ab;
  unsigned char *flags, *cconv;
  int *counts;
};

constexpr int LC_CELLS = 256;   // cells per block; one thread per cell for the flags

// Each block owns LC_CELLS consecutive cells.  Its threads sweep the
// coolants' [cell][level] arrays over that range with coalesced element
// strides, mark a cell's coolant unconverged in shared memory (an idempotent
// store), and copy SOLUTION into the populations; then one thread per cell
// combines the marks into the flags and the counts.
__global__ void __launch_bounds__(LC_CELLS) levconv_kernel(const __grid_constant__ LevConvArgs A) {
  __shared__ unsigned char bad[PDR_MAX_COOLANTS][LC_CELLS];
  const int c0 = blockIdx.x * LC_CELLS;
  const int ncb = min(LC_CELLS, A.ncell - c0);
  for (int k = 0; k < A.ncool; k++) bad[k][threadIdx.x] = 0;
  __syncthreads();
  for (int k = 0; k < A.ncool; k++) {
    const int n = A.nlev[k];
    const size_t base = (size_t)c0 * n;
    const int ne = ncb * n;
    const double *s = A.sol[k] + base;
    double *p = A.pop[k] + base;
    for (int e = threadIdx.x; e < ne; e += LC_CELLS) {
      const int cl = e / n;
      const double sv = s[e], pv = p[e];
      const double floor = __dmul_rn(A.ab[(size_t)(c0 + cl) * A.nspec + A.species[k]], 1.0e-10);
      if (sv >= floor) {
        double relch = 0.0;
        if (!(sv == 0.0 && pv == 0.0))
          relch = __dmul_rn(2.0, fabs(__ddiv_rn(__dsub_rn(sv, pv), __dadd_rn(sv, pv))));
        if (relch > 1.0e-2) bad[k][cl] = 1;
      }
      p[e] = sv;   // 3DPDR.F90:1212-1229
    }
  }
  __syncthreads();
  const int c = c0 + threadIdx.x;
  const bool live = threadIdx.x < ncb;
  unsigned conv = 0;
  if (live) {
    for (int k = 0; k < A.ncool; k++)
      if (!bad[k][threadIdx.x]) conv |= 1u << k;
    const bool all = conv == (1u << A.ncool) - 1u;
    unsigned f = A.flags[c] & ~LCONV;
    if (all) f |= LCONV;
    A.flags[c] = (unsigned char)f;
    if (A.cconv) A.cconv[c] = (unsigned char)conv;
  }
  count_add(&A.counts[0], live && conv == (1u << A.ncool) - 1u);
  for (int k = 0; k < A.ncool; k++) count_add(&A.counts[1 + k], live && ((conv >> k) & 1u));
}

// 3DPDR.F90:1202-1206: with thermal balance, all level_converged flags are
// reset once every cell has converged; decided on the device from the count.
__global__ void __launch_bounds__(256) levconv_reset_kernel(int ncell, const int *counts, unsigned char *flags) {
  if (counts[0] != ncell) return;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += gridDim.x * blockDim.x)
    flags[c] &= (unsigned char)~LCONV;
}

}  // namespace

int launch_thermal(const pdr_thermal_params &p, int level_conv, int first_time, const double *heat, int hstride,
                   int ncool, const double *const *cool, const pdr_thermal_state &s, double *total, int *nconv,
                   cudaStream_t st) {
  ThermArgs A = {};
  A.ncell = s.ncell;
  A.hstride = hstride;
  A.ncool = ncool;
  A.level_conv = level_conv != 0;
  A.first_time = first_time != 0;
  A.temp_fix = p.temp_fix != 0;
  A.Tmin = p.Tmin;
  A.Tmax = p.Tmax;
  A.Fcrit = p.Fcrit;
  A.Tdiff = p.Tdiff;
  A.heat = heat;
  for (int k = 0; k < ncool; k++) A.cool[k] = cool[k];
  A.T = s.d_T;
  A.Tprev = s.d_Tprev;
  A.Tlow = s.d_Tlow;
  A.Thigh = s.d_Thigh;
  A.Fmean = s.d_Fmean;
  A.Fratio = s.d_Fratio;
  A.flags = s.d_flags;
  A.total = total;
  A.nconv = nconv;
  cudaError_t e = cudaSuccess;
  if (nconv) e = cudaMemsetAsync(nconv, 0, sizeof(int), st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(converged count)");
  thermal_kernel<<<(s.ncell + 255) / 256, 256, 0, st>>>(A);
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "thermal_kernel launch");
}

int launch_level_convergence(int ncell, int ncool, const int *nlev, const double *const *sol, double *const *pop,
                             const double *ab, int nspec, const int *species, int thermal_balance,
                             unsigned char *flags, unsigned char *cconv, int *counts, int sm_count,
                             cudaStream_t st) {
  LevConvArgs A = {};
  A.ncell = ncell;
  A.ncool = ncool;
  A.nspec = nspec;
  for (int k = 0; k < ncool; k++) {
    A.nlev[k] = nlev[k];
    A.species[k] = species[k];
    A.sol[k] = sol[k];
    A.pop[k] = pop[k];
  }
  A.ab = ab;
  A.flags = flags;
  A.cconv = cconv;
  A.counts = counts;
  cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * (1 + ncool), st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(level convergence counts)");
  levconv_kernel<<<(ncell + LC_CELLS - 1) / LC_CELLS, LC_CELLS, 0, st>>>(A);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "levconv_kernel launch");
  if (thermal_balance) {
    const int blocks = std::max(1, std::min((ncell + 255) / 256, sm_count * 8));
    levconv_reset_kernel<<<blocks, 256, 0, st>>>(ncell, counts, flags);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "levconv_reset_kernel launch");
  }
  return 0;
}

}  // namespace pdr
