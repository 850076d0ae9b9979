// thermal.cu -- the outer-iteration controllers resident on the device:
// the per-cell thermal-balance update (3DPDR.F90:928-1050) and the
// level-population convergence check with the population update
// (3DPDR.F90:1084-1229).
//
// Both keep their per-cell state in HBM between outer iterations; the host
// reads back only the counts it prints (converged cells, level-converged
// cells per coolant).  The arithmetic is the reference's: the cooling total is
// the left-to-right sum of the coolants (3DPDR.F90:897), the 30% brackets are
// 1.3D0*T and 0.7D0*T, the binary chop (a+b)/2.0D0 (taken as (a+b)*0.5, the
// same correctly rounded value) -- no products feed an add, so nothing is
// contracted and the results are bit-identical to the host's.
#include <cstdint>

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
            t = __dmul_rn(__dadd_rn(thigh, tlow), 0.5);
            f |= CHOP;
          }
          if (fm < 0.0 && (f & HEAT)) {
            t = __dmul_rn(__dadd_rn(thigh, tlow), 0.5);
            f |= CHOP;
          }
        } else {
          if (fm > 0.0) {
            tlow = t;
            t = __dmul_rn(__dadd_rn(t, thigh), 0.5);
          }
          if (fm < 0.0) {
            thigh = t;
            t = __dmul_rn(__dadd_rn(t, tlow), 0.5);
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
  int ncell, ncool, nspec, vec;
  int copy;   // copy SOLUTION into the populations in the same sweep
  int nlev[PDR_MAX_COOLANTS], species[PDR_MAX_COOLANTS];
  float inv_nlev[PDR_MAX_COOLANTS];
  const double *sol[PDR_MAX_COOLANTS];
  double *pop[PDR_MAX_COOLANTS];
  const double *ab;
  unsigned char *flags, *cconv;
  int *counts;
};

constexpr int LC_CELLS = 256;   // cells per block; one thread per cell for the flags
constexpr int LC_BATCH = 4;     // element pairs in flight per thread

// One level's check (3DPDR.F90:1090-1102): returns true when the level is
// checked and changed by more than 1e-2, i.e. sv >= floor and
// 2|(sv-pv)/(sv+pv)| > 1e-2, in the reference's FP64 operations.
__device__ __forceinline__ bool level_moved_fp64(double sv, double pv, double floor) {
  if (!(sv >= floor)) return false;
  double relch = 0.0;
  if (!(sv == 0.0 && pv == 0.0)) relch = __dmul_rn(2.0, fabs(__ddiv_rn(__dsub_rn(sv, pv), __dadd_rn(sv, pv))));
  return relch > 1.0e-2;
}

// The same decision, settled in integer arithmetic where that is certain.
// For positive normal finite doubles the bit pattern read as an integer, over
// 2^52, is L(x) = E + f for x = 2^(E-1023) (1+f), a continuous monotone map
// whose slope against ln x lies in [1, 2): |ln s - ln p| is between
// |dL|/2 and |dL|.  The relative change 2|s-p|/(s+p) = 2 tanh(|ln s - ln p|/2)
// exceeds 1e-2 exactly when |ln s - ln p| > 0.01000008, so |dL| <= 0.0099
// means "not moved" and |dL| >= 0.0202 means "moved", with margins far beyond
// the FP64 rounding of the reference's expression.  Everything else -- the
// band between, zeros, negatives, subnormals, infinities, NaN -- takes the
// FP64 path.  Positive s passes s >= floor exactly when its bits are >= the
// floor's for floor > 0, always for floor <= 0, never for a NaN floor.
__device__ __forceinline__ bool level_moved(double sv, double pv, double floor) {
  constexpr unsigned long long MIN_NORMAL = 0x0010000000000000ull, INF = 0x7FF0000000000000ull;
  constexpr long long NOT_MOVED = 44585636310967ll;   // floor(0.0099 * 2^52)
  constexpr long long MOVED = 90972712472885ll;       // ceil(0.0202 * 2^52)
  const unsigned long long sb = __double_as_longlong(sv), pb = __double_as_longlong(pv);
  if (sb - MIN_NORMAL < INF - MIN_NORMAL && pb - MIN_NORMAL < INF - MIN_NORMAL) {
    const unsigned long long fb = __double_as_longlong(floor);
    const unsigned long long fkey =
        (fb & 0x7FFFFFFFFFFFFFFFull) > INF ? ~0ull : ((fb >> 63) ? 0ull : fb);
    if (sb < fkey) return false;
    const long long d = (long long)sb - (long long)pb;
    const long long ad = d < 0 ? -d : d;
    if (ad <= NOT_MOVED) return false;
    if (ad >= MOVED) return true;
  }
  return level_moved_fp64(sv, pv, floor);
}

// Each block owns LC_CELLS consecutive cells.  The per-cell floors
// 1e-10 * abundance(species) go to shared memory first; then the threads sweep
// each coolant's [cell][level] arrays over the block's range in 16-byte pairs
// (LC_BATCH pairs loaded before any is used), mark a cell's coolant
// unconverged in shared memory (an idempotent store) and copy SOLUTION into the
// populations; finally one thread per cell combines the marks into the flags
// and the counts.  The cell of element e is floor((e + 0.5) / nlev), taken in
// FP32: e < LC_CELLS * nlev keeps it exact.
__global__ void __launch_bounds__(LC_CELLS) levconv_kernel(const __grid_constant__ LevConvArgs A) {
  __shared__ unsigned char bad[PDR_MAX_COOLANTS][LC_CELLS];
  __shared__ double floor_of[PDR_MAX_COOLANTS][LC_CELLS];
  const int c0 = blockIdx.x * LC_CELLS;
  const int ncb = min(LC_CELLS, A.ncell - c0);
  const int t = threadIdx.x;
  for (int k = 0; k < A.ncool; k++) {
    bad[k][t] = 0;
    if (t < ncb) floor_of[k][t] = __dmul_rn(A.ab[(size_t)(c0 + t) * A.nspec + A.species[k]], 1.0e-10);
  }
  __syncthreads();
  for (int k = 0; k < A.ncool; k++) {
    const int n = A.nlev[k];
    const float inv = A.inv_nlev[k];
    const size_t base = (size_t)c0 * n;
    const int ne = ncb * n;
    const double *s = A.sol[k] + base;
    double *p = A.pop[k] + base;
    int e0 = 0;
    if (A.vec) {
      // base is a multiple of LC_CELLS elements and the arrays are 16-byte aligned
      const int npair = ne >> 1;
      const double2 *s2 = reinterpret_cast<const double2 *>(s);
      double2 *p2 = reinterpret_cast<double2 *>(p);
      for (int q0 = t; q0 < npair; q0 += LC_CELLS * LC_BATCH) {
        double2 sv[LC_BATCH], pv[LC_BATCH];
#pragma unroll
        for (int u = 0; u < LC_BATCH; u++) {
          const int q = q0 + u * LC_CELLS;
          if (q < npair) {
            sv[u] = s2[q];
            pv[u] = p2[q];
          }
        }
#pragma unroll
        for (int u = 0; u < LC_BATCH; u++) {
          const int q = q0 + u * LC_CELLS;
          if (q < npair) {
            const int ea = 2 * q, eb = ea + 1;
            const int ca = __float2int_rz(__fmul_rn(__int2float_rn(ea) + 0.5f, inv));
            const int cb = __float2int_rz(__fmul_rn(__int2float_rn(eb) + 0.5f, inv));
            if (level_moved(sv[u].x, pv[u].x, floor_of[k][ca])) bad[k][ca] = 1;
            if (level_moved(sv[u].y, pv[u].y, floor_of[k][cb])) bad[k][cb] = 1;
            if (A.copy) p2[q] = sv[u];   // 3DPDR.F90:1212-1229
          }
        }
      }
      e0 = npair * 2;
    }
    for (int e = e0 + t; e < ne; e += LC_CELLS) {
      const int cl = __float2int_rz(__fmul_rn(__int2float_rn(e) + 0.5f, inv));
      const double sv = s[e];
      if (level_moved(sv, p[e], floor_of[k][cl])) bad[k][cl] = 1;
      if (A.copy) p[e] = sv;
    }
  }
  __syncthreads();
  const int c = c0 + t;
  const bool live = t < ncb;
  const unsigned all_mask = (1u << A.ncool) - 1u;
  unsigned conv = 0;
  if (live) {
    for (int k = 0; k < A.ncool; k++)
      if (!bad[k][t]) conv |= 1u << k;
    unsigned f = A.flags[c] & ~LCONV;
    if (conv == all_mask) f |= LCONV;
    A.flags[c] = (unsigned char)f;
    if (A.cconv) A.cconv[c] = (unsigned char)conv;
  }
  count_add(&A.counts[0], live && conv == all_mask);
  for (int k = 0; k < A.ncool; k++) count_add(&A.counts[1 + k], live && ((conv >> k) & 1u));
}

// 3DPDR.F90:1202-1206: with thermal balance, all level_converged flags are
// reset once every cell has converged; decided on the device from the count.
__global__ void __launch_bounds__(256) levconv_reset_kernel(int ncell, const int *counts, unsigned char *flags) {
  if (counts[0] != ncell) return;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += gridDim.x * blockDim.x)
    flags[c] &= (unsigned char)~LCONV;
}

// Without thermal balance the reference updates the populations only while
// some cell has not converged: once every cell has, it leaves the loop before
// the update (3DPDR.F90:1161-1172, goto 2) and keeps the previous populations.
// The decision needs the count over all cells, so this pass runs after the
// check and copies SOLUTION into the populations unless counts[0] == ncell.
__global__ void __launch_bounds__(256) levconv_copy_kernel(const __grid_constant__ LevConvArgs A) {
  if (A.counts[0] == A.ncell) return;
  for (int k = 0; k < A.ncool; k++) {
    const size_t ne = (size_t)A.ncell * A.nlev[k];
    const double *s = A.sol[k];
    double *p = A.pop[k];
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    if (A.vec) {
      const size_t npair = ne >> 1;
      const double2 *s2 = reinterpret_cast<const double2 *>(s);
      double2 *p2 = reinterpret_cast<double2 *>(p);
      for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < npair; q += stride) p2[q] = s2[q];
      if ((ne & 1) && blockIdx.x == 0 && threadIdx.x == 0) p[ne - 1] = s[ne - 1];
    } else {
      for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += stride) p[e] = s[e];
    }
  }
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
  A.vec = 1;
  for (int k = 0; k < ncool; k++) {
    A.nlev[k] = nlev[k];
    A.inv_nlev[k] = 1.0f / (float)nlev[k];
    A.species[k] = species[k];
    A.sol[k] = sol[k];
    A.pop[k] = pop[k];
    if ((reinterpret_cast<uintptr_t>(sol[k]) | reinterpret_cast<uintptr_t>(pop[k])) & 15) A.vec = 0;
  }
  A.ab = ab;
  A.flags = flags;
  A.cconv = cconv;
  A.counts = counts;
  A.copy = thermal_balance ? 1 : 0;
  cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * (1 + ncool), st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(level convergence counts)");
  levconv_kernel<<<(ncell + LC_CELLS - 1) / LC_CELLS, LC_CELLS, 0, st>>>(A);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "levconv_kernel launch");
  const int blocks = std::max(1, std::min((ncell + 255) / 256, sm_count * 8));
  if (thermal_balance) {
    levconv_reset_kernel<<<blocks, 256, 0, st>>>(ncell, counts, flags);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "levconv_reset_kernel launch");
  } else {
    levconv_copy_kernel<<<blocks, 256, 0, st>>>(A);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "levconv_copy_kernel launch");
  }
  return 0;
}

}  // namespace pdr
