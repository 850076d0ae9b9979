// levpop.cu -- batched statistical-equilibrium solves for one coolant
// (the per-cell, per-coolant step of 3DPDR.F90:756-843: FIND_CCOEFF,
// escape_probability after the optical depths are known, solvlevpop).
//
// One warp per cell.  The lanes share the nlev x nlev work:
//   C_ij   linear-in-T interpolation of each partner's table, partners summed in
//          LAMDA-id order with the para/ortho split (find_Ccoeff.F90:35-147);
//   field  per radiative pair: CMB + dust Planck background, source function,
//          ray-averaged escape probability beta(tau) with the masing and
//          small-tau guards (escape_probability.F90:51-167; PSEUDO_1D uses ray 6);
//   R_ij = A_ij + B_ij <J_ij> + C_ij (|R| < 1e-50 -> 0);
//   the solvlevpop matrix (transposed rates, diagonal = -row sum, last row
//   1e-8, rhs = density*1e-8, solvlevpop.F90:18-35) held in shared memory and
//   solved either in FP64 by the reference's Gauss-Jordan elimination with full
//   pivoting (same pivot order, unfused products as in the reference), or
//   (mixed) by an FP32 Gauss-Jordan inverse of the row-equilibrated matrix
//   with partial pivoting and up to two refinement steps, the residual in FP64
//   and the correction in FP32, each accepted by the size of the next
//   correction (cells that fail the check are re-solved in FP64, status 2);
//   negative populations are set to zero.
#include <algorithm>
#include <mutex>
#include <vector>

#include "pdr_internal.h"

namespace pdr {
namespace {

constexpr double KB = 1.38065040e-16, CL = 2.99792458e+10, HP = 6.62606896e-27;
constexpr double PI = 3.141592653589793238462643383279502884197;
constexpr unsigned FULL = 0xffffffffu;

// per-warp shared memory: the nlev^2 FP64 rate matrix, the line values of the
// radiative pairs, four nlev vectors, three int vectors and, for the mixed
// solve, an nlev^2 FP32 matrix and an nlev FP32 vector
struct LevLayout {
  size_t R, lines, b, sp, x, rs, ipiv, indxr, indxc, Mf, total;
};
__host__ __device__ inline LevLayout levpop_layout(int n, int nrad, bool mixed) {
  auto al = [](size_t v) { return (v + 15) & ~size_t(15); };
  LevLayout L;
  size_t o = 0;
  L.R = o; o += al(8 * (size_t)n * n);
  L.lines = o; o += al(8 * (size_t)(nrad > 0 ? nrad : 1));
  L.b = o; o += al(8 * (size_t)n);
  L.sp = o; o += al(8 * (size_t)n);
  L.x = o; o += al(8 * (size_t)n);
  L.rs = o; o += al(8 * (size_t)n);
  L.ipiv = o; o += al(4 * (size_t)n);
  L.indxr = o; o += al(4 * (size_t)n);
  L.indxc = o; o += al(4 * (size_t)n);
  L.Mf = o;
  if (mixed) o += al(4 * (size_t)n * n) + al(4 * (size_t)n);
  L.total = o;
  return L;
}

struct LevArgs {
  int ncell, nrays, pseudo1d;
  double metallicity, g2d;
  const double *density, *T, *Td, *partner5, *cdens, *spop, *tau;
  double *pop, *cooling, *line;
  int *status;
};

// magnitude bit pattern of a value: ordered like |x| for finite values
__device__ __forceinline__ long long mag_bits(double x) { return __double_as_longlong(x) & 0x7fffffffffffffffll; }
__device__ __forceinline__ long long mag_bits(float x) { return (long long)(__float_as_int(x) & 0x7fffffff); }

// warp argmax of (value, index) with ties resolved to the larger index
__device__ __forceinline__ void argmax_last(long long &v, int &idx) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long ov = __shfl_xor_sync(FULL, v, o);
    const int oi = __shfl_xor_sync(FULL, idx, o);
    if (ov > v || (ov == v && oi > idx)) { v = ov; idx = oi; }
  }
}

// Gauss-Jordan with full pivoting on a (n x n, row stride n, n <= 64) and one
// rhs b, warp-cooperative; the result is the reference's element for element:
//  * pivot search: the last maximum in row-major order over the unpivoted rows
//    and columns (the serial scan of GAUSS_JORDAN, solvlevpop.F90:65-174),
//    lanes striding over the flattened matrix, pivoted columns in a bit mask;
//  * elimination: every (row, column) element, b as column n, updated by one
//    lane with the reference's unfused a - a_pivot*dum, so the order in which
//    lanes take the elements does not matter.
// dumv is n scratch values.  Returns false on a singular matrix.
template <class R>
__device__ bool gauss_jordan(R *a, R *b, int n, R *dumv, int *indxr, int *indxc, bool unscramble) {
  const int lane = threadIdx.x & 31;
  const int nn = n * n, w = n + 1;   // elimination width: n columns and b
  unsigned long long used = 0ull;
  for (int it = 0; it < n; it++) {
    long long best = -1;
    int bidx = -1;
    {
      int j = 0, k = lane;
      while (k >= n) { k -= n; j++; }
      for (int e = lane; e < nn; e += 32) {
        if (!((used >> j) & 1ull) && !((used >> k) & 1ull)) {
          // |a| compared through its bit pattern (the order of non-negative
          // IEEE values), on the integer pipe instead of the FP64 one
          const long long v = mag_bits(a[e]);
          if (v >= best) { best = v; bidx = e; }
        }
        k += 32;
        while (k >= n) { k -= n; j++; }
      }
    }
    argmax_last(best, bidx);
    if (bidx < 0) return false;
    const int irow = bidx / n, icol = bidx - irow * n;
    __syncwarp();
    used |= 1ull << icol;
    if (irow != icol) {
      for (int l = lane; l < n; l += 32) {
        const R d = a[irow * n + l];
        a[irow * n + l] = a[icol * n + l];
        a[icol * n + l] = d;
      }
      if (lane == 0) { const R d = b[irow]; b[irow] = b[icol]; b[icol] = d; }
    }
    if (lane == 0) { indxr[it] = irow; indxc[it] = icol; }
    __syncwarp();
    const R piv = a[icol * n + icol];
    if (piv == R(0)) return false;
    const R pivinv = R(1) / piv;
    __syncwarp();
    if (lane == 0) a[icol * n + icol] = R(1);
    __syncwarp();
    for (int l = lane; l < n; l += 32) a[icol * n + l] = a[icol * n + l] * pivinv;
    if (lane == 0) b[icol] = b[icol] * pivinv;
    // the multipliers, read before any row changes
    for (int ll = lane; ll < n; ll += 32) dumv[ll] = a[ll * n + icol];
    __syncwarp();
    {
      int ll = 0, l = lane;
      while (l >= w) { l -= w; ll++; }
      for (int e = lane; e < n * w; e += 32) {
        if (ll != icol) {
          const R dum = dumv[ll];
          const R pv = (l < n) ? a[icol * n + l] : b[icol];
          R cur = (l == icol) ? R(0) : ((l < n) ? a[ll * n + l] : b[ll]);
          if constexpr (sizeof(R) == 8) cur = __dsub_rn(cur, __dmul_rn(pv, dum));
          else cur = __fsub_rn(cur, __fmul_rn(pv, dum));
          if (l < n) a[ll * n + l] = cur;
          else b[ll] = cur;
        }
        l += 32;
        while (l >= w) { l -= w; ll++; }
      }
    }
    __syncwarp();
  }
  if (unscramble) {
    for (int l = n - 1; l >= 0; l--) {
      const int r = indxr[l], c = indxc[l];
      if (r != c)
        for (int k = lane; k < n; k += 32) {
          const R d = a[k * n + r];
          a[k * n + r] = a[k * n + c];
          a[k * n + c] = d;
        }
      __syncwarp();
    }
  }
  return true;
}

// The mixed solve's acceptance test on the correction s that a further
// refinement step would make to population x: above 1e-6 of the coolant
// density it must be below 1e-7 of x, above 1e-12 of the density below 1e-4
// of x (ten times inside the 1e-6 and 1e-3 the results are held to), and it
// must contract (at most half the previous correction, or negligible)
__device__ __forceinline__ bool refine_ok(double ax, double as, double prev, double dens) {
  const bool contracts = as <= 0.5 * prev || as <= 1.0e-12 * ax;
  if (ax > 1.0e-6 * dens) return as <= 1.0e-7 * ax && contracts;
  if (ax > 1.0e-12 * dens) return as <= 1.0e-4 * ax && contracts;
  return true;
}

// The mixed solve's FP32 inverse of the row-equilibrated matrix: Gauss-Jordan
// with partial pivoting (the largest |a_ik| among the rows not yet pivoted,
// lowest row on ties), in place.  The inverse only preconditions the FP64
// refinement, so it need not follow the reference's full-pivot order, and a
// column search costs two compares per lane where the full search scans the
// matrix.  Lanes own columns (l = lane, lane + 32); the rows are a uniform
// loop, so no element index is divided.  dumv: n floats.  Returns false on a
// zero pivot.
__device__ bool gj_inverse_pp(float *a, int n, float *dumv, int *indxr) {
  const int lane = threadIdx.x & 31;
  const int l0 = lane, l1 = lane + 32;
  for (int k = 0; k < n; k++) {
    float best = -1.0f;
    int bi = n;
    for (int i = k + lane; i < n; i += 32) {
      const float v = fabsf(a[i * n + k]);
      if (v > best) { best = v; bi = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(FULL, best, o);
      const int oi = __shfl_xor_sync(FULL, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if (!(best > 0.0f)) return false;
    if (bi != k) {
      if (l0 < n) { const float t = a[bi * n + l0]; a[bi * n + l0] = a[k * n + l0]; a[k * n + l0] = t; }
      if (l1 < n) { const float t = a[bi * n + l1]; a[bi * n + l1] = a[k * n + l1]; a[k * n + l1] = t; }
    }
    if (lane == 0) indxr[k] = bi;
    __syncwarp();
    const float pivinv = 1.0f / a[k * n + k];
    // the multipliers of column k, read before any row changes
    for (int i = lane; i < n; i += 32) dumv[i] = a[i * n + k];
    __syncwarp();
    // pivot row scaled (its column k becomes 1/pivot); the other rows take
    // a_il -= a_kl a_ik, column k from zero
    float p0 = 0.0f, p1 = 0.0f;
    if (l0 < n) { p0 = (l0 == k) ? pivinv : a[k * n + l0] * pivinv; a[k * n + l0] = p0; }
    if (l1 < n) { p1 = (l1 == k) ? pivinv : a[k * n + l1] * pivinv; a[k * n + l1] = p1; }
    for (int i = 0; i < n; i++) {
      if (i == k) continue;
      const float dum = dumv[i];
      if (l0 < n) a[i * n + l0] = fmaf(-p0, dum, (l0 == k) ? 0.0f : a[i * n + l0]);
      if (l1 < n) a[i * n + l1] = fmaf(-p1, dum, (l1 == k) ? 0.0f : a[i * n + l1]);
    }
    __syncwarp();
  }
  // the row interchanges undone on the inverse's columns, last first
  for (int k = n - 1; k >= 0; k--) {
    const int r = indxr[k];
    if (r != k)
      for (int i = lane; i < n; i += 32) {
        const float t = a[i * n + r];
        a[i * n + r] = a[i * n + k];
        a[i * n + k] = t;
      }
    __syncwarp();
  }
  return true;
}

template <bool MIXED>
__global__ void __launch_bounds__(256) levpop_kernel(const __grid_constant__ CoolantTables C,
                                                     const __grid_constant__ LevArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int n = C.nlev, nn = n * n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const LevLayout L = levpop_layout(n, C.nrad, MIXED);
  unsigned char *base = smem + L.total * warp;
  double *R = reinterpret_cast<double *>(base + L.R);          // rates, then the solvlevpop matrix
  double *lines = reinterpret_cast<double *>(base + L.lines);  // line values of the radiative pairs
  double *b = reinterpret_cast<double *>(base + L.b);
  double *sp = reinterpret_cast<double *>(base + L.sp);
  double *x = reinterpret_cast<double *>(base + L.x);
  double *rs = reinterpret_cast<double *>(base + L.rs);        // row scales of the FP32 solve
  int *ipiv = reinterpret_cast<int *>(base + L.ipiv);
  int *indxr = reinterpret_cast<int *>(base + L.indxr);
  int *indxc = reinterpret_cast<int *>(base + L.indxc);
  const int wpb = blockDim.x >> 5;
  for (int cell = blockIdx.x * wpb + warp; cell < A.ncell; cell += gridDim.x * wpb) {
    const double T = A.T[cell], Td = A.Td[cell], rho = A.density[cell];
    const double *p5 = A.partner5 + (size_t)cell * 5;
    const double nH = p5[0], nHp = p5[1], ne = p5[2], nHe = p5[3], nH2 = p5[4];
    for (int i = lane; i < n; i += 32) sp[i] = A.spop[(size_t)cell * n + i];
    // ---- collision rates ----
    double fpara = 0.0, fortho = 0.0;
    if (nH2 > 0.0) { fpara = 1.0 / (1.0 + 9.0 * exp(-170.5 / T)); fortho = 1.0 - fpara; }
    for (int e = lane; e < nn; e += 32) R[e] = 0.0;
    __syncwarp();
    for (int q = 0; q < C.npart; q++) {
      const int p = C.part[q];
      const double *tp = C.temps + (size_t)q * C.ntemp;
      int klo = 0, khi = 0;
      for (int k = 1; k <= C.ntemp; k++) {
        if (tp[k - 1] > T) { klo = k - 1; khi = k; break; }
        else if (tp[k - 1] == 0.0) { klo = k - 1; khi = k - 1; break; }
      }
      if (khi == 0) { klo = C.ntemp; khi = C.ntemp; }
      else if (khi == 1) { klo = 1; khi = 1; }
      const double step = (klo == khi) ? 0.0 : (T - tp[klo - 1]) / (tp[khi - 1] - tp[klo - 1]);
      const double *lo = C.col + ((size_t)q * C.ntemp + (klo - 1)) * nn;
      const double *hi = C.col + ((size_t)q * C.ntemp + (khi - 1)) * nn;
      const double dsingle = (p == 0 ? nH2 : p == 3 ? ne : p == 4 ? nH : p == 5 ? nHe : nHp);
      for (int e = lane; e < nn; e += 32) {
        const double tmp = lo[e] + (hi[e] - lo[e]) * step;
        double add;
        if (p == 1 || p == 2) add = tmp * nH2 * (p == 1 ? fpara : fortho);
        else add = tmp * dsingle;
        R[e] = R[e] + add;
      }
    }
    __syncwarp();
    // ---- escape probabilities and the radiative terms ----
    const double ngrain = 2.0e-12 * rho * A.metallicity * 100. / A.g2d;
    const double *tau = A.tau + (size_t)cell * C.nlin * A.nrays;
    // pairs with no radiative coupling in either direction (A = B = 0) leave
    // R unchanged and their line term zero: only the radiative pairs are visited
    for (int pe = lane; pe < C.nrad; pe += 32) {
      const int e = C.rad_pairs[pe];
      const int i = e / n, j = e - i * n;
      const double f = C.freq[e], Aij = C.A[e];
      // per-pair constants (2 h nu^3 / c^2, the 2.7 K background, the dust
      // emissivity factor) come precomputed with the coolant
      const double tmp2 = C.pair_tmp2[pe];
      double bb = C.pair_cmb[pe];
      const double emis = (2.0 * ngrain) * C.pair_emis[pe];
      bb = bb + tmp2 * (1.0 / (exp(HP * f / KB / Td) - 1.0) * emis);
      double S, beta;
      bool has_line = true;
      if (sp[i] == 0.0) {
        S = 0.0; beta = 1.0; has_line = false;
      } else {
        const double tpop = (sp[j] * C.weights[i]) / (sp[i] * C.weights[j]) - 1.0;
        if (fabs(tpop) < 1.0e-50) {
          S = HP * f * sp[i] * Aij / 4. / PI;
          beta = 1.0;
        } else {
          S = tmp2 / tpop;
          const int li = C.line_of_pair[e];
          double bsum = 0.0;
          for (int r = 0; r < A.nrays; r++) {
            double t = (A.pseudo1d && r != 6) ? 1.0e50 : (li >= 0 ? tau[li * A.nrays + r] : 0.0);
            double br;
            if (t < -5.0) br = (1.0 - exp(5.0)) / (-5.0);
            else if (fabs(t) < 1.0e-8) br = 1.0;
            else br = (1.0 - exp(-t)) / t;
            bsum += br;
          }
          beta = A.pseudo1d ? bsum : bsum / (double)A.nrays;
        }
      }
      lines[pe] = has_line ? Aij * HP * f * sp[i] * beta * (S - bb) / S : 0.0;
      const double field = (1.0 - beta) * S + beta * bb;
      const int et = j * n + i;
      R[e] = (Aij + C.B[e] * field) + R[e];
      R[et] = (C.A[et] + C.B[et] * field) + R[et];
    }
    __syncwarp();
    for (int e = lane; e < nn; e += 32)
      if (fabs(R[e]) < 1.0e-50) R[e] = 0.0;
    // the cooling rate: the line values summed over i > j in row-major order,
    // as the reference adds them; the non-radiative pairs contribute zeros,
    // which leave the sum unchanged, so only the radiative pairs are added
    if (lane == 0) {
      double cool = 0.0;
      for (int pe = 0; pe < C.nrad; pe++) cool = cool + lines[pe];
      A.cooling[cell] = cool;
    }
    if (A.line) {
      double *lo = A.line + (size_t)cell * nn;
      for (int e = lane; e < nn; e += 32) lo[e] = 0.0;
      __syncwarp();
      for (int pe = lane; pe < C.nrad; pe += 32) lo[C.rad_pairs[pe]] = lines[pe];
    }
    __syncwarp();
    // ---- solvlevpop matrix: transpose, diagonal -sum, conservation row ----
    for (int i = lane; i < n; i += 32) {
      double out = 0.0;
      for (int j = 0; j < n; j++) out = out + R[i * n + j];
      b[i] = out;
    }
    __syncwarp();
    for (int e = lane; e < nn; e += 32) {
      const int i = e / n, j = e - i * n;
      if (j > i) { const double t = R[e]; R[e] = R[j * n + i]; R[j * n + i] = t; }
    }
    __syncwarp();
    for (int i = lane; i < n; i += 32) R[i * n + i] = -b[i];
    __syncwarp();
    for (int i = lane; i < n; i += 32) { R[(n - 1) * n + i] = 1.0e-8; b[i] = 0.0; }
    __syncwarp();
    const double dens = A.cdens[cell];
    if (lane == 0) b[n - 1] = dens * 1.0e-8;
    __syncwarp();
    bool ok, redo = false;
    if constexpr (!MIXED) {
      ok = gauss_jordan<double>(R, b, n, rs, indxr, indxc, false);
      for (int i = lane; i < n; i += 32) x[i] = b[i];
    } else {
      // FP32 copy of the matrix with its rows equilibrated in FP32 (D M, D =
      // 1 / row maximum), the FP32 inverse of D M (partial pivoting), then
      // x = inv(DM) D b and up to two refinement steps x += inv(DM) D (b - M x)
      // with the residual in FP64 and the correction in FP32.  Each step is
      // accepted by the size of the correction the next would make
      // (refine_ok); otherwise the cell is re-solved by the FP64
      // Gauss-Jordan (R is intact).
      float *Mf = reinterpret_cast<float *>(base + L.Mf);
      float *rf = Mf + nn;                            // FP32 scaled residual
      float *rsf = reinterpret_cast<float *>(rs);     // FP32 row scales
      float *prev = reinterpret_cast<float *>(sp);    // |previous correction| (s_pop is no longer needed)
      float *dumv = reinterpret_cast<float *>(ipiv);
      for (int e = lane; e < nn; e += 32) Mf[e] = (float)R[e];
      __syncwarp();
      for (int i = lane; i < n; i += 32) {
        float mx = 0.0f;
        for (int l = 0; l < n; l++) mx = fmaxf(mx, fabsf(Mf[i * n + l]));
        rsf[i] = (mx > 0.0f) ? 1.0f / mx : 1.0f;
      }
      __syncwarp();
      for (int i = 0; i < n; i++) {
        const float r = rsf[i];
        for (int l = lane; l < n; l += 32) Mf[i * n + l] *= r;
      }
      __syncwarp();
      ok = gj_inverse_pp(Mf, n, dumv, indxr);
      __syncwarp();
      // b is zero but for its last entry: x = column n-1 of the inverse times D b
      const double bl = b[n - 1] * (double)rsf[n - 1];
      for (int i = lane; i < n; i += 32) x[i] = (double)Mf[i * n + n - 1] * bl;
      bool good = false;
      for (int it = 0; it < 3 && ok && !good; it++) {
        __syncwarp();
        for (int i = lane; i < n; i += 32) {
          double s = b[i];
          for (int l = 0; l < n; l++) s = fma(-R[i * n + l], x[l], s);
          rf[i] = (float)s * rsf[i];
        }
        __syncwarp();
        bool bad = false;
        for (int i = lane; i < n; i += 32) {
          float s32 = 0.0f;
          for (int l = 0; l < n; l++) s32 = fmaf(Mf[i * n + l], rf[l], s32);
          const double s = (double)s32;
          // from the second correction on, the correction is also the test of
          // the previous one
          if (it > 0 && !refine_ok(fabs(x[i]), fabs(s), (double)prev[i], dens)) bad = true;
          if (it < 2) {
            x[i] += s;
            prev[i] = fabsf(s32);
          }
        }
        good = (it > 0) && !__any_sync(FULL, bad);
      }
      if (!ok || !good) {
        __syncwarp();
        for (int i = lane; i < n; i += 32) b[i] = 0.0;
        __syncwarp();
        if (lane == 0) b[n - 1] = dens * 1.0e-8;
        __syncwarp();
        ok = gauss_jordan<double>(R, b, n, rs, indxr, indxc, false);
        for (int i = lane; i < n; i += 32) x[i] = b[i];
        redo = true;
      }
    }
    __syncwarp();
    for (int i = lane; i < n; i += 32) {
      double v = x[i];
      if (v < 0.0) v = 0.0;
      A.pop[(size_t)cell * n + i] = v;
    }
    if (lane == 0 && A.status) A.status[cell] = ok ? (redo ? 2 : 0) : 1;
    __syncwarp();
  }
}

}  // namespace

size_t levpop_smem_per_warp(int n, int nrad, bool mixed) { return levpop_layout(n, nrad, mixed).total; }

namespace {
// LTE populations of one cell per thread: CALCULATE_PARTITION_FUNCTION and
// CALCULATE_LTE_POPULATIONS (3DPDR.F90:1847-1894), the same operation order;
// the reference STOPs when the populations do not add up to the density
// within 1e-3 -- here the cell's status is set to 1 instead.
__global__ void lte_kernel(CoolantTables C, int ncell, const double *__restrict__ T,
                           const double *__restrict__ density, double *__restrict__ pop, int *status) {
  for (int cell = blockIdx.x * blockDim.x + threadIdx.x; cell < ncell; cell += gridDim.x * blockDim.x) {
    const double t = T[cell], d = density[cell];
    double z = 0.0;
    for (int i = 0; i < C.nlev; i++) z = z + C.weights[i] * exp(-C.energies[i] / KB / t);
    double tot = 0.0;
    for (int i = 0; i < C.nlev; i++) {
      const double p = d * C.weights[i] * exp(-C.energies[i] / KB / t) / z;
      pop[(size_t)cell * C.nlev + i] = p;
      tot = tot + p;
    }
    if (status) status[cell] = (fabs(tot - d) / d > 1.0e-3) ? 1 : 0;
  }
}
}  // namespace

int launch_lte(const pdr_coolant *c, int ncell, const double *T, const double *density, double *pop, int *status,
               int sm_count, cudaStream_t st) {
  const int blocks = std::min((ncell + 127) / 128, sm_count * 8);
  lte_kernel<<<blocks, 128, 0, st>>>(c->dev, ncell, T, density, pop, status);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "lte_kernel launch");
}

int launch_levpop(const pdr_coolant *c, const LevArgsHost &h, bool mixed, int sm_count, cudaStream_t st) {
  LevArgs A;
  A.ncell = h.ncell; A.nrays = h.nrays; A.pseudo1d = h.pseudo1d;
  A.metallicity = h.metallicity; A.g2d = h.g2d;
  A.density = h.density; A.T = h.T; A.Td = h.Td; A.partner5 = h.partner5; A.cdens = h.cdens;
  A.spop = h.spop; A.tau = h.tau; A.pop = h.pop; A.cooling = h.cooling; A.line = h.line; A.status = h.status;
  const int n = c->dev.nlev;
  if (n > 64) {   // the Gauss-Jordan pivot mask holds 64 levels
    set_error("pdr_levpop_batched: coolants with more than 64 levels are not supported");
    return PDR_E_ARG;
  }
  // the FP32 inverse with refinement pays off only for larger systems: the
  // 5-level coolants take the FP64 elimination in both forms
  if (n <= 8) mixed = false;
  const size_t pw = levpop_smem_per_warp(n, c->dev.nrad, mixed);
  // the block size (1..8 warps) that keeps the most warps resident per SM
  // (the shared memory of one warp bounds it for the 41-level coolant),
  // chosen once per device and warp size; the attribute is set to the largest
  // candidate and never lowered, so concurrent launches cannot undercut it
  auto kern = mixed ? levpop_kernel<true> : levpop_kernel<false>;
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  struct Shape { int dev; size_t pw; bool mixed; int wpb, per_sm; };
  static std::mutex mu;
  static std::vector<Shape> shapes;
  static size_t attr[64][2] = {};
  int wpb = 0, per_sm = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    for (const Shape &sh : shapes)
      if (sh.dev == dev && sh.pw == pw && sh.mixed == mixed) { wpb = sh.wpb; per_sm = sh.per_sm; }
    if (wpb == 0) {
      const size_t top = std::min((size_t)optin, pw * 8);
      if (top > attr[dev & 63][mixed]) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)top);
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(levpop)");
        attr[dev & 63][mixed] = top;
      }
      for (int w = 8; w >= 1; w--) {
        if (pw * w > top) continue;
        int b = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, w * 32, pw * w);
        if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor(levpop)");
        if (b * w > per_sm * wpb) { wpb = w; per_sm = b; }
      }
      if (wpb < 1) {
        set_error("pdr_levpop_batched: one warp's shared memory exceeds a block's");
        return PDR_E_ARG;
      }
      shapes.push_back({dev, pw, mixed, wpb, per_sm});
    }
  }
  const size_t smem = pw * wpb;
  long long blocks = ((long long)h.ncell + wpb - 1) / wpb;
  if (blocks > (long long)sm_count * per_sm) blocks = (long long)sm_count * per_sm;
  if (blocks < 1) blocks = 1;
  kern<<<(int)blocks, wpb * 32, smem, st>>>(c->dev, A);
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "levpop_kernel launch");
}

}  // namespace pdr
