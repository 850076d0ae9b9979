// chem_cta.cu -- batched BDF chemistry integrator, one thread block per cell.
//
// Replaces the per-cell CVODE solve of calculate_abundances.c:124-326 for
// networks of any size up to 252 ODE species (the full network has 214, the
// "mynetwork" example 57).  The block has G = 32*ceil(neq/32) threads (at
// least 64); thread i owns species i: its Nordsieck row, error weight and
// correction, and row i of the Newton matrix.  The CVODE control logic is the
// one shared with the warp-per-cell integrator (bdf_core.cuh); this file
// supplies the block-wide collectives, the network RHS and Jacobian, and the
// dense linear algebra:
//
//   RHS  fluxes phi_r = kn_r x_a x_b reaction-parallel over the block, the
//        stoichiometric sums in G balanced chunks with deterministic partial
//        sums (the same scheme as the warp integrator, stride G);
//   Jac  the entry-sorted term contributions in G balanced chunks, one
//        register sum per entry run (runs across chunks added in chunk
//        order), then the x_e chain rule J_ij += (df_i/dx_e) c_j by row;
//   LU   dense LU with partial pivoting (CVDense semantics: in each column the
//        unpivoted row of largest magnitude, lowest row on ties), rows kept in
//        place with the pivot order recorded; right-looking in panels of 8
//        columns: per panel the pivot rows' U block is formed column-parallel
//        and the trailing update is a rank-8 update applied by the row owners,
//        four columns at a time, to the columns where that U block has a
//        nonzero (the network's
//        Jacobian is sparse, so many are exactly zero -- skipping them changes
//        no result);
//   solve forward/backward substitution in 32-row blocks: the 32x32 diagonal
//        blocks of L and U are inverted in place at setup, so a block step is
//        a 32x32 product by one warp plus a rank-32 update by the row owners.
//
// The matrix is column-major, element (i, j) at j*ld + i with ld odd: thread
// i's accesses to its own row are consecutive across a warp (coalesced in
// global memory, conflict-free in shared memory) and the pivot-row reads are
// broadcasts.  PDR_MIXED keeps it in shared memory in FP32 after the
// similarity scaling W M W^-1, W = diag(1/(rtol|y|+atol)) (the full network's
// 214 x 216 FP32 matrix plus the integrator's arrays fit the 227 KB of one
// block); PDR_FP64 keeps it in FP64, in shared memory when it fits and
// otherwise in a per-block slot of global memory that stays in L2.  A cell
// whose FP32 Newton iteration fails with a fresh matrix is re-solved in FP64.
#include <cstdint>
#include <mutex>
#include <type_traits>

#include "bdf_core.cuh"
#include "pdr_internal.h"

namespace pdr {

namespace {

using namespace bdf;
constexpr unsigned FULL = 0xffffffffu;
constexpr int PB = 8;    // LU panel width
constexpr int DB = 32;   // diagonal block of the triangular solves
constexpr int MAXW = 8;  // at most 256 threads per block

struct CtaArgs {
  WarpTables tab;
  int ncell, nspec, nreac, n, ld, G;
  double *abundance;
  const double *rate;
  const double *density;
  const double *t_end_yr;
  double t_end_default_yr, start_time_yr, reltol, abstol;
  long long mxstep, max_total_steps;
  int *status;
  int *stats;
  const int *cell_list;
  int *queue;
  int *fallback_list;
  int *fallback_count;
  int refill_static;
  const int *sm_limit;    // work-queue mode: SMs the launch may keep (device word, null: all)
  int grid_sms;           // SMs the grid was sized for
  double *kn_global;      // [gridDim.x][tab.nkn + 1] rate constants (times n_H where the RHS has it)
  void *mat_global;       // [gridDim.x][(n+2)*ld] Newton matrix, when it is not in shared memory
};

// byte offsets of the block's shared arrays (host and device agree)
struct CtaLayout {
  size_t scr, xs, part, red, sig, perm, cols, bsv, ys, upan, ws, wu, mat, dinv, yv, rfs, idx, wv, total;
};

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~size_t(15); }

// sp: the mixed form's sparse Newton matrix (storage of T.sp.total values,
// the dense routines on its m x m trailing block)
__host__ __device__ inline CtaLayout cta_layout(const WarpTables &T, int ld, size_t mt, bool mat_smem,
                                                bool sp = false) {
  const int nreac = T.nreac, nparts = T.nparts, G = T.lanes;
  const int n = sp ? T.sp.m : T.neq;   // order of the dense matrix
  CtaLayout L;
  size_t o = 0;
  // scr: the RHS operands (FP64) or the two Jacobian scatter buffers
  size_t scr = (size_t)nreac * (8 > 2 * mt ? 8 : 2 * mt);
  if (8 * (size_t)T.nop > scr) scr = 8 * (size_t)T.nop;
  L.scr = o; o += al16(scr);
  L.xs = o; o += al16(8 * (size_t)(n + 2));
  L.part = o; o += al16(8 * (size_t)(nparts + 1));
  L.red = o; o += al16(2 * MAXW * (8 + 8 + 4));   // sums, argmax keys, argmax rows
  L.sig = o; o += al16(4 * (size_t)(T.neq + 2) * 2);   // column scales, then the FP32 slot values
  L.perm = o; o += al16(4 * (size_t)n);
  L.cols = o; o += al16(4 * (size_t)(n + MAXW));   // nonzero U columns of a panel, per-warp counts
  L.bsv = o; o += al16(mt * (size_t)G);
  L.ys = o; o += al16(mt * (size_t)(n + DB));
  // LU panel; also the assembly's boundary slots (at most 2G - 2)
  L.upan = o; o += al16(mt * (size_t)(PB * n > 2 * G ? PB * n : 2 * G));
  L.ws = o; o += al16(sizeof(CoefShared));
  L.wu = o; o += al16(sizeof(CoefUniform));
  L.mat = o;
  if (sp) {
    o += al16(mt * (size_t)T.sp.total);
    L.dinv = o; o += al16(mt * (size_t)(T.sp.a > 0 ? T.sp.a : 1));
    L.yv = o; o += al16(mt * (size_t)T.sp.N);
    L.rfs = o; o += al16(4 * (size_t)T.sp.N);
    // the index tables (a_col, b_col, a_ptr, a_diag, b_ptr, iperm, ul_rows)
    // and one scatter row per warp
    L.idx = o;
    o += al16(2 * (size_t)T.sp.off_ba) + al16(2 * (size_t)T.sp.nnz_b) + al16(4 * (size_t)(T.sp.a + 1)) +
         al16(4 * (size_t)T.sp.a) + al16(4 * (size_t)(T.sp.m + 1)) + al16(4 * (size_t)T.sp.N) + al16(4 * (size_t)T.sp.a);
    L.wv = o; o += al16(mt * (size_t)MAXW * T.sp.N);
  } else {
    if (mat_smem) o += al16(mt * (size_t)(n + 2) * ld);
    L.dinv = L.yv = L.rfs = L.idx = L.wv = o;
  }
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

// ordering key of a non-negative magnitude (0 = not a candidate)
__device__ __forceinline__ unsigned long long mag_key(float v, bool cand) {
  return cand ? (unsigned long long)__float_as_uint(v) : 0ull;
}
__device__ __forceinline__ unsigned long long mag_key(double v, bool cand) {
  return cand ? (unsigned long long)__double_as_longlong(v) : 0ull;
}

// SP (mixed only): the sparse bordered Newton matrix; the dense routines
// (lu, invert_diagonal_blocks, lin_solve) then act on its trailing block
template <bool MIXED, bool SP = false>
struct CtaCell : Core<CtaCell<MIXED, SP>, false, MIXED> {
  using MT = typename std::conditional<MIXED, float, double>::type;
  static_assert(!SP || MIXED, "the sparse Newton matrix is the mixed form's");
  const CtaArgs &A;
  const int tid, lane, warp, nw, n, ld;
  const bool owns;
  // the dense matrix the dense routines factorise: order dn, stride dld
  int dn, dld;
  MT *dmat;
  MT *S = nullptr;       // sparse: the matrix storage (leaf rows, trailing rows' leaf part, dense block)
  MT *dinv = nullptr;    // sparse: reciprocal pivots of the leaf rows
  MT *yv = nullptr;      // sparse: the solve's vector in elimination order
  float *rfs = nullptr;  // sparse: row factor of each species row at assembly
  // sparse: the index tables, copied to shared memory at the start
  const unsigned short *sa_col = nullptr, *sb_col = nullptr;
  const int *sa_ptr = nullptr, *sa_diag = nullptr, *sb_ptr = nullptr, *siperm = nullptr, *sul_rows = nullptr;
  MT *wv = nullptr;      // sparse: [MAXW][N] one scatter row per warp
  const double inv_n;
  double *kn;            // global, this block's slot
  double *scr, *xs, *part;
  double *red_d;         // [2][MAXW] reduction partials
  unsigned long long *red_k;  // [2][MAXW] argmax keys
  int *red_i;            // [2][MAXW] argmax rows
  float *sig;
  float *xs32;           // [n+2] FP32 copy of the slot values at setup (mixed)
  int *perm;
  int *cols, *cnt;       // nonzero columns of the current U panel; per-warp counts
  MT *bsv, *ys, *upan, *mat;
  int rbuf = 0;          // alternating reduction buffer
  double cx;
  int mystep;
  float wsc32, ssc32;    // mixed form: setup-time weight and its inverse (FP32 matrix scaling)

  __device__ __forceinline__ CtaCell(const CtaArgs &a, int t)
      : A(a), tid(t), lane(t & 31), warp(t >> 5), nw(blockDim.x >> 5), n(a.n), ld(a.ld), owns(t < a.n),
        dn(a.n), dld(a.ld), dmat(nullptr), inv_n(1.0 / a.n) {}

  __device__ __forceinline__ bool leader() const { return tid == 0; }
  __device__ __forceinline__ void sync() const { __syncthreads(); }
  __device__ __forceinline__ MT &M(int i, int j) const { return dmat[(size_t)j * dld + i]; }

  // block-wide sums and maxima in a fixed order (every thread gets the value)
  __device__ __forceinline__ double sum_all(double v) {
    v = warp_sum(v);
    double *r = red_d + rbuf * MAXW;
    rbuf ^= 1;
    if (lane == 0) r[warp] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < nw; w++) s += r[w];
    return s;
  }
  __device__ __forceinline__ float sum_all(float v) {
    v = warp_sum(v);
    float *r = reinterpret_cast<float *>(red_d + rbuf * MAXW);
    rbuf ^= 1;
    if (lane == 0) r[warp] = v;
    __syncthreads();
    float s = 0.0f;
    for (int w = 0; w < nw; w++) s += r[w];
    return s;
  }
  __device__ __forceinline__ double max_all(double v) {
    v = warp_max(v);
    double *r = red_d + rbuf * MAXW;
    rbuf ^= 1;
    if (lane == 0) r[warp] = v;
    __syncthreads();
    double s = r[0];
    for (int w = 1; w < nw; w++) s = fmax(s, r[w]);
    return s;
  }
  // row of the largest candidate (lowest row on ties), -1 if all are zero
  __device__ __forceinline__ int argmax_all(MT v, bool cand) {
    const unsigned long long key = mag_key(v, cand);
    const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
    const unsigned mh = __reduce_max_sync(FULL, hi);
    const unsigned ml = __reduce_max_sync(FULL, hi == mh ? lo : 0u);
    const unsigned b = __ballot_sync(FULL, cand && hi == mh && lo == ml);
    unsigned long long *rk = red_k + rbuf * MAXW;
    int *ri = red_i + rbuf * MAXW;
    rbuf ^= 1;
    if (lane == 0) {
      rk[warp] = ((unsigned long long)mh << 32) | ml;
      ri[warp] = b ? warp * 32 + __ffs(b) - 1 : -1;
    }
    __syncthreads();
    unsigned long long best = 0ull;
    int row = -1;
    for (int w = 0; w < nw; w++)
      if (rk[w] > best) { best = rk[w]; row = ri[w]; }
    return row;
  }

  __device__ __forceinline__ double slot_value(int s, double xe) const { return s == n ? xe : xs[s]; }

  // per-cell rate constants (kn_r = k_r, times n_H for the terms that carry
  // it), the extras |nu| kn_r of the RHS terms with |nu| > 1 and a zero for
  // the padding terms
  __device__ __forceinline__ void load_rates(const double *rate, double n_H) {
    const WarpTables &T = A.tab;
    for (int r = tid; r < T.nreac; r += blockDim.x)
      kn[r] = __ldg(&rate[r]) * (__ldg(&T.nh_mask[r]) != 0.0 ? n_H : 1.0);
    if (tid == 0) kn[T.nkn] = 0.0;
    __syncthreads();
    for (int e = tid; e < T.nkext; e += blockDim.x) {
      double k = 0.0;
      for (int q = __ldg(&T.kext_ptr[e]); q < __ldg(&T.kext_ptr[e + 1]); q++) {
        const int2 rn = __ldg(&T.kext_rn[q]);
        k = fma((double)rn.y, kn[rn.x], k);
      }
      kn[T.nreac + e] = k;
    }
  }

  // f(y): returns f of this thread's species, records x_e of this call.  The
  // operands are the slot values and the products x_a x_b of the two-body
  // reactant pairs; each stoichiometric term is one FMA with the signed rate
  // constant (the warp integrator's scheme, stride G).
  __device__ __forceinline__ double rhs(double yv) {
    const WarpTables &T = A.tab;
    const int G = T.lanes;
    double *P = scr;
    if (owns) P[tid] = yv;
    const double xe = sum_all(owns ? cx * yv : 0.0);
    this->xe_last = xe;
    if (tid == 0) {
      P[n] = xe;
      P[n + 1] = 1.0;
    }
#pragma unroll 4
    for (int p = tid; p < T.npairs; p += G) {
      const int2 ab = __ldg(&T.pairs[p]);
      P[n + 2 + p] = (ab.x == n ? xe : P[ab.x]) * (ab.y == n ? xe : P[ab.y]);
    }
    __syncthreads();
    double s = 0.0;
#pragma unroll 4
    for (int t = 0; t < T.rhs_len; t++) {
      const int2 d = __ldg(&T.rhs_t[t * G + tid]);
      const double k = kn[d.x & 0xffff];
      const double ks = __hiloint2double(__double2hiint(k) ^ (d.y & (int)0x80000000u), __double2loint(k));
      s = fma(ks, P[d.y & 0x7fffffff], s);
      const int fl = (int)((unsigned)d.x >> 16) - 1;
      if (fl >= 0) { part[fl] = s; s = 0.0; }
    }
    __syncthreads();
    double f = 0.0;
#pragma unroll 4
    for (int k = 0; k < T.plist_len; k++) f += part[__ldg(&T.plist[k * G + tid])];
    this->nfe++;
    return owns ? f : 0.0;
  }

  // Newton matrix rows: FP64 M = I - gamma J; mixed FP32 W M W^-1 (rf_d =
  // -gamma, identity); the diagnostic evaluation takes J itself (rf_d = 1, no
  // identity)
  __device__ __forceinline__ void assemble(double yv, double rf_d, bool identity = true) {
    const WarpTables &T = A.tab;
    const int G = T.lanes;
    if (owns) xs[tid] = yv;
    if constexpr (MIXED) {
      // column scales rtol|y|+atol normalised by atol, formed in FP32 from the
      // FP32 value of y (the matrix is FP32)
      const float y32 = (float)yv;
      ssc32 = fmaf(this->rtol32, fabsf(y32), this->atol32);
      wsc32 = __frcp_rn(ssc32);
      if (owns) {
        sig[tid] = ssc32 * __frcp_rn(this->atol32);
        xs32[tid] = y32;
      }
    }
    const double xe = sum_all(owns ? cx * yv : 0.0);
    MT *Da = reinterpret_cast<MT *>(scr);
    MT *Db = Da + T.nreac;
    const float xe32 = MIXED ? (float)xe : 0.0f;
#pragma unroll 4
    for (int r = tid; r < T.nreac; r += G) {
      const int2 ab = __ldg(&T.rab[r]);
      if constexpr (MIXED) {
        // one conversion of the rate constant per reaction, the rest in FP32
        const float k32 = (float)kn[r];
        Da[r] = k32 * ((ab.y == n ? xe32 : xs32[ab.y]) * sig[ab.x]);
        Db[r] = k32 * ((ab.x == n ? xe32 : xs32[ab.x]) * sig[ab.y]);
      } else {
        const double k = kn[r];
        Da[r] = k * slot_value(ab.y, xe);
        Db[r] = (ab.y == n + 1) ? 0.0 : k * slot_value(ab.x, xe);
      }
    }
    if (owns)
      for (int j = 0; j < n + 2; j++) M(tid, j) = MT(0);
    __syncthreads();
    // J entries term-parallel: every thread sums its balanced chunk of the
    // entry-sorted contributions in a register (rows with thousands of terms
    // no longer serialise on one thread); runs crossing a chunk boundary are
    // added up from their slots, in chunk order, by a second pass
    {
      MT *slots = upan;   // the LU panel buffer is free during the assembly
      MT s = MT(0);
#pragma unroll 4
      for (int t = 0; t < T.hlen; t++) {
        const int2 xy = __ldg(&T.h_xy[t * G + tid]);
        const int x = xy.x, y = xy.y;
        MT nu;
        if constexpr (MIXED) nu = (MT)(x >> 19);
        else nu = __ldg(&T.h_nu[t * G + tid]);
        const int r = x & 0xffff;
        s = fma(nu, (x & 0x10000) ? Db[r] : Da[r], s);
        const int kind = (x >> 17) & 3;
        if (kind == 1) {
          M(y & 0xff, (y >> 8) & 0xff) = s;
          s = MT(0);
        } else if (kind == 2) {
          slots[y >> 16] = s;
          s = MT(0);
        }
      }
      __syncthreads();
      for (int b = tid; b < T.nbnd; b += G) {
        const int tt = __ldg(&T.bnd_t[b]), ss = __ldg(&T.bnd_s[b]);
        MT acc = MT(0);
        for (int q = ss & 0xffff; q < (ss >> 16); q++) acc += slots[q];
        M(tt & 0xff, (tt >> 8) & 0xff) = acc;
      }
      __syncthreads();
    }
    if (owns) {
      const MT e = M(tid, n);
      MT rf;
      if constexpr (MIXED) rf = (MT)rf_d * (wsc32 * this->atol32);
      else rf = (MT)rf_d;
      for (int j = 0; j < n; j++) {
        MT cj;
        if constexpr (MIXED) cj = __ldg(&T.xe_coef_f[j]);
        else cj = __ldg(&T.xe_coef[j]);
        MT v = M(tid, j);
        if constexpr (MIXED) v = fmaf(e * cj, sig[j], v);
        else v = fma(e, cj, v);
        M(tid, j) = rf * v + ((identity && tid == j) ? MT(1) : MT(0));
      }
    }
  }

  __device__ __forceinline__ MT rcp(MT x) const {
    if constexpr (sizeof(MT) == 8) return __drcp_rn(x);
    else return __frcp_rn(x);
  }

  // the PB U-panel entries of column jj (16-byte aligned: upan is, and a
  // column holds PB = 8 values)
  __device__ __forceinline__ void load_upan(int jj, MT (&u)[PB]) const {
    if constexpr (sizeof(MT) == 4) {
      const float4 *p = reinterpret_cast<const float4 *>(upan + (size_t)jj * PB);
#pragma unroll
      for (int q = 0; q < PB / 4; q++) {
        const float4 v = p[q];
        u[4 * q] = v.x; u[4 * q + 1] = v.y; u[4 * q + 2] = v.z; u[4 * q + 3] = v.w;
      }
    } else {
      const double2 *p = reinterpret_cast<const double2 *>(upan + (size_t)jj * PB);
#pragma unroll
      for (int q = 0; q < PB / 2; q++) {
        const double2 v = p[q];
        u[2 * q] = v.x; u[2 * q + 1] = v.y;
      }
    }
  }

  // LU with partial pivoting in place; false if a column has no nonzero pivot
  __device__ __forceinline__ bool lu() {
    mystep = (tid < dn) ? -1 : dn;
    for (int k0 = 0; k0 < dn; k0 += PB) {
      const int kb = min(PB, dn - k0);
      for (int t = 0; t < kb; t++) {
        const int k = k0 + t;
        const bool cand = (mystep < 0);
        const int p = argmax_all(cand ? (MT)fabs(M(tid, k)) : MT(0), cand);
        if (p < 0) return false;
        const MT rinv = rcp(M(p, k));
        if (tid == p) { mystep = k; perm[k] = p; }
        if (mystep < 0) {
          const MT l = M(tid, k) * rinv;
          M(tid, k) = l;
          for (int j = k + 1; j < k0 + kb; j++) M(tid, j) = fma(-l, M(p, j), M(tid, j));
        }
      }
      __syncthreads();
      // U rows of this panel's pivots, columns right of the panel (at most one
      // column per thread: the block has at least n threads); the columns
      // whose U entries are all zero are left out of the trailing update
      const int j = k0 + kb + tid;
      bool nzc = false;
      if (j < dn) {
        MT u[PB];
#pragma unroll
        for (int t = 0; t < PB; t++) {
          if (t < kb) {
            const int pt = perm[k0 + t];
            MT s = M(pt, j);
#pragma unroll
            for (int t2 = 0; t2 < PB; t2++)
              if (t2 < t) s = fma(-M(pt, k0 + t2), u[t2], s);
            u[t] = s;
            M(pt, j) = s;
            nzc |= (s != MT(0));
          } else {
            u[t] = MT(0);
          }
          upan[(size_t)j * PB + t] = u[t];
        }
      }
      const unsigned bal = __ballot_sync(FULL, nzc);
      if (lane == 0) cnt[warp] = __popc(bal);
      __syncthreads();
      int base = 0, ncols = 0;
      for (int w = 0; w < nw; w++) {
        const int c = cnt[w];
        base += (w < warp) ? c : 0;
        ncols += c;
      }
      if (nzc) cols[base + __popc(bal & ((1u << lane) - 1u))] = j;
      __syncthreads();
      if (mystep < 0) {
        MT l[PB];
        bool any = false;
#pragma unroll
        for (int t = 0; t < PB; t++) {
          l[t] = (t < kb) ? M(tid, k0 + t) : MT(0);
          any |= (l[t] != MT(0));
        }
        if (any) {
          // four columns at a time: every load of the group is issued before
          // any store (the compiler cannot prove the panel buffer and the
          // matrix apart), the U entries of a column as 16-byte vectors
          constexpr int CB = 4;
          int c = 0;
          for (; c + CB <= ncols; c += CB) {
            int jj[CB];
            MT s[CB], u[CB][PB];
#pragma unroll
            for (int b = 0; b < CB; b++) {
              jj[b] = cols[c + b];
              s[b] = M(tid, jj[b]);
              load_upan(jj[b], u[b]);
            }
#pragma unroll
            for (int b = 0; b < CB; b++) {
#pragma unroll
              for (int t = 0; t < PB; t++) s[b] = fma(-l[t], u[b][t], s[b]);
              M(tid, jj[b]) = s[b];
            }
          }
          for (; c < ncols; c++) {
            const int jj = cols[c];
            MT s = M(tid, jj), u[PB];
            load_upan(jj, u);
#pragma unroll
            for (int t = 0; t < PB; t++) s = fma(-l[t], u[t], s);
            M(tid, jj) = s;
          }
        }
      }
    }
    __syncthreads();
    return true;
  }

  // invert the 32x32 diagonal blocks of L (unit lower) and U in place
  __device__ __forceinline__ void invert_diagonal_blocks() {
    const int nb = (dn + DB - 1) / DB;
    for (int c = warp; c < nb; c += nw) {
      const int k0 = c * DB, bs = min(DB, dn - k0);
      const int t = lane;  // column of the block
      MT x[DB];
      // L^-1 column t: x_t = 1, x_r = -sum_{m=t}^{r-1} L_rm x_m
#pragma unroll
      for (int r = 0; r < DB; r++) {
        if (r < bs) {
          const int pr = perm[k0 + r];
          MT s = MT(0);
#pragma unroll
          for (int m = 0; m < DB; m++)
            if (m < r && m >= t) s = fma(-M(pr, k0 + m), x[m], s);
          x[r] = (r == t) ? MT(1) : (r > t ? s : MT(0));
        } else {
          x[r] = MT(0);
        }
      }
      __syncwarp();
#pragma unroll
      for (int r = 0; r < DB; r++)
        if (r < bs && t < bs && r > t) M(perm[k0 + r], k0 + t) = x[r];
      __syncwarp();
      // U^-1 column t: y_t = 1/U_tt, y_r = -(sum_{m=r+1}^{t} U_rm y_m) / U_rr
#pragma unroll
      for (int r = DB - 1; r >= 0; r--) {
        if (r < bs) {
          const int pr = perm[k0 + r];
          MT s = MT(0);
#pragma unroll
          for (int m = 0; m < DB; m++)
            if (m > r && m <= t && m < bs) s = fma(M(pr, k0 + m), x[m], s);
          const MT d = rcp(M(pr, k0 + r));
          x[r] = (r == t) ? d : (r < t ? -s * d : MT(0));
        } else {
          x[r] = MT(0);
        }
      }
      __syncwarp();
#pragma unroll
      for (int r = 0; r < DB; r++)
        if (r < bs && t < bs && r <= t) M(perm[k0 + r], k0 + t) = x[r];
    }
    __syncthreads();
  }

  __device__ __forceinline__ bool setup(double yv) {
    bool ok;
    if constexpr (SP) {
      assemble_sparse(yv, -this->gamma);
      ok = sparse_lu();
    } else {
      assemble(yv, -this->gamma);
      ok = lu();
    }
    if (ok) {
      // any non-finite factor entry fails the setup (as a singular matrix)
      bool finite = true;
      if constexpr (SP) {
        for (int e = tid; e < A.tab.sp.total; e += blockDim.x) finite &= isfinite(S[e]);
      } else if (owns) {
        for (int j = 0; j < n; j++) finite &= isfinite(M(tid, j));
      }
      ok = __syncthreads_and(finite);
    }
    if (ok) invert_diagonal_blocks();
    this->after_setup();
    return ok;
  }

  // ---- the sparse bordered Newton matrix (mixed form) ----
  //
  // Unknowns: the species and x_e, in the plan's elimination order.  Rows:
  // species i, W (I - gamma J) W^-1 with J taken at fixed x_e (its x_e column
  // is df_i/dx_e); the x_e row, x_e - c^T x = 0 scaled the same way.  The
  // correction of the species is the chain-rule system's.

  // the matrix at y, times rf = -gamma, plus the identity, in the storage
  __device__ __forceinline__ void assemble_sparse(double yv, double rf_d) {
    const WarpTables &T = A.tab;
    const auto &Q = T.sp;
    const int G = T.lanes;
    if (owns) xs[tid] = yv;
    const float y32 = (float)yv;
    ssc32 = fmaf(this->rtol32, fabsf(y32), this->atol32);
    wsc32 = __frcp_rn(ssc32);
    const float inv_atol = __frcp_rn(this->atol32);
    if (owns) {
      sig[tid] = ssc32 * inv_atol;
      xs32[tid] = y32;
      rfs[tid] = (float)rf_d * (wsc32 * this->atol32);   // -gamma / sig_i
    }
    const double xe = sum_all(owns ? cx * yv : 0.0);
    const float xe32 = (float)xe;
    // the x_e column's scale, from x_e like the species' (every thread has it)
    const float sig_e = fmaf(this->rtol32, fabsf(xe32), this->atol32) * inv_atol;
    MT *Da = reinterpret_cast<MT *>(scr);
    MT *Db = Da + T.nreac;
#pragma unroll 4
    for (int r = tid; r < T.nreac; r += G) {
      const int2 ab = __ldg(&T.rab[r]);
      const float k32 = (float)kn[r];
      const float sa = (ab.x == n) ? sig_e : sig[ab.x];
      const float sb = (ab.y == n) ? sig_e : sig[ab.y];
      Da[r] = k32 * ((ab.y == n ? xe32 : xs32[ab.y]) * sa);
      Db[r] = k32 * ((ab.x == n ? xe32 : xs32[ab.x]) * sb);
    }
    for (int e = tid; e < Q.total; e += G) S[e] = MT(0);
    __syncthreads();
    {
      MT *slots = upan;
      MT s = MT(0);
#pragma unroll 4
      for (int t = 0; t < T.hlen; t++) {
        const int2 xy = __ldg(&T.h_xy[t * G + tid]);
        const int x = xy.x, y = xy.y;
        const MT nu = (MT)(x >> 19);
        const int r = x & 0xffff;
        s = fma(nu, (x & 0x10000) ? Db[r] : Da[r], s);
        const int kind = (x >> 17) & 3;
        if (kind == 1) {
          S[(unsigned)y >> 16] = s * rfs[y & 0xff];
          s = MT(0);
        } else if (kind == 2) {
          slots[(unsigned)y >> 16] = s;
          s = MT(0);
        }
      }
      __syncthreads();
      for (int b = tid; b < T.nbnd; b += G) {
        const int tt = __ldg(&T.bnd_t[b]), ss = __ldg(&T.bnd_s[b]);
        MT acc = MT(0);
        for (int q = ss & 0xffff; q < (ss >> 16); q++) acc += slots[q];
        S[(unsigned)tt >> 16] = acc * rfs[tt & 0xff];
      }
      __syncthreads();
    }
    // the identity, and the x_e row: -c_j sig_j / sig_e
    for (int i = tid; i < Q.N; i += G) S[__ldg(&Q.diag_loc[i])] += MT(1);
    if (owns) {
      const int l = __ldg(&Q.e_loc[tid]);
      if (l >= 0) S[l] = (MT)(-cx) * (sig[tid] * __frcp_rn(sig_e));
    }
    __syncthreads();
  }

  // in place: the leaf rows by dependency level, then the trailing rows'
  // leaf-column part with its update of the dense block (no pivoting; one
  // warp per row, the row scattered into the warp's dense row so that every
  // update finds its entry by column), then the dense block with partial
  // pivoting.  A row's eliminations run in column order; the updates of one
  // elimination step go to distinct columns, one per lane.
  __device__ __forceinline__ bool sparse_lu() {
    const auto &Q = A.tab.sp;
    const int a = Q.a;
    MT *w = wv + (size_t)warp * Q.N;
    bool ok = true;
    for (int l = 0; l < Q.nlev; l++) {
      const int r1 = __ldg(&Q.lev_ptr[l + 1]);
      for (int r = __ldg(&Q.lev_ptr[l]) + warp; r < r1; r += nw) {
        const int p0 = sa_ptr[r], pd = sa_diag[r], p1 = sa_ptr[r + 1];
        for (int p = p0 + lane; p < p1; p += 32) w[sa_col[p]] = S[p];
        __syncwarp();
        for (int p = p0; p < pd; p++) {
          const int k = sa_col[p];
          const MT lk = w[k] * dinv[k];
          const int u1 = sa_ptr[k + 1];
          for (int u = sa_diag[k] + 1 + lane; u < u1; u += 32) {
            const int j = sa_col[u];
            w[j] = fma(-lk, S[u], w[j]);
          }
          if (lane == 0) S[p] = lk;
          __syncwarp();
        }
        for (int p = pd + lane; p < p1; p += 32) S[p] = w[sa_col[p]];
        if (lane == 0) {
          const MT d = w[r];
          ok &= (d != MT(0));
          dinv[r] = rcp(d);
        }
        __syncwarp();
      }
      __syncthreads();
    }
    const int off_ba = Q.off_ba;
    MT *D = S + Q.off_d;
    for (int t = warp; t < Q.m; t += nw) {
      const int p0 = sb_ptr[t], p1 = sb_ptr[t + 1];
      for (int p = p0 + lane; p < p1; p += 32) w[sb_col[p]] = S[off_ba + p];
      __syncwarp();
      for (int p = p0; p < p1; p++) {
        const int k = sb_col[p];
        const MT lk = w[k] * dinv[k];
        const int u1 = sa_ptr[k + 1];
        for (int u = sa_diag[k] + 1 + lane; u < u1; u += 32) {
          const int j = sa_col[u];
          MT &dst = (j < a) ? w[j] : D[(size_t)(j - a) * Q.ldb + t];
          dst = fma(-lk, S[u], dst);
        }
        if (lane == 0) S[off_ba + p] = lk;
        __syncwarp();
      }
    }
    if (!__syncthreads_and(ok)) return false;
    return lu();
  }

  // x = M^-1 v (v this thread's species entry, scaled), the species part
  __device__ __forceinline__ MT sparse_solve(MT v) {
    const auto &Q = A.tab.sp;
    const int a = Q.a;
    if (owns) yv[siperm[tid]] = v;
    if (tid == 0) yv[siperm[n]] = MT(0);
    __syncthreads();
    // forward, leaf rows
    for (int l = 0; l < Q.nlev; l++) {
      const int r1 = __ldg(&Q.lev_ptr[l + 1]);
      for (int r = __ldg(&Q.lev_ptr[l]) + tid; r < r1; r += blockDim.x) {
        MT s = yv[r];
        const int pd = sa_diag[r];
        for (int p = sa_ptr[r]; p < pd; p++) s = fma(-S[p], yv[sa_col[p]], s);
        yv[r] = s;
      }
      __syncthreads();
    }
    // the trailing rows' leaf part, then the dense block
    MT bt = MT(0);
    if (tid < Q.m) {
      MT s = yv[a + tid];
      const int p1 = sb_ptr[tid + 1];
      for (int p = sb_ptr[tid]; p < p1; p++) s = fma(-S[Q.off_ba + p], yv[sb_col[p]], s);
      bt = s;
    }
    const MT xt = lin_solve(bt);
    if (tid < Q.m) yv[a + tid] = xt;
    __syncthreads();
    // backward, leaf rows by U-dependency level
    for (int l = 0; l < Q.nul; l++) {
      const int i1 = __ldg(&Q.ul_ptr[l + 1]);
      for (int i = __ldg(&Q.ul_ptr[l]) + tid; i < i1; i += blockDim.x) {
        const int r = sul_rows[i];
        MT s = yv[r];
        const int pd = sa_diag[r], p1 = sa_ptr[r + 1];
        for (int p = pd + 1; p < p1; p++) s = fma(-S[p], yv[sa_col[p]], s);
        yv[r] = s * dinv[r];
      }
      __syncthreads();
    }
    const MT x = owns ? yv[siperm[tid]] : MT(0);
    __syncthreads();
    return x;
  }

  // copy the sparse index tables to shared memory (once per block)
  __device__ __forceinline__ void stage_sparse(unsigned char *base) {
    const auto &Q = A.tab.sp;
    unsigned char *o = base;
    auto take = [&](size_t bytes) { unsigned char *p = o; o += al16(bytes); return p; };
    unsigned short *ac = reinterpret_cast<unsigned short *>(take(2 * (size_t)Q.off_ba));
    unsigned short *bc = reinterpret_cast<unsigned short *>(take(2 * (size_t)Q.nnz_b));
    int *ap = reinterpret_cast<int *>(take(4 * (size_t)(Q.a + 1)));
    int *ad = reinterpret_cast<int *>(take(4 * (size_t)Q.a));
    int *bp = reinterpret_cast<int *>(take(4 * (size_t)(Q.m + 1)));
    int *ip = reinterpret_cast<int *>(take(4 * (size_t)Q.N));
    int *ur = reinterpret_cast<int *>(take(4 * (size_t)Q.a));
    for (int i = tid; i < Q.off_ba; i += blockDim.x) ac[i] = __ldg(&Q.a_col[i]);
    for (int i = tid; i < Q.nnz_b; i += blockDim.x) bc[i] = __ldg(&Q.b_col[i]);
    for (int i = tid; i <= Q.a; i += blockDim.x) ap[i] = __ldg(&Q.a_ptr[i]);
    for (int i = tid; i < Q.a; i += blockDim.x) { ad[i] = __ldg(&Q.a_diag[i]); ur[i] = __ldg(&Q.ul_rows[i]); }
    for (int i = tid; i <= Q.m; i += blockDim.x) bp[i] = __ldg(&Q.b_ptr[i]);
    for (int i = tid; i < Q.N; i += blockDim.x) ip[i] = __ldg(&Q.iperm[i]);
    sa_col = ac; sb_col = bc; sa_ptr = ap; sa_diag = ad; sb_ptr = bp; siperm = ip; sul_rows = ur;
    __syncthreads();
  }

  // x = M^-1 b for this thread's component (FP64 form)
  __device__ __forceinline__ double solve(double b) {
    const MT xv = lin_solve(owns ? (MT)b : MT(0));
    return owns ? (double)xv : 0.0;
  }

  // mixed form: the residual converted once and scaled in FP32 (the scaling
  // of the FP32 matrix); the correction comes back times ssc*gscale, in FP32
  // for the norm and in FP64 for the state
  __device__ __forceinline__ double solve32(double b, float gs, float &x32) {
    MT xv;
    if constexpr (SP) xv = sparse_solve(owns ? (float)b * wsc32 : 0.0f);
    else xv = lin_solve(owns ? (float)b * wsc32 : 0.0f);
    x32 = owns ? xv * (ssc32 * gs) : 0.0f;
    return (double)x32;
  }

  // the triangular solves with the factors in place: v is this thread's
  // right-hand-side entry, the solution component of its species is returned
  __device__ __forceinline__ MT lin_solve(MT v) {
    const int nb = (dn + DB - 1) / DB;
    const bool downs = tid < dn;
    bsv[tid] = v;
    __syncthreads();
    // forward: L y = P b
    for (int c = 0; c < nb; c++) {
      const int k0 = c * DB, bs = min(DB, dn - k0);
      if (warp == c % nw) {
        const int pr = (lane < bs) ? perm[k0 + lane] : 0;
        const MT s = (lane < bs) ? bsv[pr] : MT(0);
        MT y = s;
#pragma unroll
        for (int t = 0; t < DB; t++) {
          const MT st = __shfl_sync(FULL, s, t);
          if (t < lane && lane < bs) y = fma(M(pr, k0 + t), st, y);
        }
        if (lane < bs) ys[k0 + lane] = y;
      }
      __syncthreads();
      if (mystep >= k0 + bs && downs) {
        MT s = v;
        for (int t = 0; t < bs; t++) s = fma(-M(tid, k0 + t), ys[k0 + t], s);
        v = s;
        bsv[tid] = v;
      }
      __syncthreads();
    }
    // backward: U x = y; the running value of logical row k is kept by its pivot row
    v = downs ? ys[mystep] : MT(0);
    bsv[tid] = v;
    __syncthreads();
    for (int c = nb - 1; c >= 0; c--) {
      const int k0 = c * DB, bs = min(DB, dn - k0);
      if (warp == c % nw) {
        // x_r = sum_{t>=r} Uinv_rt s_t, s_t the running value of logical row k0+t
        const int pr = (lane < bs) ? perm[k0 + lane] : 0;
        const MT s = (lane < bs) ? bsv[pr] : MT(0);
        MT x = MT(0);
#pragma unroll
        for (int t = 0; t < DB; t++) {
          const MT st = __shfl_sync(FULL, s, t);
          if (t >= lane && lane < bs && t < bs) x = fma(M(pr, k0 + t), st, x);
        }
        if (lane < bs) ys[k0 + lane] = x;
      }
      __syncthreads();
      if (downs && mystep < k0) {
        MT s = v;
        for (int t = 0; t < bs; t++) s = fma(-M(tid, k0 + t), ys[k0 + t], s);
        v = s;
        bsv[tid] = v;
      }
      __syncthreads();
    }
    // ys[k] is now the solution component of column k
    const MT xv = downs ? ys[tid] : MT(0);
    __syncthreads();
    return xv;
  }

  // calculate_abundances.c:132-317 for one cell
  __device__ __forceinline__ void run(int cell) {
    const int nspec = A.nspec;
    double *ab = A.abundance + (size_t)cell * nspec;
    this->rtol = A.reltol;
    this->atol = A.abstol;
    this->mxstep = A.mxstep;
    this->max_total_steps = A.max_total_steps;
    cx = owns ? __ldg(&A.tab.xe_coef[tid]) : 0.0;
    load_rates(A.rate + (size_t)cell * A.nreac, A.density[cell]);
    if (tid == 0) {
      xs[n + 1] = 1.0;
      xs32[n + 1] = 1.0f;
      part[A.tab.nparts] = 0.0;
      sig[n] = 1.0f;
      sig[n + 1] = 0.0f;
    }
    this->clear_row(owns ? ab[tid] : 0.0);
    this->xe_last = ab[nspec - 1];
    __syncthreads();
    const double tend_yr = A.t_end_yr ? A.t_end_yr[cell] : A.t_end_default_yr;
    double yv = 0.0;
    const int status = this->integrate(A.start_time_yr, tend_yr, MIXED, &yv);
    if (status == FELL_BACK) {
      if (tid == 0) {
        const int k = atomicAdd(A.fallback_count, 1);
        A.fallback_list[k] = cell;
        A.status[cell] = FELL_BACK;
      }
      return;
    }
    if (yv < this->atol) yv = 0.0;
    if (owns) ab[tid] = yv;
    if (tid == 0) {
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

template <bool MIXED, bool SP>
__global__ void __launch_bounds__(256, SP ? 2 : 1) chem_cta_kernel(const __grid_constant__ CtaArgs A, int total_cells,
                                                          const int *total_ptr, int mat_smem) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using MT = typename std::conditional<MIXED, float, double>::type;
  const CtaLayout L = cta_layout(A.tab, A.ld, sizeof(MT), mat_smem != 0, SP);
  CtaCell<MIXED, SP> c(A, threadIdx.x);
  c.kn = A.kn_global + (size_t)blockIdx.x * (A.tab.nkn + 1);
  c.scr = reinterpret_cast<double *>(smem_raw + L.scr);
  c.xs = reinterpret_cast<double *>(smem_raw + L.xs);
  c.part = reinterpret_cast<double *>(smem_raw + L.part);
  c.red_d = reinterpret_cast<double *>(smem_raw + L.red);
  c.red_k = reinterpret_cast<unsigned long long *>(smem_raw + L.red + 2 * MAXW * 8);
  c.red_i = reinterpret_cast<int *>(smem_raw + L.red + 2 * MAXW * 16);
  c.sig = reinterpret_cast<float *>(smem_raw + L.sig);
  c.xs32 = c.sig + (A.n + 2);
  c.perm = reinterpret_cast<int *>(smem_raw + L.perm);
  c.cols = reinterpret_cast<int *>(smem_raw + L.cols);
  c.cnt = c.cols + A.n;
  c.bsv = reinterpret_cast<MT *>(smem_raw + L.bsv);
  c.ys = reinterpret_cast<MT *>(smem_raw + L.ys);
  c.upan = reinterpret_cast<MT *>(smem_raw + L.upan);
  c.ws = reinterpret_cast<CoefShared *>(smem_raw + L.ws);
  c.wu = reinterpret_cast<CoefUniform *>(smem_raw + L.wu);
  c.mat = mat_smem ? reinterpret_cast<MT *>(smem_raw + L.mat)
                   : reinterpret_cast<MT *>(A.mat_global) + (size_t)blockIdx.x * (A.n + 2) * A.ld;
  c.dmat = c.mat;
  if constexpr (SP) {
    c.S = reinterpret_cast<MT *>(smem_raw + L.mat);
    c.dinv = reinterpret_cast<MT *>(smem_raw + L.dinv);
    c.yv = reinterpret_cast<MT *>(smem_raw + L.yv);
    c.rfs = reinterpret_cast<float *>(smem_raw + L.rfs);
    c.dmat = c.S + A.tab.sp.off_d;
    c.dn = A.tab.sp.m;
    c.dld = A.tab.sp.ldb;
    c.wv = reinterpret_cast<MT *>(smem_raw + L.wv);
    c.stage_sparse(smem_raw + L.idx);
  }
  c.build_uniform_table();
  if (total_ptr) total_cells = *total_ptr;
  __shared__ int next_idx;
  for (int k = 0;; k++) {
    int idx;
    if (A.refill_static) {
      idx = blockIdx.x + k * gridDim.x;
    } else {
      if (threadIdx.x == 0) {
        // blocks beyond the launch's current SM allowance take no further cells
        bool over = false;
        if (A.sm_limit) {
          const int lim = *reinterpret_cast<const volatile int *>(A.sm_limit);
          over = (long long)blockIdx.x * A.grid_sms >= (long long)lim * gridDim.x;
        }
        next_idx = over ? 0x7fffffff : atomicAdd(A.queue, 1);
      }
      __syncthreads();
      idx = next_idx;
      __syncthreads();
    }
    if (idx >= total_cells) break;
    const int cell = A.cell_list ? A.cell_list[idx] : idx;
    c.run(cell);
    __syncthreads();
  }
}

// Diagnostic evaluation of the block integrator's RHS (mode 0) or Jacobian
// with the x_e chain rule (mode 1) on given states: one block per state, the
// same device code the integrator runs (CtaCell::rhs, CtaCell::assemble), in
// FP64.  out: mode 0 [nstate][n], mode 1 [nstate][n][n] row-major.
__global__ void __launch_bounds__(256, 1) eval_cta_kernel(const __grid_constant__ CtaArgs A, int nstate,
                                                          const double *x, double *out, double *xe_out, int mode,
                                                          int mat_smem) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const CtaLayout L = cta_layout(A.tab, A.ld, 8, mat_smem != 0);
  CtaCell<false> c(A, threadIdx.x);
  const int n = A.n, tid = threadIdx.x;
  c.kn = A.kn_global + (size_t)blockIdx.x * (A.tab.nkn + 1);
  c.scr = reinterpret_cast<double *>(smem_raw + L.scr);
  c.xs = reinterpret_cast<double *>(smem_raw + L.xs);
  c.part = reinterpret_cast<double *>(smem_raw + L.part);
  c.red_d = reinterpret_cast<double *>(smem_raw + L.red);
  c.red_k = reinterpret_cast<unsigned long long *>(smem_raw + L.red + 2 * MAXW * 8);
  c.red_i = reinterpret_cast<int *>(smem_raw + L.red + 2 * MAXW * 16);
  c.sig = reinterpret_cast<float *>(smem_raw + L.sig);
  c.xs32 = c.sig + (A.n + 2);
  c.perm = reinterpret_cast<int *>(smem_raw + L.perm);
  c.cols = reinterpret_cast<int *>(smem_raw + L.cols);
  c.cnt = c.cols + n;
  c.bsv = reinterpret_cast<double *>(smem_raw + L.bsv);
  c.ys = reinterpret_cast<double *>(smem_raw + L.ys);
  c.upan = reinterpret_cast<double *>(smem_raw + L.upan);
  c.ws = reinterpret_cast<CoefShared *>(smem_raw + L.ws);
  c.wu = reinterpret_cast<CoefUniform *>(smem_raw + L.wu);
  c.mat = mat_smem ? reinterpret_cast<double *>(smem_raw + L.mat)
                   : reinterpret_cast<double *>(A.mat_global) + (size_t)blockIdx.x * (n + 2) * A.ld;
  c.dmat = c.mat;
  c.rtol = A.reltol;
  c.atol = A.abstol;
  c.cx = (tid < n) ? __ldg(&A.tab.xe_coef[tid]) : 0.0;
  for (int s = blockIdx.x; s < nstate; s += gridDim.x) {
    c.load_rates(A.rate + (size_t)s * A.nreac, A.density[s]);
    if (tid == 0) {
      c.xs[n + 1] = 1.0;
      c.part[A.tab.nparts] = 0.0;
      c.sig[n] = 1.0f;
      c.sig[n + 1] = 0.0f;
    }
    __syncthreads();
    const double yv = (tid < n) ? x[(size_t)s * n + tid] : 0.0;
    if (mode == 0) {
      const double f = c.rhs(yv);
      if (tid < n) out[(size_t)s * n + tid] = f;
      if (tid == 0 && xe_out) xe_out[s] = c.xe_last;
    } else {
      c.assemble(yv, 1.0, false);
      __syncthreads();
      for (int e = tid; e < n * n; e += blockDim.x) out[(size_t)s * n * n + e] = c.M(e / n, e % n);
    }
    __syncthreads();
  }
}

}  // namespace

#ifndef PDR_CTA_SPARSE
#define PDR_CTA_SPARSE 1
#endif

static int optin_smem() {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return optin;
}

// the mixed form runs on the sparse Newton matrix when the network has its
// plan and the block's arrays fit shared memory
static bool cta_sparse(const pdr_net *net, bool mixed) {
  const WarpTables &T = net->cta;
  if (!PDR_CTA_SPARSE || !mixed || !T.sp.ok) return false;
  return cta_layout(T, T.neq | 1, 4, true, true).total + 64 <= (size_t)optin_smem();
}

// shared memory of one block, and whether the matrix is in it
size_t chem_cta_smem(const pdr_net *net, bool mixed, bool *mat_smem) {
  const WarpTables &T = net->cta;
  const int n = T.neq, ld = n | 1;
  const size_t mt = mixed ? 4 : 8;
  if (cta_sparse(net, mixed)) { *mat_smem = true; return cta_layout(T, ld, 4, true, true).total; }
  CtaLayout with = cta_layout(T, ld, mt, true);
  if (with.total + 64 <= (size_t)optin_smem()) { *mat_smem = true; return with.total; }   // + static shared
  *mat_smem = false;
  return cta_layout(T, ld, mt, false).total;
}

using CtaKernel = void (*)(const CtaArgs, int, const int *, int);
static CtaKernel cta_kernel(int variant) {
  return variant == 0 ? chem_cta_kernel<false, false> : (variant == 1 ? chem_cta_kernel<true, false>
                                                                       : chem_cta_kernel<true, true>);
}
static int cta_variant(const pdr_net *net, bool mixed) { return !mixed ? 0 : (cta_sparse(net, mixed) ? 2 : 1); }

// Per-launch global scratch of the block integrator: rate constants and, when
// the matrix does not fit shared memory, the matrix, one slot per block.
size_t chem_cta_global_bytes(const pdr_net *net, bool mixed, int grid) {
  bool ms = false;
  chem_cta_smem(net, mixed, &ms);
  const WarpTables &T = net->cta;
  const int n = T.neq, ld = n | 1;
  size_t b = al16((size_t)grid * (T.nkn + 1) * 8);
  if (!ms) b += al16((size_t)grid * (n + 2) * ld * (mixed ? 4 : 8));
  return b;
}

// The dynamic shared-memory limit of a kernel is set per device and only ever
// grows there (networks of different sizes share the two kernels), so no call
// lowers it below what another network's launch needs.
static cudaError_t ensure_smem_attr(int variant, size_t smem) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  dev &= 63;
  static std::mutex mu;
  static size_t attr[64][3] = {};
  std::lock_guard<std::mutex> lk(mu);
  if (smem <= attr[dev][variant]) return cudaSuccess;
  e = cudaFuncSetAttribute(cta_kernel(variant), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) attr[dev][variant] = smem;
  return e;
}

// blocks per SM the block integrator runs with (0 on error)
int chem_cta_blocks_per_sm(const pdr_net *net, bool mixed) {
  bool ms = false;
  const size_t smem = chem_cta_smem(net, mixed, &ms);
  const int variant = cta_variant(net, mixed);
  auto k = cta_kernel(variant);
  if (ensure_smem_attr(variant, smem) != cudaSuccess) return 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, net->cta.lanes, smem) != cudaSuccess) return 0;
  return per_sm;
}

// Launch the persistent block integrator over `ncell` cells (or the listed
// ones) with `grid` blocks; `scratch` holds chem_cta_global_bytes(grid) bytes.
int launch_chem_cta(const pdr_net *net, int ncell, double *ab, const double *rate, const double *dens,
                    const double *tend, const pdr_chem_opts &o, int *status, int *stats, int *queue,
                    int *fb_list, int *fb_count, const int *cell_list, const int *total_ptr, bool mixed,
                    int grid, void *scratch, cudaStream_t st, const int *sm_limit, int grid_sms) {
  const WarpTables &T = net->cta;
  if (!net->cta_ok || T.lanes > 256) return PDR_E_NET;
  CtaArgs A;
  A.tab = T;
  A.ncell = ncell;
  A.nspec = net->host.nspec;
  A.nreac = net->host.nreac;
  A.n = T.neq;
  A.ld = T.neq | 1;
  A.G = T.lanes;
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
  A.grid_sms = grid_sms > 0 ? grid_sms : 1;
  A.fallback_list = fb_list;
  A.fallback_count = fb_count;
  A.refill_static = (o.refill == 1 || (o.refill == 2 && !cell_list)) ? 1 : 0;
  bool ms = false;
  const size_t smem = chem_cta_smem(net, mixed, &ms);
  A.kn_global = reinterpret_cast<double *>(scratch);
  A.mat_global = ms ? nullptr : reinterpret_cast<unsigned char *>(scratch) + al16((size_t)grid * (T.nkn + 1) * 8);
  const int variant = cta_variant(net, mixed);
  auto k = cta_kernel(variant);
  cudaError_t ea = ensure_smem_attr(variant, smem);
  if (ea != cudaSuccess) return cuda_fail(ea, "cudaFuncSetAttribute(chem_cta_kernel)");
  k<<<grid, T.lanes, smem, st>>>(A, ncell, total_ptr, ms ? 1 : 0);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "chem_cta_kernel launch");
}

}  // namespace pdr

namespace pdr {
// Diagnostic launch of eval_cta_kernel (FP64): allocates its per-block scratch
// (rate constants and, when it does not fit shared memory, the matrix) and
// frees it after the stream has finished the launch.
int launch_chem_eval_cta(const pdr_net *net, int nstate, const double *x, const double *rate, const double *dens,
                         double *out, double *xe_out, int mode, cudaStream_t st) {
  const WarpTables &T = net->cta;
  if (!net->cta_ok || T.lanes > 256) return PDR_E_NET;
  CtaArgs A{};
  A.tab = T;
  A.nspec = net->host.nspec;
  A.nreac = net->host.nreac;
  A.n = T.neq;
  A.ld = T.neq | 1;
  A.G = T.lanes;
  A.rate = rate;
  A.density = dens;
  A.reltol = 1e-8;
  A.abstol = 1e-30;
  bool ms = false;
  const size_t smem = chem_cta_smem(net, false, &ms);
  const int grid = nstate < 1024 ? nstate : 1024;
  void *scratch = nullptr;
  cudaError_t e = cudaMalloc(&scratch, chem_cta_global_bytes(net, false, grid));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(eval scratch)");
  A.kn_global = reinterpret_cast<double *>(scratch);
  A.mat_global = ms ? nullptr : reinterpret_cast<unsigned char *>(scratch) + al16((size_t)grid * (T.nkn + 1) * 8);
  e = cudaFuncSetAttribute(eval_cta_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) {
    eval_cta_kernel<<<grid, T.lanes, smem, st>>>(A, nstate, x, out, xe_out, mode, ms ? 1 : 0);
    e = cudaGetLastError();
  }
  cudaError_t e2 = cudaStreamSynchronize(st);
  cudaFree(scratch);
  if (e != cudaSuccess) return cuda_fail(e, "eval_cta_kernel launch");
  return e2 == cudaSuccess ? 0 : cuda_fail(e2, "eval_cta_kernel");
}
}  // namespace pdr
