// coolant.cpp -- LAMDA coolant-file loader and device tables for the
// level-population kernels.
//
// Follows the record sequence and conversions of read_input.F90:56-252:
// five header records, the level block (energy cm^-1 -> erg via c*h, weight),
// the radiative block (frequency GHz -> Hz, Einstein A, B_ij = A/(2h nu^3/c^2),
// B_ji = B_ij g_i/g_j), frequencies of all remaining pairs from the energies
// (a >1% mismatch with a listed frequency is an error), and per collision
// partner (LAMDA ids 1 H2, 2 p-H2, 3 o-H2, 4 e, 5 H, 6 He, 7 H+) the table
// temperatures and downward rates, with missing upward rates filled by
// detailed balance at the table temperatures (:123-126).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "pdr_internal.h"

namespace pdr {

static const double KB = 1.38065040e-16, CL = 2.99792458e+10, HP = 6.62606896e-27;

std::string load_coolant(const char *path, int nlev, int ntemp, HostCoolant &c) {
  std::ifstream in(path);
  if (!in) return std::string("cannot open ") + path;
  std::string line;
  auto next = [&](std::string &s) { return (bool)std::getline(in, s); };
  c.nlev = nlev;
  c.ntemp = ntemp;
  c.energies.assign(nlev, 0.0);
  c.weights.assign(nlev, 0.0);
  c.A.assign(nlev * nlev, 0.0);
  c.B.assign(nlev * nlev, 0.0);
  c.freq.assign(nlev * nlev, 0.0);
  c.temps.assign(7 * ntemp, 0.0);
  c.col.assign((size_t)7 * nlev * nlev * ntemp, 0.0);
  for (int k = 0; k < 5; k++) next(line);
  if (!next(line) || std::atoi(line.c_str()) != nlev) return "incorrect number of energy levels";
  next(line);
  for (int n = 0; n < nlev;) {
    if (!next(line)) return "unexpected end of file in the level block";
    std::istringstream ss(line);
    double e, w;
    if (!(ss >> n >> e >> w) || n < 1 || n > nlev) return "bad level record";
    c.energies[n - 1] = e * CL * HP;
    c.weights[n - 1] = w;
  }
  next(line);
  next(line);
  c.nlin = std::atoi(line.c_str());
  next(line);
  for (int n = 0; n < c.nlin;) {
    if (!next(line)) return "unexpected end of file in the radiative block";
    std::istringstream ss(line);
    int i, j;
    double a, f;
    if (!(ss >> n >> i >> j >> a >> f)) return "bad radiative record";
    i--; j--;
    c.freq[i * nlev + j] = f * 1.0e9;
    c.freq[j * nlev + i] = c.freq[i * nlev + j];
    c.A[i * nlev + j] = a;
    const double f3 = c.freq[i * nlev + j];
    c.B[i * nlev + j] = c.A[i * nlev + j] / (2.0 * HP * (f3 * f3 * f3) / (CL * CL));
    c.B[j * nlev + i] = c.B[i * nlev + j] * (c.weights[i] / c.weights[j]);
    c.line_up.push_back(i);
    c.line_lo.push_back(j);
  }
  for (int i = 0; i < nlev; i++)
    for (int j = 0; j < nlev; j++) {
      const double fq = std::fabs(c.energies[i] - c.energies[j]) / HP;
      double &f = c.freq[i * nlev + j];
      if (f != 0.0) {
        if (std::fabs(fq - f) / f > 1.0e-2) return "calculated frequency differs by >1% from the listed one";
      } else {
        f = fq;
      }
    }
  next(line);
  next(line);
  const int npart = std::atoi(line.c_str());
  for (int l = 0; l < npart; l++) {
    next(line);
    next(line);
    const int p = std::atoi(line.c_str());
    next(line);
    next(line);
    const int ncol = std::atoi(line.c_str());
    next(line);
    next(line);
    const int m = std::atoi(line.c_str());
    if (m > ntemp) return "too many collision temperatures";
    if (p < 1 || p > 7) return "unrecognized collision partner";
    next(line);
    int got = 0;
    while (got < m) {
      if (!next(line)) return "unexpected end of file in the temperature list";
      std::istringstream ss(line);
      double v;
      while (got < m && (ss >> v)) c.temps[(p - 1) * ntemp + got++] = v;
    }
    next(line);
    double *col = c.col.data() + (size_t)(p - 1) * nlev * nlev * ntemp;
    for (int n = 0; n < ncol;) {
      if (!next(line)) return "unexpected end of file in the collision block";
      std::istringstream ss(line);
      int i, j;
      if (!(ss >> n >> i >> j)) return "bad collision record";
      i--; j--;
      for (int k = 0; k < m; k++) {
        double v = 0.0;
        ss >> v;
        col[((size_t)i * nlev + j) * ntemp + k] = v;
        double &rev = col[((size_t)j * nlev + i) * ntemp + k];
        if (v != 0.0 && rev == 0.0)
          rev = v * (c.weights[i] / c.weights[j]) *
                std::exp(-(c.energies[i] - c.energies[j]) / (KB * c.temps[(p - 1) * ntemp + k]));
      }
    }
  }
  return std::string();
}

template <class T>
static T *up(pdr_coolant *c, const std::vector<T> &v, int &rc) {
  T *d = nullptr;
  if (v.empty()) return nullptr;
  cudaError_t e = cudaMalloc(&d, v.size() * sizeof(T));
  if (e != cudaSuccess) { rc = cuda_fail(e, "cudaMalloc(coolant tables)"); return nullptr; }
  c->allocations.push_back(d);
  e = cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpy(coolant tables)");
  return d;
}

int build_coolant_tables(pdr_coolant *c) {
  const HostCoolant &h = c->host;
  CoolantTables &t = c->dev;
  const int n = h.nlev, nn = n * n;
  t.nlev = n;
  t.ntemp = h.ntemp;
  t.nlin = h.nlin;
  t.npart = 0;
  std::vector<double> temps, col;
  for (int p = 0; p < 7; p++) {
    if (h.temps[p * h.ntemp] == 0.0) continue;   // find_Ccoeff.F90:46: partner without rates
    t.part[t.npart++] = p;
    for (int k = 0; k < h.ntemp; k++) temps.push_back(h.temps[p * h.ntemp + k]);
    for (int k = 0; k < h.ntemp; k++)
      for (int e = 0; e < nn; e++) col.push_back(h.col[((size_t)p * nn + e) * h.ntemp + k]);
  }
  std::vector<int> lop(nn, -1);
  for (int l = 0; l < h.nlin; l++) lop[h.line_up[l] * n + h.line_lo[l]] = l;
  int rc = 0;
  t.temps = up(c, temps, rc);
  t.col = up(c, col, rc);
  t.A = up(c, h.A, rc);
  t.B = up(c, h.B, rc);
  t.freq = up(c, h.freq, rc);
  t.weights = up(c, h.weights, rc);
  t.energies = up(c, h.energies, rc);
  t.line_of_pair = up(c, lop, rc);
  std::vector<int> rp;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < i; j++) {
      const int e = i * n + j, et = j * n + i;
      if (h.A[e] != 0.0 || h.B[e] != 0.0 || h.A[et] != 0.0 || h.B[et] != 0.0) rp.push_back(e);
    }
  {
    // escape_probability.F90:61 per radiative line (FRAC1 of the tau sum)
    const double CLc = 2.99792458e+10, PIc = 3.141592653589793238462643383279502884197;
    std::vector<double> f1(h.nlin);
    for (int l = 0; l < h.nlin; l++) {
      const int e = h.line_up[l] * n + h.line_lo[l];
      const double fr = h.freq[e];
      f1[l] = (h.A[e] * (CLc * CLc * CLc)) / (8.0 * PIc * (fr * fr * fr));
    }
    t.line_up = up(c, h.line_up, rc);
    t.line_lo = up(c, h.line_lo, rc);
    t.line_frac1 = up(c, f1, rc);
  }
  t.nrad = (int)rp.size();
  if (!rp.empty()) {
    // escape_probability.F90:66-71 per pair, with the reference's operation
    // order and its default-REAL literals
    const double KB = 1.38065040e-16, CL = 2.99792458e+10, HP = 6.62606896e-27;
    std::vector<double> tmp2(rp.size()), cmb(rp.size()), emis(rp.size());
    for (size_t k = 0; k < rp.size(); k++) {
      const double f = h.freq[rp[k]];
      tmp2[k] = 2.0 * HP * (f * f * f) / (CL * CL);
      cmb[k] = tmp2[k] * (1.0 / (std::exp(HP * f / KB / 2.7) - 1.0));
      emis[k] = (double)0.01f * ((double)1.3f * f / 3.0e11);
    }
    t.rad_pairs = up(c, rp, rc);
    t.pair_tmp2 = up(c, tmp2, rc);
    t.pair_cmb = up(c, cmb, rc);
    t.pair_emis = up(c, emis, rc);
  }
  return rc;
}

}  // namespace pdr
