/*
 * fortran_caller.c -- stands in for the 3D-PDR Fortran driver when testing the
 * drop-in symbol calculate_abundances_ (there is no Fortran compiler here).
 *
 * Like the gfortran program it defines the bind(c) module variables the C
 * chemistry reads (modules.F90:165-166,383,529-530) and calls the symbol with
 * every argument by reference, arrays column-major (3DPDR.F90:498).
 *
 *   fortran_caller <input> <output>
 * input : int32 npart, nspec, nreac, nelect(1-based); float64 reltol, abstol,
 *         start_time, end_time; float64 abundance[npart*nspec],
 *         rate[npart*nreac], density[npart], temperature[npart]
 * output: int32 status; float64 abundance[npart*nspec]
 */
#include <stdio.h>
#include <stdlib.h>

double chemistry_module_mp_relative_abundance_tolerance_;
double chemistry_module_mp_absolute_abundance_tolerance_;
double maincode_module_mp_start_time_;
double maincode_module_mp_end_time_;
int global_module_mp_nelect_;

int calculate_abundances_(double *abundance, double *rate, double *density, double *temperature, int *npart,
                          int *nspec, int *nreac);

static void rd(void *p, size_t sz, size_t n, FILE *f) {
  if (fread(p, sz, n, f) != n) { fprintf(stderr, "short input\n"); exit(2); }
}

int main(int argc, char **argv) {
  if (argc != 3) { fprintf(stderr, "usage: fortran_caller <input> <output>\n"); return 2; }
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  int hdr[4];
  double par[4];
  rd(hdr, sizeof(int), 4, f);
  rd(par, sizeof(double), 4, f);
  int npart = hdr[0], nspec = hdr[1], nreac = hdr[2];
  global_module_mp_nelect_ = hdr[3];
  chemistry_module_mp_relative_abundance_tolerance_ = par[0];
  chemistry_module_mp_absolute_abundance_tolerance_ = par[1];
  maincode_module_mp_start_time_ = par[2];
  maincode_module_mp_end_time_ = par[3];
  double *ab = malloc(sizeof(double) * (size_t)npart * nspec);
  double *rate = malloc(sizeof(double) * (size_t)npart * nreac);
  double *dens = malloc(sizeof(double) * (size_t)npart);
  double *temp = malloc(sizeof(double) * (size_t)npart);
  rd(ab, sizeof(double), (size_t)npart * nspec, f);
  rd(rate, sizeof(double), (size_t)npart * nreac, f);
  rd(dens, sizeof(double), (size_t)npart, f);
  rd(temp, sizeof(double), (size_t)npart, f);
  fclose(f);
  int status = calculate_abundances_(ab, rate, dens, temp, &npart, &nspec, &nreac);
  FILE *o = fopen(argv[2], "wb");
  if (!o) return 2;
  fwrite(&status, sizeof(int), 1, o);
  fwrite(ab, sizeof(double), (size_t)npart * nspec, o);
  fclose(o);
  return 0;
}
