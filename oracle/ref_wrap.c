/*
 * ref_wrap.c -- C entry points around the reference's generated f() and Jac()
 * (odes_<net>.c:26, jacobian_<net>.c:26), compiled together with those files
 * into oracle/_ref/libref_<net>.so.  TEST INFRASTRUCTURE ONLY: it lets the
 * tests evaluate the reference RHS/Jacobian on the same states as the oracle
 * and the GPU path.
 */
#include <stdlib.h>
#include <sundials/sundials_types.h>
#include <nvector/nvector_serial.h>
#include <sundials/sundials_dense.h>

typedef struct {
  realtype *rate, n_H, T_g, x_e;
} *User_Data;

int f(realtype t, N_Vector y, N_Vector ydot, void *user_data);
int Jac(long int N, realtype t, N_Vector y, N_Vector fy, DlsMat J, void *user_data, N_Vector tmp1,
        N_Vector tmp2, N_Vector tmp3);

/* ode[neq]; returns the x_e the generated code stores in user_data */
double ref_rhs(int neq, const double *x, double *ode, double *rate, double n_H, double T) {
  (void)neq;
  struct shim_nvec vy = {(double *)x}, vd = {ode};
  typeof(*(User_Data)0) ud = {rate, n_H, T, 0.0};
  f(0.0, &vy, &vd, &ud);
  return ud.x_e;
}

/* J column-major J[j*neq+i] = dfi/dxj with x_e held at the given value */
void ref_jac(int neq, const double *x, double *J, double *rate, double n_H, double T, double x_e) {
  struct shim_nvec vy = {(double *)x};
  double **cols = (double **)malloc(sizeof(double *) * neq);
  for (int j = 0; j < neq; j++) {
    cols[j] = J + (size_t)j * neq;
    for (int i = 0; i < neq; i++) cols[j][i] = 0.0;
  }
  struct shim_dlsmat m = {neq, neq, cols};
  typeof(*(User_Data)0) ud = {rate, n_H, T, x_e};
  Jac(neq, 0.0, &vy, NULL, &m, &ud, NULL, NULL, NULL);
  free(cols);
}
