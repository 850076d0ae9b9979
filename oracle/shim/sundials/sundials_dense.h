/* Type shim (oracle build only): dense matrix as an array of column pointers. */
#ifndef SHIM_SUNDIALS_DENSE_H
#define SHIM_SUNDIALS_DENSE_H
#include <sundials/sundials_types.h>
struct shim_dlsmat { long M, N; realtype **cols; };
typedef struct shim_dlsmat *DlsMat;
#endif
