/* Type shim (oracle build only): a serial vector is a bare data pointer. */
#ifndef SHIM_NVECTOR_SERIAL_H
#define SHIM_NVECTOR_SERIAL_H
#include <sundials/sundials_types.h>
struct shim_nvec { realtype *data; };
typedef struct shim_nvec *N_Vector;
#define NV_DATA_S(v) ((v)->data)
#endif
