/* Type shim (oracle build only). */
#include <sundials/sundials_dense.h>
