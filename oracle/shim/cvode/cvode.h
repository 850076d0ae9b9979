/* Type shim (oracle build only). */
#include <sundials/sundials_types.h>
#include <nvector/nvector_serial.h>
