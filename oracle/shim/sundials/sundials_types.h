/* Type shim so the reference's generated network code (odes_<net>.c,
 * jacobian_<net>.c) compiles without SUNDIALS.  Oracle build only. */
#ifndef SHIM_SUNDIALS_TYPES_H
#define SHIM_SUNDIALS_TYPES_H
typedef double realtype;
#define RCONST(x) x
#endif
