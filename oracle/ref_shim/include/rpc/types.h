/* Stand-in for <rpc/types.h> (absent on this machine); see rpc/xdr.h. */
#ifndef DMANN_SHIM_RPC_TYPES_H
#define DMANN_SHIM_RPC_TYPES_H
/* The system header pulls in the C library declarations (malloc, exit, ...)
 * that the reference relies on without including them itself. */
#include <stdlib.h>
#include <string.h>
typedef int bool_t;
#endif
