/* Stand-in for <rpc/xdr.h> (absent on this machine).  The reference's
 * translation units include it for the Tipsy XDR reader only; the shim
 * provides the type and the decode-side entry points the reader calls
 * (ref_shim.cpp), reading big-endian values from the FILE. */
#ifndef DMANN_SHIM_RPC_XDR_H
#define DMANN_SHIM_RPC_XDR_H
#include <stdio.h>
#include "types.h"
enum xdr_op { XDR_ENCODE = 0, XDR_DECODE = 1, XDR_FREE = 2 };
typedef struct { int x_op; FILE *fp; } XDR;
#ifdef __cplusplus
extern "C" {
#endif
void xdrstdio_create(XDR *xdrs, FILE *file, enum xdr_op op);
void xdr_destroy(XDR *xdrs);
#ifdef __cplusplus
}
#endif
#endif
