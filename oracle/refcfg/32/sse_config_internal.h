/* Configuration header for building the reference scalar library from its own
 * sources with oracle/Makefile.  Autotools would generate this file from
 * include/sse_config_internal.h.in; it is written by hand here because
 * autotools are not installed.  Scalar (single node) build, 32-bit. */
#define SSE_PRECISION 32
#define SSE_SCALAR 1
#define PACKAGE "sse_wilson_dslash"
#define VERSION "reference"
