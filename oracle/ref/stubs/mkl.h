/* Test-only stub: just enough Intel MKL type names for the reference
 * headers to parse.  No MKL routine is called on the spatial-statistics
 * path, so nothing here is implemented. */
#ifndef PP_ORACLE_STUB_MKL_H
#define PP_ORACLE_STUB_MKL_H
typedef long MKL_LONG;
typedef struct { float real; float imag; } MKL_Complex8;
#endif
