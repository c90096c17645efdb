/* Test-only stub: DFTI handle types named by the reference's MKL wrapper
 * header (never called on the spatial-statistics path). */
#ifndef PP_ORACLE_STUB_MKL_DFTI_H
#define PP_ORACLE_STUB_MKL_DFTI_H
#include "mkl.h"
typedef int DFTI_CONFIG_VALUE;
typedef void* DFTI_DESCRIPTOR_HANDLE;
#endif
