/* Test-only stub: libnuma's bitmask type, named by a reference header. */
#ifndef PP_ORACLE_STUB_NUMA_H
#define PP_ORACLE_STUB_NUMA_H
struct bitmask { unsigned long size; unsigned long* maskp; };
#endif
