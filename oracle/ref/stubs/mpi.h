/* Test-only stub: the reference units used by the oracle only call
 * MPI_Wtime (for their profiling prints).  Declared here as a wall clock.
 * The Hoshen-Kopelman unit also names MPI file I/O in a debug dump that is
 * off by default (Settings::IORAWHKClusterID); those calls compile to no-ops
 * here and report failure if ever reached. */
#ifndef PP_ORACLE_STUB_MPI_H
#define PP_ORACLE_STUB_MPI_H
#include <chrono>
typedef int MPI_Datatype;
typedef int MPI_Comm;
typedef int MPI_File;
typedef int MPI_Status;
typedef long MPI_Offset;
typedef long MPI_Aint;
#define MPI_COMM_WORLD 0
#define MPI_COMM_SELF 0
#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 2
#define MPI_INFO_NULL 0
#define MPI_SEEK_SET 0
#define MPI_UNSIGNED 0
static inline int MPI_File_open(MPI_Comm, const char*, int, int, MPI_File*) { return 1; }
static inline int MPI_File_seek(MPI_File, MPI_Offset, int) { return 1; }
static inline int MPI_File_write(MPI_File, const void*, int, MPI_Datatype, MPI_Status*) { return 1; }
static inline int MPI_File_close(MPI_File*) { return 1; }
static inline double MPI_Wtime() {
  return std::chrono::duration<double>(
      std::chrono::steady_clock::now().time_since_epoch()).count();
}
#endif
