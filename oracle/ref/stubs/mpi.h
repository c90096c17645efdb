/* Test-only stub: the reference units used by the oracle only call
 * MPI_Wtime (for their profiling prints).  Declared here as a wall clock. */
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
static inline double MPI_Wtime() {
  return std::chrono::duration<double>(
      std::chrono::steady_clock::now().time_since_epoch()).count();
}
#endif
