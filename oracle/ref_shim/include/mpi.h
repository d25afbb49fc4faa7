/* Stub MPI header used only to compile the reference's CPU setup code as a
 * test-only checker. Single process: rank 0, abort exits. */
#pragma once
#include <stdlib.h>
typedef int MPI_Comm;
#define MPI_COMM_WORLD 0
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Abort(MPI_Comm, int code) { exit(code); return 0; }
static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline double MPI_Wtime(void) { return 0.0; }
