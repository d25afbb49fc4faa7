/* Stub HYPRE header used only to compile the reference's CPU setup code as a
 * test-only checker. No solver exists behind these names: every function
 * returns an error code and is never called by the checker. */
#pragma once
typedef int HYPRE_Int;
typedef double HYPRE_Complex;
typedef double HYPRE_Real;
typedef struct hypre_stub_obj *HYPRE_StructGrid, *HYPRE_StructStencil, *HYPRE_StructMatrix,
    *HYPRE_StructVector, *HYPRE_StructSolver;
typedef HYPRE_Int (*HYPRE_PtrToStructSolverFcn)(...);
#define HYPRE_ERROR_CONV 256
#define HYPRE_MEMORY_DEVICE 1
#define HYPRE_EXEC_DEVICE 1
#define HYPRE_STUB(name) static inline HYPRE_Int name(...) { return -1; }
HYPRE_STUB(HYPRE_ClearError)
HYPRE_STUB(HYPRE_Initialize)
HYPRE_STUB(HYPRE_Finalize)
HYPRE_STUB(HYPRE_SetMemoryLocation)
HYPRE_STUB(HYPRE_SetExecutionPolicy)
