// Forwards to the single-rank PETSc/HYPRE/MPI stand-in.
#include "petsc_shim.h"
