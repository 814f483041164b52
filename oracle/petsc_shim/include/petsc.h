/* TEST INFRASTRUCTURE ONLY: the PETSc umbrella header some reference files include. */
#include "petsc_shim.h"
