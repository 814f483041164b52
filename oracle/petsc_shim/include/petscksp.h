/* TEST INFRASTRUCTURE ONLY: forwards to the single-process API shim. */
#include "petsc_shim.h"
