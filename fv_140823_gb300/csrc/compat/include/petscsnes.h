/* Resolves to the single PETSc declaration the reference program needs. */
#include "petsc.h"
