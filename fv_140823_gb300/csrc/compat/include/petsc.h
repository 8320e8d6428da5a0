/*
 * petsc.h -- the one PETSc call of the reference's host program
 * (PetscInitialize, main.c:28); nothing on its explicit path uses PETSc
 * objects.  The reference's header also includes petscsys.h, petscksp.h,
 * petscmat.h, petscsnes.h, petscvec.h and petscts.h, which resolve here.
 * Definition in fvcompat.c.
 */
#ifndef FVCOMPAT_PETSC_H
#define FVCOMPAT_PETSC_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int PetscErrorCode;
PetscErrorCode PetscInitialize(int *argc, char ***args, const char *file, const char *help);
PetscErrorCode PetscFinalize(void);

#ifdef __cplusplus
}
#endif
#endif
