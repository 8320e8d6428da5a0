/*
 * fvcompat_cpu.c -- the time step the reference's loop calls
 * (advancetimeexplicit, loop.c:48; strdata.h:568-569) for a build of the
 * reference program that keeps its own residual code (no drop-in shim, no
 * GPU).  One step of con->dt: RK(0), then per stage faceinterp (MUSCL),
 * gradcalc (viscous), RHS and RK(k).  The stage list follows the deck's RK
 * method (CON.method, inputset.c:47) as the drop-in shim reads it: 1 forward
 * Euler {1}, 2 SSP-RK2 {1, 4}, anything else SSP-RK3 {1, 2, 3} (RK.c:16-47).
 * Link either this file or fvshim.c, not both.
 */
#include "strdata.h"

void advancetimeexplicit(struct RUN *run) {
  static const int kEuler[] = {1}, kSsp2[] = {1, 4}, kSsp3[] = {1, 2, 3};
  const int method = run->con->method;
  const int *stages = method == 1 ? kEuler : (method == 2 ? kSsp2 : kSsp3);
  const int nstages = method == 1 ? 1 : (method == 2 ? 2 : 3);
  RK(0, run);
  for (int s = 0; s < nstages; ++s) {
    if (run->con->ischeme == 2) faceinterp(run);
    if (run->con->ns == 1) gradcalc(run);
    RHS(run);
    RK(stages[s], run);
  }
}

void advancetimeexplicit_nb(struct RUN *run) { advancetimeexplicit(run); }
