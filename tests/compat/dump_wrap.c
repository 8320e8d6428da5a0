/*
 * dump_wrap.c -- TEST INFRASTRUCTURE ONLY.  Linked into builds of the
 * reference's host program with -Wl,--wrap=advancetimeexplicit, it runs the
 * real time step and, after the loop's last one (istep == nstep, loop.c:34),
 * writes every leaf's state to the file named by FVCOMPAT_DUMP:
 *   int64 leaf count, int32 neq, then per leaf in list order
 *   int32 root (the input element), double S[neq], double Vol, xc, yc, zc.
 * With the drop-in shim it first copies the device state into the leaves.
 */
#include "strdata.h"

#include <stdint.h>

void __real_advancetimeexplicit(struct RUN *run);
void fvshim_sync_host(struct RUN *run, int fields) __attribute__((weak));

void __wrap_advancetimeexplicit(struct RUN *run) {
  __real_advancetimeexplicit(run);
  if (run->con->istep != run->con->nstep) return;
  if (fvshim_sync_host) fvshim_sync_host(run, 1);
  const char *path = getenv("FVCOMPAT_DUMP");
  if (!path) return;
  FILE *fp = fopen(path, "wb");
  if (!fp) {
    fprintf(stderr, "dump_wrap: cannot open %s\n", path);
    exit(1);
  }
  int64_t n = 0;
  for (BRANCH *b = run->topo->locl; b; b = b->lnxt) ++n;
  const int32_t neq = run->con->neq;
  fwrite(&n, sizeof n, 1, fp);
  fwrite(&neq, sizeof neq, 1, fp);
  for (BRANCH *b = run->topo->locl; b; b = b->lnxt) {
    const int32_t root = b->root;
    fwrite(&root, sizeof root, 1, fp);
    fwrite(b->el->S, sizeof(double), (size_t)neq, fp);
    const double geo[4] = {b->cl->Vol, b->cl->xc, b->cl->yc, b->cl->zc};
    fwrite(geo, sizeof(double), 4, fp);
  }
  fclose(fp);
}
