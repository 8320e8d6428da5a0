/*
 * fvshim.h -- link-time drop-in of libfvgpu for the FV_140823 host program.
 *
 * fvshim.c is compiled against the host's own strdata.h and linked into the
 * host executable in place of the reference objects RHS.o, RHS_nb.o, RK.o,
 * faceinterp.o and gradcalc.o.  It defines the reference's symbols with the
 * reference's signatures (strdata.h:568-569, 642, 654-656, 675):
 *
 *     void RHS(struct RUN *run);                    RHS.c:3-13
 *     void RHS_nb(struct RUN *run, int inner_outer); RHS_nb.c:3-15
 *     void RK(int irk, RUN *run);                   RK.c:3-56
 *     void faceinterp(struct RUN *run);             faceinterp.c:21-61
 *     void gradcalc(struct RUN *run);               gradcalc.c:9-47
 *     void advancetimeexplicit(struct RUN *run);    declared, never defined (loop.c:48)
 *     void advancetimeexplicit_nb(struct RUN *run); declared, never defined
 *
 * and keeps the state on the GPU between calls.  The leaf list is flattened
 * (with the host's own distance() for the MUSCL distances) and uploaded on
 * the first call and after every mesh change; LEAF.S is gathered from the
 * leaves at those points and written back only where the host reads it:
 *   - gradcalc(run) called by the host (loop.c:51, before export) downloads
 *     S and the gradients SG into the leaves;
 *   - advancetimeexplicit downloads S after the steps that precede a
 *     restart save (con->ststep), an export (con->exstep) or an adaptation
 *     (con->adapthstep), and re-flattens on adaptation steps;
 *   - fvshim_sync_host() does it on demand (conservationcalc, custom I/O).
 * Errors print the library's message and exit(0), as the reference does on
 * a NaN residual (residual_faces_AMR.c:186-194); fvshim_set_error_handler()
 * replaces that behaviour.
 */
#ifndef FVSHIM_H
#define FVSHIM_H

#ifdef __cplusplus
extern "C" {
#endif

struct RUN;

/* fields for fvshim_sync_host */
#define FVSHIM_S 1    /* LEAF.S   */
#define FVSHIM_SN 2   /* LEAF.SN  */
#define FVSHIM_RHS 4  /* LEAF.RHS */
#define FVSHIM_SF 8   /* LEAF.SF (ischeme 2) */
#define FVSHIM_SG 16  /* LEAF.SG (once a gradcalc or a viscous step ran) */

/* Copy device fields into the leaves of run->topo->locl. */
void fvshim_sync_host(struct RUN *run, int fields);
/* The mesh or the leaves' S changed on the host (adaptation, restart load,
 * initialisation): flatten and upload again before the next call. */
void fvshim_invalidate(struct RUN *run);
/* RK scheme of advancetimeexplicit: FVGPU_SCHEME_EULER / SSPRK2 / SSPRK3,
 * or 0 (the default) for the deck's method (CON.method, inputset.c:47):
 * 1 Euler, 2 SSP-RK2, anything else SSP-RK3. */
void fvshim_set_scheme(int scheme);
/* FVGPU_FP64 (default, bit-identical to the reference) or FVGPU_MIXED. */
void fvshim_set_precision(int precision);
/* Called with the library's error code and message instead of exit(0). */
void fvshim_set_error_handler(void (*handler)(int code, const char *msg));
/* Release the GPU context and the flattened tables. */
void fvshim_release(void);
/* Number of flatten + mesh uploads and of host syncs so far (diagnostics). */
void fvshim_counters(long *uploads, long *syncs);

#ifdef __cplusplus
}
#endif
#endif
