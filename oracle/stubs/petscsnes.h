/* Empty stand-in for <petscsnes.h>: the reference header includes it, but nothing on
 * the residual/RK path uses its declarations. Written for the oracle harness. */
