/* Linear-system plugin interface of libgDMR (GB300 build).
 *
 * Same entry points and meaning as the reference's gDMRC.h (the interface
 * progDMR.c is written against), implemented by this library's own plugin:
 * it owns the operator A, the source vector x and the image vector b on the
 * device and passes linOptLS to the solver as its operator hook.  A is dense
 * (impOptLS, column-major n x n complex64, as in the reference) or sparse
 * (impCsrLS in gdmr_ext.h).  Plain C99: no CUDA headers needed.
 */
#ifndef GDMR_GB300_GDMRC_H
#define GDMR_GB300_GDMRC_H
#ifdef __cplusplus
extern "C" {
#endif

/* Initialise the system and the solver (reference gDMRC.h:6 / testLS.cu:131-192).
 * The dense operator starts as the identity. */
void initLS(int blocksMDR, int threadsPerBlockMDR, int devNumLO, int cells, int *devListMDR, int numDevsMDR,
            int basisSizeMDR, int deflatSizeMDR);
/* Free the system and the solver (reference gDMRC.h:8 / testLS.cu:195-244). */
void freeLS(void);
/* Copy b (image) to / from the device (reference gDMRC.h:10-11). */
void impImgLS(float _Complex *cImg);
void expImgLS(float _Complex *cImg);
/* Copy x (source) to / from the device (reference gDMRC.h:13-14). */
void impSrcLS(float _Complex *cSrc);
void expSrcLS(float _Complex *cSrc);
/* Copy the dense operator to / from the device (reference gDMRC.h:16-17). */
void impOptLS(float _Complex *cOpt);
void expOptLS(float _Complex *cOpt);
/* Solve, returning solverDMR's value (reference gDMRC.h:21 / testLS.cu:387-390). */
float solveLS(int mode, float solTol, int matRank, int *numIts);
/* x <- A x in place (reference gDMRC.h:23 / testLS.cu:97-128); no aliased
 * input/output buffers are used internally. */
void linOptLS(void);
/* Deflation vector import / export, as in gDMR.h (reference gDMRC.h:27-28). */
void impSVDMR(float _Complex *cMem);
void expSVDMR(float _Complex *cMem);

#ifdef __cplusplus
}
#endif
#endif
