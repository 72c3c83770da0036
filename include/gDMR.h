/* Solver interface of libgDMR (GB300 build).
 *
 * Same entry points, argument meaning and return values as the reference's
 * gDMR.h, so callers written against it (plugins, progDMR-style control
 * programs) compile and link unchanged.  As in the reference, include
 * <cuComplex.h> and the CUDA runtime types before this header.
 *
 * Differences a caller may notice: the solver runs on one GPU (devList[0];
 * repeated ids, the reference's "virtual devices", are accepted), never calls
 * cudaDeviceReset, and reports error details through gdmrLastError() in
 * gdmr_ext.h.
 */
#ifndef GDMR_GB300_GDMR_H
#define GDMR_GB300_GDMR_H
#ifdef __cplusplus
extern "C" {
#endif

/* Initialise the solver (replaces initDMR, reference gDMR.h:13 / gDMR.cu:842-1208).
 * blocks, threadsPerBlock: accepted for compatibility; launch shapes are chosen
 *   per kernel from the device's SM count.
 * devList, numDevs: devices; the solver runs on devList[0].
 * elements: vector length n.  basisDim: m, total basis (deflation + Krylov),
 *   at most 160; basisDim + 1 and deflatDim must be divisible by numDevs, and
 *   basisDim - deflatDim >= 2, as in the reference.
 * linComp: the operator hook; it must overwrite the plugin's source vector x
 *   with A x on the stream later passed to solverDMR. */
void initDMR(int blocks, int threadsPerBlock, int *devList, int numDevs, int elements, int basisDim, int deflatDim,
             void (*linComp)(void));

/* Free solver memory (replaces freeDMR, reference gDMR.h:15 / gDMR.cu:1211-1475). */
void freeDMR(void);

/* Solve A x = b (replaces solverDMR, reference gDMR.h:29 / gDMR.cu:2638-2900).
 * mode != 0 reuses the deflation space left by an earlier solve.
 * extSrcVec: device x (initial guess in, solution out; overwritten by the
 *   hook's products during the solve).  extImgVec: device b (read only).
 * extStream, extDevNum: the hook's stream and device.  solTol: relative
 * tolerance (also the absolute breakdown threshold, as in the reference).
 * matRank: restart-cycle cap.  numIts: restart cycles - 1.
 * Returns ||r||/||b|| from the recursively updated residual; the absolute
 * ||r|| when the initial guess already meets the tolerance. */
float solverDMR(int mode, cuComplex *extSrcVec, cuComplex *extImgVec, cudaStream_t extStream, int extDevNum,
                float solTol, int matRank, int *numIts);

/* Import / export the source-side deflation vectors Z, deflatDim x elements
 * complex64, vector-contiguous (replaces impSVDMR/expSVDMR, reference
 * gDMR.h:33-34 / gDMR.cu:431-477; the export copies device to host). */
void impSVDMR(float _Complex *cMem);
void expSVDMR(float _Complex *cMem);

#ifdef __cplusplus
}
#endif
#endif
