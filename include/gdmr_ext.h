/* Extensions of libgDMR (GB300 build): status reporting, the complex128
 * drop-in (the reference is complex64 only), sparse plugins, and a
 * context API for the batched FP64-refined mixed-precision solver.
 *
 * None of these symbols exists in the reference; each names the reference
 * interface it extends.  Complex values cross the ABI as interleaved
 * (re, im) doubles or floats, or as C99 _Complex, so plain C callers need no
 * CUDA headers (only the *_z solver entry points take cudaStream_t).
 */
#ifndef GDMR_GB300_EXT_H
#define GDMR_GB300_EXT_H
#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (the reference prints to stderr and resets the device instead,
 * gDMR.cu:409-429; this library never resets a device). */
enum {
    GDMR_OK = 0,
    GDMR_EINVAL = 1,     /* bad argument or size */
    GDMR_ENOMEM = 2,     /* device allocation failed */
    GDMR_ENOCONV = 3,    /* cycle cap reached (reference: "failed to converge", gDMR.cu:2816) */
    GDMR_ERUNAWAY = 4,   /* residual above ||b|| (reference: "Runaway", gDMR.cu:2823) */
    GDMR_ECUDA = 5,      /* CUDA runtime error */
    GDMR_ENOTINIT = 6,   /* used before init */
    GDMR_EBREAKDOWN = 7,
    GDMR_ETIMEOUT = 8,   /* a bounded device wait ran out during the call (gdmrWaitLimit); its results,
                            and the deflation space, are dropped */
    GDMR_ENONFINITE = 9  /* NaN or Inf in a residual: the operator or the data produced it (the
                            reference's loop test treats NaN as converged, gDMR.cu:2814) */
};

/* Last status and message of any entry point (process-wide). */
int gdmrLastStatus(void);
const char *gdmrLastError(void);
/* Library version string, e.g. "1.0.1-gb300". */
const char *gdmrVersion(void);

/* ---- complex128 drop-in: reference solver semantics in FP64 ----------------
 * Same arguments and behaviour as initDMR/freeDMR/solverDMR/impSVDMR/expSVDMR
 * (gDMR.h), with complex128 vectors and a double tolerance.  The hook must
 * overwrite the complex128 source buffer passed to solverDMR_z. */
#ifdef GDMR_WITH_CUDA_TYPES
void initDMR_z(int blocks, int threadsPerBlock, int *devList, int numDevs, int elements, int basisDim, int deflatDim,
               void (*linComp)(void));
void freeDMR_z(void);
double solverDMR_z(int mode, cuDoubleComplex *extSrcVec, cuDoubleComplex *extImgVec, cudaStream_t extStream,
                   int extDevNum, double solTol, int matRank, int *numIts);
#endif
void impSVDMR_z(double _Complex *cMem);
void expSVDMR_z(double _Complex *cMem);

/* ---- plugin extensions (extend gDMRC.h) ------------------------------------
 * impCsrLS: make the plugin's operator the CSR matrix (int32 row pointers of
 * length cells+1, int32 column indices, complex64 values), stored on the
 * device in SELL-32 form; replaces any dense operator. */
int impCsrLS(int nnz, const int *rowPtr, const int *colIdx, const float _Complex *vals);
/* The complex128 plugin: the same functions with a _z suffix, solving through
 * solverDMR_z. */
void initLS_z(int blocksMDR, int threadsPerBlockMDR, int devNumLO, int cells, int *devListMDR, int numDevsMDR,
              int basisSizeMDR, int deflatSizeMDR);
void freeLS_z(void);
void impImgLS_z(double _Complex *cImg);
void expImgLS_z(double _Complex *cImg);
void impSrcLS_z(double _Complex *cSrc);
void expSrcLS_z(double _Complex *cSrc);
void impOptLS_z(double _Complex *cOpt);
int impCsrLS_z(int nnz, const int *rowPtr, const int *colIdx, const double _Complex *vals);
double solveLS_z(int mode, double solTol, int matRank, int *numIts);
void linOptLS_z(void);
/* Statistics of the last solveLS/solveLS_z/solverDMR/solverDMR_z call. */
typedef struct {
    int cycles;            /* restart cycles run */
    int its;               /* reference convention: cycles - 1 */
    long long matvecs;     /* operator applications */
    double rel_res;        /* value returned by the solve */
    double true_rel_res;   /* FP64 ||b - A x|| / ||b|| when measured, else -1 */
    int status;            /* GDMR_* */
    int breakdowns;        /* cycles that ended in a Krylov breakdown */
    double latency_ms;     /* batched solves: time from the call's start to this solution's return */
} gdmr_stats;
void gdmrLastStats(gdmr_stats *out);
/* One restart cycle of the last reference-semantics solve (solverDMR/solveLS and their _z twins,
 * gdmr_solve), as the host saw it after the cycle. */
typedef struct {
    double rho;        /* ||r_new|| / ||r_old||: the cycle's residual reduction (gDMR.cu:2491-2503) */
    double rel_res;    /* the recursive residual over ||b|| after the cycle */
    int kk;            /* deflation vectors the cycle used (0 on a first cycle with mode 0) */
    int restart;       /* 0: the cycle started from the residual; otherwise the stagnation rule
                          (arnoldiSetupDMR, gDMR.cu:2600-2621) restarted it from the Krylov vector
                          at this index of the reference's [W V] storage, kk + (m - k) / 2 */
    int breakdown;     /* Krylov step of an absolute breakdown in the cycle (gDMR.cu:2256), 0: none */
    int stagnated;     /* 1 when rho > 0.995, which sets the reference's stagnation flag (gDMR.cu:2506) */
} gdmr_cycle;
/* Copies up to max cycles of the last reference-semantics solve into out; returns how many
 * cycles it had. */
int gdmrLastHistory(gdmr_cycle *out, int max);

/* ---- instrumentation --------------------------------------------------------
 * Kernel launches issued by this library since load.  With profiling on, each
 * launch is bracketed by CUDA events on its stream and booked, with its
 * algorithmic bytes, to a kernel class: 0 projection [W V]^H w, 1 update
 * w - [W V] c, 2 operator products, 3 cycle-end combinations, 4 deflation
 * update, 5 FP64 true residual, 6 least squares, 7 SVD, 8 other. */
long long gdmrKernelLaunches(void);
/* Bounded mbarrier waits (tensor-core and bulk-copy pipelines) that ran out since load: every
 * such wait gives up after about two seconds and the kernel returns with its results unset, so
 * a nonzero count means a result of this process is not to be trusted. */
unsigned gdmrAsyncTimeouts(void);
/* Bound, in milliseconds at the GB300's 2.07 GHz clock, of every wait a kernel makes on another
 * part of the GPU: the stage waits of the tensor-core and bulk-copy pipelines and the grid-wide
 * barriers of the fused small-system Krylov kernel (default 2000).  A wait that runs out stops
 * its kernel, counts in gdmrAsyncTimeouts, and the solve returns GDMR_ETIMEOUT.  The waits in
 * which a kernel drains its own copies and tensor-core operations before it frees TMEM keep a
 * fixed two-second bound.  Takes effect at the next solve (or server start); ms < 0 only reads.
 * Returns the previous value. */
double gdmrWaitLimit(double ms);
/* Failure-path testing: the nth device allocation that a solver engine makes from now on fails
 * as if cudaMalloc had (GDMR_ENOMEM, everything allocated so far is freed); 0 disarms. */
void gdmrInjectAllocFailure(int nth);
void gdmrProfile(int on);
void gdmrProfileReset(void);
int gdmrProfileRead(int kernelClass, double *bytes, double *ms, long long *launches);
/* The singular value decomposition of the deflation update on its own (svDecompHessDMR,
 * gDMR.cu:638): H is (m+1) x m complex128 (re, im interleaved), column-major with leading
 * dimension m+1, in host memory; sigma receives the m singular values in descending order and
 * vs the right singular vectors of the k smallest (k x m: vector t, of the (m-k+t)-th
 * largest value, contiguous).  The vectors are accurate to about 1e-13 (double-float), the
 * other values to FP32 refinement.  sweeps (may be NULL) receives 1000 * (FP32 Jacobi sweeps,
 * plus 100 if the unpivoted fallback ran) + double-float sweeps.  Runs on the current device
 * with device scratch of its own.  1 <= k <= m <= 160, else GDMR_EINVAL. */
int gdmr_hessenberg_svd(int m, int k, const double *H, double *sigma, double *vs, int *sweeps);
/* The tensor-core kernels of a batched cycle's shared deflation segment on their own (the
 * deflator w -= W W^H w of deflatorDMR, gDMR.cu:1710-1787, for nsys systems that share W), run
 * once on host data so that their results can be checked against a host product:
 *   coef[s*k + p] = <W_p, Y_s> = sum_i conj(W_p[i]) Y_s[i]   (split-K projection, 3xTF32)
 *   P[s*n + i]    = sum_p c[s*k + p] W_p[i]                    (apply, 3xTF32)
 * W: k x n and Y, P: nsys x n complex64 (interleaved floats); c, coef: nsys x k complex128
 * (interleaved doubles).  Needs an even n, 1 <= k <= 32, 8 <= nsys <= 64 (GDMR_EINVAL
 * otherwise).  Allocates its own device buffers and synchronises the device. */
int gdmr_shared_basis_check(int n, int k, int nsys, const float *W, const float *Y, const double *c, double *coef,
                            float *P);
/* Gram-Schmidt kernel autotuning: the first launch of a shape times the kernel variants
 * and keeps the fastest for the process (on by default; off selects the first variant).
 * The report lists one line per tuned shape with the time of every variant. */
void gdmrTune(int on);
const char *gdmrTuneReport(void);
/* Pins the Gram-Schmidt variants by their index in the tuner report (-1: tuner).  Used to
 * check every variant against the others; an index a launch cannot use falls back to 0.
 * complex64 projection 0-10, update 0-11; complex128 and fp64e projection 0-8, update 0-7
 * (projection 8 and update 7 prefetch the next group of basis vectors).
 * Batched shared-deflation-basis variants (8 to 64 systems, k <= 32): complex64 projection 9
 * (CUDA cores) and 10 (tensor cores), update 8 (CUDA cores), 9 (shared part on the tensor cores
 * into the next basis slot, then the per-system update), 10 (one kernel: the shared part on
 * the tensor cores, subtracted from TMEM while the own basis streams; at most 32 own vectors)
 * and 11 (one kernel, every system of the batch per CTA with the rows of the shared part in
 * registers; at most 128 systems); complex128 projection 7 and update 6 (CUDA cores). */
void gdmrTuneForce(int projectionVariant, int updateVariant);

/* Structured-grid operator kernel (on by default).  A CSR matrix whose non-zeros all lie on the
 * 5- or 7-point offsets (-nx ny, -nx, -1, 0, +1, +nx, +nx ny) of a lexicographic nx x ny (x nz)
 * grid, none coupling two rows across the grid's edge, is also kept as coefficient planes, and
 * its products run on a kernel that walks the grid's planes with the x values in registers
 * instead of gathering them per row.  It adds the terms in the order the SELL-32 kernels do, so
 * a matrix with sorted, duplicate-free CSR rows gives the same values either way.  0 sends the
 * products launched after the call to the SELL-32 kernels (CUDA graphs already captured keep
 * the kernels they captured). */
void gdmrGridOperator(int enable);
/* Products over several systems at once (the batched solves) take the grid kernel only when
 * this is 1, 2 or 4 (systems a thread; the coefficients are loaded once for them); 0, the
 * default, keeps them on the SELL-32 kernel, which measured faster for the 64-system batch. */
void gdmrGridBatch(int systemsPerThread);

/* The cycle-end combinations (r -= [W V] t, x += rho [Z V] y) of batches of four or more
 * systems with a deflation segment run four systems a CTA, each element of the shared W and Z
 * loaded once for the four (on by default); 0 returns them to one system a CTA. */
void gdmrCombineGroup(int enable);

/* The refined solves' FP64 residual b - A x on its own stream, beside the next restart cycle's
 * deflation loop (which needs only the deflation space), from a system's third cycle on when the
 * cycle is not a CUDA graph: ctasPerSm (1-8) caps its grid so that the loop's kernels keep room
 * on the SMs; 0, the default, runs it before the loop.  The results are the same bit for bit
 * either way.  ctasPerSm < 0 only reads; returns the previous setting. */
int gdmrOverlapResidual(int ctasPerSm);

/* Host-only check of a CSR matrix (complex values interleaved re, im) for the structured-grid
 * form: dims[0..2] <- (nx, ny, nz), zeros if it has none.  GDMR_EINVAL for malformed arrays. */
int gdmr_csr_grid_form(int n, const int *rowPtr, const int *colIdx, const double *vals_ri, int *dims);

/* ---- context API: one resident operator, many right-hand sides -------------
 * A gdmr_system holds a CSR operator on the device (SELL-32, complex64 and
 * complex128 values), a solver engine of `capacity` systems and one recycled
 * deflation space shared by every right-hand side solved through it.
 * precision 0: plain FP64 inner iteration; 1: complex64 inner iteration;
 * 2: "fp64e", the FP64 iteration carried in double-float arithmetic (pairs of
 * FP32 values, about 48 significant bits) on the FP32 pipes, for GPUs whose
 * native FP64 rate caps the streaming kernels well below memory bandwidth;
 * the least squares, SVD and Hessenberg stay native FP64.  The batched form
 * checks convergence on the true FP64 residual b - A x. */
typedef struct gdmr_system gdmr_system;
int gdmr_system_create(gdmr_system **out, int n, const int *rowPtr, const int *colIdx, const double *vals_ri,
                       int basisDim, int deflatDim, int capacity, int precision, int device);
int gdmr_system_destroy(gdmr_system *sys);
/* Bytes of device memory the system holds. */
long long gdmr_system_bytes(const gdmr_system *sys);
/* Jacobi sweeps of the last deflation-space SVD: 1000 * (FP32 sweeps) + (FP64 sweeps). */
int gdmr_system_svd_sweeps(const gdmr_system *sys);
/* Matrix-free operator: a constant-coefficient stencil on an nx x ny x nz grid (nz = 1 for the
 * 5-point 2D form), unknowns numbered i + nx (j + ny l), Dirichlet boundary:
 *   y = d x + wx (x[i-1] + x[i+1]) + wy (x[j-1] + x[j+1]) + wz (x[l-1] + x[l+1]),
 * coef_ri = {d, wx, wy, wz} as interleaved complex128.  It replaces the inner operator of the
 * system (the FP64 true residual keeps the CSR operator) after an FP64 check that it reproduces
 * the CSR operator on a pseudo-random vector (GDMR_EINVAL if not, to 1e-12 relative).
 * gdmr_system_clear_stencil returns to the CSR operator. */
int gdmr_system_set_stencil(gdmr_system *sys, int nx, int ny, int nz, const double *coef_ri);
int gdmr_system_clear_stencil(gdmr_system *sys);
/* Restart cycles of small systems (n x batch <= 2^20) replay as CUDA graphs after the first
 * cycle (on by default); 0 launches every kernel eagerly. */
int gdmr_system_set_graphs(gdmr_system *sys, int on);
/* One system with a CSR operator, complex128 or fp64e, and n up to 32 x (CTAs the device holds
 * at once): the Krylov loop of a restart cycle runs as one cooperative kernel (on by default;
 * 0 launches its operator, projection, update and scaling kernels step by step). */
int gdmr_system_set_fused(gdmr_system *sys, int on);

/* The Hessenberg's identity tail after a Krylov breakdown.  1 (default): the reference's, from
 * column j of a breakdown at step j (eyeArrayDMR, gDMR.cu:2256-2289), which in a deflated cycle
 * overwrites the diagonal of valid columns, so the least squares and with it the recursive
 * residual go wrong while the solve reports convergence (the true FP64 residual in the stats
 * shows it).  0: the tail starts after the last valid column, kk + j. */
int gdmr_system_set_compat_eye(gdmr_system *sys, int on);
/* dims[0..2] <- the grid's edge lengths (nx, ny, nz) if the system's CSR operator has the
 * structured-grid form (gdmrGridOperator), zeros if not. */
int gdmr_system_grid(const gdmr_system *sys, int *dims);

/* Reference-semantics solve of one right-hand side (solverDMR's algorithm,
 * complex128, complex64 or double-float per the system's precision), then the true FP64
 * residual.  b, x: interleaved complex128, on the host (on_device = 0) or the
 * device (on_device = 1); x is the initial guess on entry. */
int gdmr_solve(gdmr_system *sys, int mode, const double *b, double *x, double tol, int matRank, int on_device,
               gdmr_stats *stats);

/* Batched FP64-refined solve of nrhs right-hand sides (right-hand side s at
 * offset s*n, interleaved complex128), all sharing the system's deflation
 * space.  Each restart cycle starts from the true FP64 residual; a system
 * leaves the batch when ||b - A x|| <= tol[s] ||b||.  nrhs may exceed the
 * capacity: the batch is refilled as systems converge.  stats: nrhs entries
 * or NULL. */
int gdmr_solve_batch(gdmr_system *sys, int nrhs, const double *b, double *x, const double *tol, int maxCycles,
                     int on_device, gdmr_stats *stats);

/* Many operators at once, in lockstep (no counterpart in the reference, which solves one
 * system per solverDMR call): the FP64-refined batched solve of nrhs[o] right-hand sides through
 * each of nops systems (all of one precision, on one device, with CSR operators), their restart
 * cycles in lockstep and, every cycle, the Krylov loops of all right-hand sides in flight, of
 * all operators, in one cooperative launch, with the converged ones left out of it.  b[o], x[o]:
 * host arrays of nrhs[o] x n_o interleaved complex128 (x the initial guess on entry); tol[o]
 * the relative tolerance of system o's right-hand sides; stats[o]: nrhs[o] entries or NULL.
 * The systems' own deflation spaces are used and updated as by gdmr_solve_batch.
 * GDMR_EINVAL if more right-hand sides are in flight than the launch can hold (the sum of the
 * capacities must stay within the CTAs resident at once, a few hundred on a GB300). */
int gdmr_multi_solve(int nops, gdmr_system *const *systems, const int *nrhs, const double *const *b, double *const *x,
                     const double *tol, int maxCycles, gdmr_stats *const *stats);
/* gdmr_multi_solve's tail: once every right-hand side has been admitted and at most this many
 * systems remain in flight (default 48), the remaining ones finish on each system's own batched
 * cycles (as gdmr_solve_batch), one host thread per system driving its own stream, instead of in
 * the lockstep launch; 0 keeps the lockstep to the end.  systems < 0 only reads.  Returns the
 * previous value. */
int gdmrMultiTail(int systems);

/* FP64 ||b_s - A x_s|| / ||b_s|| for nrhs pairs. */
int gdmr_true_residual(gdmr_system *sys, int nrhs, const double *b, const double *x, int on_device, double *relres);

/* Allocation-free residual check (no counterpart in the reference): the FP64
 * ||b_s - A x_s|| / ||b_s|| of nrhs <= 64 pairs, b, x and relres all caller-owned device
 * buffers (complex128 interleaved; relres nrhs doubles), enqueued on `stream` (a
 * cudaStream_t, NULL for the default stream) without synchronising.  For callers that
 * cannot call cudaMalloc: hosts whose own allocator owns the device-memory pool (a library
 * cudaMalloc would fail or fragment it) and latency-critical loops (a cudaMalloc can
 * synchronise the device).  It uses a 256 KB static device array as
 * reduction scratch instead of allocating; the first call on a device sets that up
 * (cudaGetSymbolAddress), so make it before any stream capture.  Calls share the array:
 * calls that overlap on the GPU race.  nrhs above 64 is rejected with GDMR_EINVAL. */
int gdmr_true_residual_noalloc(gdmr_system *sys, int nrhs, const double *b, const double *x, double *relres,
                               void *stream);

/* Deflation space in and out: deflatDim x n interleaved complex128 on the host.
 * Import makes the next solve start from it; drop forgets it. */
int gdmr_export_deflation(gdmr_system *sys, double *z);
int gdmr_import_deflation(gdmr_system *sys, const double *z);
int gdmr_drop_deflation(gdmr_system *sys);

/* Deflation spaces on disk, versioned (magic "GDMRDEFL", format 1, k, n, FNV-1a hash, then
 * k x n complex128 little endian): the reference's impSVDMR/expSVDMR only move them between
 * host and device.  write/read are host-only; read checks magic, version, sizes and hash.
 * save/load go through a system (export + write, read + import). */
int gdmr_deflation_write(const char *path, int n, int k, const double *z);
int gdmr_deflation_read(const char *path, int n, int k, double *z);
int gdmr_save_deflation(gdmr_system *sys, const char *path);
int gdmr_load_deflation(gdmr_system *sys, const char *path);

/* ---- serving: resident operators, HBM-budget admission, continuous batching ----
 * A server holds several resident operators.  Each has its matrix, its recycled
 * deflation space and an engine of `capacity` slots: device memory fixed at
 * registration and bounded by the server's budget (capacity 0: as many slots as
 * the remaining budget allows, at most 256).  After gdmr_server_start, one worker
 * per operator admits queued requests into free slots between restart cycles and
 * runs FP64-refined cycles for all requests in flight; operators run on separate
 * streams.  b and x are caller-owned host buffers (n interleaved complex128) that
 * must stay valid until the request completes. */
typedef struct gdmr_server gdmr_server;
int gdmr_server_create(gdmr_server **out, long long budgetBytes, int device);
/* A server over several devices, each with its own budget of budgetBytesPerDevice (a device
 * listed twice gets two budgets on one GPU).  Independent operators shard across them with no
 * collective, replacing the reference's split of one basis across devices with peer copies
 * (gDMR.cu:1478-1520, 871-872): gdmr_server_add_operator places each operator, with its
 * matrix, deflation space, engine, stream and queue, on the device that keeps the most budget
 * free after taking it (gdmr_place_operator). */
int gdmr_server_create_multi(gdmr_server **out, long long budgetBytesPerDevice, const int *devices, int ndevices);
/* Index into the server's device list of the device an operator was placed on (-1: none). */
int gdmr_server_operator_device(gdmr_server *srv, int opId);
/* Host-only placement rule of gdmr_server_add_operator: for devices with budget[d] and used[d]
 * bytes, the device that keeps the most budget free after taking fixedBytes plus capacity
 * slots of perSlotBytes (capacity <= 0: as many slots as fit, at most 256, on the device with
 * the most room).  Returns the device index and the capacity granted, or -1 if none fits. */
int gdmr_place_operator(int ndev, const long long *budget, const long long *used, long long fixedBytes,
                        long long perSlotBytes, int capacity, int *capacityOut);
int gdmr_server_add_operator(gdmr_server *srv, int n, const int *rowPtr, const int *colIdx, const double *vals_ri,
                             int basisDim, int deflatDim, int capacity, int precision, int *opId);
/* Device bytes one slot costs (basis, work vectors, FP64 slot vectors). */
long long gdmr_server_slot_bytes(int n, int basisDim, int precision);
int gdmr_server_operator_capacity(gdmr_server *srv, int opId);
long long gdmr_server_bytes(gdmr_server *srv);
int gdmr_server_start(gdmr_server *srv);
int gdmr_server_submit(gdmr_server *srv, int opId, const double *b, double *x, double tol, int maxCycles,
                       long long *ticket);
/* Blocks until the request is done (or timeout_s passes; <= 0 waits without limit). */
int gdmr_server_wait(gdmr_server *srv, long long ticket, double timeout_s, gdmr_stats *stats);
/* Up to max completed requests since the last poll; returns how many. */
int gdmr_server_poll(gdmr_server *srv, long long *tickets, gdmr_stats *stats, int max);
/* Drains the queues, stops the workers and frees everything. */
int gdmr_server_destroy(gdmr_server *srv);

#ifdef __cplusplus
}
#endif
#endif
