// C ABI of libgDMR (GB300 build): the reference's gDMR.h / gDMRC.h entry
// points, their complex128 twins, and the context API of gdmr_ext.h.
#include <cuComplex.h>
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>
#include <type_traits>
#include <vector>

#include "gdmr_engine.h"

#define GDMR_WITH_CUDA_TYPES 1
extern "C" {
#include "../../include/gDMR.h"
#include "../../include/gDMRC.h"
#include "../../include/gdmr_ext.h"
}

using namespace gdmr;

namespace {

std::mutex g_api_mu;     // the legacy entry points are process-global, as in the reference
gdmr_stats g_last_stats{0, 0, 0, 0.0, -1.0, GDMR_OK, 0, 0.0};
std::mutex g_hist_mu;
std::vector<CycleRecord> g_last_history;

void record_history(const std::vector<CycleRecord> &h) {
    std::lock_guard<std::mutex> lk(g_hist_mu);
    g_last_history = h;
}

void record(const SolveStats &s) {
    g_last_stats.cycles = s.cycles;
    g_last_stats.its = s.its;
    g_last_stats.matvecs = s.matvecs;
    g_last_stats.rel_res = s.rel_res;
    g_last_stats.true_rel_res = s.true_rel_res;
    g_last_stats.status = s.status;
    g_last_stats.breakdowns = s.breakdowns;
}

int fail(int status, const char *where, const char *what) {
    char buf[512];
    snprintf(buf, sizeof buf, "%s: %s", where, what);
    set_last_error(status, buf);
    fprintf(stderr, "%s\n", buf);
    return status;
}

// ---------------------------------------------------------------- legacy solver state
template <class R> struct LegacySolver {
    Engine<R> eng;
    void (*hook)(void) = nullptr;
    int device = 0;
};
LegacySolver<float> g_s32;
LegacySolver<double> g_s64;

template <class R>
void legacy_init(LegacySolver<R> &S, const char *name, int blocks, int tpb, int *devList, int numDevs, int elements,
                 int basisDim, int deflatDim, void (*linComp)(void)) {
    (void)blocks;
    (void)tpb;
    // the reference's validation (gDMR.cu:844-860): print and return with nothing allocated
    if (numDevs < 1 || !devList) { fail(GDMR_EINVAL, name, "at least one device is required"); return; }
    if ((basisDim + 1) % numDevs != 0) {
        fail(GDMR_EINVAL, name, "The dimension basisDim + 1 must be divisible by the number of requested devices.");
        return;
    }
    if (deflatDim % numDevs != 0) {
        fail(GDMR_EINVAL, name, "The deflation space dimension must be divisible by the number of requested devices.");
        return;
    }
    if (basisDim - deflatDim < 2) {
        fail(GDMR_EINVAL, name,
             "After removing the deflation space, the basis dimension is too small to perform Arnoldi iterations.");
        return;
    }
    if (!linComp) { fail(GDMR_EINVAL, name, "a linear operator hook is required"); return; }
    S.device = devList[0];
    if (S.eng.init(elements, basisDim, deflatDim, 1, S.device) != GDMR_OK) {
        fprintf(stderr, "%s: %s\n", name, last_error());
        return;
    }
    S.hook = linComp;
    S.eng.op.kind = Operator<R>::HOOK;
    S.eng.op.hook = linComp;
    set_last_error(GDMR_OK, "ok");
}

template <class R>
double legacy_solve(LegacySolver<R> &S, const char *name, int mode, typename CT<R>::t *src, typename CT<R>::t *img,
                    cudaStream_t st, int dev, double tol, int matRank, int *numIts) {
    if (!S.eng.ready()) {
        fail(GDMR_ENOTINIT, name, "solver not initialised");
        if (numIts) *numIts = matRank * matRank;
        return 1.0;
    }
    if (!src || !img) {
        fail(GDMR_EINVAL, name, "null source or image vector");
        return 1.0;
    }
    if (dev != S.device) fprintf(stderr, "%s: operator device %d differs from solver device %d; using %d\n", name, dev,
                                 S.device, S.device);
    cudaSetDevice(S.device);
    S.eng.stream = st;
    S.eng.op.ext = src;
    SolveStats stats;
    double r = S.eng.solve_reference(mode, img, src, tol, matRank, &stats);
    if (numIts) *numIts = stats.its;
    record(stats);
    record_history(S.eng.history());
    if (stats.status == GDMR_ENOCONV)
        fprintf(stderr, "%s Inverse Solve Error: failed to converge to a solution after %d iterations.\n", name,
                stats.cycles);
    else if (stats.status == GDMR_ERUNAWAY)
        fprintf(stderr, "%s Inverse Solve Error: Runaway!\n", name);
    else if (stats.status == GDMR_OK && stats.cycles == 0)
        fprintf(stdout, "Initial guess within solution tolerance.\n");
    return r;
}

template <class R> void legacy_imp_z(LegacySolver<R> &S, const void *host, const char *name) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    if (!S.eng.ready()) { fail(GDMR_ENOTINIT, name, "solver not initialised"); return; }
    cudaSetDevice(S.device);
    if (S.eng.import_deflation((const typename CT<R>::t *)host) != GDMR_OK) fprintf(stderr, "%s: %s\n", name, last_error());
}
template <class R> void legacy_exp_z(LegacySolver<R> &S, void *host, const char *name) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    if (!S.eng.ready()) { fail(GDMR_ENOTINIT, name, "solver not initialised"); return; }
    cudaSetDevice(S.device);
    if (S.eng.export_deflation((typename CT<R>::t *)host) != GDMR_OK) fprintf(stderr, "%s: %s\n", name, last_error());
}

// ---------------------------------------------------------------- plugin (testLS.cu's role)
template <class R> struct Plugin {
    using C = typename CT<R>::t;
    int n = 0, dev = 0;
    C *src = nullptr, *img = nullptr, *tmp = nullptr, *opt = nullptr;
    int *zero = nullptr;   // active list {0} of the one-system operator product, on this device
    DeviceSell csr;
    bool use_csr = false;
    cudaStream_t st = nullptr;
    bool ready = false;
};
Plugin<float> g_p32;
Plugin<double> g_p64;

template <class C> __global__ void k_identity(int n, C *A) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < (long)n * n; i += (long)gridDim.x * blockDim.x) {
        C v;
        v.x = (i / n == i % n) ? 1 : 0;
        v.y = 0;
        A[i] = v;
    }
}

template <class R> void plugin_apply(Plugin<R> &P) {
    if (!P.ready) { fail(GDMR_ENOTINIT, "linOptLS", "linear system not initialised"); return; }
    cudaSetDevice(P.dev);
    // y = A x into a separate buffer, then copy back: the reference's hook aliases input and output
    if (P.use_csr) {
        SellMatrix A = sizeof(R) == 4 ? P.csr.view32() : P.csr.view64();
        launch_spmm<R>(A, P.src, 0, P.tmp, 0, P.zero, 1, P.st);
    } else {
        launch_dense_gemv<R>(P.n, P.opt, P.src, P.tmp, P.st);
    }
    cudaMemcpyAsync(P.src, P.tmp, sizeof(typename Plugin<R>::C) * P.n, cudaMemcpyDeviceToDevice, P.st);
}

void linop32(void) { plugin_apply(g_p32); }
void linop64(void) { plugin_apply(g_p64); }

template <class R> void plugin_free(Plugin<R> &P) {
    if (P.src) cudaFree(P.src);
    if (P.img) cudaFree(P.img);
    if (P.tmp) cudaFree(P.tmp);
    if (P.opt) cudaFree(P.opt);
    if (P.zero) cudaFree(P.zero);
    sell_free(P.csr);
    if (P.st) cudaStreamDestroy(P.st);
    P = Plugin<R>();
}

template <class R>
bool plugin_init(Plugin<R> &P, const char *name, int devNumLO, int cells) {
    using C = typename Plugin<R>::C;
    plugin_free(P);
    if (cells <= 0) { fail(GDMR_EINVAL, name, "cells must be positive"); return false; }
    P.n = cells;
    P.dev = devNumLO;
    if (cudaSetDevice(devNumLO) != cudaSuccess) { fail(GDMR_ECUDA, name, "Failed to set device"); return false; }
    const size_t vb = sizeof(C) * (size_t)cells;
    if (cudaMalloc(&P.src, vb) != cudaSuccess || cudaMalloc(&P.img, vb) != cudaSuccess ||
        cudaMalloc(&P.tmp, vb) != cudaSuccess || cudaMalloc(&P.opt, vb * (size_t)cells) != cudaSuccess ||
        cudaMalloc(&P.zero, sizeof(int)) != cudaSuccess) {
        plugin_free(P);
        fail(GDMR_ENOMEM, name, "Failed to allocate device memory");
        return false;
    }
    cudaMemset(P.src, 0, vb);
    cudaMemset(P.img, 0, vb);
    cudaMemset(P.zero, 0, sizeof(int));
    if (cudaStreamCreate(&P.st) != cudaSuccess) { plugin_free(P); fail(GDMR_ECUDA, name, "stream"); return false; }
    k_identity<C><<<1024, 256, 0, P.st>>>(cells, P.opt);
    cudaStreamSynchronize(P.st);
    P.ready = true;
    return true;
}

template <class R> void copy_in(Plugin<R> &P, typename Plugin<R>::C *dst, const void *host, size_t count, const char *name) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    if (!P.ready) { fail(GDMR_ENOTINIT, name, "linear system not initialised"); return; }
    cudaSetDevice(P.dev);
    cudaStreamSynchronize(P.st);
    if (cudaMemcpy(dst, host, sizeof(typename Plugin<R>::C) * count, cudaMemcpyHostToDevice) != cudaSuccess)
        fail(GDMR_ECUDA, name, "Failed to copy memory from host to device");
}
template <class R> void copy_out(Plugin<R> &P, void *host, const typename Plugin<R>::C *src, size_t count, const char *name) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    if (!P.ready) { fail(GDMR_ENOTINIT, name, "linear system not initialised"); return; }
    cudaSetDevice(P.dev);
    cudaStreamSynchronize(P.st);
    if (cudaMemcpy(host, src, sizeof(typename Plugin<R>::C) * count, cudaMemcpyDeviceToHost) != cudaSuccess)
        fail(GDMR_ECUDA, name, "Failed to copy memory from device to host");
}

template <class R>
int plugin_csr(Plugin<R> &P, int nnz, const int *rowPtr, const int *colIdx, const R *vals_ri, const char *name) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    if (!P.ready) return fail(GDMR_ENOTINIT, name, "linear system not initialised");
    if (!rowPtr || !colIdx || !vals_ri || nnz < 0 || rowPtr[P.n] - rowPtr[0] != nnz)
        return fail(GDMR_EINVAL, name, "CSR arrays inconsistent with nnz");
    cudaSetDevice(P.dev);
    std::vector<double> v((size_t)2 * nnz);
    for (size_t i = 0; i < v.size(); ++i) v[i] = (double)vals_ri[i];
    int rc = sell_from_csr(P.csr, P.n, rowPtr, colIdx, v.data(), sizeof(R) == 4, sizeof(R) == 8, P.st);
    if (rc != GDMR_OK) return rc;
    P.use_csr = true;
    return GDMR_OK;
}

}  // namespace

// ================================================================ gDMR.h
extern "C" void initDMR(int blocks, int threadsPerBlock, int *devList, int numDevs, int elements, int basisDim,
                        int deflatDim, void (*linComp)(void)) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    legacy_init(g_s32, "initDMR", blocks, threadsPerBlock, devList, numDevs, elements, basisDim, deflatDim, linComp);
}

extern "C" void freeDMR(void) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    g_s32.eng.release();
    g_s32.hook = nullptr;
}

extern "C" float solverDMR(int mode, cuComplex *extSrcVec, cuComplex *extImgVec, cudaStream_t extStream,
                           int extDevNum, float solTol, int matRank, int *numIts) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    return (float)legacy_solve(g_s32, "solverDMR", mode, (float2 *)extSrcVec, (float2 *)extImgVec, extStream,
                               extDevNum, (double)solTol, matRank, numIts);
}

extern "C" void impSVDMR(float _Complex *cMem) { legacy_imp_z(g_s32, cMem, "impSVDMR"); }
extern "C" void expSVDMR(float _Complex *cMem) { legacy_exp_z(g_s32, cMem, "expSVDMR"); }

// ================================================================ complex128 drop-in
extern "C" void initDMR_z(int blocks, int threadsPerBlock, int *devList, int numDevs, int elements, int basisDim,
                          int deflatDim, void (*linComp)(void)) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    legacy_init(g_s64, "initDMR_z", blocks, threadsPerBlock, devList, numDevs, elements, basisDim, deflatDim, linComp);
}
extern "C" void freeDMR_z(void) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    g_s64.eng.release();
    g_s64.hook = nullptr;
}
extern "C" double solverDMR_z(int mode, cuDoubleComplex *extSrcVec, cuDoubleComplex *extImgVec, cudaStream_t extStream,
                              int extDevNum, double solTol, int matRank, int *numIts) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    return legacy_solve(g_s64, "solverDMR_z", mode, (double2 *)extSrcVec, (double2 *)extImgVec, extStream, extDevNum,
                        solTol, matRank, numIts);
}
extern "C" void impSVDMR_z(double _Complex *cMem) { legacy_imp_z(g_s64, cMem, "impSVDMR_z"); }
extern "C" void expSVDMR_z(double _Complex *cMem) { legacy_exp_z(g_s64, cMem, "expSVDMR_z"); }

// ================================================================ gDMRC.h plugin (complex64)
extern "C" void initLS(int blocksMDR, int threadsPerBlockMDR, int devNumLO, int cells, int *devListMDR, int numDevsMDR,
                       int basisSizeMDR, int deflatSizeMDR) {
    {
        std::lock_guard<std::mutex> lk(g_api_mu);
        if (!plugin_init(g_p32, "initLS", devNumLO, cells)) return;
    }
    initDMR(blocksMDR, threadsPerBlockMDR, devListMDR, numDevsMDR, cells, basisSizeMDR, deflatSizeMDR, linop32);
}
extern "C" void freeLS(void) {
    {
        std::lock_guard<std::mutex> lk(g_api_mu);
        plugin_free(g_p32);
    }
    freeDMR();
}
extern "C" void impImgLS(float _Complex *c) { copy_in(g_p32, g_p32.img, c, g_p32.n, "impImgLS"); }
extern "C" void expImgLS(float _Complex *c) { copy_out(g_p32, c, g_p32.img, g_p32.n, "expImgLS"); }
extern "C" void impSrcLS(float _Complex *c) { copy_in(g_p32, g_p32.src, c, g_p32.n, "impSrcLS"); }
extern "C" void expSrcLS(float _Complex *c) { copy_out(g_p32, c, g_p32.src, g_p32.n, "expSrcLS"); }
extern "C" void impOptLS(float _Complex *c) {
    copy_in(g_p32, g_p32.opt, c, (size_t)g_p32.n * g_p32.n, "impOptLS");
    g_p32.use_csr = false;
}
extern "C" void expOptLS(float _Complex *c) { copy_out(g_p32, c, g_p32.opt, (size_t)g_p32.n * g_p32.n, "expOptLS"); }
extern "C" float solveLS(int mode, float solTol, int matRank, int *numIts) {
    if (!g_p32.ready) {
        fail(GDMR_ENOTINIT, "solveLS", "linear system not initialised");
        return 1.0f;
    }
    return solverDMR(mode, (cuComplex *)g_p32.src, (cuComplex *)g_p32.img, g_p32.st, g_p32.dev, solTol, matRank,
                     numIts);
}
extern "C" void linOptLS(void) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    plugin_apply(g_p32);
    cudaStreamSynchronize(g_p32.st);
}
extern "C" int impCsrLS(int nnz, const int *rowPtr, const int *colIdx, const float _Complex *vals) {
    return plugin_csr(g_p32, nnz, rowPtr, colIdx, (const float *)vals, "impCsrLS");
}

// ================================================================ complex128 plugin
extern "C" void initLS_z(int blocksMDR, int threadsPerBlockMDR, int devNumLO, int cells, int *devListMDR,
                         int numDevsMDR, int basisSizeMDR, int deflatSizeMDR) {
    {
        std::lock_guard<std::mutex> lk(g_api_mu);
        if (!plugin_init(g_p64, "initLS_z", devNumLO, cells)) return;
    }
    initDMR_z(blocksMDR, threadsPerBlockMDR, devListMDR, numDevsMDR, cells, basisSizeMDR, deflatSizeMDR, linop64);
}
extern "C" void freeLS_z(void) {
    {
        std::lock_guard<std::mutex> lk(g_api_mu);
        plugin_free(g_p64);
    }
    freeDMR_z();
}
extern "C" void impImgLS_z(double _Complex *c) { copy_in(g_p64, g_p64.img, c, g_p64.n, "impImgLS_z"); }
extern "C" void expImgLS_z(double _Complex *c) { copy_out(g_p64, c, g_p64.img, g_p64.n, "expImgLS_z"); }
extern "C" void impSrcLS_z(double _Complex *c) { copy_in(g_p64, g_p64.src, c, g_p64.n, "impSrcLS_z"); }
extern "C" void expSrcLS_z(double _Complex *c) { copy_out(g_p64, c, g_p64.src, g_p64.n, "expSrcLS_z"); }
extern "C" void impOptLS_z(double _Complex *c) {
    copy_in(g_p64, g_p64.opt, c, (size_t)g_p64.n * g_p64.n, "impOptLS_z");
    g_p64.use_csr = false;
}
extern "C" int impCsrLS_z(int nnz, const int *rowPtr, const int *colIdx, const double _Complex *vals) {
    return plugin_csr(g_p64, nnz, rowPtr, colIdx, (const double *)vals, "impCsrLS_z");
}
extern "C" double solveLS_z(int mode, double solTol, int matRank, int *numIts) {
    if (!g_p64.ready) {
        fail(GDMR_ENOTINIT, "solveLS_z", "linear system not initialised");
        return 1.0;
    }
    return solverDMR_z(mode, (cuDoubleComplex *)g_p64.src, (cuDoubleComplex *)g_p64.img, g_p64.st, g_p64.dev, solTol,
                       matRank, numIts);
}
extern "C" void linOptLS_z(void) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    plugin_apply(g_p64);
    cudaStreamSynchronize(g_p64.st);
}

// ================================================================ status
extern "C" int gdmrLastStatus(void) { return last_status(); }
extern "C" const char *gdmrLastError(void) { return last_error(); }
extern "C" const char *gdmrVersion(void) { return "1.0.1-gb300"; }
extern "C" void gdmrLastStats(gdmr_stats *out) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    if (out) *out = g_last_stats;
}

// ================================================================ instrumentation
extern "C" int gdmrLastHistory(gdmr_cycle *out, int max) {
    std::lock_guard<std::mutex> lk(g_hist_mu);
    const int cnt = (int)g_last_history.size();
    for (int i = 0; out && i < cnt && i < max; ++i) {
        const CycleRecord &c = g_last_history[i];
        out[i].rho = c.rho;
        out[i].rel_res = c.rel_res;
        out[i].kk = c.kk;
        out[i].restart = c.restart;
        out[i].breakdown = c.breakdown;
        out[i].stagnated = c.stagnated;
    }
    return cnt;
}

extern "C" long long gdmrKernelLaunches(void) { return launch_count(); }
extern "C" unsigned gdmrAsyncTimeouts(void) { return wproj_tc_timeouts() + bulk_timeouts(); }
extern "C" double gdmrWaitLimit(double ms) {
    const double prev = wait_limit_ms();
    if (ms >= 0) set_wait_limit_ms(ms);
    return prev;
}
extern "C" void gdmrInjectAllocFailure(int nth) { inject_alloc_failure(nth); }
extern "C" void gdmrCombineGroup(int enable) { set_combine_group(enable); }
extern "C" int gdmrOverlapResidual(int ctasPerSm) { return set_overlap_residual(ctasPerSm); }
// Systems in flight at or below which gdmr_multi_solve finishes on the engines' own cycles.
static std::atomic<int> g_multi_tail{48};
extern "C" int gdmrMultiTail(int systems) {
    const int prev = g_multi_tail.load();
    if (systems >= 0) g_multi_tail.store(systems);
    return prev;
}
extern "C" void gdmrProfile(int on) { profile_enable(on != 0); }
extern "C" void gdmrProfileReset(void) { profile_reset(); }
extern "C" void gdmrTune(int on) { tune_enable(on != 0); }
extern "C" void gdmrTuneForce(int projectionVariant, int updateVariant) {
    tune_force(projectionVariant, updateVariant);
}
extern "C" void gdmrGridOperator(int enable) { set_grid_operator(enable); }
extern "C" void gdmrGridBatch(int systemsPerThread) { set_grid_batch(systemsPerThread); }
extern "C" const char *gdmrTuneReport(void) {
    static thread_local std::string rep;
    rep = tune_report();
    return rep.c_str();
}
extern "C" int gdmrProfileRead(int kernelClass, double *bytes, double *ms, long long *launches) {
    if (kernelClass < 0 || kernelClass >= KC_COUNT) return fail(GDMR_EINVAL, "gdmrProfileRead", "no such kernel class");
    profile_flush();
    profile_read(kernelClass, bytes, ms, launches);
    return GDMR_OK;
}

// The deflation update's SVD on its own (svDecompHessDMR, gDMR.cu:638): host buffers in and
// out, device scratch for the call, the current device and the null stream.
extern "C" int gdmr_hessenberg_svd(int m, int k, const double *H_ri, double *sigma, double *vs_ri, int *sweeps) {
    const char *W = "gdmr_hessenberg_svd";
    if (m < 1 || m > 160 || k < 1 || k > m) return fail(GDMR_EINVAL, W, "need 1 <= k <= m <= 160");
    if (!H_ri || !sigma || !vs_ri) return fail(GDMR_EINVAL, W, "null buffer");
    const size_t hb = sizeof(double2) * (size_t)(m + 1) * m, vb = sizeof(double2) * (size_t)k * m;
    double2 *Hd = nullptr, *vsd = nullptr, *work = nullptr;
    double *sd = nullptr;
    int *ints = nullptr;                    // [0] = lead system (0), [1] = sweeps
    auto release = [&]() {
        cudaFree(Hd);
        cudaFree(vsd);
        cudaFree(work);
        cudaFree(sd);
        cudaFree(ints);
    };
    if (cudaMalloc(&Hd, hb) != cudaSuccess || cudaMalloc(&vsd, vb) != cudaSuccess ||
        cudaMalloc(&work, svd_smem_bytes(m)) != cudaSuccess || cudaMalloc(&sd, sizeof(double) * m) != cudaSuccess ||
        cudaMalloc(&ints, 2 * sizeof(int)) != cudaSuccess) {
        release();
        return fail(GDMR_ENOMEM, W, "device allocation failed");
    }
    cudaError_t e = cudaMemcpy(Hd, H_ri, hb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(ints, 0, 2 * sizeof(int));
    if (e == cudaSuccess) {
        launch_svd_smallest(m, k, Hd, 0, ints, vsd, sd, work, ints + 1, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(sigma, sd, sizeof(double) * m, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(vs_ri, vsd, vb, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && sweeps) e = cudaMemcpy(sweeps, ints + 1, sizeof(int), cudaMemcpyDeviceToHost);
    release();
    if (e != cudaSuccess) return fail(GDMR_ECUDA, W, cudaGetErrorString(e));
    return GDMR_OK;
}

// ================================================================ shared-basis kernels on their own
// The tensor-core kernels of a batched cycle's shared deflation segment (the deflator of the
// reference, gDMR.cu:1710-1787, for a batch of systems that share W): the split-K projection
// coef_s = W^H y_s (k_wproj_tc) and the apply P_s = W c_s (k_wapply_tc), run once on the
// caller's host data so that a test can check them against a host product.
extern "C" int gdmr_shared_basis_check(int n, int k, int nsys, const float *W_ri, const float *Y_ri,
                                       const double *c_ri, double *coef_ri, float *P_ri) {
    const char *F = "gdmr_shared_basis_check";
    if (n < 2 || n % 2 != 0 || k < 1 || k > 32 || nsys < 8 || nsys > 64)
        return fail(GDMR_EINVAL, F, "need an even n >= 2, 1 <= k <= 32 and 8 <= nsys <= 64");
    if (!W_ri || !Y_ri || !c_ri || !coef_ri || !P_ri) return fail(GDMR_EINVAL, F, "null buffer");
    const size_t ldc = (size_t)k + 1;   // the apply writes a unit coefficient at index k
    float2 *Wd = nullptr, *Yd = nullptr, *Pd = nullptr;
    double2 *coef = nullptr, *capp = nullptr;
    double *part = nullptr;
    int *act = nullptr;
    auto release = [&]() {
        cudaFree(Wd);
        cudaFree(Yd);
        cudaFree(Pd);
        cudaFree(coef);
        cudaFree(capp);
        cudaFree(part);
        cudaFree(act);
    };
    const size_t wb = sizeof(float2) * (size_t)k * n, yb = sizeof(float2) * (size_t)nsys * n;
    const size_t pb = sizeof(double) * (size_t)wproj_tc_grid(n) * k * nsys * 2;
    if (cudaMalloc(&Wd, wb) != cudaSuccess || cudaMalloc(&Yd, yb) != cudaSuccess || cudaMalloc(&Pd, yb) != cudaSuccess ||
        cudaMalloc(&coef, sizeof(double2) * ldc * nsys) != cudaSuccess ||
        cudaMalloc(&capp, sizeof(double2) * ldc * nsys) != cudaSuccess || cudaMalloc(&part, pb) != cudaSuccess ||
        cudaMalloc(&act, sizeof(int) * nsys) != cudaSuccess) {
        release();
        return fail(GDMR_ENOMEM, F, "device allocation failed");
    }
    std::vector<int> ident(nsys);
    for (int i = 0; i < nsys; ++i) ident[i] = i;
    if (!wproj_tc_ok(n, k, nsys, Wd, Yd, (size_t)n) || !wapply_tc_ok(n, k, nsys)) {
        release();
        return fail(GDMR_EINVAL, F, "the tensor-core kernels do not apply to these sizes");
    }
    const unsigned t0 = wproj_tc_timeouts();
    cudaError_t e = cudaMemcpy(Wd, W_ri, wb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(Yd, Y_ri, yb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(act, ident.data(), sizeof(int) * nsys, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy2D(capp, sizeof(double2) * ldc, c_ri, sizeof(double2) * k, sizeof(double2) * k, nsys,
                         cudaMemcpyHostToDevice);
    if (e == cudaSuccess && push_wait_limit() != 0) e = cudaErrorUnknown;
    if (e == cudaSuccess) {
        launch_wproj_tc(n, k, Wd, Yd, (size_t)n, act, nsys, part, coef, ldc, 0);
        launch_wapply_tc(n, k, Wd, capp, ldc, act, nsys, Pd, (size_t)n, k, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = cudaMemcpy2D(coef_ri, sizeof(double2) * k, coef, sizeof(double2) * ldc, sizeof(double2) * k, nsys,
                         cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(P_ri, Pd, yb, cudaMemcpyDeviceToHost);
    release();
    if (e != cudaSuccess) return fail(GDMR_ECUDA, F, cudaGetErrorString(e));
    if (wproj_tc_timeouts() != t0) return fail(GDMR_ETIMEOUT, F, "a pipeline wait ran out");
    return GDMR_OK;
}

// ================================================================ context API
// complex128 <-> complex64 helpers used by the context API
namespace {
__global__ void k_demote(int n, const double2 *a, float2 *b) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        b[i] = make_float2((float)a[i].x, (float)a[i].y);
}
__global__ void k_promote(int n, const float2 *a, double2 *b) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        b[i] = make_double2(a[i].x, a[i].y);
}
__global__ void k_to_dfc(int n, const double2 *a, dfc *b) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        dfc c;
        c.x = dfr(a[i].x);
        c.y = dfr(a[i].y);
        b[i] = c;
    }
}
__global__ void k_from_dfc(int n, const dfc *a, double2 *b) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        b[i] = make_double2((double)a[i].x, (double)a[i].y);
}
}  // namespace
static void gdmr_demote_vec(int n, const double2 *a, float2 *b, cudaStream_t st) {
    k_demote<<<std::min((n + 255) / 256, 4096), 256, 0, st>>>(n, a, b);
}
static void gdmr_promote_vec(int n, const float2 *a, double2 *b, cudaStream_t st) {
    k_promote<<<std::min((n + 255) / 256, 4096), 256, 0, st>>>(n, a, b);
}
static void gdmr_to_dfc_vec(int n, const double2 *a, dfc *b, cudaStream_t st) {
    k_to_dfc<<<std::min((n + 255) / 256, 4096), 256, 0, st>>>(n, a, b);
}
static void gdmr_from_dfc_vec(int n, const dfc *a, double2 *b, cudaStream_t st) {
    k_from_dfc<<<std::min((n + 255) / 256, 4096), 256, 0, st>>>(n, a, b);
}

struct gdmr_system {
    int n = 0, m = 0, k = 0, cap = 0, precision = 0, device = 0;
    DeviceSell A;
    Engine<float> e32;
    Engine<double> e64;
    Engine<dfr> edf;   // precision 2: FP64-class double-float on the FP32 pipes
    cudaStream_t st = nullptr;
    double2 *db = nullptr, *dx = nullptr;   // staging for host-buffer calls (cap vectors each)
    std::mutex mu;
    // frees everything, also when creation failed part of the way
    ~gdmr_system() {
        cudaSetDevice(device);
        if (st) cudaStreamSynchronize(st);
        e32.release();
        e64.release();
        edf.release();
        sell_free(A);
        if (db) cudaFree(db);
        if (dx) cudaFree(dx);
        if (st) cudaStreamDestroy(st);
    }
};

namespace {
template <class R> Engine<R> &eng_of(gdmr_system *s);
template <> Engine<float> &eng_of<float>(gdmr_system *s) { return s->e32; }
template <> Engine<double> &eng_of<double>(gdmr_system *s) { return s->e64; }
template <> Engine<dfr> &eng_of<dfr>(gdmr_system *s) { return s->edf; }

void to_stats(const SolveStats &s, gdmr_stats *o) {
    o->cycles = s.cycles;
    o->its = s.its;
    o->matvecs = s.matvecs;
    o->rel_res = s.rel_res;
    o->true_rel_res = s.true_rel_res;
    o->status = s.status;
    o->breakdowns = s.breakdowns;
    o->latency_ms = s.latency_ms;
}

template <class R>
int batch_impl(gdmr_system *S, int nrhs, const double *b, double *x, const double *tol, int maxCycles, int on_device,
               gdmr_stats *stats) {
    Engine<R> &E = eng_of<R>(S);
    const size_t vb = sizeof(double2) * (size_t)S->n;
    int rc = E.refine_setup(S->A.view64());
    if (rc != GDMR_OK) return rc;
    std::vector<int> slot_of(E.capacity(), -1);
    int next = 0, finished = 0, worst = GDMR_OK;
    const auto t0 = std::chrono::steady_clock::now();
    while (finished < nrhs) {
        for (int s = 0; s < E.capacity() && next < nrhs; ++s) {
            if (slot_of[s] >= 0) continue;
            const double2 *bsrc, *xsrc;
            if (on_device) {
                bsrc = (const double2 *)b + (size_t)next * S->n;
                xsrc = (const double2 *)x + (size_t)next * S->n;
            } else {
                if (cudaMemcpyAsync(S->db + (size_t)s * S->n, b + (size_t)2 * next * S->n, vb, cudaMemcpyHostToDevice,
                                    S->st) != cudaSuccess ||
                    cudaMemcpyAsync(S->dx + (size_t)s * S->n, x + (size_t)2 * next * S->n, vb, cudaMemcpyHostToDevice,
                                    S->st) != cudaSuccess)
                    return fail(GDMR_ECUDA, "gdmr_solve_batch", "host to device copy failed");
                bsrc = S->db + (size_t)s * S->n;
                xsrc = S->dx + (size_t)s * S->n;
            }
            if ((rc = E.refine_admit(s, bsrc, xsrc, tol ? tol[next] : 1e-10, maxCycles)) != GDMR_OK) return rc;
            slot_of[s] = next++;
        }
        std::vector<int> done;
        if ((rc = E.refine_cycle(&done)) != GDMR_OK) return rc;
        for (int s : done) {
            const int r = slot_of[s];
            if (on_device)
                cudaMemcpyAsync((double2 *)x + (size_t)r * S->n, E.slot_x(s), vb, cudaMemcpyDeviceToDevice, S->st);
            else
                cudaMemcpyAsync(x + (size_t)2 * r * S->n, E.slot_x(s), vb, cudaMemcpyDeviceToHost, S->st);
            if (stats) {
                to_stats(E.slot_stats(s), &stats[r]);
                stats[r].latency_ms =
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            }
            worst = std::max(worst, E.slot_stats(s).status);
            slot_of[s] = -1;
            ++finished;
        }
    }
    if (cudaStreamSynchronize(S->st) != cudaSuccess) return fail(GDMR_ECUDA, "gdmr_solve_batch", "synchronise");
    if (worst != GDMR_OK)
        set_last_error(worst, worst == GDMR_ETIMEOUT
                                  ? "gdmr_solve_batch: a bounded device wait ran out (gdmrWaitLimit); see the stats"
                                  : "gdmr_solve_batch: some right-hand sides did not converge; see the stats");
    else set_last_error(GDMR_OK, "ok");
    return worst;
}

template <class R>
int single_impl(gdmr_system *S, int mode, const double *b, double *x, double tol, int matRank, int on_device,
                gdmr_stats *stats) {
    using C = typename CT<R>::t;
    Engine<R> &E = eng_of<R>(S);
    const int n = S->n;
    const size_t vb = sizeof(double2) * (size_t)n;
    double2 *db = S->db, *dx = S->dx;
    if (on_device) {
        cudaMemcpyAsync(db, b, vb, cudaMemcpyDeviceToDevice, S->st);
        cudaMemcpyAsync(dx, x, vb, cudaMemcpyDeviceToDevice, S->st);
    } else {
        cudaMemcpyAsync(db, b, vb, cudaMemcpyHostToDevice, S->st);
        cudaMemcpyAsync(dx, x, vb, cudaMemcpyHostToDevice, S->st);
    }
    C *bR, *xR;
    if constexpr (std::is_same<R, double>::value) {
        bR = (C *)db;
        xR = (C *)dx;
    } else {
        // complex64 / double-float working copies live in the staging area's second half
        bR = (C *)(db + (size_t)n);
        xR = (C *)(dx + (size_t)n);
        if constexpr (std::is_same<R, float>::value) {
            gdmr_demote_vec(n, db, (float2 *)bR, S->st);
            gdmr_demote_vec(n, dx, (float2 *)xR, S->st);
        } else {
            gdmr_to_dfc_vec(n, db, (dfc *)bR, S->st);
            gdmr_to_dfc_vec(n, dx, (dfc *)xR, S->st);
        }
    }
    SolveStats st;
    E.solve_reference(mode, bR, xR, tol, matRank, &st);
    if constexpr (std::is_same<R, float>::value) gdmr_promote_vec(n, (const float2 *)xR, dx, S->st);
    if constexpr (std::is_same<R, dfr>::value) gdmr_from_dfc_vec(n, (const dfc *)xR, dx, S->st);
    // true FP64 residual
    double rel = -1;
    if (E.refine_setup(S->A.view64()) == GDMR_OK) E.true_residual(1, db, dx, &rel);
    st.true_rel_res = rel;
    if (on_device) cudaMemcpyAsync(x, dx, vb, cudaMemcpyDeviceToDevice, S->st);
    else cudaMemcpyAsync(x, dx, vb, cudaMemcpyDeviceToHost, S->st);
    cudaStreamSynchronize(S->st);
    if (stats) to_stats(st, stats);
    record(st);
    record_history(E.history());
    return st.status;
}

}  // namespace

extern "C" int gdmr_system_create(gdmr_system **out, int n, const int *rowPtr, const int *colIdx, const double *vals_ri,
                                  int basisDim, int deflatDim, int capacity, int precision, int device) {
    if (!out) return fail(GDMR_EINVAL, "gdmr_system_create", "null output pointer");
    *out = nullptr;
    if (precision < 0 || precision > 2) return fail(GDMR_EINVAL, "gdmr_system_create", "precision must be 0, 1 or 2");
    if (capacity < 1) return fail(GDMR_EINVAL, "gdmr_system_create", "capacity must be >= 1");
    if (cudaSetDevice(device) != cudaSuccess) return fail(GDMR_ECUDA, "gdmr_system_create", "cudaSetDevice");
    std::unique_ptr<gdmr_system> S(new gdmr_system());
    S->n = n; S->m = basisDim; S->k = deflatDim; S->cap = capacity; S->precision = precision; S->device = device;
    if (cudaStreamCreateWithFlags(&S->st, cudaStreamNonBlocking) != cudaSuccess)
        return fail(GDMR_ECUDA, "gdmr_system_create", "stream");
    int rc = sell_from_csr(S->A, n, rowPtr, colIdx, vals_ri, precision == 1, true, S->st, precision == 2);
    if (rc != GDMR_OK) return rc;
    if (precision == 1) {
        rc = S->e32.init(n, basisDim, deflatDim, capacity, device);
        S->e32.op.kind = Operator<float>::SELL;
        S->e32.op.sell = S->A.view32();
        S->e32.stream = S->st;
    } else if (precision == 2) {
        rc = S->edf.init(n, basisDim, deflatDim, capacity, device);
        S->edf.op.kind = Operator<dfr>::SELL;
        S->edf.op.sell = S->A.viewdf();
        S->edf.stream = S->st;
    } else {
        rc = S->e64.init(n, basisDim, deflatDim, capacity, device);
        S->e64.op.kind = Operator<double>::SELL;
        S->e64.op.sell = S->A.view64();
        S->e64.stream = S->st;
    }
    if (rc != GDMR_OK) return rc;
    const size_t stage = sizeof(double2) * (size_t)n * std::max(capacity, 2);
    if (cudaMalloc(&S->db, stage) != cudaSuccess || cudaMalloc(&S->dx, stage) != cudaSuccess)
        return fail(GDMR_ENOMEM, "gdmr_system_create", "staging buffers");
    *out = S.release();
    set_last_error(GDMR_OK, "ok");
    return GDMR_OK;
}

extern "C" int gdmr_system_destroy(gdmr_system *S) {
    delete S;   // the destructor frees the engines, the matrix, the staging buffers and the stream
    return GDMR_OK;
}

extern "C" long long gdmr_system_bytes(const gdmr_system *S) {
    if (!S) return 0;
    return (long long)(S->A.bytes() + S->e32.device_bytes() + S->e64.device_bytes() + S->edf.device_bytes() +
                       2 * sizeof(double2) * (size_t)S->n * std::max(S->cap, 2));
}

// Switches the inner operator of the system's engine to the matrix-free stencil after checking,
// in FP64, that it reproduces the system's CSR operator on a fixed pseudo-random vector.  The
// FP64 true residual keeps using the CSR operator.
extern "C" int gdmr_system_set_stencil(gdmr_system *S, int nx, int ny, int nz, const double *coef_ri) {
    if (!S || !coef_ri) return fail(GDMR_EINVAL, "gdmr_system_set_stencil", "null argument");
    if (nx < 1 || ny < 1 || nz < 1 || (long)nx * ny * nz != (long)S->n)
        return fail(GDMR_EINVAL, "gdmr_system_set_stencil", "nx * ny * nz must equal the system size");
    std::lock_guard<std::mutex> lk(S->mu);
    cudaSetDevice(S->device);
    Stencil7 st{nx, ny, nz, make_double2(coef_ri[0], coef_ri[1]), make_double2(coef_ri[2], coef_ri[3]),
                make_double2(coef_ri[4], coef_ri[5]), make_double2(coef_ri[6], coef_ri[7])};
    const int n = S->n;
    std::vector<double2> hx(n), h1(n), h2(n);
    uint64_t z = 0x2545F4914F6CDD1DULL;
    for (int i = 0; i < n; ++i) {   // xorshift64*: values in [-1, 1)
        z ^= z >> 12; z ^= z << 25; z ^= z >> 27;
        const uint64_t r = z * 0x2545F4914F6CDD1DULL;
        hx[i] = make_double2((double)(r >> 11) * 0x1.0p-52 - 1.0, (double)((r >> 11) ^ 0x5555555555555ULL) * 0x1.0p-52 - 1.0);
    }
    int *dact = nullptr;
    const int zero = 0;
    double2 *x = S->db, *y1 = S->dx, *y2 = S->dx + (size_t)n;
    if (cudaMalloc(&dact, sizeof(int)) != cudaSuccess) return fail(GDMR_ENOMEM, "gdmr_system_set_stencil", "scratch");
    cudaMemcpyAsync(dact, &zero, sizeof(int), cudaMemcpyHostToDevice, S->st);
    cudaMemcpyAsync(x, hx.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, S->st);
    launch_spmm<double>(S->A.view64(), x, 0, y1, 0, dact, 1, S->st);
    launch_stencil<double>(st, x, 0, y2, 0, dact, 1, S->st);
    cudaMemcpyAsync(h1.data(), y1, sizeof(double2) * n, cudaMemcpyDeviceToHost, S->st);
    cudaMemcpyAsync(h2.data(), y2, sizeof(double2) * n, cudaMemcpyDeviceToHost, S->st);
    const cudaError_t e = cudaStreamSynchronize(S->st);
    cudaFree(dact);
    if (e != cudaSuccess) return fail(GDMR_ECUDA, "gdmr_system_set_stencil", cudaGetErrorString(e));
    double err = 0, mag = 0;
    for (int i = 0; i < n; ++i) {
        err = std::max(err, std::hypot(h1[i].x - h2[i].x, h1[i].y - h2[i].y));
        mag = std::max(mag, std::hypot(h1[i].x, h1[i].y));
    }
    if (!(err <= 1e-12 * mag))
        return fail(GDMR_EINVAL, "gdmr_system_set_stencil", "the stencil does not reproduce the system's operator");
    if (S->precision == 1) {
        S->e32.op.kind = Operator<float>::STENCIL;
        S->e32.op.stencil = st;
    } else if (S->precision == 2) {
        S->edf.op.kind = Operator<dfr>::STENCIL;
        S->edf.op.stencil = st;
    } else {
        S->e64.op.kind = Operator<double>::STENCIL;
        S->e64.op.stencil = st;
    }
    set_last_error(GDMR_OK, "ok");
    return GDMR_OK;
}

extern "C" int gdmr_system_clear_stencil(gdmr_system *S) {
    if (!S) return fail(GDMR_EINVAL, "gdmr_system_clear_stencil", "null system");
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->precision == 1) S->e32.op.kind = Operator<float>::SELL;
    else if (S->precision == 2) S->edf.op.kind = Operator<dfr>::SELL;
    else S->e64.op.kind = Operator<double>::SELL;
    return GDMR_OK;
}

extern "C" int gdmr_system_set_graphs(gdmr_system *S, int on) {
    if (!S) return fail(GDMR_EINVAL, "gdmr_system_set_graphs", "null system");
    std::lock_guard<std::mutex> lk(S->mu);
    S->e32.use_graphs = on != 0;
    S->e64.use_graphs = on != 0;
    S->edf.use_graphs = on != 0;
    return GDMR_OK;
}

extern "C" int gdmr_system_set_fused(gdmr_system *S, int on) {
    if (!S) return fail(GDMR_EINVAL, "gdmr_system_set_fused", "null system");
    std::lock_guard<std::mutex> lk(S->mu);
    S->e32.fused_small = on != 0;
    S->e64.fused_small = on != 0;
    S->edf.fused_small = on != 0;
    return GDMR_OK;
}

extern "C" int gdmr_system_set_compat_eye(gdmr_system *S, int on) {
    if (!S) return fail(GDMR_EINVAL, "gdmr_system_set_compat_eye", "null system");
    std::lock_guard<std::mutex> lk(S->mu);
    cudaSetDevice(S->device);
    S->e32.set_compat_eye(on != 0);
    S->e64.set_compat_eye(on != 0);
    S->edf.set_compat_eye(on != 0);
    return GDMR_OK;
}

extern "C" int gdmr_system_grid(const gdmr_system *S, int *dims) {
    if (!S || !dims) return fail(GDMR_EINVAL, "gdmr_system_grid", "null system or dims");
    dims[0] = S->A.gx;
    dims[1] = S->A.gy;
    dims[2] = S->A.gz;
    return GDMR_OK;
}

extern "C" int gdmr_csr_grid_form(int n, const int *rowPtr, const int *colIdx, const double *vals_ri, int *dims) {
    if (!dims) return fail(GDMR_EINVAL, "gdmr_csr_grid_form", "null dims");
    const int rc = csr_grid_form(n, rowPtr, colIdx, vals_ri, dims);
    if (rc == GDMR_OK) set_last_error(GDMR_OK, "ok");
    return rc;
}

extern "C" int gdmr_system_svd_sweeps(const gdmr_system *S) {
    if (!S) return 0;
    return S->precision == 1 ? S->e32.last_svd_sweeps()
                             : S->precision == 2 ? S->edf.last_svd_sweeps() : S->e64.last_svd_sweeps();
}

extern "C" int gdmr_solve(gdmr_system *S, int mode, const double *b, double *x, double tol, int matRank, int on_device,
                          gdmr_stats *stats) {
    if (!S || !b || !x) return fail(GDMR_EINVAL, "gdmr_solve", "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    cudaSetDevice(S->device);
    if (S->precision == 1) return single_impl<float>(S, mode, b, x, tol, matRank, on_device, stats);
    if (S->precision == 2) return single_impl<dfr>(S, mode, b, x, tol, matRank, on_device, stats);
    return single_impl<double>(S, mode, b, x, tol, matRank, on_device, stats);
}

extern "C" int gdmr_solve_batch(gdmr_system *S, int nrhs, const double *b, double *x, const double *tol,
                                int maxCycles, int on_device, gdmr_stats *stats) {
    if (!S || !b || !x || nrhs < 1) return fail(GDMR_EINVAL, "gdmr_solve_batch", "null argument or nrhs < 1");
    std::lock_guard<std::mutex> lk(S->mu);
    cudaSetDevice(S->device);
    if (S->precision == 1) return batch_impl<float>(S, nrhs, b, x, tol, maxCycles, on_device, stats);
    if (S->precision == 2) return batch_impl<dfr>(S, nrhs, b, x, tol, maxCycles, on_device, stats);
    return batch_impl<double>(S, nrhs, b, x, tol, maxCycles, on_device, stats);
}

// ================================================================ many operators in lockstep
// gdmr_multi_solve: the refined batched solve of several systems (operators) at once, their
// restart cycles in lockstep and the Krylov loops of every right-hand side in flight, across all
// operators, in one cooperative launch a cycle (k_krylov_multi), instead of one engine and stream
// per operator each launching its own kernels.  The rest of a cycle (true residual, deflation
// loop, least squares, combinations, deflation update) stays on each operator's own stream.
namespace {
template <class R>
int multi_impl(int nops, gdmr_system *const *sys, const int *nrhs, const double *const *b, double *const *x,
               const double *tol, int maxCycles, gdmr_stats *const *stats) {
    const char *F = "gdmr_multi_solve";
    const int dev = sys[0]->device;
    std::vector<Engine<R> *> E(nops);
    int total = 0, max_jobs = 0, qmax = 0;
    for (int o = 0; o < nops; ++o) {
        E[o] = &eng_of<R>(sys[o]);
        int rc = E[o]->refine_setup(sys[o]->A.view64());
        if (rc != GDMR_OK) return rc;
        total += nrhs[o];
        max_jobs += E[o]->capacity();
        qmax = std::max(qmax, sys[o]->m + 1);
    }
    const int resident = krylov_multi_resident();
    if (resident < 1) return fail(GDMR_ECUDA, F, "the many-system kernel cannot be resident");
    // driver-owned device buffers: jobs, the job of each CTA, partial sums, barrier counters
    KrylovJob<R> *djobs = nullptr, *hjobs = nullptr;
    int *dcta = nullptr, *hcta = nullptr, *dabort = nullptr;
    double *dpart = nullptr;
    unsigned *dbar = nullptr;
    cudaStream_t ms = nullptr;
    cudaEvent_t ev_kernel = nullptr;
    std::vector<cudaEvent_t> ev_front(nops, nullptr);
    auto release = [&]() {
        cudaFree(djobs);
        cudaFreeHost(hjobs);
        cudaFree(dcta);
        cudaFreeHost(hcta);
        cudaFree(dabort);
        cudaFree(dpart);
        cudaFree(dbar);
        if (ev_kernel) cudaEventDestroy(ev_kernel);
        for (auto &e : ev_front)
            if (e) cudaEventDestroy(e);
        if (ms) cudaStreamDestroy(ms);
    };
    const size_t part_doubles = (size_t)resident * (2 * (size_t)qmax + 3);
    if (cudaMalloc(&djobs, sizeof(KrylovJob<R>) * max_jobs) != cudaSuccess ||
        cudaMallocHost(&hjobs, sizeof(KrylovJob<R>) * max_jobs) != cudaSuccess ||
        cudaMalloc(&dcta, sizeof(int) * resident) != cudaSuccess ||
        cudaMallocHost(&hcta, sizeof(int) * resident) != cudaSuccess || cudaMalloc(&dabort, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&dpart, sizeof(double) * part_doubles) != cudaSuccess ||
        cudaMalloc(&dbar, sizeof(unsigned) * max_jobs) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ms, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev_kernel, cudaEventDisableTiming) != cudaSuccess) {
        release();
        return fail(GDMR_ENOMEM, F, "driver buffers");
    }
    for (auto &e : ev_front)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            release();
            return fail(GDMR_ECUDA, F, "events");
        }
    std::vector<std::vector<int>> slot_of(nops);
    std::vector<int> next(nops, 0);
    for (int o = 0; o < nops; ++o) slot_of[o].assign(E[o]->capacity(), -1);
    int finished = 0, worst = GDMR_OK;
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<KrylovJob<R>> jobs;
    std::vector<long> job_nnz;   // non-zeros of each job's operator (algorithmic bytes)
    while (finished < total) {
        // admission into free slots, then the true residuals of every operator (enqueued)
        for (int o = 0; o < nops; ++o) {
            gdmr_system *S = sys[o];
            const size_t vb = sizeof(double2) * (size_t)S->n;
            for (int sl = 0; sl < E[o]->capacity() && next[o] < nrhs[o]; ++sl) {
                if (slot_of[o][sl] >= 0) continue;
                const int r = next[o]++;
                if (cudaMemcpyAsync(S->db + (size_t)sl * S->n, b[o] + (size_t)2 * r * S->n, vb, cudaMemcpyHostToDevice,
                                    S->st) != cudaSuccess ||
                    cudaMemcpyAsync(S->dx + (size_t)sl * S->n, x[o] + (size_t)2 * r * S->n, vb, cudaMemcpyHostToDevice,
                                    S->st) != cudaSuccess) {
                    release();
                    return fail(GDMR_ECUDA, F, "host to device copy failed");
                }
                int rc = E[o]->refine_admit(sl, S->db + (size_t)sl * S->n, S->dx + (size_t)sl * S->n,
                                            tol ? tol[o] : 1e-10, maxCycles);
                if (rc != GDMR_OK) { release(); return rc; }
                slot_of[o][sl] = r;
            }
            int rc = E[o]->multi_residual();
            if (rc != GDMR_OK) { release(); return rc; }
        }
        // convergence and retirement of every operator
        auto retire = [&](int o, const std::vector<int> &done) {
            gdmr_system *S = sys[o];
            for (int sl : done) {
                const int r = slot_of[o][sl];
                cudaMemcpyAsync(x[o] + (size_t)2 * r * S->n, E[o]->slot_x(sl), sizeof(double2) * (size_t)S->n,
                                cudaMemcpyDeviceToHost, S->st);
                if (stats && stats[o]) {
                    to_stats(E[o]->slot_stats(sl), &stats[o][r]);
                    stats[o][r].latency_ms =
                        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
                }
                worst = std::max(worst, E[o]->slot_stats(sl).status);
                slot_of[o][sl] = -1;
                ++finished;
            }
        };
        std::vector<int> nrun(nops, 0);
        int in_flight = 0;
        bool all_admitted = true;
        for (int o = 0; o < nops; ++o) {
            std::vector<int> done;
            nrun[o] = E[o]->multi_select(&done);
            if (nrun[o] < 0) { release(); return GDMR_ECUDA; }
            retire(o, done);
            in_flight += nrun[o];
            all_admitted &= next[o] >= nrhs[o];
        }
        // the tail: with every right-hand side admitted and few systems left, a lockstep cycle is
        // as long as its largest system's Krylov loop run by a fraction of the CTAs; the engines'
        // own batched cycles finish the remaining systems, operator by operator
        const int tail = g_multi_tail.load();
        if (all_admitted && in_flight > 0 && in_flight <= tail) {
            // one host thread per remaining operator drives its engine (each engine has its own
            // stream and buffers, as the server's workers do), so their cycles overlap on the GPU
            std::vector<std::thread> th;
            std::vector<int> trc(nops, GDMR_OK);
            std::vector<std::vector<std::pair<int, double>>> tdone(nops);
            for (int o = 0; o < nops; ++o) {
                if (E[o]->active_count() == 0) continue;
                th.emplace_back([&, o] {
                    if (cudaSetDevice(dev) != cudaSuccess) { trc[o] = GDMR_ECUDA; return; }
                    while (E[o]->active_count() > 0) {
                        std::vector<int> done;
                        const int rc = E[o]->refine_cycle(&done);
                        if (rc != GDMR_OK) { trc[o] = rc; return; }
                        const double ms =
                            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
                        for (int sl : done) tdone[o].emplace_back(sl, ms);
                    }
                });
            }
            for (auto &t : th) t.join();
            for (int o = 0; o < nops; ++o) {
                if (trc[o] != GDMR_OK) {
                    release();
                    return fail(trc[o], F, "a system's own cycles failed in the tail");
                }
                for (auto &d : tdone[o]) {
                    const int r = slot_of[o][d.first];
                    retire(o, std::vector<int>{d.first});
                    if (stats && stats[o]) stats[o][r].latency_ms = d.second;   // when its thread saw it finish
                }
            }
            break;
        }
        // the front of the cycle of each operator
        jobs.clear();
        job_nnz.clear();
        for (int o = 0; o < nops; ++o) {
            gdmr_system *S = sys[o];
            if (nrun[o] > 0) {
                int rc = E[o]->multi_front();
                if (rc != GDMR_OK) { release(); return rc; }
                if (cudaEventRecord(ev_front[o], E[o]->main_stream()) != cudaSuccess ||
                    cudaStreamWaitEvent(ms, ev_front[o], 0) != cudaSuccess) {
                    release();
                    return fail(GDMR_ECUDA, F, "events");
                }
                E[o]->multi_jobs(jobs);
                job_nnz.resize(jobs.size(), S->A.nnz);
            }
        }
        if (jobs.empty()) continue;
        const int njobs = (int)jobs.size();
        if (njobs > resident || njobs > max_jobs) {
            release();
            return fail(GDMR_EINVAL, F, "more right-hand sides in flight than the persistent launch holds");
        }
        // CTAs to jobs in proportion to n (at least one, at most one per slice); partials and
        // barrier counters per job
        double sum_n = 0;
        for (auto &j : jobs) sum_n += j.n;
        int ctas = 0;
        size_t poff = 0;
        double bytes = 0;
        for (int i = 0; i < njobs; ++i) {
            KrylovJob<R> &j = jobs[i];
            const int left = resident - ctas - (njobs - 1 - i);   // keep one for each job after this
            int c = (int)((double)resident * j.n / sum_n);
            c = std::max(1, std::min(c, std::min(j.nslices, left)));
            j.cta0 = ctas;
            j.ncta = c;
            j.part = dpart + poff;
            j.bar = dbar + i;
            poff += (size_t)c * (2 * (size_t)j.qmax + 3);
            for (int q = 0; q < c; ++q) hcta[ctas + q] = i;
            ctas += c;
            const SellMatrix A{j.n, j.nslices, j.slice_ptr, j.cols, j.vals, job_nnz[i]};
            bytes += krylov_loop_bytes(A, sizeof(typename CT<R>::t), j.kk, j.m);
            hjobs[i] = j;
        }
        if (cudaMemcpyAsync(djobs, hjobs, sizeof(KrylovJob<R>) * njobs, cudaMemcpyHostToDevice, ms) != cudaSuccess ||
            cudaMemcpyAsync(dcta, hcta, sizeof(int) * ctas, cudaMemcpyHostToDevice, ms) != cudaSuccess ||
            cudaMemsetAsync(dbar, 0, sizeof(unsigned) * njobs, ms) != cudaSuccess ||
            cudaMemsetAsync(dabort, 0, sizeof(int), ms) != cudaSuccess ||
            launch_krylov_multi<R>(djobs, dcta, ctas, dabort, bytes, ms) != 1 ||
            cudaEventRecord(ev_kernel, ms) != cudaSuccess) {
            release();
            return fail(GDMR_ECUDA, F, "the many-system launch failed");
        }
        for (int o = 0; o < nops; ++o) {
            int rc = E[o]->multi_back(ev_kernel);
            if (rc != GDMR_OK) { release(); return rc; }
        }
        // the host buffers of this launch are reused only after every operator's stream, which
        // waits for it, has been synchronised by the next round's multi_select
    }
    for (int o = 0; o < nops; ++o) cudaStreamSynchronize(sys[o]->st);
    cudaStreamSynchronize(ms);
    release();
    (void)dev;
    if (worst != GDMR_OK)
        set_last_error(worst, "gdmr_multi_solve: some right-hand sides did not converge; see the stats");
    else
        set_last_error(GDMR_OK, "ok");
    return worst;
}
}  // namespace

extern "C" int gdmr_multi_solve(int nops, gdmr_system *const *systems, const int *nrhs, const double *const *b,
                                double *const *x, const double *tol, int maxCycles, gdmr_stats *const *stats) {
    if (nops < 1 || !systems || !nrhs || !b || !x) return fail(GDMR_EINVAL, "gdmr_multi_solve", "null argument");
    const int prec = systems[0] ? systems[0]->precision : -1, dev = systems[0] ? systems[0]->device : -1;
    for (int o = 0; o < nops; ++o) {
        if (!systems[o] || !b[o] || !x[o] || nrhs[o] < 0)
            return fail(GDMR_EINVAL, "gdmr_multi_solve", "null system or buffer, or a negative count");
        if (systems[o]->precision != prec || systems[o]->device != dev)
            return fail(GDMR_EINVAL, "gdmr_multi_solve", "all systems need the same precision and device");
    }
    std::vector<std::unique_lock<std::mutex>> locks;
    for (int o = 0; o < nops; ++o) {
        bool seen = false;   // the same system twice: lock it once
        for (int p = 0; p < o; ++p) seen |= systems[p] == systems[o];
        if (seen) return fail(GDMR_EINVAL, "gdmr_multi_solve", "a system is listed twice");
        locks.emplace_back(systems[o]->mu);
    }
    cudaSetDevice(dev);
    if (prec == 1) return multi_impl<float>(nops, systems, nrhs, b, x, tol, maxCycles, stats);
    if (prec == 2) return multi_impl<dfr>(nops, systems, nrhs, b, x, tol, maxCycles, stats);
    return multi_impl<double>(nops, systems, nrhs, b, x, tol, maxCycles, stats);
}

extern "C" int gdmr_true_residual(gdmr_system *S, int nrhs, const double *b, const double *x, int on_device,
                                  double *relres) {
    if (!S || !b || !x || !relres || nrhs < 1) return fail(GDMR_EINVAL, "gdmr_true_residual", "bad argument");
    std::lock_guard<std::mutex> lk(S->mu);
    cudaSetDevice(S->device);
    const size_t vb = sizeof(double2) * (size_t)S->n;
    auto run = [&](auto &E) -> int {
        int rc = E.refine_setup(S->A.view64());
        if (rc != GDMR_OK) return rc;
        if (on_device) return E.true_residual(nrhs, (const double2 *)b, (const double2 *)x, relres);
        for (int r = 0; r < nrhs; r += S->cap) {
            const int cnt = std::min(S->cap, nrhs - r);
            cudaMemcpyAsync(S->db, b + (size_t)2 * r * S->n, vb * cnt, cudaMemcpyHostToDevice, S->st);
            cudaMemcpyAsync(S->dx, x + (size_t)2 * r * S->n, vb * cnt, cudaMemcpyHostToDevice, S->st);
            if ((rc = E.true_residual(cnt, S->db, S->dx, relres + r)) != GDMR_OK) return rc;
        }
        return GDMR_OK;
    };
    return S->precision == 1 ? run(S->e32) : S->precision == 2 ? run(S->edf) : run(S->e64);
}

extern "C" int gdmr_export_deflation(gdmr_system *S, double *z) {
    if (!S || !z) return fail(GDMR_EINVAL, "gdmr_export_deflation", "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    cudaSetDevice(S->device);
    if (S->precision == 0) return S->e64.export_deflation((double2 *)z);
    if (S->precision == 2) {
        std::vector<dfc> tmp((size_t)S->k * S->n);
        int rc = S->edf.export_deflation(tmp.data());
        for (size_t i = 0; i < tmp.size(); ++i) {
            z[2 * i] = (double)tmp[i].x;
            z[2 * i + 1] = (double)tmp[i].y;
        }
        return rc;
    }
    std::vector<float2> tmp((size_t)S->k * S->n);
    int rc = S->e32.export_deflation(tmp.data());
    for (size_t i = 0; i < tmp.size(); ++i) { z[2 * i] = tmp[i].x; z[2 * i + 1] = tmp[i].y; }
    return rc;
}

extern "C" int gdmr_import_deflation(gdmr_system *S, const double *z) {
    if (!S || !z) return fail(GDMR_EINVAL, "gdmr_import_deflation", "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    cudaSetDevice(S->device);
    if (S->precision == 0) return S->e64.import_deflation((const double2 *)z);
    if (S->precision == 2) {
        std::vector<dfc> tmp((size_t)S->k * S->n);
        for (size_t i = 0; i < tmp.size(); ++i) {
            tmp[i].x = dfr(z[2 * i]);
            tmp[i].y = dfr(z[2 * i + 1]);
        }
        return S->edf.import_deflation(tmp.data());
    }
    std::vector<float2> tmp((size_t)S->k * S->n);
    for (size_t i = 0; i < tmp.size(); ++i) tmp[i] = make_float2((float)z[2 * i], (float)z[2 * i + 1]);
    return S->e32.import_deflation(tmp.data());
}

extern "C" int gdmr_save_deflation(gdmr_system *S, const char *path) {
    if (!S || !path) return fail(GDMR_EINVAL, "gdmr_save_deflation", "null argument");
    std::vector<double> z((size_t)2 * S->k * S->n);
    int rc = gdmr_export_deflation(S, z.data());
    if (rc != GDMR_OK) return rc;
    return gdmr_deflation_write(path, S->n, S->k, z.data());
}

extern "C" int gdmr_load_deflation(gdmr_system *S, const char *path) {
    if (!S || !path) return fail(GDMR_EINVAL, "gdmr_load_deflation", "null argument");
    std::vector<double> z((size_t)2 * S->k * S->n);
    int rc = gdmr_deflation_read(path, S->n, S->k, z.data());
    if (rc != GDMR_OK) return rc;
    return gdmr_import_deflation(S, z.data());
}

extern "C" int gdmr_drop_deflation(gdmr_system *S) {
    if (!S) return fail(GDMR_EINVAL, "gdmr_drop_deflation", "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    S->e32.drop_deflation();
    S->e64.drop_deflation();
    S->edf.drop_deflation();
    return GDMR_OK;
}

// ================================================================ allocation-free residual check
// gdmr_true_residual_noalloc: the FP64 relative residual ||b_s - A x_s|| / ||b_s|| of up to
// 64 pairs on the caller's device buffers, for callers that must not allocate device memory:
// hosts whose own allocator owns the whole device-memory pool (a fixed arena carved up at
// start-up, where a cudaMalloc from a library would fail or fragment it), and latency-critical
// loops, where a cudaMalloc can synchronise the device and stall.  It allocates nothing: the
// cross-CTA reduction scratch is the file-scope array below (256 KB of partial sums plus the
// arrival counters), which every GPU that loads this library holds until the process exits.
//
// Set-up: the first call on a device (with that device current) looks the arrays up with
// cudaGetSymbolAddress and zeroes the counters; make that first call before any stream
// capture.  All calls share the arrays, which keep the last call's contents: the counters
// return to zero at the end of every call, and calls that overlap on the GPU race on them.
namespace {

constexpr int NOALLOC_MAX_RHS = 64;
constexpr int NOALLOC_CTAS = 256;                  // CTAs per right-hand side (grid-stride)
__device__ __align__(256) double g_noalloc_partials[NOALLOC_MAX_RHS * 2 * NOALLOC_CTAS];
__device__ __align__(256) unsigned g_noalloc_tickets[NOALLOC_MAX_RHS];

struct NoallocScratch {
    double *partials = nullptr;
    unsigned *tickets = nullptr;
};
constexpr int NOALLOC_MAX_DEVICES = 64;
NoallocScratch g_noalloc[NOALLOC_MAX_DEVICES];
std::mutex g_noalloc_mu;

int noalloc_scratch(int device, NoallocScratch *out) {
    if (device < 0 || device >= NOALLOC_MAX_DEVICES)
        return fail(GDMR_EINVAL, "gdmr_true_residual_noalloc", "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoallocScratch &s = g_noalloc[device];
    if (!s.partials) {
        void *p = nullptr, *t = nullptr;
        cudaError_t e1 = cudaGetSymbolAddress(&p, g_noalloc_partials);
        cudaError_t e2 = cudaGetSymbolAddress(&t, g_noalloc_tickets);
        if (e1 != cudaSuccess || e2 != cudaSuccess)
            return fail(GDMR_ECUDA, "gdmr_true_residual_noalloc", "cudaGetSymbolAddress failed");
        if (cudaMemset(t, 0, sizeof(g_noalloc_tickets)) != cudaSuccess)
            return fail(GDMR_ECUDA, "gdmr_true_residual_noalloc", "clearing the arrival counters failed");
        s.partials = (double *)p;
        s.tickets = (unsigned *)t;
    }
    *out = s;
    return GDMR_OK;
}

// One kernel: ||b - A x||^2 and ||b||^2 per right-hand side over a grid-stride row loop, CTA
// partials into the static scratch, the last CTA of each right-hand side sums them in order.
template <int NCX, int WID>
__global__ void __launch_bounds__(256) k_relres_noalloc(int n, const int *__restrict__ slice_ptr,
                                                        const int *__restrict__ cols,
                                                        const double2 *__restrict__ vals,
                                                        const double2 *__restrict__ b0,
                                                        const double2 *__restrict__ x0, double *partials,
                                                        unsigned *tickets, double *relres, ResidPattern rp) {
    const int s = blockIdx.x, G = gridDim.y, tid = threadIdx.x;
    const double2 *b = b0 + (size_t)s * n;
    const double2 *x = x0 + (size_t)s * n;
    double r2 = 0, b2 = 0;
    for (long row = (long)blockIdx.y * 256 + tid; row < n; row += (long)G * 256) {
        const double2 bv = b[row];
        // the row code of the allocating residual kernel: near convergence the residual cancels
        // ~10 digits, so the per-entry operations and their order must match exactly
        const double2 acc = resid_row<NCX, WID>(bv, row, slice_ptr, cols, vals, x, rp);
        r2 += acc.x * acc.x + acc.y * acc.y;
        b2 += bv.x * bv.x + bv.y * bv.y;
    }
    __shared__ double red[2][8];
    __shared__ unsigned last;
    for (int o = 16; o > 0; o >>= 1) {
        r2 += __shfl_xor_sync(0xffffffffu, r2, o);
        b2 += __shfl_xor_sync(0xffffffffu, b2, o);
    }
    if ((tid & 31) == 0) { red[0][tid >> 5] = r2; red[1][tid >> 5] = b2; }
    __syncthreads();
    double *part = partials + (size_t)s * 2 * NOALLOC_CTAS;
    if (tid == 0) {
        double a = 0, c = 0;
        for (int w = 0; w < 8; ++w) { a += red[0][w]; c += red[1][w]; }
        part[blockIdx.y] = a;
        part[NOALLOC_CTAS + blockIdx.y] = c;
        __threadfence();
        last = atomicAdd(&tickets[s], 1u) == (unsigned)G - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (tid == 0) {
        double a = 0, c = 0;
        for (int g = 0; g < G; ++g) { a += __ldcg(part + g); c += __ldcg(part + NOALLOC_CTAS + g); }
        relres[s] = c > 0 ? sqrt(a) / sqrt(c) : sqrt(a);
        tickets[s] = 0;   // ready for the next call
    }
}

}  // namespace

extern "C" int gdmr_true_residual_noalloc(gdmr_system *S, int nrhs, const double *b, const double *x,
                                          double *relres, void *stream) {
    if (!S || !b || !x || !relres) return fail(GDMR_EINVAL, "gdmr_true_residual_noalloc", "null argument");
    if (nrhs < 1 || nrhs > NOALLOC_MAX_RHS)
        return fail(GDMR_EINVAL, "gdmr_true_residual_noalloc",
                    "nrhs must be between 1 and 64 (the size of the static reduction scratch)");
    if (!S->A.vals64) return fail(GDMR_ENOTINIT, "gdmr_true_residual_noalloc", "system has no FP64 operator");
    if (cudaSetDevice(S->device) != cudaSuccess)
        return fail(GDMR_ECUDA, "gdmr_true_residual_noalloc", "cudaSetDevice failed");
    NoallocScratch sc;
    int rc = noalloc_scratch(S->device, &sc);
    if (rc != GDMR_OK) return rc;
    int G = (S->n + 255) / 256;
    if (G > NOALLOC_CTAS) G = NOALLOC_CTAS;
    if (G < 1) G = 1;
    const SellMatrix A = S->A.view64();
    ResidPattern rp{};
    const int ncx = resid_pattern(A, rp);
    resid_dispatch(A.npat, ncx, [&](auto ncx_c, auto wid_c) {
        k_relres_noalloc<decltype(ncx_c)::value, decltype(wid_c)::value>
            <<<dim3((unsigned)nrhs, (unsigned)G), 256, 0, (cudaStream_t)stream>>>(
                S->n, S->A.slice_ptr, S->A.cols, S->A.vals64, (const double2 *)b, (const double2 *)x, sc.partials,
                sc.tickets, relres, rp);
    });
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(GDMR_ECUDA, "gdmr_true_residual_noalloc", cudaGetErrorString(e));
    return GDMR_OK;
}
