// Device kernels of the GB300 DMR restart cycle (sm_103a).
//
// Every kernel here is HBM-bound streaming work over n-long complex vectors,
// except the small dense FP64 problems on the Hessenberg matrix (least squares
// by Givens rotations, one-sided Jacobi SVD), which are latency-bound and run
// one CTA per system.  Vectors are complex64 (float2) or complex128 (double2);
// cross-thread reductions accumulate in double and finish deterministically
// (fixed grid, fixed order, last-CTA-done ticket), replacing the racy
// innerProdKerDMR reduction of the reference (gDMR.cu:268-326).
//
// Batching: most kernels run over an "active list" of systems (blockIdx.y
// indexes the list), each system s owning a Krylov basis V_s of (m+1)
// vectors at V + s*sysStride, while the deflation vectors W and Z are shared.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include <type_traits>

namespace gdmr {

// Double-float real: value = hi + lo with |lo| <= ulp(hi)/2, about 48 significant bits.  It
// carries the FP64-class "fp64e" precision form through the streaming kernels on the FP32
// pipes (GB300 retires FP32 at 69 TFLOP/s but FP64 at 1 TFLOP/s, too slow for HBM-rate
// complex dot products).  Products use the exact FMA two-product, sums the two-sum of Knuth
// (Dekker 1971; Knuth, TAOCP vol. 2, 4.2.2), each result renormalised by fast-two-sum.
struct dfr {
    float hi, lo;
    dfr() = default;
    __host__ __device__ constexpr dfr(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ dfr(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    __host__ __device__ dfr(int v) : hi((float)v), lo(0.f) {}
    __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};
// complex double-float: (re.hi, re.lo, im.hi, im.lo), one 16-byte load
struct __align__(16) dfc {
    dfr x, y;
};

template <class R> struct CT;
template <> struct CT<float> { using t = float2; };
template <> struct CT<double> { using t = double2; };
template <> struct CT<dfr> { using t = dfc; };

// Tuner / report key of a precision: 4 complex64, 8 complex128, 9 double-float complex.
template <class R> constexpr int prec_key() { return sizeof(R) == 4 ? 4 : 8; }
template <> constexpr int prec_key<dfr>() { return 9; }

__host__ __device__ inline float2 mk(float a, float b) { return make_float2(a, b); }
__host__ __device__ inline double2 mk(double a, double b) { return make_double2(a, b); }

#ifdef __CUDACC__
__device__ __forceinline__ dfr df_renorm(float s, float e) {   // fast-two-sum, |s| >= |e|
    const float h = s + e;
    return dfr(h, e - (h - s));
}
__device__ __forceinline__ dfr operator+(dfr a, dfr b) {
    const float s = a.hi + b.hi, bb = s - a.hi;
    const float e = ((a.hi - (s - bb)) + (b.hi - bb)) + (a.lo + b.lo);
    return df_renorm(s, e);
}
__device__ __forceinline__ dfr operator-(dfr a) { return dfr(-a.hi, -a.lo); }
__device__ __forceinline__ dfr operator-(dfr a, dfr b) { return a + (-b); }
__device__ __forceinline__ dfr operator*(dfr a, dfr b) {
    const float p = a.hi * b.hi;
    const float e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p)));
    return df_renorm(p, e);
}
// a * b + c
__device__ __forceinline__ dfr fma(dfr a, dfr b, dfr c) {
    const float p = a.hi * b.hi;
    const float pe = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p)));
    const float s = p + c.hi, bb = s - p;
    const float e = ((p - (s - bb)) + (c.hi - bb)) + (pe + c.lo);
    return df_renorm(s, e);
}
__device__ __forceinline__ dfr &operator+=(dfr &a, dfr b) { return a = a + b; }
__device__ __forceinline__ dfr &operator-=(dfr &a, dfr b) { return a = a - b; }
__device__ __forceinline__ dfr &operator*=(dfr &a, dfr b) { return a = a * b; }
#endif

// Per-system state that the device kernels update and the host reads once per cycle.
struct SysState {
    double nrm2;        // last reduced squared norm
    double cross_re;    // last reduced <w_new, w_orig>
    double cross_im;
    double alpha;       // scale for the pending normalisation (1/norm, 0 after breakdown)
    double rho;         // ||r_new|| / ||r_old|| of the last cycle (unit residual direction)
    double rho_abs;     // absolute residual norm carried by the recursion
    double bnorm;       // ||b||
    double true_res;    // last FP64 ||b - A x|| (refined form)
    int broken;         // Krylov step at which breakdown happened this cycle (0 = none)
    int bad;            // non-finite value met
    int pad[2];
};

// Finishing actions run by the last CTA of a reduction kernel.
enum FinishMode : int {
    FIN_NONE = 0,       // store nrm2/cross only
    FIN_KRYLOV = 1,     // Krylov step: H column, breakdown test, alpha
    FIN_DEFLATION = 2,  // deflation step: H[i,i] = <w,Az>/||w||, alpha
    FIN_UNIT = 3,       // alpha = 1/||w||
    FIN_RESIDUAL = 4,   // cycle end: rho, alpha = 1/rho
};

struct FinishArgs {
    int mode;
    int col;            // Hessenberg column being completed
    int nco;            // number of projection coefficients in that column (rows 0..nco-1)
    int ldH;            // m + 1
    int m;              // Hessenberg columns
    int kk;             // deflation dimension in this cycle
    int compat_eye;     // breakdown identity tail starts at column j (reference) instead of kk+j
    double tol;         // absolute breakdown threshold (the reference's solTol)
    double2 *H;         // H of system 0; system s at H + s*strideH
    size_t strideH;
    const double2 *coef;  // projection coefficients of system 0; s at coef + s*strideC
    size_t strideC;
};

#ifdef __CUDACC__
// The finishing step of a reduction kernel's last CTA: stores the reduced norm and cross term,
// then, per mode, the Hessenberg column with the breakdown test and the reference's identity
// tail (gDMR.cu:2256-2289), the deflation loop's diagonal, or the cycle-end residual factor.
__device__ inline void run_finish(const FinishArgs &f, int s, SysState &st, double n2, double cre, double cim) {
    st.nrm2 = n2;
    st.cross_re = cre;
    st.cross_im = cim;
    const double nrm = sqrt(n2);
    if (!isfinite(nrm)) st.bad = 1;
    switch (f.mode) {
    case FIN_KRYLOV: {
        double2 *H = f.H + (size_t)s * f.strideH;
        const double2 *c = f.coef + (size_t)s * f.strideC;
        for (int p = 0; p < f.nco; ++p) H[(size_t)f.col * f.ldH + p] = c[p];
        const int j = f.col - f.kk + 1;
        if (nrm < f.tol) {   // absolute breakdown threshold, gDMR.cu:2256
            st.broken = j;
            st.alpha = 0.0;
            for (int cc = f.compat_eye ? j : f.kk + j; cc < f.m; ++cc) H[(size_t)cc * f.ldH + cc] = make_double2(1.0, 0.0);
        } else {
            st.alpha = 1.0 / nrm;
            H[(size_t)f.col * f.ldH + f.col + 1] = make_double2(cre / nrm, cim / nrm);
        }
        break;
    }
    case FIN_DEFLATION: {
        double2 *H = f.H;
        const double2 *c = f.coef;
        for (int p = 0; p < f.nco; ++p) H[(size_t)f.col * f.ldH + p] = c[p];
        st.alpha = 1.0 / nrm;
        H[(size_t)f.col * f.ldH + f.col] = make_double2(cre / nrm, cim / nrm);
        break;
    }
    case FIN_UNIT:
        st.alpha = 1.0 / nrm;
        break;
    case FIN_RESIDUAL:
        st.rho = nrm;
        st.alpha = 1.0 / nrm;
        st.rho_abs = st.rho_abs * nrm;
        break;
    default:
        break;
    }
}
#endif

// ----------------------------------------------------------------- instrumentation
// Every launcher counts its kernel launches.  With profiling on, it also brackets
// each launch with CUDA events on its stream and books the launch's algorithmic
// bytes (the minimum HBM traffic of the operation) to its kernel class;
// profile_flush() (after the stream is synchronised) turns the events into times.
enum KernelClass : int {
    KC_MDOT = 0,      // projection coefficients  [W V]^H w
    KC_UPDATE = 1,    // w - [W V] c with norms
    KC_SPMM = 2,      // SELL operator products (inner precision)
    KC_COMBINE = 3,   // cycle-end residual / solution combinations
    KC_ZUPDATE = 4,   // deflation-space update
    KC_RESID64 = 5,   // FP64 true residual
    KC_LS = 6,        // Givens least squares
    KC_SVD = 7,       // Jacobi SVD
    KC_OTHER = 8,     // scales, copies, norms, refinement updates
    KC_COUNT = 9
};
long long launch_count();
void profile_enable(bool on);
bool profile_enabled();
void profile_flush();
void profile_read(int kc, double *bytes, double *ms, long long *launches);
void profile_reset();
// Gram-Schmidt variant autotuning (on by default) and its report, one line per tuned shape.
void tune_enable(bool on);
// Pins the projection and update variants (-1 returns each to the tuner).
void tune_force(int projection, int update);
// Marks the calling thread as capturing a CUDA graph: launchers then use cached choices only.
void set_capturing(bool on);
std::string tune_report();

// ----------------------------------------------------------------- launchers
// All launchers enqueue on `st` and never synchronise.

// Reduction scratch: every reducing kernel below needs `partials` of at least
// scratch_doubles(qmax, nsys) doubles and `tickets` of nsys zero-initialised
// counters (each kernel resets the counters it used).  Kernels on one stream
// may share both.
size_t scratch_doubles(int qmax, int nsys, int n);
// Reduction scratch handed to the Gram-Schmidt launchers must be registered with its size.
void register_scratch(const void *p, size_t doubles);
void unregister_scratch(const void *p);

template <class R>
void launch_mdot(int n, const typename CT<R>::t *segA, int qa, const typename CT<R>::t *segB, size_t strideB, int qb,
                 const typename CT<R>::t *w, size_t strideW, const int *act, int nsys, double2 *partials, int qmax,
                 unsigned *tickets, double2 *coef, size_t strideC, SysState *state, bool skip_broken, cudaStream_t st);

// out = w - [segA segB] coef, reduces ||out||^2 and <out, w>, then runs `fin` in the last CTA.
template <class R>
void launch_update(int n, const typename CT<R>::t *segA, int qa, const typename CT<R>::t *segB, size_t strideB, int qb,
                   const typename CT<R>::t *w, size_t strideW, typename CT<R>::t *out, size_t strideO, const int *act,
                   int nsys, const double2 *coef, size_t strideC, double2 *partials, unsigned *tickets,
                   SysState *state, FinishArgs fin, bool skip_broken, cudaStream_t st);

// Tensor-core split-K projection of a batch onto the shared deflation vectors (complex64;
// gdmr_tc.cu): coef[act[s]*strideC + p] = <W_p, y_s> for p < kk, s < nsys, through per-CTA
// partials in `part` (wproj_tc_grid(n) x kk x nsys x 2 doubles); returns the number of
// kernels launched.  wproj_tc_ok says when it applies (kk <= 32, 8 <= nsys <= 64, even n and
// stride, 16-byte aligned vectors).
bool wproj_tc_ok(int n, int kk, int nsys, const void *W, const void *Y, size_t strideY);
int wproj_tc_grid(int n);
int launch_wproj_tc(int n, int kk, const float2 *W, const float2 *Y, size_t strideY, const int *act, int nsys,
                    double *part, double2 *coef, size_t strideC, cudaStream_t st);
// Tensor-core apply of the shared deflation vectors for a batch (complex64; gdmr_tc.cu):
// P[act[s]*strideP + i] = sum_p coef[act[s]*strideC + p] W_p[i] for p < kk, and
// coef[act[s]*strideC + unit_idx] = 1, so that a per-system update with P as one more basis
// vector subtracts W c_s.  wapply_tc_ok: kk <= 32, 8 <= nsys <= 64.
bool wapply_tc_ok(int n, int kk, int nsys);
int launch_wapply_tc(int n, int kk, const float2 *W, double2 *coef, size_t strideC, const int *act, int nsys,
                     float2 *P, size_t strideP, int unit_idx, cudaStream_t st);
// The batched update with its shared part on the tensor cores in one kernel (complex64;
// gdmr_tc.cu): out_s = w_s - V_s c_s[kk..kk+qb) - W c_s[0..kk) for the active systems, with
// ||out_s||^2 and <out_s, w_s> reduced through partials (wupdate_tc_grid(n) x 3 x nsys doubles)
// and tickets (nsys counters) and `fin` run per system, as launch_update does.  wupdate_tc_ok:
// kk <= 32, qb <= 32, 8 <= nsys <= 64.
bool wupdate_tc_ok(int n, int kk, int qb, int nsys);
int wupdate_tc_grid(int n);
int launch_wupdate_tc(int n, int kk, const float2 *W, const float2 *V, size_t strideV, int qb, const float2 *w,
                      size_t strideW, float2 *out, size_t strideO, const int *act, int nsys, const double2 *coef,
                      size_t strideC, double *partials, unsigned *tickets, SysState *state, FinishArgs fin,
                      bool skip_broken, cudaStream_t st);
// mbarrier waits of the tensor-core kernels that ran out of time (0 in a healthy process).
unsigned wproj_tc_timeouts();
// Bounded mbarrier waits of the bulk-copy Gram-Schmidt pipelines and grid barriers of the fused
// Krylov kernel that ran out (0 in a healthy run).
unsigned bulk_timeouts();
// The same two counters read on `st` into pinned host memory: host2[0] tensor-core kernels,
// host2[1] bulk-copy pipelines and grid barriers (valid once `st` is synchronised).
void enqueue_timeout_read(unsigned *host2, cudaStream_t st);

// Bound of the waits a kernel makes on other parts of the GPU: the stage waits of the
// tensor-core and bulk-copy pipelines and the grid barriers of the fused Krylov kernel, in
// milliseconds at the GB300's 2.07 GHz clock (default 2000).  A wait that runs out makes its
// kernel stop and return, and counts in the timeout counters.  The drain waits, where a kernel
// waits for its own copies and tensor-core operations in flight before it frees TMEM and exits,
// keep a fixed bound of about two seconds whatever this is set to.
void set_wait_limit_ms(double ms);
double wait_limit_ms();
// Copies the process's wait limit to the current device if it differs from what that device
// holds (a synchronous copy: never call it while a stream capture is open on this thread).
int push_wait_limit();
// The tensor-core translation unit's copy of the limit (clock cycles) on the current device.
int push_wait_limit_tc(long long cycles);

// out1 (and out2 if non-null) = alpha_s * in; zeros when the system broke down.
template <class R>
void launch_scale(int n, const typename CT<R>::t *in, size_t strideI, typename CT<R>::t *out1, size_t strideO1,
                  typename CT<R>::t *out2, size_t strideO2, const int *act, int nsys, const SysState *state,
                  bool honour_broken, cudaStream_t st);

// Cycle-end combinations: r -= [W V] t ; x += rho_abs [Z V] y ; reduce ||r||^2, finish FIN_RESIDUAL.
template <class R>
void launch_combine(int n, int kk, int m, const typename CT<R>::t *W, const typename CT<R>::t *Z,
                    const typename CT<R>::t *V, size_t strideV, typename CT<R>::t *r, size_t strideR,
                    typename CT<R>::t *x, size_t strideX, const double2 *t, const double2 *y, size_t strideC,
                    const int *act, int nsys, double2 *partials, unsigned *tickets, SysState *state, cudaStream_t st);

// Batches of four or more systems with a deflation segment take a grouped form of the cycle-end
// combination (W and Z loaded once for four systems); 0 returns them to one system a CTA.
void set_combine_group(int on);
int combine_group();
// The refined form's FP64 residual beside the next cycle's deflation loop, on its own stream,
// on about ctas_per_sm CTAs an SM (0, the default: the residual before the loop).  ctas_per_sm < 0 only
// reads; returns the previous setting.
int set_overlap_residual(int ctas_per_sm);
int overlap_residual();
// Z_new[t] = [Z V] vs[:, t] for t < k, plus squared norms into znorm2 (k doubles).
// V: basis of system 0 (system s at V + s*strideV); the lead system is read from device memory.
template <class R>
void launch_zupdate(int n, int kk, int m, int k, const typename CT<R>::t *Z, const typename CT<R>::t *V,
                    size_t strideV, const int *lead, const double2 *vs, typename CT<R>::t *Znew, double2 *partials,
                    unsigned *ticket, double *znorm2, cudaStream_t st);
// Z[t] = Znew[t] / sqrt(znorm2[t]).
template <class R>
void launch_znormalise(int n, int k, const typename CT<R>::t *Znew, const double *znorm2, typename CT<R>::t *Z,
                       cudaStream_t st);

// Batched least squares min ||H_s y - g_s|| (FP64 Givens), t_s = H_s y_s.
void launch_ls(int m, const double2 *H, size_t strideH, const double2 *g, double2 *y, double2 *t, size_t strideC,
               const int *act, int nsys, cudaStream_t st);
// Right singular vectors of the k smallest singular values of H ((m+1) x m) in one CTA: FP32
// pivoted QR and one-sided Jacobi, then a double-float polar correction and restricted Jacobi
// (about 1e-13).  vs: m x k column-major, vector t for the (m-k+t)-th largest value; sigma: m
// values (descending); work: global scratch of svd_smem_bytes(m) = 3*m*(m+1) double2.
// H: Hessenberg of system 0 (system s at H + s*strideH); the lead system is read from device memory.
// sweeps: 1000 * (FP32 sweeps, +100 when the unpivoted fallback ran) + double-float sweeps.
void launch_svd_smallest(int m, int k, const double2 *H, size_t strideH, const int *lead, double2 *vs, double *sigma,
                         double2 *work, int *sweeps, cudaStream_t st);
size_t svd_smem_bytes(int m);

// SELL-32 sparse matrix times a batch of vectors: y_s = A x_s over the active systems.
constexpr int SELL_PATTERN = 8;   // most distinct column offsets stored as a pattern
// Column offsets of a pattern-stored slice, passed to the operator kernels by value.
struct SellPattern {
    const unsigned char *uniform;
    int off[SELL_PATTERN];
};
struct SellMatrix {
    int n;              // rows
    int nslices;        // ceil(n/32)
    const int *slice_ptr;   // nslices+1 offsets (entries), int32
    const int *cols;        // padded column indices
    const void *vals;       // padded values (float2 or double2)
    long nnz;               // non-zeros of the source matrix (for algorithmic byte counts)
    const unsigned char *uniform = nullptr;   // per slice: 1 = column of entry e is row + pat[e]
    int npat = 0;                              // offset pattern (0: none)
    int pat[SELL_PATTERN] = {};
    // Structured-grid form (null: none): the same matrix as coefficient planes on a gx x gy x gz
    // grid, plane p = A[r][r + off_p] for every row r, offsets ascending (-P, -Q, -1, 0, +1, +Q,
    // +P with Q = gx, P = gx gy; 2D (gz = 1): the middle five), values of the same type as `vals`.
    const void *grid = nullptr;
    int gx = 0, gy = 0, gz = 0;
    unsigned greal = 0;   // bit p: every value of plane p has a zero imaginary part
    unsigned preal = 0;   // bit e: entry e of every pattern-stored slice has a zero imaginary part
};
// Process-wide switch for the structured-grid operator kernel (on by default); launch_spmm
// takes the SELL kernels when it is off or the matrix has no grid form.  grid_batch: systems a
// thread of a launch over several systems (1, 2 or 4); 0 (default) keeps those launches on the
// SELL kernel.
void set_grid_operator(int enable);
int grid_operator();
void set_grid_batch(int sg);
int grid_batch();
// Matrix-free constant-coefficient stencil on an nx x ny x nz grid (nz = 1: 5-point 2D),
// unknowns numbered i + nx (j + ny l), Dirichlet boundary (neighbours outside are dropped):
//   y = d x + wx (x[i-1] + x[i+1]) + wy (x[j-1] + x[j+1]) + wz (x[l-1] + x[l+1]).
struct Stencil7 {
    int nx, ny, nz;
    double2 d, wx, wy, wz;
};
// `scale` / vout: the pending normalisation, as for launch_spmm.
template <class R>
void launch_stencil(const Stencil7 &S, const typename CT<R>::t *x, size_t strideX, typename CT<R>::t *y,
                    size_t strideY, const int *act, int nsys, cudaStream_t st, const SysState *scale = nullptr,
                    typename CT<R>::t *vout = nullptr, size_t strideVO = 0);

// With `scale` (the pending normalisation): x holds the unnormalised Krylov vectors w_s, y_s =
// a_s (A w_s) and v_s = a_s w_s (zero after a breakdown) is written to vout (a_s = scale[s].alpha).
template <class R>
void launch_spmm(const SellMatrix &A, const typename CT<R>::t *x, size_t strideX, typename CT<R>::t *y,
                 size_t strideY, const int *act, int nsys, cudaStream_t st, const SysState *scale = nullptr,
                 typename CT<R>::t *vout = nullptr, size_t strideVO = 0);

// The Krylov loop of a restart cycle for one system act[0] with a SELL operator (complex128 or
// double-float) as one cooperative kernel, CTA b on SELL slice b; partials: the engine's scratch
// (G x qmax x 2 + G x 3 doubles), bar: 2 unsigned (zeroed here).  Returns false, launching
// nothing, when it does not apply (complex64, more slices than CTAs resident at once, scratch).
template <class R>
bool launch_krylov_small(int n, int kk, int m, const SellMatrix &A, const typename CT<R>::t *W,
                         typename CT<R>::t *V, size_t strideV, const int *act, SysState *state, double2 *H,
                         size_t strideH, double2 *coef, size_t strideC, double *partials, int qmax, unsigned *bar,
                         double tol, bool compat_eye, cudaStream_t st);

// One system's Krylov loop in the many-system persistent launch (launch_krylov_multi): its
// operator (SELL-32), its operator's shared deflation vectors, its basis with v_0 normalised,
// a scratch vector, its state, Hessenberg and coefficients, and its share of the launch's CTAs
// (cta0 .. cta0 + ncta - 1) with partial sums and a barrier counter of its own.
template <class R> struct KrylovJob {
    using C = typename CT<R>::t;
    int n, nslices, kk, m, compat_eye, qmax, cta0, ncta;
    double tol;
    const int *slice_ptr, *cols;
    const C *vals;          // the job's operator
    const C *W;             // its operator's shared deflation vectors (kk x n)
    C *V;                   // the system's basis ((m + 1) x n, v_0 normalised)
    C *y;                   // the system's scratch vector (n)
    SysState *state;
    double2 *H;             // the system's Hessenberg (ld m + 1)
    double2 *coef;          // the system's projection coefficients
    double *part;           // ncta x qmax x 2 projection partials, then ncta x 3 norm partials
    unsigned *bar;          // the job's barrier counter (zeroed before the launch)
};
// CTAs of the many-system launch that fit on the current device at once (the launch is
// cooperative: every CTA resident).
int krylov_multi_resident();
// The Krylov loops of njobs systems (jobs and cta_job, the job of each CTA, in device memory;
// every job's barrier counter and *abort zeroed before it on `st`) as one cooperative launch of
// ctas CTAs.  algorithmic_bytes: booked to the update class when profiling.
template <class R>
int launch_krylov_multi(const KrylovJob<R> *jobs, const int *cta_job, int ctas, int *abort, double algorithmic_bytes,
                        cudaStream_t st);
// Algorithmic bytes of one system's Krylov loop (operator products, projections, updates).
double krylov_loop_bytes(const SellMatrix &A, size_t vs, int kk, int m);

// The FP64 residual's row: acc - sum_e A[row][e] x[col_e].  A pattern-stored slice adds its
// complex pattern entries (idx[0..NCX-1]) with four FP64 FMAs each, then its real ones (zero
// imaginary part in every pattern-stored slice, decided on the host) with two; the FP64 pipe
// bounds this product on GB300 and a 7-point Helmholtz row goes from 28 FMAs to 16.  Both loops
// have compile-time trip counts (nothing predicated; the entry list stays in parameter space).
// Other slices take the SELL loop.  Every residual kernel uses it, so they agree bit for bit.
struct ResidPattern {
    const unsigned char *uniform;   // per slice: pattern-stored (null: none)
    int idx[SELL_PATTERN];          // pattern entries, complex ones first
    int off[SELL_PATTERN];          // column offset of entry idx[j]
};
// Fills rp for A and returns the number of complex entries, or -1 when every slice takes the
// SELL loop (no pattern, or no real entry).
int resid_pattern(const SellMatrix &A, ResidPattern &rp);
// Calls f(NCX, WID) with compile-time constants for the instantiated shapes (5- and 7-entry
// patterns with up to two complex entries), or f(0, 0) (the SELL loop).
template <class F> void resid_dispatch(int npat, int ncx, F &&f) {
    using std::integral_constant;
    if (npat == 7 && ncx == 1) f(integral_constant<int, 1>{}, integral_constant<int, 7>{});
    else if (npat == 7 && ncx == 0) f(integral_constant<int, 0>{}, integral_constant<int, 7>{});
    else if (npat == 7 && ncx == 2) f(integral_constant<int, 2>{}, integral_constant<int, 7>{});
    else if (npat == 5 && ncx == 1) f(integral_constant<int, 1>{}, integral_constant<int, 5>{});
    else if (npat == 5 && ncx == 0) f(integral_constant<int, 0>{}, integral_constant<int, 5>{});
    else if (npat == 5 && ncx == 2) f(integral_constant<int, 2>{}, integral_constant<int, 5>{});
    else f(integral_constant<int, 0>{}, integral_constant<int, 0>{});
}
#ifdef __CUDACC__
template <int NCX, int WID>
__device__ __forceinline__ double2 resid_row(double2 acc, long row, const int *__restrict__ slice_ptr,
                                             const int *__restrict__ cols, const double2 *__restrict__ vals,
                                             const double2 *__restrict__ x, const ResidPattern &rp) {
    const int slice = (int)(row >> 5), lane = (int)(row & 31);
    const int beg = slice_ptr[slice], width = (slice_ptr[slice + 1] - beg) >> 5;
    if (WID > 0 && rp.uniform[slice]) {
#pragma unroll
        for (int j = 0; j < NCX; ++j) {
            const double2 a = vals[beg + rp.idx[j] * 32 + lane], xv = x[row + rp.off[j]];
            acc.x = ::fma(-a.x, xv.x, acc.x);
            acc.x = ::fma(a.y, xv.y, acc.x);
            acc.y = ::fma(-a.x, xv.y, acc.y);
            acc.y = ::fma(-a.y, xv.x, acc.y);
        }
#pragma unroll
        for (int j = NCX; j < WID; ++j) {
            const double a = vals[beg + rp.idx[j] * 32 + lane].x;
            const double2 xv = x[row + rp.off[j]];
            acc.x = ::fma(-a, xv.x, acc.x);
            acc.y = ::fma(-a, xv.y, acc.y);
        }
    } else {
        for (int c = 0; c < width; ++c) {
            const int e = beg + c * 32 + lane;
            const double2 a = vals[e], xv = x[cols[e]];
            acc.x = ::fma(-a.x, xv.x, acc.x);
            acc.x = ::fma(a.y, xv.y, acc.x);
            acc.y = ::fma(-a.x, xv.y, acc.y);
            acc.y = ::fma(-a.y, xv.x, acc.y);
        }
    }
    return acc;
}
#endif

// y_s = b_s - A x_s in FP64 with ||y_s||^2 reduced into state[s].nrm2 (refined form).
// per_sm > 0 caps the grid near per_sm CTAs an SM (to share the SMs with another stream); the
// result is the same bit for bit whatever the cap.
void launch_residual64(const SellMatrix &A, const double2 *b, size_t strideB, const double2 *x, size_t strideX,
                       double2 *r, size_t strideR, const int *act, int nsys, double2 *partials, unsigned *tickets,
                       SysState *state, cudaStream_t st, int per_sm = 0);
// Dense column-major n x n operator (the reference's impOptLS form): y = A x.
template <class R>
void launch_dense_gemv(int n, const typename CT<R>::t *A, const typename CT<R>::t *x, typename CT<R>::t *y,
                       cudaStream_t st);

// Small helpers.
template <class R>
void launch_copy_vec(int n, const typename CT<R>::t *src, size_t strideS, typename CT<R>::t *dst, size_t strideD,
                     const int *act, int nsys, cudaStream_t st);
// x64_s += scale_s * d_s (d complex64/128 inner correction), then d_s = 0.
template <class R>
void launch_refine_update(int n, double2 *x, size_t strideX, typename CT<R>::t *d, size_t strideD,
                          const int *act, int nsys, const SysState *state, cudaStream_t st);
// rhat_s = (R) (r64_s / sqrt(nrm2_s)); also into v0_s (the cycle's first basis vector) unless
// v0 is null.
template <class R>
void launch_demote_unit(int n, const double2 *r64, size_t strideR, typename CT<R>::t *rhat, size_t strideH,
                        typename CT<R>::t *v0, size_t strideV, const int *act, int nsys, const SysState *state,
                        cudaStream_t st);
// Squared norm of each active vector into state[s].nrm2 (and bnorm if set_bnorm).
// mode 0: nrm2 only; 1: also bnorm = ||v||; 2: also rho_abs = ||v|| and alpha = 1/||v||.
template <class R>
void launch_norm(int n, const typename CT<R>::t *v, size_t strideV, const int *act, int nsys, double2 *partials,
                 unsigned *tickets, SysState *state, int mode, cudaStream_t st);
// Deflation block broadcast: H_s[0:kk, 0:kk] = Hd[0:kk, 0:kk] (ld m+1) for each active system.
void launch_broadcast_hdef(int m, int kk, const double2 *Hd, double2 *H, size_t strideH, const int *act, int nsys,
                           cudaStream_t st);

}  // namespace gdmr
