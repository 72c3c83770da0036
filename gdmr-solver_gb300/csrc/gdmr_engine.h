// Host engine of the GB300 DMR solver: the restart cycle over B systems that
// share one operator and one recycled deflation space.
//
// One engine owns every device buffer of a solve (no globals, no managed
// memory, no per-call allocation); all work is enqueued on one stream and the
// host synchronises once per restart cycle, to read the per-system residuals
// that decide convergence.  B = 1 with reference semantics is the drop-in for
// the reference's solverDMR (gDMR.cu:2638-2900); B > 1 with FP64 refinement is
// the batched mixed-precision form.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gdmr_kernels.cuh"

extern "C" {
#include "../../include/gdmr_ext.h"   // status codes GDMR_*
}

namespace gdmr {

void set_last_error(int status, const std::string &msg);
int last_status();
const char *last_error();
// Failure-path testing: the nth device allocation an engine makes from now on fails (0: none).
void inject_alloc_failure(int nth);

// A sparse operator resident on the device in SELL-32 form, with values in
// complex64 and (optionally) complex128 sharing one index structure.
struct DeviceSell {
    int n = 0;
    long nnz = 0;        // non-zeros of the source CSR
    long padded = 0;     // stored entries (slices padded to their widest row)
    int nslices = 0;
    int *slice_ptr = nullptr;
    int *cols = nullptr;
    float2 *vals32 = nullptr;
    double2 *vals64 = nullptr;
    dfc *valsdf = nullptr;   // double-float values of the fp64e form
    int device = 0;
    int band = 0;                      // max |column - row|
    unsigned char *uniform = nullptr;  // per slice: 1 = columns are row + pat[e]
    int npat = 0;                      // offset pattern (0: none)
    int pat[SELL_PATTERN] = {};
    // structured-grid coefficient planes per precision (null: the matrix is not a grid stencil)
    float2 *grid32 = nullptr;
    double2 *grid64 = nullptr;
    dfc *griddf = nullptr;
    int gx = 0, gy = 0, gz = 0;
    unsigned greal = 0;                // bit p: plane p is real (imaginary parts all zero)
    unsigned preal = 0;                // bit e: entry e of every pattern-stored slice is real
    SellMatrix view(const void *v, const void *g) const {
        SellMatrix m{n, nslices, slice_ptr, cols, v, nnz};
        m.uniform = uniform;
        m.npat = npat;
        for (int e = 0; e < SELL_PATTERN; ++e) m.pat[e] = pat[e];
        m.grid = g;
        m.gx = gx;
        m.gy = gy;
        m.gz = gz;
        m.greal = greal;
        m.preal = preal;
        return m;
    }
    SellMatrix view32() const { return view(vals32, grid32); }
    SellMatrix view64() const { return view(vals64, grid64); }
    SellMatrix viewdf() const { return view(valsdf, griddf); }
    int grid_planes() const { return gx == 0 ? 0 : (gz > 1 ? 7 : 5); }
    size_t bytes() const;
};
// Builds the SELL-32 form of a CSR matrix (values interleaved re,im doubles).
int sell_from_csr(DeviceSell &out, int n, const int *rowptr, const int *colidx, const double *vals_ri, bool want32,
                  bool want64, cudaStream_t st, bool wantdf = false);
void sell_free(DeviceSell &s);
// Host check of a CSR matrix for the structured-grid form: dims <- {nx, ny, nz}, zeros if none.
int csr_grid_form(int n, const int *rowptr, const int *colidx, const double *vals_ri, int dims[3]);

// Operator seen by an engine of precision R.
template <class R> struct Operator {
    using C = typename CT<R>::t;
    enum Kind { NONE, HOOK, SELL, DENSE, STENCIL } kind = NONE;
    Stencil7 stencil{};             // STENCIL: matrix-free constant-coefficient operator
    void (*hook)(void) = nullptr;   // reference hook: applies A in place to `ext`
    C *ext = nullptr;
    SellMatrix sell{};
    const C *dense = nullptr;      // column-major n x n
};

// One restart cycle of a reference-semantics solve, as the host saw it.
struct CycleRecord {
    double rho = 0;       // ||r_new|| / ||r_old|| of the cycle (the recursion's reduction factor)
    double rel_res = 0;   // the recursive residual over ||b|| after the cycle
    int kk = 0;           // deflation vectors the cycle used
    int restart = 0;      // 0: started from the residual; else the reference's basis-storage index of
                          // the mid-Krylov vector it restarted from (gDMR.cu:2600-2621)
    int breakdown = 0;    // Krylov step of a breakdown, 0 if none
    int stagnated = 0;    // 1: rho > 0.995, the reference's stagnation flag (gDMR.cu:2506)
};

struct SolveStats {
    int cycles = 0;
    int its = 0;             // reference convention: cycles - 1
    long matvecs = 0;
    double rel_res = 0;      // what solverDMR returns
    double true_rel_res = -1; // FP64 ||b - A x|| / ||b|| when measured
    int status = GDMR_OK;
    int breakdowns = 0;
    double latency_ms = 0;
};

template <class R> class Engine {
  public:
    using C = typename CT<R>::t;
    Engine() = default;
    ~Engine();
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;

    // Allocates every buffer for `capacity` systems of size n, basis m, deflation k.
    int init(int n, int m, int k, int capacity, int device);
    void release();
    bool ready() const { return n_ > 0; }

    Operator<R> op;
    cudaStream_t stream = nullptr;
    bool use_graphs = true;     // capture restart cycles of small systems as CUDA graphs
    bool fused_small = true;    // one small system: the Krylov loop as one cooperative kernel
    bool compat_eye = true;     // reproduce the reference's breakdown identity tail (gDMR.cu:2275)
    // Changes compat_eye; restart-cycle graphs captured with the other setting are dropped.
    void set_compat_eye(bool on) {
        if (on == compat_eye) return;
        compat_eye = on;
        for (auto &g : graphs_) cudaGraphExecDestroy(g.exec);
        graphs_.clear();
    }

    // Reference semantics on system 0 (solverDMR): b, x are device vectors of precision R;
    // x holds x0 on entry and the solution on exit.  With a hook operator x must be the hook's
    // buffer (op.ext).  Returns the reference's return value.
    double solve_reference(int mode, const C *b, C *x, double tol, int mat_rank, SolveStats *stats);

    // FP64-refined batched form, driven one restart cycle at a time so that
    // systems can join and leave between cycles (continuous batching).  Each
    // slot holds b and x in complex128 on the device; every cycle starts from
    // the true FP64 residual b - A64 x, runs one DMR cycle in precision R on
    // the unit residual, and adds the correction to x in FP64.  The SELL
    // operator in `op` is the inner operator; A64 the FP64 one.
    int refine_setup(const SellMatrix &A64);
    // Copies b (and x0, or zeros when null) from device memory into a free slot.
    int refine_admit(int slot, const double2 *b, const double2 *x0, double tol, int max_cycles);
    // Residual check for every active slot, then one cycle for those not done.
    // Slots that finished (converged, cycle cap, non-finite) are appended to `done`.
    int refine_cycle(std::vector<int> *done);
    double2 *slot_x(int s) const { return x64_ + (size_t)s * n_; }
    double2 *slot_b(int s) const { return b64_ + (size_t)s * n_; }
    const SolveStats &slot_stats(int s) const { return slot_[s].stats; }
    int active_count() const { return (int)act_h_.size(); }
    int capacity() const { return cap_; }
    // FP64 relative residual ||b_s - A64 x_s|| / ||b_s|| of arbitrary device pairs (s < capacity slots used as scratch).
    int true_residual(int count, const double2 *b, const double2 *x, double *relres);

    // Lockstep driving of several engines, the Krylov loops of all their systems in one launch
    // (the many-operator form, gdmr_multi_solve).  A refined cycle in five parts:
    // multi_residual enqueues the true FP64 residual of the active slots; multi_select
    // synchronises, books the previous cycle, retires finished slots into `done` and returns how
    // many systems run a cycle now; multi_front enqueues the cycle up to its Krylov loop;
    // multi_jobs appends one Krylov job per such system; multi_back waits for the event `after`
    // (the launch) and enqueues the rest of the cycle and the FP64 correction.  SELL operators.
    int multi_residual();
    void restart_vectors(const std::vector<int> &next, int kk);
    int multi_select(std::vector<int> *done);
    int multi_front();
    void multi_jobs(std::vector<KrylovJob<R>> &jobs) const;
    int multi_back(cudaEvent_t after);
    cudaStream_t main_stream() const { return stream; }

    // Deflation basis (k x n, vector-contiguous) between host and device, precision R.
    int import_deflation(const C *host);
    int export_deflation(C *host);
    bool has_deflation() const { return have_z_; }
    void drop_deflation() {
        sync_deflation();
        have_z_ = false;
    }
    // The reference keeps its stagnation counter across solves (gDMR.cu:2646-2655); reset on init.
    int flag_count() const { return flag_count_; }
    // Cycles of the last solve_reference call.
    const std::vector<CycleRecord> &history() const { return hist_; }

    // FP32 and FP64 Jacobi sweeps of the last deflation update (read after a cycle).
    int last_svd_sweeps() const { return svd_sweeps_; }
    int n() const { return n_; }
    int m() const { return m_; }
    int k() const { return k_; }
    size_t device_bytes() const { return bytes_; }

  private:
    int n_ = 0, m_ = 0, k_ = 0, cap_ = 0, dev_ = 0;
    size_t bytes_ = 0;
    std::vector<CycleRecord> hist_;
    // bounded device waits that ran out (process-wide counters, read with every state read):
    // the value at the start of the current solve and the latest one
    unsigned *hto_ = nullptr;     // pinned: [tensor-core, bulk-copy and grid barriers]
    unsigned to_base_ = 0;
    unsigned timeouts_now() const { return hto_ ? hto_[0] + hto_[1] : 0; }
    int begin_solve();            // pushes the wait limit, takes the timeout baseline
    bool timed_out() const { return timeouts_now() != to_base_; }
    bool have_z_ = false;
    int flag_count_ = 0;        // reference kryFlagCountDMR (system 0)
    // device buffers
    C *V_ = nullptr, *W_ = nullptr, *Z_ = nullptr, *Znew_ = nullptr;
    C *R_ = nullptr, *X_ = nullptr, *Y_ = nullptr, *T_ = nullptr, *AZ_ = nullptr;
    double2 *H_ = nullptr, *Hd_ = nullptr, *coef_ = nullptr, *coefD_ = nullptr, *g_ = nullptr, *y_ = nullptr,
            *t_ = nullptr;
    double2 *vs_ = nullptr, *svdwork_ = nullptr, *partials_ = nullptr, *r64_ = nullptr;
    double *sigma_ = nullptr, *znorm2_ = nullptr;
    int *sweeps_ = nullptr;
    unsigned *tickets_ = nullptr;
    unsigned *ks_bar_ = nullptr;   // grid barrier + abort flag of the fused small-system Krylov loop
    SysState *state_ = nullptr, *hstate_ = nullptr;
    int *act_ = nullptr;        // active list (device)
    int *ident_ = nullptr;      // 0..cap (device), ident_[cap] is the deflation pseudo-system
    std::vector<int> act_h_;
    std::vector<void *> allocs_;
    // refined form
    struct Slot {
        bool active = false;
        int loop_flag = 0, flag_count = 0, max_cycles = 0;
        double bnorm = 0, tol = 0;
        SolveStats stats;
    };
    std::vector<Slot> slot_;
    SellMatrix A64_{};
    double2 *b64_ = nullptr, *x64_ = nullptr;
    int kk_prev_ = 0;
    int svd_sweeps_ = 0;
    int hsweeps_ = 0;
    // The deflation-space update (SVD of the lead Hessenberg, Z <- [Z V] Vs) runs on a side
    // stream, overlapped with the rest of the cycle and the next cycle's residual; the main
    // stream joins it before anything writes the basis or reads the new Z.
    cudaStream_t side_ = nullptr;
    cudaEvent_t ev_krylov_ = nullptr, ev_zdone_ = nullptr;
    bool z_pending_ = false;
    double2 *partials_side_ = nullptr;
    unsigned *ticket_side_ = nullptr;
    int sync_deflation();
    // The refined form's FP64 residual can run on its own stream beside the next cycle's
    // deflation loop, which needs only Z (front_done_: the loop is already enqueued).
    cudaStream_t res_ = nullptr;
    cudaEvent_t ev_x_ = nullptr, ev_res_ = nullptr;
    double2 *partials_res_ = nullptr;
    bool front_done_ = false;
    void enqueue_deflation_loop(int kk, long *matvecs);
    bool graph_ok(int nsys) const;
    // restart-cycle graphs (key: deflation dimension, batch size, Z buffer parity, tolerance)
    struct GraphEntry {
        int kk, nsys, zpar;
        double tol;
        cudaGraphExec_t exec;
    };
    std::vector<GraphEntry> graphs_;
    int cycles_run_ = 0, zpar_ = 0, lead_host_ = 0;
    int *lead_dev_ = nullptr;
    int enqueue_cycle(int kk, int nsys, double tol, long *matvecs, bool join);
    int enqueue_front(int kk, int nsys, long *matvecs);
    int enqueue_krylov(int kk, int nsys, double tol, long *matvecs);
    int enqueue_back(int kk, int nsys, bool join);
    // lockstep (many-operator) form: the cycle the last multi_front set up
    int mf_kk_ = 0, mf_nsys_ = 0;
    bool mf_ran_ = false;       // a cycle ran since the last multi_select
    double mf_tol_ = 0;
    std::vector<int> mf_act_;   // the slots of that cycle

    size_t strideV() const { return (size_t)(m_ + 1) * n_; }
    size_t strideH() const { return (size_t)(m_ + 1) * m_; }
    size_t strideC() const { return (size_t)(m_ + 1); }
    int qmax() const { return m_ + 1; }
    C *Vs(int s) const { return V_ + (size_t)s * strideV(); }

    int alloc(void **p, size_t bytes);
    int set_active(const std::vector<int> &act);
    int read_state(int count);
    void apply(const C *x0, size_t strideX, C *y0, size_t strideY, int nsys, long *matvecs);
    C *op_out(int s) const { return op.kind == Operator<R>::HOOK ? op.ext : Y_ + (size_t)s * n_; }
    size_t op_out_stride() const { return op.kind == Operator<R>::HOOK ? 0 : (size_t)n_; }
    // One restart cycle over the active systems with deflation dimension kk; lead
    // selects the system whose Hessenberg updates the shared deflation space.
    int run_cycle(int kk, int nsys, int lead, double tol, long *matvecs);
};

}  // namespace gdmr
