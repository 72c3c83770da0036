// Host engine of the GB300 DMR solver.  See gdmr_engine.h.
#include "gdmr_engine.h"

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace gdmr {

// ----------------------------------------------------------------- errors
namespace {
std::mutex g_err_mu;
int g_status = GDMR_OK;
std::string g_msg = "ok";
}  // namespace

void set_last_error(int status, const std::string &msg) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_status = status;
    g_msg = msg;
}
int last_status() {
    std::lock_guard<std::mutex> lk(g_err_mu);
    return g_status;
}
const char *last_error() {
    static thread_local std::string copy;
    std::lock_guard<std::mutex> lk(g_err_mu);
    copy = g_msg;
    return copy.c_str();
}

namespace {
std::atomic<int> g_alloc_countdown{0};   // > 0: the allocation that takes it to 0 fails
}
void inject_alloc_failure(int nth) { g_alloc_countdown.store(nth > 0 ? nth : 0); }

// NVTX ranges around the phases of a solve (free when no tool is attached).
struct Range {
    explicit Range(const char *name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
};

#define GDMR_CK(call)                                                                                                  \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) {                                                                                       \
            set_last_error(GDMR_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));                            \
            return GDMR_ECUDA;                                                                                         \
        }                                                                                                              \
    } while (0)

// ----------------------------------------------------------------- helper kernels
namespace {

template <class C> __global__ void k_sub(int n, const C *__restrict__ a, const C *__restrict__ b, C *__restrict__ out) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        C u = a[i], v = b[i];
        u.x -= v.x;
        u.y -= v.y;
        out[i] = u;
    }
}

__global__ void k_cycle_reset(const int *__restrict__ act, int nsys, SysState *state, int set_unit) {
    for (int i = threadIdx.x; i < nsys; i += blockDim.x) {
        SysState &st = state[act[i]];
        st.broken = 0;
        if (set_unit) st.rho_abs = 1.0;
    }
}

__global__ void k_state_init(SysState *state, int count) {
    for (int i = threadIdx.x; i < count; i += blockDim.x) {
        SysState z{};
        state[i] = z;
    }
}

template <class C> void sub(int n, const C *a, const C *b, C *out, cudaStream_t st) {
    int blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_sub<C><<<blocks, 256, 0, st>>>(n, a, b, out);
}

}  // namespace

// ----------------------------------------------------------------- SELL build
size_t DeviceSell::bytes() const {
    return sizeof(int) * ((size_t)nslices + 1 + padded) + (size_t)nslices + (vals32 ? sizeof(float2) * padded : 0) +
           (vals64 ? sizeof(double2) * padded : 0) + (valsdf ? sizeof(dfc) * padded : 0) +
           (size_t)grid_planes() * n * ((grid32 ? sizeof(float2) : 0) + (grid64 ? sizeof(double2) : 0) +
                                        (griddf ? sizeof(dfc) : 0));
}

// Checks a CSR matrix's arrays (row pointers from 0 up, non-decreasing; columns in 0..n-1) and
// collects its offset pattern: every distinct column - row, ascending, if there are at most
// SELL_PATTERN of them (else none).
static int csr_offsets(int n, const int *rowptr, const int *colidx, std::vector<int> &pat, const char *who) {
    pat.clear();
    if (n <= 0 || !rowptr || !colidx) {
        set_last_error(GDMR_EINVAL, std::string(who) + ": empty matrix or null arrays");
        return GDMR_EINVAL;
    }
    if (rowptr[0] < 0) {
        set_last_error(GDMR_EINVAL, std::string(who) + ": negative row pointer");
        return GDMR_EINVAL;
    }
    bool over = false;
    for (int r = 0; r < n; ++r) {
        if (rowptr[r + 1] < rowptr[r]) {
            set_last_error(GDMR_EINVAL, std::string(who) + ": row pointers are not non-decreasing");
            return GDMR_EINVAL;
        }
        for (int q = rowptr[r]; q < rowptr[r + 1]; ++q) {
            const int col = colidx[q];
            if (col < 0 || col >= n) {
                set_last_error(GDMR_EINVAL, std::string(who) + ": column index out of range");
                return GDMR_EINVAL;
            }
            if (!over && std::find(pat.begin(), pat.end(), col - r) == pat.end()) {
                pat.push_back(col - r);
                over = pat.size() > (size_t)SELL_PATTERN;
            }
        }
    }
    if (over) pat.clear();
    std::sort(pat.begin(), pat.end());
    return GDMR_OK;
}

// Structured-grid form: the pattern is the 7-point (-P, -Q, -1, 0, 1, Q, P) or 5-point
// (-Q, -1, 0, 1, Q) offset set of a lexicographic grid, nx = Q, P = nx ny, n = P nz, and no
// non-zero couples two rows across the grid's edge (the grid kernel leaves those terms out).
// dims <- {nx, ny, nz}, zeros if the matrix has no such form.
static void grid_form(int n, const int *rowptr, const int *colidx, const double *vals_ri, const std::vector<int> &pat,
                      int dims[3]) {
    dims[0] = dims[1] = dims[2] = 0;
    const int np = (int)pat.size();
    if (np != 7 && np != 5) return;
    const int b = np == 7 ? 1 : 0;
    const long Q = -(long)pat[b], P = np == 7 ? -(long)pat[0] : (long)n;
    bool ok = Q > 1 && pat[b + 1] == -1 && pat[b + 2] == 0 && pat[b + 3] == 1 && pat[b + 4] == Q && P % Q == 0 &&
              n % P == 0 && P / Q > 1;
    if (np == 7) ok = ok && pat[6] == P && n / P > 1;
    if (!ok) return;
    const int gx = (int)Q, gy = (int)(P / Q), gz = (int)(n / P);
    for (int r = 0; r < n; ++r) {
        const int ix = r % gx, iy = (r / gx) % gy, iz = (int)(r / P);
        for (int q = rowptr[r]; q < rowptr[r + 1]; ++q) {
            const long dlt = (long)colidx[q] - r;
            if (vals_ri[2 * (size_t)q] == 0.0 && vals_ri[2 * (size_t)q + 1] == 0.0) continue;
            if ((dlt == -1 && ix == 0) || (dlt == 1 && ix == gx - 1) || (dlt == -Q && iy == 0) ||
                (dlt == Q && iy == gy - 1) || (np == 7 && ((dlt == -P && iz == 0) || (dlt == P && iz == gz - 1))))
                return;
        }
    }
    dims[0] = gx;
    dims[1] = gy;
    dims[2] = gz;
}

int csr_grid_form(int n, const int *rowptr, const int *colidx, const double *vals_ri, int dims[3]) {
    dims[0] = dims[1] = dims[2] = 0;
    std::vector<int> pat;
    const int rc = csr_offsets(n, rowptr, colidx, pat, "csr_grid_form");
    if (rc != GDMR_OK) return rc;
    if (!vals_ri) {
        set_last_error(GDMR_EINVAL, "csr_grid_form: null values");
        return GDMR_EINVAL;
    }
    grid_form(n, rowptr, colidx, vals_ri, pat, dims);
    return GDMR_OK;
}

// SELL-32 with an offset pattern.  When the column offsets (column - row) of all non-zeros form
// a set of at most SELL_PATTERN values (a 5- or 7-point stencil on a lexicographic grid), a
// slice all of whose rows can use every offset (rows whose neighbours stay inside 0..n-1) is
// stored "uniform": entry e of row r is A[r][r + off[e]], zero where A has no such entry, so the
// kernels form the column as r + off[e] instead of loading it (the column-index load, then the
// dependent gather, was the latency chain of the operator kernels).  The explicit column array
// is filled for every slice, so kernels that do not use the pattern read the same matrix.  A
// matrix with the structured-grid form also gets its coefficient planes (SellMatrix::grid).
int sell_from_csr(DeviceSell &out, int n, const int *rowptr, const int *colidx, const double *vals_ri, bool want32,
                  bool want64, cudaStream_t st, bool wantdf) {
    std::vector<int> pat;
    int rc = csr_offsets(n, rowptr, colidx, pat, "sell_from_csr");
    if (rc != GDMR_OK) return rc;
    if (!vals_ri) {
        set_last_error(GDMR_EINVAL, "sell_from_csr: null values");
        return GDMR_EINVAL;
    }
    const int ns = (n + 31) / 32;
    const int np = (int)pat.size();
    std::vector<unsigned char> uni(ns, 0);
    std::vector<int> sp(ns + 1, 0);
    for (int s = 0; s < ns; ++s) {
        int w = 0;
        bool u = np > 0;
        for (int r = s * 32; r < std::min(n, s * 32 + 32); ++r) {
            w = std::max(w, rowptr[r + 1] - rowptr[r]);
            if (np > 0 && (r + pat.front() < 0 || r + pat.back() >= n)) u = false;
        }
        if (u) {
            uni[s] = 1;
            w = np;
        }
        long next = (long)sp[s] + 32L * w;
        if (next > 0x7fffffffL) {
            set_last_error(GDMR_EINVAL, "sell_from_csr: more than 2^31 stored entries");
            return GDMR_EINVAL;
        }
        sp[s + 1] = (int)next;
    }
    const long padded = sp[ns];
    int band = 0;
    std::vector<int> cols(padded);
    std::vector<float2> v32(want32 ? padded : 0);
    std::vector<double2> v64(want64 ? padded : 0);
    std::vector<dfc> vdf(wantdf ? padded : 0);
    auto put = [&](long e, int col, double re, double im) {
        cols[e] = col;
        if (want32) v32[e] = make_float2((float)re, (float)im);
        if (want64) v64[e] = make_double2(re, im);
        if (wantdf) {
            vdf[e].x = dfr(re);
            vdf[e].y = dfr(im);
        }
    };
    for (int s = 0; s < ns; ++s) {
        const int w = (sp[s + 1] - sp[s]) / 32;
        for (int lane = 0; lane < 32; ++lane) {
            const int r = s * 32 + lane;
            const int beg = r < n ? rowptr[r] : 0, len = r < n ? rowptr[r + 1] - rowptr[r] : 0;
            for (int q = beg; q < beg + len; ++q) band = std::max(band, std::abs(colidx[q] - r));
            if (uni[s]) {
                // pattern order; duplicate entries of one column add up, as in CSR
                std::vector<double> re(np, 0.0), im(np, 0.0);
                for (int q = beg; q < beg + len; ++q) {
                    const int e = (int)(std::find(pat.begin(), pat.end(), colidx[q] - r) - pat.begin());
                    re[e] += vals_ri[2 * (size_t)q];
                    im[e] += vals_ri[2 * (size_t)q + 1];
                }
                for (int e = 0; e < np; ++e)
                    put((long)sp[s] + (long)e * 32 + lane, r < n ? r + pat[e] : 0, re[e], im[e]);
            } else {
                for (int c = 0; c < w; ++c) {
                    const long e = (long)sp[s] + (long)c * 32 + lane;
                    if (c < len)
                        put(e, colidx[beg + c], vals_ri[2 * (size_t)(beg + c)], vals_ri[2 * (size_t)(beg + c) + 1]);
                    else
                        put(e, r < n ? r : 0, 0.0, 0.0);
                }
            }
        }
    }
    int gdims[3];
    grid_form(n, rowptr, colidx, vals_ri, pat, gdims);
    const int gx = gdims[0], gy = gdims[1], gz = gdims[2];
    // coefficient planes, duplicates of one column added in CSR order as for uniform slices
    const size_t gsz = gx ? (size_t)np * n : 0;
    std::vector<double> gre(gsz, 0.0), gim(gsz, 0.0);
    if (gx)
        for (int r = 0; r < n; ++r)
            for (int q = rowptr[r]; q < rowptr[r + 1]; ++q) {
                const size_t e = (size_t)(std::find(pat.begin(), pat.end(), colidx[q] - r) - pat.begin());
                gre[e * n + r] += vals_ri[2 * (size_t)q];
                gim[e * n + r] += vals_ri[2 * (size_t)q + 1];
            }
    DeviceSell d;
    // a failed allocation or copy frees what was already allocated
#define SELL_CK_(call)                                                                                                 \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) {                                                                                       \
            sell_free(d);                                                                                              \
            set_last_error(GDMR_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));                            \
            return GDMR_ECUDA;                                                                                         \
        }                                                                                                              \
    } while (0)
    d.n = n;
    d.nnz = rowptr[n] - rowptr[0];
    d.padded = padded;
    d.nslices = ns;
    d.band = band;
    d.npat = np;
    for (int e = 0; e < np; ++e) d.pat[e] = pat[e];
    // pattern entries that are real in every pattern-stored slice (conservatively: no CSR value
    // stored there has a non-zero imaginary part; padding zeros are real)
    if (np > 0) {
        unsigned real = (1u << np) - 1u;
        for (int s = 0; s < ns && real; ++s) {
            if (!uni[s]) continue;
            for (int r = s * 32; r < std::min(n, s * 32 + 32); ++r)
                for (int q = rowptr[r]; q < rowptr[r + 1]; ++q)
                    if (vals_ri[2 * (size_t)q + 1] != 0.0) {
                        const int e = (int)(std::find(pat.begin(), pat.end(), colidx[q] - r) - pat.begin());
                        real &= ~(1u << e);
                    }
        }
        d.preal = real;
    }
    SELL_CK_(cudaGetDevice(&d.device));
    SELL_CK_(cudaMalloc(&d.slice_ptr, sizeof(int) * (ns + 1)));
    SELL_CK_(cudaMalloc(&d.cols, sizeof(int) * std::max<long>(padded, 1)));
    SELL_CK_(cudaMalloc(&d.uniform, (size_t)ns));
    SELL_CK_(cudaMemcpyAsync(d.slice_ptr, sp.data(), sizeof(int) * (ns + 1), cudaMemcpyHostToDevice, st));
    SELL_CK_(cudaMemcpyAsync(d.cols, cols.data(), sizeof(int) * padded, cudaMemcpyHostToDevice, st));
    SELL_CK_(cudaMemcpyAsync(d.uniform, uni.data(), (size_t)ns, cudaMemcpyHostToDevice, st));
    if (want32) {
        SELL_CK_(cudaMalloc(&d.vals32, sizeof(float2) * std::max<long>(padded, 1)));
        SELL_CK_(cudaMemcpyAsync(d.vals32, v32.data(), sizeof(float2) * padded, cudaMemcpyHostToDevice, st));
    }
    if (want64) {
        SELL_CK_(cudaMalloc(&d.vals64, sizeof(double2) * std::max<long>(padded, 1)));
        SELL_CK_(cudaMemcpyAsync(d.vals64, v64.data(), sizeof(double2) * padded, cudaMemcpyHostToDevice, st));
    }
    if (wantdf) {
        SELL_CK_(cudaMalloc(&d.valsdf, sizeof(dfc) * std::max<long>(padded, 1)));
        SELL_CK_(cudaMemcpyAsync(d.valsdf, vdf.data(), sizeof(dfc) * padded, cudaMemcpyHostToDevice, st));
    }
    if (gx) {
        d.gx = gx;
        d.gy = gy;
        d.gz = gz;
        // real planes (the off-diagonals of a Helmholtz operator): the kernels skip the products
        // with their zero imaginary parts, which add nothing
        for (int e = 0; e < np; ++e) {
            bool real = true;
            for (int r = 0; real && r < n; ++r) real = gim[(size_t)e * n + r] == 0.0;
            if (real) d.greal |= 1u << e;
        }
        // one precision at a time, each host copy released after its upload
        if (want32) {
            std::vector<float2> g(gsz);
            for (size_t e = 0; e < gsz; ++e) g[e] = make_float2((float)gre[e], (float)gim[e]);
            SELL_CK_(cudaMalloc(&d.grid32, sizeof(float2) * gsz));
            SELL_CK_(cudaMemcpyAsync(d.grid32, g.data(), sizeof(float2) * gsz, cudaMemcpyHostToDevice, st));
            SELL_CK_(cudaStreamSynchronize(st));
        }
        if (want64) {
            std::vector<double2> g(gsz);
            for (size_t e = 0; e < gsz; ++e) g[e] = make_double2(gre[e], gim[e]);
            SELL_CK_(cudaMalloc(&d.grid64, sizeof(double2) * gsz));
            SELL_CK_(cudaMemcpyAsync(d.grid64, g.data(), sizeof(double2) * gsz, cudaMemcpyHostToDevice, st));
            SELL_CK_(cudaStreamSynchronize(st));
        }
        if (wantdf) {
            std::vector<dfc> g(gsz);
            for (size_t e = 0; e < gsz; ++e) {
                g[e].x = dfr(gre[e]);
                g[e].y = dfr(gim[e]);
            }
            SELL_CK_(cudaMalloc(&d.griddf, sizeof(dfc) * gsz));
            SELL_CK_(cudaMemcpyAsync(d.griddf, g.data(), sizeof(dfc) * gsz, cudaMemcpyHostToDevice, st));
            SELL_CK_(cudaStreamSynchronize(st));
        }
    }
    SELL_CK_(cudaStreamSynchronize(st));
#undef SELL_CK_
    sell_free(out);
    out = d;
    return GDMR_OK;
}

void sell_free(DeviceSell &s) {
    if (s.slice_ptr) cudaFree(s.slice_ptr);
    if (s.cols) cudaFree(s.cols);
    if (s.uniform) cudaFree(s.uniform);
    if (s.vals32) cudaFree(s.vals32);
    if (s.vals64) cudaFree(s.vals64);
    if (s.valsdf) cudaFree(s.valsdf);
    if (s.grid32) cudaFree(s.grid32);
    if (s.grid64) cudaFree(s.grid64);
    if (s.griddf) cudaFree(s.griddf);
    s = DeviceSell();
}

// ----------------------------------------------------------------- engine
template <class R> Engine<R>::~Engine() { release(); }

template <class R> int Engine<R>::alloc(void **p, size_t bytes) {
    int c = g_alloc_countdown.load();
    while (c > 0 && !g_alloc_countdown.compare_exchange_weak(c, c - 1)) {
    }
    if (c == 1) {   // an injected failure (failure-path tests)
        *p = nullptr;
        set_last_error(GDMR_ENOMEM, std::string("cudaMalloc of ") + std::to_string(bytes) +
                                        " bytes: injected allocation failure");
        return GDMR_ENOMEM;
    }
    cudaError_t e = cudaMalloc(p, bytes > 0 ? bytes : 16);
    if (e != cudaSuccess) {
        set_last_error(GDMR_ENOMEM, std::string("cudaMalloc of ") + std::to_string(bytes) + " bytes: " +
                                        cudaGetErrorString(e));
        return GDMR_ENOMEM;
    }
    allocs_.push_back(*p);
    bytes_ += bytes;
    return GDMR_OK;
}

template <class R> void Engine<R>::release() {
    for (auto &g : graphs_) cudaGraphExecDestroy(g.exec);
    graphs_.clear();
    cycles_run_ = 0;
    zpar_ = 0;
    lead_dev_ = nullptr;
    if (side_) {
        cudaStreamSynchronize(side_);
        cudaStreamDestroy(side_);
        side_ = nullptr;
    }
    if (res_) {
        cudaStreamSynchronize(res_);
        cudaStreamDestroy(res_);
        res_ = nullptr;
    }
    if (ev_krylov_) cudaEventDestroy(ev_krylov_);
    if (ev_zdone_) cudaEventDestroy(ev_zdone_);
    if (ev_x_) cudaEventDestroy(ev_x_);
    if (ev_res_) cudaEventDestroy(ev_res_);
    ev_krylov_ = ev_zdone_ = ev_x_ = ev_res_ = nullptr;
    z_pending_ = false;
    front_done_ = false;
    partials_res_ = nullptr;
    if (partials_) unregister_scratch(partials_);
    partials_side_ = nullptr;
    ticket_side_ = nullptr;
    ks_bar_ = nullptr;
    for (void *p : allocs_) cudaFree(p);
    allocs_.clear();
    if (hstate_) cudaFreeHost(hstate_);
    hstate_ = nullptr;
    if (hto_) cudaFreeHost(hto_);
    hto_ = nullptr;
    hist_.clear();
    V_ = W_ = Z_ = Znew_ = R_ = X_ = Y_ = T_ = AZ_ = nullptr;
    H_ = Hd_ = coef_ = coefD_ = g_ = y_ = t_ = vs_ = svdwork_ = partials_ = r64_ = b64_ = x64_ = nullptr;
    slot_.clear();
    act_h_.clear();
    sigma_ = znorm2_ = nullptr;
    sweeps_ = nullptr;
    tickets_ = nullptr;
    state_ = nullptr;
    act_ = ident_ = nullptr;
    n_ = m_ = k_ = cap_ = 0;
    bytes_ = 0;
    have_z_ = false;
}

template <class R> int Engine<R>::init(int n, int m, int k, int capacity, int device) {
    release();
    if (n <= 0 || m < 2 || k < 0 || m - k < 2 || capacity < 1) {
        set_last_error(GDMR_EINVAL, "engine: need n > 0, basisDim - deflatDim >= 2, capacity >= 1");
        return GDMR_EINVAL;
    }
    if (m > 160) {
        set_last_error(GDMR_EINVAL, "engine: basisDim above 160 is not supported (device least squares)");
        return GDMR_EINVAL;
    }
    GDMR_CK(cudaSetDevice(device));
    n_ = n; m_ = m; k_ = k; cap_ = capacity; dev_ = device;
    const size_t vn = (size_t)n * sizeof(C);
    int rc = GDMR_OK;
#define A_(ptr, bytes)                                                                                                 \
    if ((rc = alloc((void **)&ptr, bytes)) != GDMR_OK) { release(); return rc; }
    A_(V_, vn * (m + 1) * capacity);
    A_(W_, vn * std::max(k, 1));
    A_(Z_, vn * std::max(k, 1));
    A_(Znew_, vn * std::max(k, 1));
    A_(R_, vn * capacity);
    A_(X_, vn * capacity);
    A_(Y_, vn * capacity);
    A_(T_, vn * capacity);
    A_(AZ_, vn);
    A_(H_, sizeof(double2) * strideH() * capacity);
    A_(Hd_, sizeof(double2) * strideH());
    A_(coef_, sizeof(double2) * strideC() * (capacity + 1));
    A_(coefD_, sizeof(double2) * strideC());
    A_(g_, sizeof(double2) * strideC() * capacity);
    A_(y_, sizeof(double2) * strideC() * capacity);
    A_(t_, sizeof(double2) * strideC() * capacity);
    A_(vs_, sizeof(double2) * (size_t)m * std::max(k, 1));
    A_(svdwork_, sizeof(double2) * 3 * (size_t)m * (m + 1));
    A_(sigma_, sizeof(double) * m);
    A_(znorm2_, sizeof(double) * std::max(k, 1));
    A_(sweeps_, sizeof(int));
    A_(partials_, sizeof(double) * scratch_doubles(qmax() + 16, capacity + 1, n));
    register_scratch(partials_, scratch_doubles(qmax() + 16, capacity + 1, n));
    A_(tickets_, sizeof(unsigned) * (capacity + 1));
    A_(state_, sizeof(SysState) * (capacity + 1));
    A_(act_, sizeof(int) * (capacity + 1));
    // 0..max(cap, k - 1): the batch's identity list (entry cap is the deflation pseudo-system)
    // and the deflation loop's batched operator product over the k vectors of Z
    const int nident = std::max(capacity + 1, k);
    A_(ident_, sizeof(int) * nident);
    A_(partials_side_, sizeof(double) * scratch_doubles(16, 1, 1));
    A_(partials_res_, sizeof(double) * scratch_doubles(0, capacity + 1, 1));
    A_(lead_dev_, sizeof(int));
    A_(ticket_side_, sizeof(unsigned));
    A_(ks_bar_, 2 * sizeof(unsigned));
#undef A_
    if (cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&res_, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev_krylov_, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev_zdone_, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev_x_, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev_res_, cudaEventDisableTiming) != cudaSuccess) {
        release();
        set_last_error(GDMR_ECUDA, "engine: side stream or events");
        return GDMR_ECUDA;
    }
    if (cudaMallocHost(&hstate_, sizeof(SysState) * (capacity + 1)) != cudaSuccess ||
        cudaMallocHost(&hto_, 2 * sizeof(unsigned)) != cudaSuccess) {
        release();
        set_last_error(GDMR_ENOMEM, "engine: pinned host state");
        return GDMR_ENOMEM;
    }
    hto_[0] = hto_[1] = 0;
    std::vector<int> id(nident);
    for (int i = 0; i < nident; ++i) id[i] = i;
    GDMR_CK(cudaMemcpy(ident_, id.data(), sizeof(int) * nident, cudaMemcpyHostToDevice));
    GDMR_CK(cudaMemset(tickets_, 0, sizeof(unsigned) * (capacity + 1)));
    GDMR_CK(cudaMemset(ticket_side_, 0, sizeof(unsigned)));
    GDMR_CK(cudaMemset(V_, 0, vn * (m + 1) * capacity));
    GDMR_CK(cudaMemset(Z_, 0, vn * std::max(k, 1)));
    GDMR_CK(cudaMemset(X_, 0, vn * capacity));
    k_state_init<<<1, 256>>>(state_, capacity + 1);
    GDMR_CK(cudaGetLastError());
    GDMR_CK(cudaDeviceSynchronize());
    flag_count_ = 0;
    have_z_ = false;
    return GDMR_OK;
}

template <class R> int Engine<R>::set_active(const std::vector<int> &act) {
    act_h_ = act;
    if (!act.empty()) GDMR_CK(cudaMemcpyAsync(act_, act.data(), sizeof(int) * act.size(), cudaMemcpyHostToDevice, stream));
    return GDMR_OK;
}

template <class R> int Engine<R>::read_state(int count) {
    GDMR_CK(cudaMemcpyAsync(hstate_, state_, sizeof(SysState) * count, cudaMemcpyDeviceToHost, stream));
    if (k_ > 0) GDMR_CK(cudaMemcpyAsync(&hsweeps_, sweeps_, sizeof(int), cudaMemcpyDeviceToHost, stream));
    enqueue_timeout_read(hto_, stream);
    GDMR_CK(cudaStreamSynchronize(stream));
    svd_sweeps_ = hsweeps_;
    if (profile_enabled()) profile_flush();
    return GDMR_OK;
}

// A solve begins: the process's wait limit goes to this device and the timeout counters are
// read, so that a wait that runs out during the solve shows up as a rise above this baseline.
template <class R> int Engine<R>::begin_solve() {
    if (push_wait_limit() != 0) {
        set_last_error(GDMR_ECUDA, "engine: copying the wait limit to the device failed");
        return GDMR_ECUDA;
    }
    enqueue_timeout_read(hto_, stream);
    GDMR_CK(cudaStreamSynchronize(stream));
    to_base_ = timeouts_now();
    return GDMR_OK;
}

// y_s = A x_s for the active systems (nsys of them; the active list is act_).
template <class R>
void Engine<R>::apply(const C *x0, size_t strideX, C *y0, size_t strideY, int nsys, long *matvecs) {
    *matvecs += nsys;
    switch (op.kind) {
    case Operator<R>::SELL:
        launch_spmm<R>(op.sell, x0, strideX, y0, strideY, act_, nsys, stream);
        break;
    case Operator<R>::STENCIL:
        launch_stencil<R>(op.stencil, x0, strideX, y0, strideY, act_, nsys, stream);
        break;
    case Operator<R>::DENSE:
        for (int i = 0; i < nsys; ++i) {
            const int s = act_h_[i];
            launch_dense_gemv<R>(n_, op.dense, x0 + s * strideX, y0 + s * strideY, stream);
        }
        break;
    case Operator<R>::HOOK: {
        // the hook reads and overwrites its own buffer in place, on this stream
        if (x0 != op.ext) cudaMemcpyAsync(op.ext, x0, sizeof(C) * n_, cudaMemcpyDeviceToDevice, stream);
        op.hook();
        if (y0 != op.ext) cudaMemcpyAsync(y0, op.ext, sizeof(C) * n_, cudaMemcpyDeviceToDevice, stream);
        break;
    }
    default:
        break;
    }
}

template <class R> int Engine<R>::sync_deflation() {
    if (!z_pending_) return GDMR_OK;
    GDMR_CK(cudaStreamWaitEvent(stream, ev_zdone_, 0));
    std::swap(Z_, Znew_);
    zpar_ ^= 1;
    have_z_ = true;
    z_pending_ = false;
    return GDMR_OK;
}

template <class R> int Engine<R>::run_cycle(int kk, int nsys, int lead, double tol, long *matvecs) {
    if (sync_deflation() != GDMR_OK) return GDMR_ECUDA;
    lead_host_ = lead;
    GDMR_CK(cudaMemcpyAsync(lead_dev_, &lead_host_, sizeof(int), cudaMemcpyHostToDevice, stream));
    // a cycle whose deflation loop is already enqueued runs eagerly (a graph holds whole cycles)
    const bool graphable = !front_done_ && graph_ok(nsys);
    ++cycles_run_;
    if (!graphable) return enqueue_cycle(kk, nsys, tol, matvecs, false);
    const int zpar = zpar_;
    cudaGraphExec_t exec = nullptr;
    for (auto &g : graphs_)
        if (g.kk == kk && g.nsys == nsys && g.zpar == zpar && g.tol == tol) exec = g.exec;
    if (!exec) {
        if (graphs_.size() >= 32) {
            for (auto &g : graphs_) cudaGraphExecDestroy(g.exec);
            graphs_.clear();
        }
        GDMR_CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        set_capturing(true);
        long mv = 0;
        const bool hz = have_z_, zp = z_pending_;
        int rc = enqueue_cycle(kk, nsys, tol, &mv, true);
        set_capturing(false);
        have_z_ = hz;
        z_pending_ = zp;
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(stream, &graph);
        if (rc != GDMR_OK) { if (graph) cudaGraphDestroy(graph); return rc; }
        if (e != cudaSuccess) {
            set_last_error(GDMR_ECUDA, std::string("restart-cycle capture: ") + cudaGetErrorString(e));
            return GDMR_ECUDA;
        }
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            set_last_error(GDMR_ECUDA, std::string("restart-cycle graph: ") + cudaGetErrorString(e));
            return GDMR_ECUDA;
        }
        graphs_.push_back(GraphEntry{kk, nsys, zpar, tol, exec});
    }
    GDMR_CK(cudaGraphLaunch(exec, stream));
    // the graph joins the deflation update into the main stream: the new Z is ready in order
    *matvecs += kk + (long)nsys * (m_ - kk);
    if (k_ > 0) {
        std::swap(Z_, Znew_);
        zpar_ ^= 1;
        have_z_ = true;
        z_pending_ = false;
    }
    return GDMR_OK;
}

// CUDA graphs pay off where launch overhead is comparable to the work: small n x batch.  The
// first two cycles of an engine run eagerly: they tune the kernels of both cycle shapes
// (without and with the deflation space) before anything is captured.
template <class R> bool Engine<R>::graph_ok(int nsys) const {
    return use_graphs && op.kind != Operator<R>::HOOK && !profile_enabled() && cycles_run_ > 1 &&
           (long)n_ * nsys <= (1L << 20);
}

template <class R> int Engine<R>::enqueue_cycle(int kk, int nsys, double tol, long *matvecs, bool join) {
    int rc = enqueue_front(kk, nsys, matvecs);
    if (rc != GDMR_OK) return rc;
    if ((rc = enqueue_krylov(kk, nsys, tol, matvecs)) != GDMR_OK) return rc;
    return enqueue_back(kk, nsys, join);
}

// The cycle up to its Krylov loop: H cleared, the deflation loop (W = orth(A Z), the shared
// block of H) and v_0 <- (I - W W^H) v_0 / ||.||.
template <class R> int Engine<R>::enqueue_front(int kk, int nsys, long *matvecs) {
    const int n = n_, m = m_;
    const size_t sV = strideV(), sC = strideC();
    const bool hook = op.kind == Operator<R>::HOOK;
    GDMR_CK(cudaMemsetAsync(H_, 0, sizeof(double2) * strideH() * cap_, stream));
    k_cycle_reset<<<1, 256, 0, stream>>>(act_, nsys, state_, 0);
    if (kk > 0) {
        if (!front_done_) enqueue_deflation_loop(kk, matvecs);
        front_done_ = false;
        launch_broadcast_hdef(m, kk, Hd_, H_, strideH(), act_, nsys, stream);
        // v0 <- (I - W W^H) v0 / ||.||  (deflatorDMR(0,0), gDMR.cu:2033-2059)
        launch_mdot<R>(n, W_, kk, nullptr, 0, 0, V_, sV, act_, nsys, partials_, qmax(), tickets_, coef_, sC, state_,
                       false, stream);
        FinishArgs f{};
        f.mode = FIN_UNIT;
        launch_update<R>(n, W_, kk, nullptr, 0, 0, V_, sV, T_, n, act_, nsys, coef_, sC, partials_, tickets_, state_, f,
                         false, stream);
        launch_scale<R>(n, T_, n, V_, sV, hook ? op.ext : nullptr, 0, act_, nsys, state_, false, stream);
    } else if (hook) {
        cudaMemcpyAsync(op.ext, V_, sizeof(C) * n, cudaMemcpyDeviceToDevice, stream);
    }
    GDMR_CK(cudaGetLastError());
    return GDMR_OK;
}

// Deflation loop (arnoldiDMR, gDMR.cu:1823-2030): W_i = orth(A z_i), H[:i+1, i] into Hd_.  It
// reads only Z and writes only W, Hd, T's slot 0 and the shared pseudo-system (state index cap_,
// active list ident_+cap_, tickets_[cap_]); no system's own data.
template <class R> void Engine<R>::enqueue_deflation_loop(int kk, long *matvecs) {
    const int n = n_, m = m_;
    const bool hook = op.kind == Operator<R>::HOOK;
    cudaMemsetAsync(Hd_, 0, sizeof(double2) * strideH(), stream);
    int *pact = ident_ + cap_;
    // SELL and stencil operators: the kk products A z_i are independent, so they run as one
    // batched product straight into W's slots (the matrix read once, not kk times); step i
    // then orthogonalises slot i against the finished slots 0..i-1 and normalises it in place
    const bool batched = op.kind == Operator<R>::SELL || op.kind == Operator<R>::STENCIL;
    if (batched) {
        *matvecs += kk;
        if (op.kind == Operator<R>::SELL) launch_spmm<R>(op.sell, Z_, n, W_, n, ident_, kk, stream);
        else launch_stencil<R>(op.stencil, Z_, n, W_, n, ident_, kk, stream);
    }
    for (int i = 0; i < kk; ++i) {
        C *az = batched ? W_ + (size_t)i * n : (hook ? op.ext : AZ_);
        if (!batched) {
            std::vector<int> keep = act_h_;
            act_h_ = {0};
            apply(Z_ + (size_t)i * n, 0, az, 0, 1, matvecs);
            act_h_ = keep;
        }
        if (i > 0)
            launch_mdot<R>(n, W_, i, nullptr, 0, 0, az, 0, pact, 1, partials_, qmax(), tickets_ + cap_, coefD_, 0,
                           state_, false, stream);
        FinishArgs f{};
        f.mode = FIN_DEFLATION; f.col = i; f.nco = i; f.ldH = m + 1; f.m = m; f.kk = kk;
        f.H = Hd_; f.strideH = 0; f.coef = coefD_; f.strideC = 0;
        launch_update<R>(n, W_, i, nullptr, 0, 0, az, 0, T_, 0, pact, 1, coefD_, 0, partials_, tickets_ + cap_,
                         state_, f, false, stream);
        launch_scale<R>(n, T_, 0, W_ + (size_t)i * n, 0, nullptr, 0, pact, 1, state_, false, stream);
    }
}

// The Krylov loop (gDMR.cu:2069-2328): classical Gram-Schmidt against [W V] in one pass.
template <class R> int Engine<R>::enqueue_krylov(int kk, int nsys, double tol, long *matvecs) {
    const int n = n_, m = m_;
    const size_t sV = strideV(), sC = strideC();
    const bool hook = op.kind == Operator<R>::HOOK;
    // One small system with a SELL operator runs the whole loop as one cooperative kernel.
    const bool fused = nsys == 1 && op.kind == Operator<R>::SELL && fused_small &&
                       launch_krylov_small<R>(n, kk, m, op.sell, W_, V_, sV, act_, state_, H_, strideH(), coef_, sC,
                                              (double *)partials_, qmax(), ks_bar_, tol, compat_eye, stream);
    if (fused) *matvecs += m - kk;
    // With a SELL or stencil operator, the normalisation of v_{j-1} = a w_{j-1} happens inside the operator
    // product of step j (launch_spmm with `scale`), which reads w_{j-1} from T anyway; only the
    // last vector of the cycle is normalised on its own.
    const bool fold = !fused && (op.kind == Operator<R>::SELL || op.kind == Operator<R>::STENCIL);
    for (int j = 1; !fused && j <= m - kk; ++j) {
        const int col = kk + j - 1;
        if (hook) {
            *matvecs += 1;
            op.hook();      // v_{j-1} is already in the hook buffer
        } else if (fold && j > 1) {
            *matvecs += nsys;
            if (op.kind == Operator<R>::SELL)
                launch_spmm<R>(op.sell, T_, n, Y_, n, act_, nsys, stream, state_, V_ + (size_t)(j - 1) * n, sV);
            else
                launch_stencil<R>(op.stencil, T_, n, Y_, n, act_, nsys, stream, state_, V_ + (size_t)(j - 1) * n, sV);
        } else {
            apply(V_ + (size_t)(j - 1) * n, sV, Y_, n, nsys, matvecs);
        }
        const C *w = op_out(0);
        const size_t sW = op_out_stride();
        launch_mdot<R>(n, W_, kk, V_, sV, j, w, sW, act_, nsys, partials_, qmax(), tickets_, coef_, sC, state_, true,
                       stream);
        FinishArgs f{};
        f.mode = FIN_KRYLOV; f.col = col; f.nco = kk + j; f.ldH = m + 1; f.m = m; f.kk = kk;
        f.compat_eye = compat_eye ? 1 : 0; f.tol = tol; f.H = H_; f.strideH = strideH(); f.coef = coef_; f.strideC = sC;
        launch_update<R>(n, W_, kk, V_, sV, j, w, sW, T_, n, act_, nsys, coef_, sC, partials_, tickets_, state_, f, true,
                         stream);
        if (!fold || j == m - kk)
            launch_scale<R>(n, T_, n, V_ + (size_t)j * n, sV, hook ? op.ext : nullptr, 0, act_, nsys, state_, true,
                            stream);
    }
    GDMR_CK(cudaGetLastError());
    return GDMR_OK;
}

// The cycle after its Krylov loop: the deflation-space update on the side stream, g, the
// least squares, the residual and solution combinations.
template <class R> int Engine<R>::enqueue_back(int kk, int nsys, bool join) {
    const int n = n_, m = m_;
    const size_t sV = strideV(), sC = strideC();
    // deflation-space update from the lead system (genDeflatDMR, gDMR.cu:1583-1704), on the
    // side stream: it needs only H_lead and the basis, which nothing below modifies
    if (k_ > 0) {
        GDMR_CK(cudaEventRecord(ev_krylov_, stream));
        GDMR_CK(cudaStreamWaitEvent(side_, ev_krylov_, 0));
        launch_svd_smallest(m, k_, H_, strideH(), lead_dev_, vs_, sigma_, svdwork_, sweeps_, side_);
        launch_zupdate<R>(n, kk, m, k_, Z_, V_, sV, lead_dev_, vs_, Znew_, partials_side_, ticket_side_, znorm2_,
                          side_);
        launch_znormalise<R>(n, k_, Znew_, znorm2_, Znew_, side_);
        GDMR_CK(cudaEventRecord(ev_zdone_, side_));
        z_pending_ = true;
    }
    // g = [W V]^H r (updateTrgCoeffsDMR, gDMR.cu:2334-2408)
    launch_mdot<R>(n, W_, kk, V_, sV, m + 1 - kk, R_, n, act_, nsys, partials_, qmax(), tickets_, g_, sC, state_, false,
                   stream);
    // y = argmin ||H y - g||, t = H y (qrHessArrDMR/qrSolveDMR/hessenbergMultDMR)
    launch_ls(m, H_, strideH(), g_, y_, t_, sC, act_, nsys, stream);
    // r -= [W V] t ; x += rho_abs [Z V] y ; rho = ||r|| (updateAppResDMR, gDMR.cu:2411-2582)
    launch_combine<R>(n, kk, m, W_, Z_, V_, sV, R_, n, X_, n, t_, y_, sC, act_, nsys, partials_, tickets_, state_,
                      stream);
    launch_scale<R>(n, R_, n, R_, n, nullptr, 0, act_, nsys, state_, false, stream);
    // a captured cycle must join the side stream before the capture ends
    if (join && k_ > 0) GDMR_CK(cudaStreamWaitEvent(stream, ev_zdone_, 0));
    GDMR_CK(cudaGetLastError());
    return GDMR_OK;
}

template <class R>
double Engine<R>::solve_reference(int mode, const C *b, C *x, double tol, int mat_rank, SolveStats *stats) {
    SolveStats local;
    SolveStats &S = stats ? *stats : local;
    S = SolveStats();
    const int n = n_, m = m_, k = k_;
    auto fail = [&](double ret) {
        S.status = last_status();
        S.rel_res = ret;
        return ret;
    };
    if (!ready()) {
        set_last_error(GDMR_ENOTINIT, "solver used before initialisation");
        S.status = GDMR_ENOTINIT;
        return 1.0;
    }
    Range range("gdmr solve");
    hist_.clear();
    S.its = mat_rank * mat_rank;
    const bool hook = op.kind == Operator<R>::HOOK;
    if (set_active({0}) != GDMR_OK) return fail(1.0);
    if (begin_solve() != GDMR_OK) return fail(1.0);
    // ends the solve with x~ exported, for the exits after the restart loop has started
    auto stop = [&](int status, const char *msg, int cycle, double ret) {
        sync_deflation();
        set_last_error(status, msg);
        S.its = cycle;
        S.cycles = cycle;
        S.status = status;
        S.rel_res = ret;
        cudaMemcpyAsync(x, X_, sizeof(C) * n, cudaMemcpyDeviceToDevice, stream);
        cudaStreamSynchronize(stream);
        return ret;
    };
    // ||b||
    launch_norm<R>(n, b, 0, act_, 1, partials_, tickets_, state_, 1, stream);
    // x~ = x0; r = b - A x0  (the hook overwrites x with A x0, as the reference's does)
    cudaMemcpyAsync(X_, x, sizeof(C) * n, cudaMemcpyDeviceToDevice, stream);
    apply(X_, 0, hook ? op.ext : Y_, 0, 1, &S.matvecs);
    sub<C>(n, b, hook ? op.ext : Y_, R_, stream);
    launch_norm<R>(n, R_, 0, act_, 1, partials_, tickets_, state_, 2, stream);
    if (read_state(1) != GDMR_OK) return fail(1.0);
    const double bnorm = hstate_[0].bnorm;
    double rho_abs = hstate_[0].rho_abs;
    if (!std::isfinite(bnorm) || !std::isfinite(rho_abs)) {
        // the reference's loop test is false for NaN, so it returns NaN as if converged, with
        // numIts = -1; the same value is returned here, with a status that says what happened
        const double ret = stop(GDMR_ENONFINITE,
                                "non-finite residual: the operator or the right-hand side produced NaN or Inf", 0,
                                rho_abs / bnorm);
        S.its = -1;
        return ret;
    }
    if (rho_abs < bnorm * tol) {     // gDMR.cu:2785-2796: absolute norm returned, x unchanged
        cudaMemcpyAsync(x, X_, sizeof(C) * n, cudaMemcpyDeviceToDevice, stream);
        cudaStreamSynchronize(stream);
        S.rel_res = rho_abs;
        S.cycles = 0;
        return rho_abs;
    }
    launch_scale<R>(n, R_, 0, R_, 0, nullptr, 0, act_, 1, state_, false, stream);
    const int first_def = mode == 0 ? 0 : k;
    int loop_flag = 0, cycle = 0, kk_prev = 0;
    while (rho_abs > tol * bnorm) {
        if (cycle > mat_rank)
            return stop(GDMR_ENOCONV, "solver failed to converge within matRank restart cycles", cycle,
                        rho_abs / bnorm);
        if (rho_abs / bnorm > 1.0)
            return stop(GDMR_ERUNAWAY, "solver runaway: residual above the right-hand side norm", cycle,
                        rho_abs / bnorm);
        const int kk = (cycle == 0 && first_def == 0) ? 0 : k;
        if (sync_deflation() != GDMR_OK) return fail(1.0);
        // restart vector (arnoldiSetupDMR, gDMR.cu:2600-2621); a zero period would divide by zero there
        CycleRecord rec;
        rec.kk = kk;
        const int period = (2 * mat_rank) / (m - k);
        if (loop_flag == 0 || (period != 0 && flag_count_ % period == 0)) {
            cudaMemcpyAsync(V_, R_, sizeof(C) * n, cudaMemcpyDeviceToDevice, stream);
        } else {
            const int idx = kk + (m - k) / 2 - kk_prev;   // the reference indexes its [W|V] storage
            rec.restart = kk + (m - k) / 2;
            if (idx > 0 && idx <= m) cudaMemcpyAsync(V_, V_ + (size_t)idx * n, sizeof(C) * n, cudaMemcpyDeviceToDevice, stream);
        }
        {
            Range rc("gdmr cycle");
            if (run_cycle(kk, 1, 0, tol, &S.matvecs) != GDMR_OK) return fail(1.0);
            if (read_state(1) != GDMR_OK) return fail(1.0);
        }
        const SysState &st = hstate_[0];
        if (timed_out()) {
            // a bounded wait ran out: this cycle's results, and the deflation space it updated,
            // are not to be trusted
            drop_deflation();
            return stop(GDMR_ETIMEOUT, "a bounded device wait ran out during the solve (gdmrWaitLimit)", cycle + 1,
                        rho_abs / bnorm);
        }
        if (st.broken) S.breakdowns++;
        const double rho = st.rho;
        if (rho > 0.995) {            // gDMR.cu:2506-2514
            loop_flag = 1;
            ++flag_count_;
        } else {
            loop_flag = 0;
        }
        rho_abs = st.rho_abs;
        rec.rho = rho;
        rec.rel_res = rho_abs / bnorm;
        rec.breakdown = st.broken;
        rec.stagnated = loop_flag;
        hist_.push_back(rec);
        kk_prev = kk;
        ++cycle;
        if (!std::isfinite(rho_abs))
            return stop(GDMR_ENONFINITE, "non-finite residual: the operator produced NaN or Inf", cycle,
                        rho_abs / bnorm);
    }
    S.its = cycle - 1;
    S.cycles = cycle;
    S.rel_res = rho_abs / bnorm;
    if (sync_deflation() != GDMR_OK) return fail(rho_abs / bnorm);
    cudaMemcpyAsync(x, X_, sizeof(C) * n, cudaMemcpyDeviceToDevice, stream);
    if (cudaStreamSynchronize(stream) != cudaSuccess) {
        set_last_error(GDMR_ECUDA, "solver: final synchronisation failed");
        return fail(rho_abs / bnorm);
    }
    return rho_abs / bnorm;
}

template <class R> int Engine<R>::refine_setup(const SellMatrix &A64) {
    if (!ready()) {
        set_last_error(GDMR_ENOTINIT, "solver used before initialisation");
        return GDMR_ENOTINIT;
    }
    if ((op.kind != Operator<R>::SELL && op.kind != Operator<R>::STENCIL) || !A64.vals) {
        set_last_error(GDMR_EINVAL, "refined solve: needs a SELL or stencil operator and FP64 SELL values");
        return GDMR_EINVAL;
    }
    A64_ = A64;
    front_done_ = false;
    if (!r64_) {
        int rc;
        if ((rc = alloc((void **)&r64_, sizeof(double2) * (size_t)n_ * cap_)) != GDMR_OK) return rc;
        if ((rc = alloc((void **)&b64_, sizeof(double2) * (size_t)n_ * cap_)) != GDMR_OK) return rc;
        if ((rc = alloc((void **)&x64_, sizeof(double2) * (size_t)n_ * cap_)) != GDMR_OK) return rc;
    }
    slot_.assign(cap_, Slot());
    act_h_.clear();
    kk_prev_ = 0;
    GDMR_CK(cudaMemsetAsync(X_, 0, sizeof(C) * (size_t)n_ * cap_, stream));
    return begin_solve();
}

template <class R>
int Engine<R>::refine_admit(int slot, const double2 *b, const double2 *x0, double tol, int max_cycles) {
    if (slot < 0 || slot >= cap_ || slot_[slot].active) {
        set_last_error(GDMR_EINVAL, "refine_admit: slot out of range or busy");
        return GDMR_EINVAL;
    }
    const size_t vb = sizeof(double2) * (size_t)n_;
    GDMR_CK(cudaMemcpyAsync(slot_b(slot), b, vb, cudaMemcpyDeviceToDevice, stream));
    if (x0) GDMR_CK(cudaMemcpyAsync(slot_x(slot), x0, vb, cudaMemcpyDeviceToDevice, stream));
    else GDMR_CK(cudaMemsetAsync(slot_x(slot), 0, vb, stream));
    GDMR_CK(cudaMemsetAsync(X_ + (size_t)slot * n_, 0, sizeof(C) * (size_t)n_, stream));
    Slot &S = slot_[slot];
    S = Slot();
    S.active = true;
    S.tol = tol;
    S.max_cycles = max_cycles;
    S.bnorm = -1;   // measured with the first residual
    act_h_.push_back(slot);
    return GDMR_OK;
}

// The stagnation rule of the restart (arnoldiSetupDMR, gDMR.cu:2600-2621): a system whose last
// cycle stagnated starts from the Krylov vector at storage index kk + (m - k)/2 of that cycle
// instead of from the unit residual, which k_demote_unit has already written as basis vector 0.
template <class R> void Engine<R>::restart_vectors(const std::vector<int> &next, int kk) {
    const int n = n_, m = m_, k = k_;
    for (int s : next) {
        Slot &S = slot_[s];
        const int period = (2 * S.max_cycles) / (m - k);
        if (S.loop_flag == 0 || (period != 0 && S.flag_count % period == 0)) continue;
        const int idx = kk + (m - k) / 2 - kk_prev_;
        if (idx > 0 && idx <= m)
            cudaMemcpyAsync(Vs(s), Vs(s) + (size_t)idx * n, sizeof(C) * n, cudaMemcpyDeviceToDevice, stream);
    }
}

template <class R> int Engine<R>::refine_cycle(std::vector<int> *done) {
    const int n = n_, m = m_, k = k_;
    if (act_h_.empty()) return GDMR_OK;
    std::vector<int> act = act_h_;
    if (set_active(act) != GDMR_OK) return GDMR_ECUDA;
    int na = (int)act.size();
    // ||b|| for newcomers
    std::vector<int> fresh;
    for (int s : act)
        if (slot_[s].bnorm < 0) fresh.push_back(s);
    if (!fresh.empty()) {
        if (set_active(fresh) != GDMR_OK) return GDMR_ECUDA;
        launch_norm<double>(n, b64_, n, act_, (int)fresh.size(), partials_, tickets_, state_, 1, stream);
        if (set_active(act) != GDMR_OK) return GDMR_ECUDA;
    }
    // true FP64 residual of every active system.  With gdmrOverlapResidual(n > 0), from the
    // engine's third cycle on, with a deflation space and no cycle graph, it runs on its own
    // stream on about n CTAs an SM, beside the next cycle's deflation loop on the main stream
    // (W = orth(A Z) needs only Z); the host reads the states once both are done.  The 96^3
    // batch measured the same cycle time either way, so it is off by default.
    Range range("gdmr refined cycle");
    const int res_per_sm = overlap_residual();
    const bool early = k > 0 && res_per_sm > 0 && cycles_run_ > 1 && !graph_ok(na) && (have_z_ || z_pending_);
    if (early) {
        GDMR_CK(cudaEventRecord(ev_x_, stream));
        GDMR_CK(cudaStreamWaitEvent(res_, ev_x_, 0));
        launch_residual64(A64_, b64_, n, x64_, n, r64_, n, act_, na, partials_res_, tickets_, state_, res_,
                          res_per_sm);
        GDMR_CK(cudaEventRecord(ev_res_, res_));
        if (sync_deflation() != GDMR_OK) return GDMR_ECUDA;
        long dmv = 0;
        enqueue_deflation_loop(k, &dmv);
        front_done_ = true;
        GDMR_CK(cudaStreamWaitEvent(stream, ev_res_, 0));
    } else {
        launch_residual64(A64_, b64_, n, x64_, n, r64_, n, act_, na, partials_, tickets_, state_, stream);
    }
    if (read_state(cap_) != GDMR_OK) return GDMR_ECUDA;
    // a bounded wait that ran out since the last look (the previous cycle's kernels) leaves
    // every system in flight, and the shared deflation space, untrustworthy
    const bool lost = timed_out();
    if (lost) {
        to_base_ = timeouts_now();
        drop_deflation();
        set_last_error(GDMR_ETIMEOUT, "a bounded device wait ran out during the solve (gdmrWaitLimit)");
    }
    std::vector<int> next;
    int lead = -1;
    double worst = -1;
    for (int s : act) {
        Slot &S = slot_[s];
        const SysState &st = hstate_[s];
        if (S.bnorm < 0) S.bnorm = st.bnorm;
        const double rel = S.bnorm > 0 ? st.true_res / S.bnorm : 0.0;
        S.stats.true_rel_res = rel;
        S.stats.rel_res = rel;
        S.stats.matvecs += 1;   // the FP64 residual product
        int fin = -1;
        if (lost && S.stats.cycles > 0) fin = GDMR_ETIMEOUT;
        else if (st.bad || !std::isfinite(rel)) fin = GDMR_ENONFINITE;
        else if (rel <= S.tol) fin = GDMR_OK;
        else if (S.stats.cycles >= S.max_cycles) fin = GDMR_ENOCONV;
        if (fin >= 0) {
            S.stats.status = fin;
            S.stats.its = S.stats.cycles > 0 ? S.stats.cycles - 1 : 0;
            S.active = false;
            if (done) done->push_back(s);
            continue;
        }
        next.push_back(s);
        if (rel > worst) { worst = rel; lead = s; }
    }
    act_h_ = next;
    if (next.empty()) {
        front_done_ = false;
        return sync_deflation();
    }
    if (set_active(next) != GDMR_OK) return GDMR_ECUDA;
    na = (int)next.size();
    // unit residual direction in precision R, also the first basis vector of every system (the
    // side stream's deflation update reads the previous cycle's basis: join it first); the
    // inner recursion starts at rho_abs = 1
    if (sync_deflation() != GDMR_OK) return GDMR_ECUDA;
    launch_demote_unit<R>(n, r64_, n, R_, n, V_, strideV(), act_, na, state_, stream);
    k_cycle_reset<<<1, 256, 0, stream>>>(act_, na, state_, 1);
    const int kk = (k > 0 && have_z_) ? k : 0;
    if (kk == 0) front_done_ = false;   // the deflation space was dropped after a timeout
    restart_vectors(next, kk);
    long mv = 0;
    // breakdown of unit vectors: an invariant subspace at working precision
    const double inner_tol = sizeof(R) == 4 ? 1e-6 : 1e-14;
    if (run_cycle(kk, na, lead, inner_tol, &mv) != GDMR_OK) return GDMR_ECUDA;
    launch_refine_update<R>(n, x64_, n, X_, n, act_, na, state_, stream);
    if (read_state(cap_) != GDMR_OK) return GDMR_ECUDA;
    for (int s : next) {
        Slot &S = slot_[s];
        const SysState &st = hstate_[s];
        if (st.rho > 0.995) { S.loop_flag = 1; ++S.flag_count; } else S.loop_flag = 0;
        S.stats.cycles += 1;
        S.stats.matvecs += m;
        if (st.broken) S.stats.breakdowns++;
    }
    kk_prev_ = kk;
    return GDMR_OK;
}

// ----------------------------------------------------------------- lockstep (many-operator) form
template <class R> int Engine<R>::multi_residual() {
    if (act_h_.empty()) return GDMR_OK;
    const int n = n_;
    std::vector<int> act = act_h_;
    if (set_active(act) != GDMR_OK) return GDMR_ECUDA;
    std::vector<int> fresh;
    for (int s : act)
        if (slot_[s].bnorm < 0) fresh.push_back(s);
    if (!fresh.empty()) {
        if (set_active(fresh) != GDMR_OK) return GDMR_ECUDA;
        launch_norm<double>(n, b64_, n, act_, (int)fresh.size(), partials_, tickets_, state_, 1, stream);
        if (set_active(act) != GDMR_OK) return GDMR_ECUDA;
    }
    launch_residual64(A64_, b64_, n, x64_, n, r64_, n, act_, (int)act.size(), partials_, tickets_, state_, stream);
    GDMR_CK(cudaGetLastError());
    return GDMR_OK;
}

template <class R> int Engine<R>::multi_select(std::vector<int> *done) {
    mf_nsys_ = 0;
    if (act_h_.empty()) return 0;
    if (read_state(cap_) != GDMR_OK) return -1;
    // the last cycle's bookkeeping (refine_cycle does it right after its cycle)
    if (mf_ran_) {
        for (int s : mf_act_) {
            Slot &S = slot_[s];
            const SysState &st = hstate_[s];
            if (st.rho > 0.995) { S.loop_flag = 1; ++S.flag_count; } else S.loop_flag = 0;
            S.stats.cycles += 1;
            S.stats.matvecs += m_;
            if (st.broken) S.stats.breakdowns++;
        }
        kk_prev_ = mf_kk_;
        mf_ran_ = false;
    }
    const bool lost = timed_out();
    if (lost) {
        to_base_ = timeouts_now();
        drop_deflation();
        set_last_error(GDMR_ETIMEOUT, "a bounded device wait ran out during the solve (gdmrWaitLimit)");
    }
    std::vector<int> next;
    int lead = -1;
    double worst = -1;
    for (int s : act_h_) {
        Slot &S = slot_[s];
        const SysState &st = hstate_[s];
        if (S.bnorm < 0) S.bnorm = st.bnorm;
        const double rel = S.bnorm > 0 ? st.true_res / S.bnorm : 0.0;
        S.stats.true_rel_res = rel;
        S.stats.rel_res = rel;
        S.stats.matvecs += 1;
        int fin = -1;
        if (lost && S.stats.cycles > 0) fin = GDMR_ETIMEOUT;
        else if (st.bad || !std::isfinite(rel)) fin = GDMR_ENONFINITE;
        else if (rel <= S.tol) fin = GDMR_OK;
        else if (S.stats.cycles >= S.max_cycles) fin = GDMR_ENOCONV;
        if (fin >= 0) {
            S.stats.status = fin;
            S.stats.its = S.stats.cycles > 0 ? S.stats.cycles - 1 : 0;
            S.active = false;
            if (done) done->push_back(s);
            continue;
        }
        next.push_back(s);
        if (rel > worst) { worst = rel; lead = s; }
    }
    act_h_ = next;
    if (next.empty()) {
        if (sync_deflation() != GDMR_OK) return -1;
        return 0;
    }
    lead_host_ = lead;
    mf_nsys_ = (int)next.size();
    return mf_nsys_;
}

template <class R> int Engine<R>::multi_front() {
    if (mf_nsys_ == 0) return GDMR_OK;
    if (op.kind != Operator<R>::SELL) {
        set_last_error(GDMR_EINVAL, "many-operator solve: needs a SELL operator");
        return GDMR_EINVAL;
    }
    const int n = n_, m = m_, k = k_;
    const std::vector<int> next = act_h_;
    const int na = (int)next.size();
    if (set_active(next) != GDMR_OK) return GDMR_ECUDA;
    if (sync_deflation() != GDMR_OK) return GDMR_ECUDA;
    launch_demote_unit<R>(n, r64_, n, R_, n, V_, strideV(), act_, na, state_, stream);
    k_cycle_reset<<<1, 256, 0, stream>>>(act_, na, state_, 1);
    const int kk = (k > 0 && have_z_) ? k : 0;
    restart_vectors(next, kk);
    GDMR_CK(cudaMemcpyAsync(lead_dev_, &lead_host_, sizeof(int), cudaMemcpyHostToDevice, stream));
    long mv = 0;
    int rc = enqueue_front(kk, na, &mv);
    if (rc != GDMR_OK) return rc;
    ++cycles_run_;
    mf_kk_ = kk;
    mf_tol_ = sizeof(R) == 4 ? 1e-6 : 1e-14;   // breakdown of unit vectors, as refine_cycle
    mf_act_ = next;
    return GDMR_OK;
}

template <class R> void Engine<R>::multi_jobs(std::vector<KrylovJob<R>> &jobs) const {
    for (int s : mf_act_) {
        KrylovJob<R> j{};
        j.n = n_;
        j.nslices = op.sell.nslices;
        j.kk = mf_kk_;
        j.m = m_;
        j.compat_eye = compat_eye ? 1 : 0;
        j.qmax = qmax();
        j.tol = mf_tol_;
        j.slice_ptr = op.sell.slice_ptr;
        j.cols = op.sell.cols;
        j.vals = (const C *)op.sell.vals;
        j.W = W_;
        j.V = Vs(s);
        j.y = Y_ + (size_t)s * n_;
        j.state = state_ + s;
        j.H = H_ + (size_t)s * strideH();
        j.coef = coef_ + (size_t)s * strideC();
        jobs.push_back(j);
    }
}

template <class R> int Engine<R>::multi_back(cudaEvent_t after) {
    if (mf_nsys_ == 0) return GDMR_OK;
    GDMR_CK(cudaStreamWaitEvent(stream, after, 0));
    int rc = enqueue_back(mf_kk_, mf_nsys_, false);
    if (rc != GDMR_OK) return rc;
    launch_refine_update<R>(n_, x64_, n_, X_, n_, act_, mf_nsys_, state_, stream);
    GDMR_CK(cudaGetLastError());
    mf_ran_ = true;
    return GDMR_OK;
}

template <class R> int Engine<R>::true_residual(int count, const double2 *b, const double2 *x, double *relres) {
    if (!A64_.vals || !r64_) {
        set_last_error(GDMR_ENOTINIT, "true_residual: refined form not set up");
        return GDMR_ENOTINIT;
    }
    for (int c0 = 0; c0 < count; c0 += cap_) {
        const int cnt = std::min(cap_, count - c0);
        std::vector<int> act(cnt);
        for (int i = 0; i < cnt; ++i) act[i] = i;
        std::vector<int> keep = act_h_;
        if (set_active(act) != GDMR_OK) return GDMR_ECUDA;
        act_h_ = keep;
        launch_norm<double>(n_, b + (size_t)c0 * n_, n_, act_, cnt, partials_, tickets_, state_, 1, stream);
        launch_residual64(A64_, b + (size_t)c0 * n_, n_, x + (size_t)c0 * n_, n_, r64_, n_, act_, cnt, partials_,
                          tickets_, state_, stream);
        if (read_state(cnt) != GDMR_OK) return GDMR_ECUDA;
        for (int i = 0; i < cnt; ++i)
            relres[c0 + i] = hstate_[i].bnorm > 0 ? hstate_[i].true_res / hstate_[i].bnorm : hstate_[i].true_res;
    }
    return GDMR_OK;
}

template <class R> int Engine<R>::import_deflation(const C *host) {
    if (!ready() || k_ == 0) return GDMR_OK;
    if (sync_deflation() != GDMR_OK) return GDMR_ECUDA;
    GDMR_CK(cudaStreamSynchronize(stream));
    GDMR_CK(cudaMemcpy(Z_, host, sizeof(C) * (size_t)k_ * n_, cudaMemcpyHostToDevice));
    have_z_ = true;
    return GDMR_OK;
}

template <class R> int Engine<R>::export_deflation(C *host) {
    if (!ready() || k_ == 0) return GDMR_OK;
    if (sync_deflation() != GDMR_OK) return GDMR_ECUDA;
    GDMR_CK(cudaStreamSynchronize(stream));
    GDMR_CK(cudaMemcpy(host, Z_, sizeof(C) * (size_t)k_ * n_, cudaMemcpyDeviceToHost));
    return GDMR_OK;
}

template class Engine<float>;
template class Engine<double>;
template class Engine<dfr>;

}  // namespace gdmr
