// Host restatement of the reference DMR iteration -- TEST INFRASTRUCTURE ONLY.
//
// This file is the oracle: the GPU library (libgDMR) is checked against it, and
// bench.py times it as the CPU baseline.  Nothing in the product links it.
//
// Parity status: unpinned.  seanMolesky/gDMR-solver has no tests, fixtures or
// golden vectors, and its only implementation is CUDA (gDMR.cu), which cannot
// run in the CPU-only build container; its sources do not travel to the GPU
// machine.  The oracle is pinned instead by (1) a sparse direct solve (SciPy
// SuperLU) of the same systems, (2) a second, independent numpy restatement
// (dmr_numpy.py) that must agree cycle by cycle, and (3) LAPACK (numpy.linalg)
// for the QR least-squares and SVD building blocks.
//
// Scalar type: complex<R> for R = double (the plain-FP64 form) or R = float
// (an emulation of the reference's complex64 arithmetic: float storage, float
// products, float accumulation, as innerProdKerDMR does).  The small dense
// problems (least squares on H, SVD of H) run in double for both, like the GPU
// library; the reference runs them in float through cuSOLVER.
//
// Steps and their reference lines (one device, natural Krylov order):
//   solve()          solverDMR           gDMR.cu:2638-2900
//   restart vector   arnoldiSetupDMR     gDMR.cu:2586-2632 (0.995 rule gDMR.cu:2506)
//   arnoldi()        arnoldiDMR          gDMR.cu:1790-2332
//   deflate()        deflatorDMR         gDMR.cu:1710-1787
//   g = B^H r        updateTrgCoeffsDMR  gDMR.cu:2334-2408
//   LS + updates     updateAppResDMR     gDMR.cu:2411-2582
//   Z update         genDeflatDMR        gDMR.cu:1583-1704
//   dot convention   innerProdKerDMR     gDMR.cu:268-326   <a,b> = sum conj(a_i) b_i
//
// Built by oracle/build_oracle.sh into oracle/_build/liboracle.so (C ABI, used
// through ctypes by tests and bench.py).

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename R> struct C {
    R re, im;
};
template <typename R> inline C<R> cadd(C<R> a, C<R> b) { return {a.re + b.re, a.im + b.im}; }
template <typename R> inline C<R> csub(C<R> a, C<R> b) { return {a.re - b.re, a.im - b.im}; }
template <typename R> inline C<R> cmul(C<R> a, C<R> b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
template <typename R> inline C<R> cconjmul(C<R> a, C<R> b) { return {a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re}; }
template <typename R> inline C<R> cscale(C<R> a, R s) { return {a.re * s, a.im * s}; }

using Z64 = C<double>;

// ---------------------------------------------------------------- small dense
// Column-major (rows x cols) complex double, ld = rows.

// Least squares argmin ||H y - g|| by Householder QR (H is (m+1) x m).
// Replaces cusolverDnCgeqrf/Cungqr + cublasCgemv/Ctrsv, gDMR.cu:691-839.
static void ls_householder(int rows, int cols, const Z64 *Hin, const Z64 *gin, Z64 *y) {
    std::vector<Z64> H(Hin, Hin + (size_t)rows * cols), g(gin, gin + rows);
    for (int c = 0; c < cols; ++c) {
        double alpha2 = 0;
        for (int r = c; r < rows; ++r) alpha2 += H[c * rows + r].re * H[c * rows + r].re + H[c * rows + r].im * H[c * rows + r].im;
        double alpha = std::sqrt(alpha2);
        if (alpha == 0) continue;
        Z64 x0 = H[c * rows + c];
        double ax0 = std::hypot(x0.re, x0.im);
        Z64 phase = ax0 > 0 ? Z64{x0.re / ax0, x0.im / ax0} : Z64{1, 0};
        // v = x + phase*alpha e1, H -> (I - 2 v v^H / v^H v) H
        std::vector<Z64> v(rows - c);
        for (int r = c; r < rows; ++r) v[r - c] = H[c * rows + r];
        v[0] = cadd(v[0], cscale(phase, alpha));
        double vv = 0;
        for (auto &e : v) vv += e.re * e.re + e.im * e.im;
        if (vv == 0) continue;
        for (int cc = c; cc < cols; ++cc) {
            Z64 s{0, 0};
            for (int r = c; r < rows; ++r) s = cadd(s, cconjmul(v[r - c], H[cc * rows + r]));
            s = cscale(s, 2.0 / vv);
            for (int r = c; r < rows; ++r) H[cc * rows + r] = csub(H[cc * rows + r], cmul(v[r - c], s));
        }
        Z64 s{0, 0};
        for (int r = c; r < rows; ++r) s = cadd(s, cconjmul(v[r - c], g[r]));
        s = cscale(s, 2.0 / vv);
        for (int r = c; r < rows; ++r) g[r] = csub(g[r], cmul(v[r - c], s));
    }
    for (int c = cols - 1; c >= 0; --c) {
        Z64 s = g[c];
        for (int cc = c + 1; cc < cols; ++cc) s = csub(s, cmul(H[cc * rows + c], y[cc]));
        Z64 d = H[c * rows + c];
        double dd = d.re * d.re + d.im * d.im;
        y[c] = dd > 0 ? Z64{(s.re * d.re + s.im * d.im) / dd, (s.im * d.re - s.re * d.im) / dd} : Z64{0, 0};
    }
}

// One-sided Jacobi SVD (Hestenes 1958) of a (rows x cols) matrix, rows >= cols.
// Returns singular values descending and the matching right singular vectors
// (columns of V, cols x cols).  Replaces cusolverDnCgesvdj, gDMR.cu:637-689.
static void svd_jacobi(int rows, int cols, const Z64 *Ain, double *sigma, Z64 *Vout) {
    std::vector<Z64> A(Ain, Ain + (size_t)rows * cols), V((size_t)cols * cols, Z64{0, 0});
    for (int i = 0; i < cols; ++i) V[i * cols + i] = {1, 0};
    const double eps = 4.0 * 2.220446049250313e-16 * cols;   // pairwise orthogonality target
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0;
        for (int p = 0; p < cols - 1; ++p)
            for (int q = p + 1; q < cols; ++q) {
                double a = 0, b = 0;
                Z64 gm{0, 0};
                for (int r = 0; r < rows; ++r) {
                    Z64 ap = A[p * rows + r], aq = A[q * rows + r];
                    a += ap.re * ap.re + ap.im * ap.im;
                    b += aq.re * aq.re + aq.im * aq.im;
                    gm = cadd(gm, cconjmul(ap, aq));
                }
                double ag = std::hypot(gm.re, gm.im);
                if (ag == 0 || ag <= eps * std::sqrt(a * b)) continue;
                off = std::max(off, ag / std::sqrt(a * b));
                Z64 ph{gm.re / ag, gm.im / ag};          // gamma = |gamma| e^{i phi}
                Z64 phc{ph.re, -ph.im};                  // e^{-i phi}
                double zeta = (b - a) / (2 * ag);
                double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1 + zeta * zeta));
                double c = 1 / std::sqrt(1 + t * t), s = c * t;
                for (int r = 0; r < rows; ++r) {
                    Z64 ap = A[p * rows + r], aq = cmul(A[q * rows + r], phc);
                    A[p * rows + r] = csub(cscale(ap, c), cscale(aq, s));
                    A[q * rows + r] = cadd(cscale(ap, s), cscale(aq, c));
                }
                for (int r = 0; r < cols; ++r) {
                    Z64 vp = V[p * cols + r], vq = cmul(V[q * cols + r], phc);
                    V[p * cols + r] = csub(cscale(vp, c), cscale(vq, s));
                    V[q * cols + r] = cadd(cscale(vp, s), cscale(vq, c));
                }
            }
        if (off < eps) break;
    }
    std::vector<double> sv(cols);
    for (int c = 0; c < cols; ++c) {
        double s = 0;
        for (int r = 0; r < rows; ++r) s += A[c * rows + r].re * A[c * rows + r].re + A[c * rows + r].im * A[c * rows + r].im;
        sv[c] = std::sqrt(s);
    }
    std::vector<int> order(cols);
    for (int i = 0; i < cols; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return sv[x] > sv[y]; });
    for (int i = 0; i < cols; ++i) {
        sigma[i] = sv[order[i]];
        std::memcpy(&Vout[(size_t)i * cols], &V[(size_t)order[i] * cols], sizeof(Z64) * cols);
    }
}

// ---------------------------------------------------------------- the solver
template <typename R> struct Oracle {
    using T = C<R>;
    int n, m, k;
    bool compat_eye;     // reproduce the breakdown identity tail starting at column j (gDMR.cu:2275)
    bool fuse_deflation; // project against [W V] in one classical Gram-Schmidt pass
    std::vector<int32_t> indptr, indices;
    std::vector<T> vals;
    std::vector<T> Z, Znew, basis;   // defBasisDMR (k x n), itrBasisDMR ((m+1) x n)
    std::vector<Z64> H;              // (m+1) x m column-major, ld m+1 (gDMR.cu:875)
    int flag_count = 0, loop_flag = 0;
    long matvecs = 0;
    std::vector<double> cycle_rho;
    std::vector<int> cycle_restart;   // 0, or the storage index of the mid-Krylov restart vector
    std::vector<int> cycle_broken;    // Krylov step of a breakdown, 0 if none
    std::vector<double> cycle_ms;     // wall time of each cycle (the CPU baseline times deflated ones)

    void matvec(const T *x, T *y) {
        ++matvecs;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            T s{0, 0};
            for (int p = indptr[i]; p < indptr[i + 1]; ++p) s = cadd(s, cmul(vals[p], x[indices[p]]));
            y[i] = s;
        }
    }
    // sum conj(a_i) b_i, accumulated in R like the reference; fixed chunks summed in order,
    // so the result does not depend on the thread count or on scheduling
    T dot(const T *a, const T *b) {
        const int CH = 4096;
        const int nch = (n + CH - 1) / CH;
        std::vector<T> part(nch);
#pragma omp parallel for schedule(static)
        for (int c = 0; c < nch; ++c) {
            R re = 0, im = 0;
            const int hi = std::min(n, (c + 1) * CH);
            for (int i = c * CH; i < hi; ++i) {
                T p = cconjmul(a[i], b[i]);
                re += p.re;
                im += p.im;
            }
            part[c] = {re, im};
        }
        R re = 0, im = 0;
        for (int c = 0; c < nch; ++c) { re += part[c].re; im += part[c].im; }
        return {re, im};
    }
    R norm(const T *a) { return std::sqrt(dot(a, a).re); }
    void scale(T *a, R s) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) a[i] = cscale(a[i], s);
    }
    // c = B^H w over q vectors (cublasCgemv OP_C in basisProjDMR, gDMR.cu:550-590)
    void project(const T *B, int q, const T *w, T *c) {
        for (int p = 0; p < q; ++p) c[p] = dot(B + (size_t)p * n, w);
    }
    // w = w - B c (vecScaleDiffDMR with scale 1, gDMR.cu:229-248)
    void subtract(const T *B, int q, const T *c, T *w) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            T s = w[i];
            for (int p = 0; p < q; ++p) s = csub(s, cmul(c[p], B[(size_t)p * n + i]));
            w[i] = s;
        }
    }
    // y += sum_p c_p B_p (addBasisVecsDMR, gDMR.cu:250-266)
    void combine(const T *B, int q, const T *c, T *y) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            T s = y[i];
            for (int p = 0; p < q; ++p) s = cadd(s, cmul(c[p], B[(size_t)p * n + i]));
            y[i] = s;
        }
    }
    static Z64 up(T a) { return {(double)a.re, (double)a.im}; }
    static T down(Z64 a) { return {(R)a.re, (R)a.im}; }
    Z64 &h(int r, int c) { return H[(size_t)c * (m + 1) + r]; }

    // Returns the Krylov step at which breakdown happened, or 0.
    int arnoldi(int kk, R tol) {
        std::fill(H.begin(), H.end(), Z64{0, 0});
        std::vector<T> w(n), worig(n), c(m + 1);
        T *B = basis.data();
        for (int i = 0; i < kk; ++i) {   // deflation loop, gDMR.cu:1823-2030
            matvec(&Z[(size_t)i * n], w.data());
            worig = w;
            if (i > 0) {
                project(B, i, w.data(), c.data());
                subtract(B, i, c.data(), w.data());
                for (int p = 0; p < i; ++p) h(p, i) = up(c[p]);
            }
            scale(w.data(), R(1) / norm(w.data()));
            std::copy(w.begin(), w.end(), B + (size_t)i * n);
            h(i, i) = up(dot(w.data(), worig.data()));
        }
        if (kk > 0) {                    // gDMR.cu:2033-2059
            T *v0 = B + (size_t)kk * n;
            project(B, kk, v0, c.data());
            subtract(B, kk, c.data(), v0);
            scale(v0, R(1) / norm(v0));
        }
        for (int j = 1; j <= m - kk; ++j) {   // Krylov loop, gDMR.cu:2069-2328
            int col = kk + j - 1;
            matvec(B + (size_t)(kk + j - 1) * n, w.data());
            worig = w;
            if (fuse_deflation) {
                project(B, kk + j, w.data(), c.data());
                subtract(B, kk + j, c.data(), w.data());
                for (int p = 0; p < kk + j; ++p) h(p, col) = up(c[p]);
            } else {
                if (kk > 0) {
                    project(B, kk, w.data(), c.data());
                    for (int p = 0; p < kk; ++p) h(p, col) = up(c[p]);
                    subtract(B, kk, c.data(), w.data());
                }
                project(B + (size_t)kk * n, j, w.data(), c.data());
                subtract(B + (size_t)kk * n, j, c.data(), w.data());
                for (int p = 0; p < j; ++p) h(kk + p, col) = up(c[p]);
            }
            R nrm = norm(w.data());
            if (nrm < tol) {                 // gDMR.cu:2256-2289
                std::fill(basis.begin() + (size_t)(kk + j) * n, basis.end(), T{0, 0});
                for (int cc = compat_eye ? j : kk + j; cc < m; ++cc) h(cc, cc) = {1, 0};
                return j;
            }
            scale(w.data(), R(1) / nrm);
            std::copy(w.begin(), w.end(), B + (size_t)(kk + j) * n);
            h(kk + j, col) = up(dot(w.data(), worig.data()));
        }
        return 0;
    }

    // Returns the relative residual as solverDMR does; fills its/cycles/status.
    double solve(int mode, const T *b, T *x, double tol_in, int mat_rank, int *its, int *cycles, int *status) {
        R tol = (R)tol_in;
        loop_flag = 0;
        cycle_rho.clear();
        cycle_restart.clear();
        cycle_broken.clear();
        cycle_ms.clear();
        std::vector<T> r(n), t(n), u(n);
        *its = mat_rank * mat_rank;
        *cycles = 0;
        R bnorm = norm(b);
        matvec(x, t.data());
        for (int i = 0; i < n; ++i) r[i] = csub(b[i], t[i]);
        R rho_abs = norm(r.data());
        if (rho_abs < bnorm * tol) {        // gDMR.cu:2785-2796 returns the absolute norm
            *status = 1;
            return rho_abs;
        }
        scale(r.data(), R(1) / rho_abs);
        int cycle = 0;
        int first_def = mode == 0 ? 0 : k;
        std::vector<Z64> g(m + 1), y(m), hy(m + 1), sig(m);
        std::vector<double> sv(m);
        std::vector<Z64> Vs((size_t)m * m);
        std::vector<T> cT(m + 1);
        while (rho_abs > tol * bnorm) {
            if (cycle > mat_rank) { *its = cycle; *cycles = cycle; *status = 3; return rho_abs / bnorm; }
            if (rho_abs / bnorm > 1) { *its = cycle; *cycles = cycle; *status = 4; return rho_abs / bnorm; }
            const auto t_cycle = std::chrono::steady_clock::now();
            int kk = (cycle == 0 && first_def == 0) ? 0 : k;
            int period = (2 * mat_rank) / (m - k);
            T *v0 = &basis[(size_t)kk * n];
            int restart = 0;
            if (loop_flag == 0 || (period != 0 && flag_count % period == 0)) {
                std::copy(r.begin(), r.end(), v0);
            } else {                      // arnoldiSetupDMR, gDMR.cu:2610-2621
                restart = kk + (m - k) / 2;
                std::copy(&basis[(size_t)restart * n], &basis[(size_t)(restart + 1) * n], v0);
            }
            const int broken = arnoldi(kk, tol);
            project(basis.data(), m + 1, r.data(), cT.data());   // g, gDMR.cu:2334-2408
            for (int p = 0; p <= m; ++p) g[p] = up(cT[p]);
            ls_householder(m + 1, m, H.data(), g.data(), y.data());
            for (int rr = 0; rr <= m; ++rr) {
                Z64 s{0, 0};
                for (int c = 0; c < m; ++c) s = cadd(s, cmul(h(rr, c), y[c]));
                hy[rr] = s;
            }
            std::fill(t.begin(), t.end(), T{0, 0});
            for (int p = 0; p <= m; ++p) cT[p] = down(hy[p]);
            combine(basis.data(), m + 1, cT.data(), t.data());
            for (int i = 0; i < n; ++i) r[i] = csub(r[i], t[i]);
            R rho = norm(r.data());
            if (rho > (R)0.995) { loop_flag = 1; ++flag_count; } else loop_flag = 0;
            scale(r.data(), R(1) / rho);
            std::fill(u.begin(), u.end(), T{0, 0});
            for (int p = 0; p < m; ++p) cT[p] = down(y[p]);
            if (kk > 0) {
                combine(Z.data(), kk, cT.data(), u.data());
                combine(&basis[(size_t)kk * n], m - kk, cT.data() + kk, u.data());
            } else {
                combine(basis.data(), m, cT.data(), u.data());
            }
            scale(u.data(), rho_abs);
            for (int i = 0; i < n; ++i) x[i] = cadd(x[i], u[i]);
            rho_abs = rho * rho_abs;
            cycle_rho.push_back((double)rho);
            cycle_restart.push_back(restart);
            cycle_broken.push_back(broken);
            if (k > 0) {                                      // gDMR.cu:1583-1704
                svd_jacobi(m + 1, m, H.data(), sv.data(), Vs.data());
                for (int tI = 0; tI < k; ++tI) {
                    const Z64 *vcol = &Vs[(size_t)(m - k + tI) * m];
                    for (int p = 0; p < m; ++p) cT[p] = down(vcol[p]);
                    T *zt = &Znew[(size_t)tI * n];
                    std::fill(zt, zt + n, T{0, 0});
                    if (kk > 0) {
                        combine(Z.data(), kk, cT.data(), zt);
                        combine(&basis[(size_t)kk * n], m - kk, cT.data() + kk, zt);
                    } else {
                        combine(basis.data(), m, cT.data(), zt);
                    }
                    scale(zt, R(1) / norm(zt));
                }
                std::swap(Z, Znew);
            }
            cycle_ms.push_back(
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_cycle).count());
            ++cycle;
        }
        *its = cycle - 1;
        *cycles = cycle;
        *status = 0;
        return rho_abs / bnorm;
    }
};

struct Handle {
    int precision;   // 0 = complex128, 1 = complex64
    Oracle<double> *d = nullptr;
    Oracle<float> *f = nullptr;
};

template <typename R>
Oracle<R> *make(int n, int m, int k, const int32_t *indptr, const int32_t *indices, const double *vals_ri,
                int compat_eye, int fuse) {
    auto *o = new Oracle<R>();
    o->n = n; o->m = m; o->k = k;
    o->compat_eye = compat_eye != 0;
    o->fuse_deflation = fuse != 0;
    o->indptr.assign(indptr, indptr + n + 1);
    int nnz = indptr[n];
    o->indices.assign(indices, indices + nnz);
    o->vals.resize(nnz);
    for (int p = 0; p < nnz; ++p) o->vals[p] = {(R)vals_ri[2 * p], (R)vals_ri[2 * p + 1]};
    o->Z.assign((size_t)k * n, {0, 0});
    o->Znew.assign((size_t)k * n, {0, 0});
    o->basis.assign((size_t)(m + 1) * n, {0, 0});
    o->H.assign((size_t)(m + 1) * m, {0, 0});
    return o;
}

}  // namespace

extern "C" {

// Creates an oracle for the CSR operator (values interleaved re,im as double).
// precision 0 = complex128, 1 = complex64 (reference arithmetic).
void *oracle_create(int n, int m, int k, const int32_t *indptr, const int32_t *indices, const double *vals_ri,
                    int precision, int compat_eye, int fuse_deflation) {
    if (m - k < 2 || n <= 0 || k < 0) return nullptr;
    auto *h = new Handle();
    h->precision = precision;
    if (precision == 0) h->d = make<double>(n, m, k, indptr, indices, vals_ri, compat_eye, fuse_deflation);
    else h->f = make<float>(n, m, k, indptr, indices, vals_ri, compat_eye, fuse_deflation);
    return h;
}

void oracle_destroy(void *hp) {
    auto *h = (Handle *)hp;
    delete h->d;
    delete h->f;
    delete h;
}

void oracle_set_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// b and x are interleaved (re,im) doubles; x is the initial guess on entry and the
// solution on exit.  Returns solverDMR's return value.
double oracle_solve(void *hp, int mode, const double *b_ri, double *x_ri, double tol, int mat_rank,
                    int *its, int *cycles, int *status, long *matvecs) {
    auto *h = (Handle *)hp;
    if (h->precision == 0) {
        auto *o = h->d;
        o->matvecs = 0;
        double r = o->solve(mode, (const C<double> *)b_ri, (C<double> *)x_ri, tol, mat_rank, its, cycles, status);
        *matvecs = o->matvecs;
        return r;
    }
    auto *o = h->f;
    int n = o->n;
    std::vector<C<float>> b(n), x(n);
    for (int i = 0; i < n; ++i) {
        b[i] = {(float)b_ri[2 * i], (float)b_ri[2 * i + 1]};
        x[i] = {(float)x_ri[2 * i], (float)x_ri[2 * i + 1]};
    }
    o->matvecs = 0;
    double r = o->solve(mode, b.data(), x.data(), tol, mat_rank, its, cycles, status);
    *matvecs = o->matvecs;
    for (int i = 0; i < n; ++i) { x_ri[2 * i] = x[i].re; x_ri[2 * i + 1] = x[i].im; }
    return r;
}

// Per-cycle residual reduction factors of the last solve (rho = ||r_new|| / ||r_old||).
int oracle_cycle_log(void *hp, double *out, int cap) {
    auto *h = (Handle *)hp;
    const std::vector<double> &v = h->precision == 0 ? h->d->cycle_rho : h->f->cycle_rho;
    int c = std::min<int>(cap, (int)v.size());
    std::copy(v.begin(), v.begin() + c, out);
    return (int)v.size();
}

// Wall time (ms) of each cycle of the last solve.
int oracle_cycle_ms(void *hp, double *out, int cap) {
    auto *h = (Handle *)hp;
    const std::vector<double> &v = h->precision == 0 ? h->d->cycle_ms : h->f->cycle_ms;
    const int c = std::min<int>(cap, (int)v.size());
    std::copy(v.begin(), v.begin() + c, out);
    return (int)v.size();
}

// Per cycle of the last solve: the restart vector's storage index (0: the residual) and the
// Krylov step of a breakdown (0: none).
int oracle_cycle_info(void *hp, int *restart, int *broken, int cap) {
    auto *h = (Handle *)hp;
    const std::vector<int> &rs = h->precision == 0 ? h->d->cycle_restart : h->f->cycle_restart;
    const std::vector<int> &bk = h->precision == 0 ? h->d->cycle_broken : h->f->cycle_broken;
    const int c = std::min<int>(cap, (int)rs.size());
    std::copy(rs.begin(), rs.begin() + c, restart);
    std::copy(bk.begin(), bk.begin() + c, broken);
    return (int)rs.size();
}

// Deflation basis Z (k x n, vector-contiguous) in and out, interleaved doubles.
void oracle_get_Z(void *hp, double *out) {
    auto *h = (Handle *)hp;
    if (h->precision == 0) std::memcpy(out, h->d->Z.data(), sizeof(double) * 2 * h->d->Z.size());
    else for (size_t i = 0; i < h->f->Z.size(); ++i) { out[2 * i] = h->f->Z[i].re; out[2 * i + 1] = h->f->Z[i].im; }
}
void oracle_set_Z(void *hp, const double *in) {
    auto *h = (Handle *)hp;
    if (h->precision == 0) std::memcpy(h->d->Z.data(), in, sizeof(double) * 2 * h->d->Z.size());
    else for (size_t i = 0; i < h->f->Z.size(); ++i) h->f->Z[i] = {(float)in[2 * i], (float)in[2 * i + 1]};
}

// Building blocks exposed for the LAPACK cross-checks.
void oracle_ls(int rows, int cols, const double *H_ri, const double *g_ri, double *y_ri) {
    ls_householder(rows, cols, (const Z64 *)H_ri, (const Z64 *)g_ri, (Z64 *)y_ri);
}
void oracle_svd(int rows, int cols, const double *A_ri, double *sigma, double *V_ri) {
    svd_jacobi(rows, cols, (const Z64 *)A_ri, sigma, (Z64 *)V_ri);
}

}  // extern "C"
