// Truncated SVD / symmetric eigendecomposition on the device
// (replaces MatrixAlgebraKit's svd_trunc / eigh_trunc! with truncrank(k)).
//
// GB300 runs FP64 at ~2 DFMA/clk/SM, so FP64 work that lives on one SM (Jacobi
// sweeps, Cholesky) is avoided on the iteration path:
//  * randomized subspace iteration with r = min(3k, 128) columns, orthonormalised
//    every half-step with shifted CholeskyQR3 (FP64 Gram and Cholesky in FP64
//    precision; split-kernel Grams and FP32 Cholesky in split precision): stable for
//    the steep spectra of ordered phases and for numerically low-rank matrices, whose
//    noise columns are nearly dependent; the sigma estimates come from aligning the
//    basis with the Ritz vectors (FP32 Jacobi on the r x r Gram) at two iterations;
//  * the number of iterations comes from the estimated gap (sigma_r / sigma_k)^2
//    per iteration, so the kept subspace reaches the target angle;
//  * one final Rayleigh-Ritz in FP64: polar correction of the basis (GEMMs only),
//    FP32 Jacobi to align, FP64 Jacobi cleanup of the nearly diagonal remainder,
//    singular values as column norms (one-sided, accurate for graded spectra).
//  * min(m, n) <= 128: the same final step on the whole matrix (exact).
#include "common.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace tnr {

constexpr int RDIRECT = 128;
constexpr int RMAX = 128;
constexpr int MAXIT = 40;
constexpr int RSMALL = 160;     // largest matrix of the one-CTA Jacobi solvers

static void check_status(Ctx& c, const char* where) {
    int st = c.read_status_and_clear();
    if (st & ST_NONFINITE) throw Error(TNR_ERR_NONFINITE, std::string(where) + ": non-finite values");
    if (st & ST_JACOBI_NOCONV) throw Error(TNR_ERR_NOT_CONVERGED, std::string(where) + ": Jacobi sweep cap reached");
}

static std::vector<double> to_host(Ctx& c, const double* d, int n) {
    std::vector<double> h(n);
    if (n) TNR_CUDA(cudaMemcpyAsync(h.data(), d, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    return h;
}

// Q (m x r) <- orthonormal basis of span(Y); Y is overwritten.  Shifted CholeskyQR3 on the
// column-scaled Gram: a shifted pass, then two more, which orthonormalises any column
// grading and nearly dependent columns (the noise columns of a numerically low-rank M).
// FP64 precision: FP64 Gram and Cholesky, first shift 11 (m r + r (r + 1)) eps, then none.
// Split precision: Grams on the split kernel (FP32-level), FP32 Cholesky, shifts
// 1e-6 max(1, r/16) then 1e-7.
void orth_scaled(Ctx& c, double* Y, int64_t m, int r, double* Q) {
    const bool f64 = c.precision == TNR_PREC_F64;
    const int passes = f64 ? 3 : TNR_SPLIT_ORTH_PASSES;
    Buf G(c.pool.get(), (size_t)r * r * sizeof(double));
    Buf ds(c.pool.get(), (size_t)r * sizeof(double));
    double* src = Y;
    for (int pass = 0; pass < passes; ++pass) {
        double shift = f64 ? (pass == 0 ? 11.0 * ((double)m * r + (double)r * (r + 1)) * 2.220446049250313e-16 : 0.0)
                           : (pass == 0 ? 1e-6 * std::max(1, r / 16) : 1e-7);
        for (int attempt = 0;; ++attempt) {
            gemm_bulk(c, true, false, r, r, m, 1.0, src, m, 0, src, m, 0, 0.0, G.d(), r, 0);
            gram_unit_diag(c, G.d(), r, ds.d());
            if (f64) chol_inv(c, G.d(), r, shift);
            else chol_inv_f32(c, G.d(), r, shift);
            int st = c.read_status_and_clear();
            if (!(st & ST_CHOL_BREAKDOWN)) break;
            TNR_REQUIRE(attempt < 5, TNR_ERR_NOT_CONVERGED, "orth: Cholesky breakdown");
            shift = std::max(shift * 30.0, 1e-14);
        }
        col_scale(c, G.d(), r, r, r, ds.d(), 0);         // Linv D
        double* dst = (src == Q) ? Y : Q;
        gemm_bulk(c, false, true, m, r, r, 1.0, src, m, 0, G.d(), r, 0, 0.0, dst, m, 0);
        src = dst;
    }
    if (src != Q) copy_f64(c, Q, src, m * (int64_t)r);
}

// Q <- Q (I - E/2 + 3E^2/8), E = Q^T Q - I: cubic correction to FP64 orthonormality (GEMMs only).
// Its inputs (CholeskyQR3 bases, FP32 Jacobi rotations) are orthonormal to FP32 level or better,
// ||E|| <~ 1e-7, so one step leaves O(||E||^3) ~ 1e-21, below FP64 rounding.
constexpr int POLAR_STEPS = 1;
static void polar(Ctx& c, double* Q, int64_t m, int r) {
    Buf E(c.pool.get(), (size_t)r * r * sizeof(double));
    Buf E2(c.pool.get(), (size_t)r * r * sizeof(double));
    Buf T(c.pool.get(), (size_t)m * r * sizeof(double));
    for (int it = 0; it < POLAR_STEPS; ++it) {
        gemm_f64(c, true, false, r, r, m, 1.0, Q, m, 0, Q, m, 0, 0.0, E.d(), r, 0);
        add_identity(c, E.d(), r, -1.0);
        gemm_f64(c, false, false, r, r, r, 1.0, E.d(), r, 0, E.d(), r, 0, 0.0, E2.d(), r, 0);
        polar_coeff(c, E.d(), E2.d(), E.d(), r);
        gemm_f64(c, false, false, m, r, r, 1.0, Q, m, 0, E.d(), r, 0, 0.0, T.d(), m, 0);
        copy_f64(c, Q, T.d(), m * (int64_t)r);
    }
}

// Q (m x r) <- Q L^-T with Q^T Q = L L^T (FP64 Gram and Cholesky): exactly orthonormal whatever
// Q's departure from orthonormality (a tiny shift only if the Gram is numerically singular).
// The split CholeskyQR3 can leave the noise directions of a numerically rank-deficient M far
// from orthonormal, where the cubic polar step would not hold.
static void orth_exact(Ctx& c, double* Q, int64_t m, int r) {
    Buf G(c.pool.get(), (size_t)r * r * sizeof(double));
    Buf L(c.pool.get(), (size_t)r * r * sizeof(double));
    Buf T(c.pool.get(), (size_t)m * r * sizeof(double));
    gemm_f64(c, true, false, r, r, m, 1.0, Q, m, 0, Q, m, 0, 0.0, G.d(), r, 0);
    double shift = 0.0;
    for (int attempt = 0;; ++attempt) {
        copy_f64(c, L.d(), G.d(), (int64_t)r * r);
        chol_inv(c, L.d(), r, shift);
        int st = c.read_status_and_clear();
        if (!(st & ST_CHOL_BREAKDOWN)) break;
        TNR_REQUIRE(attempt < 8, TNR_ERR_NOT_CONVERGED, "orth_exact: basis Gram not positive definite");
        shift = std::max(shift * 30.0, 1e-14);
    }
    gemm_f64(c, false, true, m, r, r, 1.0, Q, m, 0, L.d(), r, 0, 0.0, T.d(), m, 0);
    copy_f64(c, Q, T.d(), m * (int64_t)r);
}

// Exact SVD of the tall X = op(M) (m x p, p <= 128): X V = Ux diag(s), Ux unit columns.
// trans=false: X = M (ld m); trans=true: X = M^T with M stored p x m (ld p).
// FP64 cleanup Jacobi of the final decompositions: rotations stop at 1e-12 of the diagonal,
// which leaves vectors of values that differ by a relative gap g rotated by ~1e-12 / g.  The gap
// fallback converges it to 1e-15 (FP64 rounding of the Gram), for gaps down to ~1e-5.
static void jacobi_final(Ctx& c, const double* G, int p, double* W, double* lam) {
    if (c.exact_jacobi) jacobi_eigh_tol(c, G, p, p, W, lam, 1, 0, 1e-15, 1e-22);
    else jacobi_eigh(c, G, p, p, W, lam);
}

static void final_svd(Ctx& c, const double* M, bool trans, int64_t m, int p, double* Ux, double* s, double* V) {
    Buf G(c.pool.get(), (size_t)p * p * sizeof(double));
    Buf W1(c.pool.get(), (size_t)p * p * sizeof(double));
    Buf W2(c.pool.get(), (size_t)p * p * sizeof(double));
    Buf lam(c.pool.get(), (size_t)p * sizeof(double));
    const int64_t ldm = trans ? p : m;
    // pass 1: align with the eigenvectors of X^T X (FP32 Jacobi), W1 made orthogonal in FP64
    gemm_f64(c, !trans, trans, p, p, m, 1.0, M, ldm, 0, M, ldm, 0, 0.0, G.d(), p, 0);
    jacobi_eigh_f32(c, G.d(), p, p, W1.d(), lam.d());
    polar(c, W1.d(), p, p);
    // pass 2: X W1 has nearly orthogonal columns; FP64 Jacobi cleans up the rest
    gemm_f64(c, trans, false, m, p, p, 1.0, M, ldm, 0, W1.d(), p, 0, 0.0, Ux, m, 0);
    gemm_f64(c, true, false, p, p, m, 1.0, Ux, m, 0, Ux, m, 0, 0.0, G.d(), p, 0);
    jacobi_final(c, G.d(), p, W2.d(), lam.d());
    gemm_f64(c, false, false, p, p, p, 1.0, W1.d(), p, 0, W2.d(), p, 0, 0.0, V, p, 0);
    gemm_f64(c, trans, false, m, p, p, 1.0, M, ldm, 0, V, p, 0, 0.0, Ux, m, 0);
    col_norms(c, Ux, m, p, m, s);
    col_scale(c, Ux, m, p, m, s, 2);
    check_status(c, "final_svd");
}

// symmetric H (p x p): eigenvectors W (FP64-orthogonal) and eigenvalues, |lambda| descending
static void final_eigh(Ctx& c, const double* H, int p, double* W, double* lam) {
    Buf W1(c.pool.get(), (size_t)p * p * sizeof(double));
    Buf W2(c.pool.get(), (size_t)p * p * sizeof(double));
    Buf G(c.pool.get(), (size_t)p * p * sizeof(double));
    Buf T(c.pool.get(), (size_t)p * p * sizeof(double));
    jacobi_eigh_f32(c, H, p, p, W1.d(), lam);
    polar(c, W1.d(), p, p);
    gemm_f64(c, false, false, p, p, p, 1.0, H, p, 0, W1.d(), p, 0, 0.0, T.d(), p, 0);
    gemm_f64(c, true, false, p, p, p, 1.0, W1.d(), p, 0, T.d(), p, 0, 0.0, G.d(), p, 0);
    jacobi_final(c, G.d(), p, W2.d(), lam);
    gemm_f64(c, false, false, p, p, p, 1.0, W1.d(), p, 0, W2.d(), p, 0, 0.0, W, p, 0);
    check_status(c, "final_eigh");
}

static void transpose2d(Ctx& c, const double* in, int64_t m, int64_t n, double* out) {
    int64_t d[2] = {m, n};
    int perm[2] = {1, 0};
    permute(c, in, d, 2, perm, out);
}

void svd_r_factor(Ctx& c, const double* M, int64_t m, int n, double* R) {
    TNR_REQUIRE(m >= n && n >= 1 && n <= RSMALL, TNR_ERR_UNSUPPORTED, "svd_r_factor: needs m >= n and n <= 160");
    Buf Ux(c.pool.get(), (size_t)m * n * sizeof(double));
    Buf V(c.pool.get(), (size_t)n * n * sizeof(double));
    Buf sv(c.pool.get(), (size_t)n * sizeof(double));
    final_svd(c, M, false, m, n, Ux.d(), sv.d(), V.d());
    transpose2d(c, V.d(), n, n, R);
    row_scale(c, R, n, n, n, sv.d(), 0);
}

// iterations needed so the kept subspace reaches the target angle: one iteration
// contracts the error by rho = (v[r-1] / v[k-1])^power, v = FP64 estimates of |values|
// (column norms of the aligned basis) sorted descending
// Subspace iterations for the kept subspace to reach the target angle, from the sigma
// estimates v: one iteration contracts the angle by (sigma_r / sigma_k)^power.  A kept
// tail below 1e-13 sigma_1 is numerically zero (2 iterations).  `cap` bounds the count:
// the split precision caps at 16, since its products resolve no direction below ~1e-7
// sigma_1 and a noise ratio near 1 there would otherwise run to the FP64 cap of 40 (and
// in a lockstep group hold every member there).
int iterations_needed(std::vector<double> v, int k, int r, int power, double target, int cap) {
    std::sort(v.begin(), v.end(), [](double a, double b) { return std::fabs(a) > std::fabs(b); });
    const double vk = std::fabs(v[k - 1]), v1 = std::fabs(v[0]);
    double vr = std::fabs(v[r - 1]);
    if (!(v1 > 0)) return 2;
    if (vk <= 1e-13 * v1) return 2;
    vr = std::max(vr, 1e-15 * v1);
    double rho = std::pow(vr / vk, (double)power);
    if (rho >= 0.999) return cap;
    // +2: the column-norm estimates of the smallest values are upper bounds, and vk is an
    // estimate too; two spare iterations keep the kept subspace at the target angle
    int n = (int)std::ceil(std::log(target) / std::log(rho)) + 2;
    return std::max(2, std::min(cap, n));
}

int iteration_cap(const Ctx& c) { return c.precision == TNR_PREC_F64 ? MAXIT : 16; }

// The spectral gap at k is too small for the subspace iteration: the estimates say the kept
// subspace would not reach the target angle within the iteration cap (sigma_r / sigma_k too
// close to 1).  Same estimate rules as iterations_needed, without the cap.  In split precision
// estimates below ~1e-7 sigma_1 are product noise, so only a kept tail above 1e-5 sigma_1
// counts (no TRG/BTRG decomposition of the Ising model at chi 24-32, beta 0.30-0.60, needs more
// than the split cap of 16 iterations by the exact spectra).
bool gap_too_small(const Ctx& c, std::vector<double> v, int k, int r, int power, double target, int cap) {
    std::sort(v.begin(), v.end(), [](double a, double b) { return std::fabs(a) > std::fabs(b); });
    const double vk = std::fabs(v[k - 1]), v1 = std::fabs(v[0]);
    if (!(v1 > 0) || vk <= 1e-13 * v1) return false;
    if (c.precision != TNR_PREC_F64 && vk <= 1e-5 * v1) return false;
    const double vr = std::max(std::fabs(v[r - 1]), 1e-15 * v1);
    const double rho = std::pow(vr / vk, (double)power);
    if (rho >= 0.999) return true;
    return std::ceil(std::log(target) / std::log(rho)) + 2 > cap;
}

// runs the decomposition in FP64 precision whatever the context's precision (the gap fallback)
struct F64Scope {
    Ctx& c;
    int saved;
    bool saved_exact;
    explicit F64Scope(Ctx& cc) : c(cc), saved(cc.precision), saved_exact(cc.exact_jacobi) {
        c.precision = TNR_PREC_F64;
        c.exact_jacobi = true;
    }
    ~F64Scope() { c.precision = saved; c.exact_jacobi = saved_exact; }
};

// sigma estimates of the columns of X (n x r, batch B of stride n r): column norms of X
// aligned with its Ritz vectors.  One FP32 Jacobi on the FP64 Gram leaves ~1e-7 of the
// leading directions in the small columns; FP64 precision aligns the aligned basis once
// more (its Gram is nearly diagonal, so the second FP32 rotation removes that leakage and
// the FP64 products keep the cancellation exact), which resolves estimates down to FP64
// noise.  G, W: r x r scratch per matrix; Xa: n x r scratch per matrix.
void sigma_estimates(Ctx& c, const double* X, int64_t n, int r, int B, double* G, double* W, double* Xa, double* lam) {
    Batch2 g, rot;
    g.n1 = B; g.sA1 = n * r; g.sB1 = n * r; g.sC1 = (int64_t)r * r;
    rot.n1 = B; rot.sA1 = n * r; rot.sB1 = (int64_t)r * r; rot.sC1 = n * r;
    gemm_bulk(c, true, false, r, r, n, 1.0, X, n, X, n, 0.0, G, r, g);
    jacobi_eigh_f32(c, G, r, r, W, lam, B, (int64_t)r * r);
    gemm_bulk(c, false, false, n, r, r, 1.0, X, n, W, r, 0.0, Xa, n, rot);
    if (c.precision == TNR_PREC_F64) {
        Buf X2(c.pool.get(), (size_t)B * n * r * sizeof(double));
        gemm_f64(c, true, false, r, r, n, 1.0, Xa, n, Xa, n, 0.0, G, r, g);
        jacobi_eigh_f32(c, G, r, r, W, lam, B, (int64_t)r * r);
        gemm_f64(c, false, false, n, r, r, 1.0, Xa, n, W, r, 0.0, X2.d(), n, rot);
        col_norms(c, X2.d(), n, (int64_t)r * B, n, lam);
    } else {
        col_norms(c, Xa, n, (int64_t)r * B, n, lam);
    }
}

static bool debug_on() {
    static int on = -1;
    if (on < 0) {
        const char* e = getenv("TNR_DEBUG");
        on = (e && *e && *e != '0') ? 1 : 0;
    }
    return on == 1;
}

#ifndef TNR_TARGET_F64
#define TNR_TARGET_F64 1e-15
#endif
static double target_angle(Ctx& c) { return c.precision == TNR_PREC_F64 ? TNR_TARGET_F64 : 1e-9; }

// r_override > 0: the subspace width (the gap fallback's widest subspace)
static TsvdOut tsvd_impl(Ctx& c, const double* M, int64_t m, int64_t n, int k, double* U, double* s, double* Vt,
                         int direct_max, int r_override);

TsvdOut tsvd(Ctx& c, const double* M, int64_t m, int64_t n, int k, double* U, double* s, double* Vt, int direct_max) {
    ++c.decompositions;
    TsvdOut o = tsvd_impl(c, M, m, n, k, U, s, Vt, std::min(direct_max, RDIRECT), 0);
    c.max_iters = std::max(c.max_iters, o.iters);
    return o;
}

TsvdOut tsvd_gap_fallback(Ctx& c, const double* M, int64_t m, int64_t n, int k, double* U, double* s, double* Vt) {
    ++c.gap_fallbacks;
    F64Scope scope(c);
    if (std::min(m, n) <= RSMALL) return tsvd_impl(c, M, m, n, k, U, s, Vt, RSMALL, 0);
    return tsvd_impl(c, M, m, n, k, U, s, Vt, RDIRECT, RSMALL);
}

static TsvdOut tsvd_impl(Ctx& c, const double* M, int64_t m, int64_t n, int k, double* U, double* s, double* Vt,
                         int direct_max, int r_override) {
    TsvdOut out;
    const int64_t p = std::min(m, n);
    k = (int)std::min<int64_t>(k, p);
    out.k = k;
    if (k <= 0) return out;
    if (p <= direct_max) {
        const int pp = (int)p;
        const bool wide = m < n;
        const int64_t rows = wide ? n : m;               // X = M (tall) or M^T
        Buf Ux(c.pool.get(), (size_t)rows * pp * sizeof(double));
        Buf V(c.pool.get(), (size_t)pp * pp * sizeof(double));
        Buf sv(c.pool.get(), (size_t)pp * sizeof(double));
        final_svd(c, M, wide, rows, pp, Ux.d(), sv.d(), V.d());
        if (!wide) {
            copy_f64(c, U, Ux.d(), m * (int64_t)k);
            transpose2d(c, V.d(), pp, k, Vt);
        } else {
            copy_f64(c, U, V.d(), m * (int64_t)k);
            transpose2d(c, Ux.d(), n, k, Vt);
        }
        copy_f64(c, s, sv.d(), k);
        std::vector<double> vals = to_host(c, sv.d(), pp);
        double tot = 0, kept = 0;
        for (int i = 0; i < pp; ++i) { tot += vals[i] * vals[i]; if (i < k) kept += vals[i] * vals[i]; }
        out.fro2 = tot;
        out.err = std::sqrt(std::max(tot - kept, 0.0));
        out.vals.assign(vals.begin(), vals.begin() + k);
        return out;
    }
    int r = (int)std::min<int64_t>({p, (int64_t)RMAX, (int64_t)((3 * k + 7) / 8 * 8)});
    r = std::max(r, std::min((int)p, k + 8));
    if (r_override > 0) r = (int)std::min<int64_t>(p, r_override);
    Buf Om(c.pool.get(), (size_t)n * r * sizeof(double));
    Buf Y(c.pool.get(), (size_t)m * r * sizeof(double));
    Buf Uq(c.pool.get(), (size_t)m * r * sizeof(double));
    Buf Z(c.pool.get(), (size_t)n * r * sizeof(double));
    Buf Vq(c.pool.get(), (size_t)n * r * sizeof(double));
    Buf G(c.pool.get(), (size_t)r * r * sizeof(double));
    Buf W(c.pool.get(), (size_t)r * r * sizeof(double));
    Buf lam(c.pool.get(), (size_t)r * sizeof(double));
    fill_normal(c, Om.d(), n * (int64_t)r, c.seed + 0x1000193ull * (++c.call_counter));
    // the split precision splits M into BF16 planes once for every product of the iteration
    const Batch2 one;
    SplitA PM, PMt;
    split_a_prepare(c, PM, false, M, m, m, n, r, one);
    split_a_prepare(c, PMt, true, M, m, n, m, r, one);
    gemm_bulk_a(c, PM, false, false, m, r, n, 1.0, M, m, Om.d(), n, 0.0, Y.d(), m, one);
    orth_scaled(c, Y.d(), m, r, Uq.d());
    int need = MAXIT, it = 0;
    for (; it < need; ++it) {
        // Z = M^T U; at two iterations its columns aligned with the Ritz vectors of Z^T Z
        // (FP32 Jacobi) give the sigma estimates that set the iteration count
        gemm_bulk_a(c, PMt, true, false, n, r, m, 1.0, M, m, Uq.d(), m, 0.0, Z.d(), n, one);
        if (it == 0 || it == 2) sigma_estimates(c, Z.d(), n, r, 1, G.d(), W.d(), Vq.d(), lam.d());
        orth_scaled(c, Z.d(), n, r, Vq.d());
        gemm_bulk_a(c, PM, false, false, m, r, n, 1.0, M, m, Vq.d(), n, 0.0, Y.d(), m, one);
        orth_scaled(c, Y.d(), m, r, Uq.d());
        if (it == 0 || it == 2) {
            std::vector<double> est = to_host(c, lam.d(), r);
            check_status(c, "tsvd");
            if (it == 0 && r_override == 0 && gap_too_small(c, est, k, r, 2, target_angle(c), iteration_cap(c))) {
                // the gap at k is too small for the iteration: a matrix the one-CTA solvers hold
                // is decomposed exactly in FP64 (the full Jacobi path); a larger one is iterated
                // in FP64 on the widest subspace they hold
                return tsvd_gap_fallback(c, M, m, n, k, U, s, Vt);
            }
            need = std::max(it + 1, iterations_needed(est, k, r, 2, target_angle(c), iteration_cap(c)));
        }
    }
    out.iters = it;
    c.last_iters = it;
    if (debug_on()) fprintf(stderr, "[tnr] tsvd m=%lld n=%lld k=%d r=%d iters=%d\n", (long long)m, (long long)n, k, r, it);
    if (c.precision == TNR_PREC_SPLIT) {
        // the split path's final step with its polar factor folded into the r x r problems
        std::vector<double> kept = final_rr_split(c, PMt, M, m, n, r, k, 1, Uq.d(), U, s, Vt);
        sum_squares(c, M, m * n, c.d_scalar);
        std::vector<double> f = to_host(c, c.d_scalar, 1);
        out.fro2 = f[0];
        double kept2 = 0;
        for (double v : kept) kept2 += v * v;
        out.err = std::sqrt(std::max(out.fro2 - kept2, 0.0));
        out.vals = kept;
        return out;
    }
    // final Rayleigh-Ritz in FP64: M ~ U (U^T M) = U B, B^T = M^T U
    polar(c, Uq.d(), m, r);
    Buf Ub(c.pool.get(), (size_t)n * r * sizeof(double));
    Buf Vb(c.pool.get(), (size_t)r * r * sizeof(double));
    Buf sb(c.pool.get(), (size_t)r * sizeof(double));
    // split precision: the projection on the tensor cores with chunked (unbiased) accumulation
    gemm_bulk_a(c, PMt, true, false, n, r, m, 1.0, M, m, Uq.d(), m, 0.0, Z.d(), n, one, true);
    final_svd(c, Z.d(), false, n, r, Ub.d(), sb.d(), Vb.d());      // B^T = Ub s Vb^T -> M ~ (U Vb) s Ub^T
    gemm_f64(c, false, false, m, k, r, 1.0, Uq.d(), m, 0, Vb.d(), r, 0, 0.0, U, m, 0);
    copy_f64(c, s, sb.d(), k);
    transpose2d(c, Ub.d(), n, k, Vt);
    std::vector<double> cur = to_host(c, sb.d(), r);
    sum_squares(c, M, m * n, c.d_scalar);
    std::vector<double> f = to_host(c, c.d_scalar, 1);
    out.fro2 = f[0];
    double kept = 0, ritz_tail = 0;
    for (int i = 0; i < r; ++i) { if (i < k) kept += cur[i] * cur[i]; else ritz_tail += cur[i] * cur[i]; }
    out.err = std::sqrt(ritz_tail + std::max(out.fro2 - kept - ritz_tail, 0.0));
    out.vals.assign(cur.begin(), cur.begin() + k);
    return out;
}

static TsvdOut teigh_impl(Ctx& c, const double* M, int64_t n, int k, double* U, double* lamk, int direct_max,
                          int r_override);

TsvdOut teigh(Ctx& c, const double* M, int64_t n, int k, double* U, double* lamk, int direct_max) {
    ++c.decompositions;
    TsvdOut o = teigh_impl(c, M, n, k, U, lamk, std::min(direct_max, RDIRECT), 0);
    c.max_iters = std::max(c.max_iters, o.iters);
    return o;
}

static TsvdOut teigh_impl(Ctx& c, const double* M, int64_t n, int k, double* U, double* lamk, int direct_max,
                          int r_override) {
    TsvdOut out;
    k = (int)std::min<int64_t>(k, n);
    out.k = k;
    if (k <= 0) return out;
    sum_squares(c, M, n * n, c.d_scalar);
    if (n <= direct_max) {
        const int nn = (int)n;
        Buf W(c.pool.get(), (size_t)nn * nn * sizeof(double));
        Buf l(c.pool.get(), (size_t)nn * sizeof(double));
        Buf Hs(c.pool.get(), (size_t)nn * nn * sizeof(double));
        copy_f64(c, Hs.d(), M, n * n);
        final_eigh(c, Hs.d(), nn, W.d(), l.d());
        copy_f64(c, U, W.d(), n * (int64_t)k);
        copy_f64(c, lamk, l.d(), k);
        std::vector<double> all = to_host(c, l.d(), nn);
        double disc = 0, tot = 0;
        for (int i = 0; i < nn; ++i) { tot += all[i] * all[i]; if (i >= k) disc += all[i] * all[i]; }
        out.err = std::sqrt(disc);
        out.fro2 = tot;
        out.vals.assign(all.begin(), all.begin() + k);
        return out;
    }
    int r = (int)std::min<int64_t>({n, (int64_t)RMAX, (int64_t)((3 * k + 7) / 8 * 8)});
    r = std::max(r, std::min((int)n, k + 8));
    if (r_override > 0) r = (int)std::min<int64_t>(n, r_override);
    Buf Om(c.pool.get(), (size_t)n * r * sizeof(double));
    Buf Y(c.pool.get(), (size_t)n * r * sizeof(double));
    Buf Q(c.pool.get(), (size_t)n * r * sizeof(double));
    Buf T(c.pool.get(), (size_t)n * r * sizeof(double));
    Buf H(c.pool.get(), (size_t)r * r * sizeof(double));
    Buf W(c.pool.get(), (size_t)r * r * sizeof(double));
    Buf l(c.pool.get(), (size_t)r * sizeof(double));
    fill_normal(c, Om.d(), n * (int64_t)r, c.seed + 0x1000193ull * (++c.call_counter));
    // M is symmetric: M Q = M^T Q, whose planes are K-contiguous; split once for every product
    const Batch2 one;
    SplitA PMt;
    split_a_prepare(c, PMt, true, M, n, n, n, r, one);
    gemm_bulk_a(c, PMt, true, false, n, r, n, 1.0, M, n, Om.d(), n, 0.0, Y.d(), n, one);
    orth_scaled(c, Y.d(), n, r, Q.d());
    int need = MAXIT, it = 0;
    for (; it < need; ++it) {
        gemm_bulk_a(c, PMt, true, false, n, r, n, 1.0, M, n, Q.d(), n, 0.0, Y.d(), n, one);
        if (it == 0 || it == 2) sigma_estimates(c, Y.d(), n, r, 1, H.d(), W.d(), T.d(), l.d());   // ~ |lambda_i|
        orth_scaled(c, Y.d(), n, r, Q.d());
        if (it == 0 || it == 2) {
            std::vector<double> est = to_host(c, l.d(), r);
            check_status(c, "teigh");
            if (it == 0 && r_override == 0 && gap_too_small(c, est, k, r, 1, target_angle(c), iteration_cap(c))) {
                // the gap fallback, as in tsvd
                ++c.gap_fallbacks;
                F64Scope scope(c);
                if (n <= RSMALL) return teigh_impl(c, M, n, k, U, lamk, RSMALL, 0);
                return teigh_impl(c, M, n, k, U, lamk, direct_max, RSMALL);
            }
            need = std::max(it + 1, iterations_needed(est, k, r, 1, target_angle(c), iteration_cap(c)));
        }
    }
    out.iters = it;
    c.last_iters = it;
    if (debug_on()) fprintf(stderr, "[tnr] teigh n=%lld k=%d r=%d iters=%d\n", (long long)n, k, r, it);
    // final Rayleigh-Ritz in FP64 on an exactly orthonormal basis
    if (c.precision == TNR_PREC_F64) polar(c, Q.d(), n, r);
    else orth_exact(c, Q.d(), n, r);
    gemm_bulk_a(c, PMt, true, false, n, r, n, 1.0, M, n, Q.d(), n, 0.0, Y.d(), n, one, true);
    gemm_f64(c, true, false, r, r, n, 1.0, Q.d(), n, 0, Y.d(), n, 0, 0.0, H.d(), r, 0);
    final_eigh(c, H.d(), r, W.d(), l.d());
    gemm_f64(c, false, false, n, k, r, 1.0, Q.d(), n, 0, W.d(), r, 0, 0.0, U, n, 0);
    copy_f64(c, lamk, l.d(), k);
    std::vector<double> cur = to_host(c, l.d(), r);
    std::vector<double> f = to_host(c, c.d_scalar, 1);
    out.fro2 = f[0];
    double kept = 0, ritz_tail = 0;
    for (int i = 0; i < r; ++i) { if (i < k) kept += cur[i] * cur[i]; else ritz_tail += cur[i] * cur[i]; }
    out.err = std::sqrt(ritz_tail + std::max(out.fro2 - kept - ritz_tail, 0.0));
    out.vals.assign(cur.begin(), cur.begin() + k);
    return out;
}

}  // namespace tnr
