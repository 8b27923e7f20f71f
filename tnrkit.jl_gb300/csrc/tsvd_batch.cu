// Truncated SVD of a batch of equal-shaped matrices, stepped in lockstep: the same
// algorithm as tsvd() (randomized subspace iteration orthonormalised with shifted
// CholeskyQR3, final FP64 Rayleigh-Ritz), with every GEMM batched and every
// one-CTA solver launched once with one CTA per instance.  The iteration count is the
// largest any instance of the batch needs.
#include "common.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace tnr {

namespace {

constexpr int RDIRECT = 128;
constexpr int RMAX = 128;
constexpr int MAXIT = 40;

#ifndef TNR_TARGET_F64
#define TNR_TARGET_F64 1e-15
#endif

std::vector<double> to_host(Ctx& c, const double* d, int64_t n) {
    std::vector<double> h((size_t)n);
    if (n) TNR_CUDA(cudaMemcpyAsync(h.data(), d, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    return h;
}

void check_status(Ctx& c, const char* where) {
    int st = c.read_status_and_clear();
    if (st & ST_NONFINITE) throw Error(TNR_ERR_NONFINITE, std::string(where) + ": non-finite values");
    if (st & ST_JACOBI_NOCONV) throw Error(TNR_ERR_NOT_CONVERGED, std::string(where) + ": Jacobi sweep cap reached");
}

Batch2 strided(int B, int64_t sA, int64_t sB, int64_t sC) {
    Batch2 bt;
    bt.n1 = B;
    bt.sA1 = sA;
    bt.sB1 = sB;
    bt.sC1 = sC;
    return bt;
}

// Q[b] (m x r) <- orthonormal basis of span(Y[b]) (Y overwritten): shifted CholeskyQR3 on
// the column-scaled Gram, as orth_scaled() in tsvd.cu (FP64 Gram and Cholesky in FP64
// precision; split-kernel Grams and FP32 Cholesky in split precision)
void orth_b(Ctx& c, double* Y, int64_t m, int r, int B, double* Q) {
    const bool f64 = c.precision == TNR_PREC_F64;
    const int passes = f64 ? 3 : TNR_SPLIT_ORTH_PASSES;
    Buf G(c.pool.get(), (size_t)B * r * r * sizeof(double));
    Buf ds(c.pool.get(), (size_t)B * r * sizeof(double));
    double* src = Y;
    for (int pass = 0; pass < passes; ++pass) {
        double shift = f64 ? (pass == 0 ? 11.0 * ((double)m * r + (double)r * (r + 1)) * 2.220446049250313e-16 : 0.0)
                           : (pass == 0 ? 1e-6 * std::max(1, r / 16) : 1e-7);
        for (int attempt = 0;; ++attempt) {
            gemm_bulk(c, true, false, r, r, m, 1.0, src, m, src, m, 0.0, G.d(), r, strided(B, m * r, m * r, r * r));
            gram_unit_diag(c, G.d(), r, ds.d(), B);
            if (f64) chol_inv(c, G.d(), r, shift, B);
            else chol_inv_f32(c, G.d(), r, shift, B);
            int st = c.read_status_and_clear();
            if (!(st & ST_CHOL_BREAKDOWN)) break;
            TNR_REQUIRE(attempt < 5, TNR_ERR_NOT_CONVERGED, "orth: Cholesky breakdown");
            shift = std::max(shift * 30.0, 1e-14);
        }
        col_scale(c, G.d(), r, (int64_t)r * B, r, ds.d(), 0);        // Linv D per instance
        double* dst = (src == Q) ? Y : Q;
        gemm_bulk(c, false, true, m, r, r, 1.0, src, m, G.d(), r, 0.0, dst, m, strided(B, m * r, r * r, m * r));
        src = dst;
    }
    if (src != Q) copy_f64(c, Q, src, m * (int64_t)r * B);
}

// Q[b] <- Q[b] (I - E/2 + 3E^2/8), E = Q^T Q - I; one step, as polar() in tsvd.cu
void polar_b(Ctx& c, double* Q, int64_t m, int r, int B) {
    Buf E(c.pool.get(), (size_t)B * r * r * sizeof(double));
    Buf E2(c.pool.get(), (size_t)B * r * r * sizeof(double));
    Buf T(c.pool.get(), (size_t)B * m * r * sizeof(double));
    for (int it = 0; it < 1; ++it) {
        gemm_f64(c, true, false, r, r, m, 1.0, Q, m, Q, m, 0.0, E.d(), r, strided(B, m * r, m * r, r * r));
        add_identity(c, E.d(), r, -1.0, B);
        gemm_f64(c, false, false, r, r, r, 1.0, E.d(), r, E.d(), r, 0.0, E2.d(), r, strided(B, r * r, r * r, r * r));
        polar_coeff(c, E.d(), E2.d(), E.d(), r, B);
        gemm_f64(c, false, false, m, r, r, 1.0, Q, m, E.d(), r, 0.0, T.d(), m, strided(B, m * r, r * r, m * r));
        copy_f64(c, Q, T.d(), m * (int64_t)r * B);
    }
}

// exact SVD of each tall X[b] = op(M[b]) (m x p, p <= 128): X V = Ux diag(s)
void final_svd_b(Ctx& c, const double* M, bool trans, int64_t m, int p, int B, int64_t strideM, double* Ux, double* s,
                 double* V) {
    Buf G(c.pool.get(), (size_t)B * p * p * sizeof(double));
    Buf W1(c.pool.get(), (size_t)B * p * p * sizeof(double));
    Buf W2(c.pool.get(), (size_t)B * p * p * sizeof(double));
    Buf lam(c.pool.get(), (size_t)B * p * sizeof(double));
    const int64_t ldm = trans ? p : m;
    const int64_t pp = (int64_t)p * p, mp = m * p;
    gemm_f64(c, !trans, trans, p, p, m, 1.0, M, ldm, M, ldm, 0.0, G.d(), p, strided(B, strideM, strideM, pp));
    jacobi_eigh_f32(c, G.d(), p, p, W1.d(), lam.d(), B, pp);
    polar_b(c, W1.d(), p, p, B);
    gemm_f64(c, trans, false, m, p, p, 1.0, M, ldm, W1.d(), p, 0.0, Ux, m, strided(B, strideM, pp, mp));
    gemm_f64(c, true, false, p, p, m, 1.0, Ux, m, Ux, m, 0.0, G.d(), p, strided(B, mp, mp, pp));
    jacobi_eigh(c, G.d(), p, p, W2.d(), lam.d(), B, pp);
    gemm_f64(c, false, false, p, p, p, 1.0, W1.d(), p, W2.d(), p, 0.0, V, p, strided(B, pp, pp, pp));
    gemm_f64(c, trans, false, m, p, p, 1.0, M, ldm, V, p, 0.0, Ux, m, strided(B, strideM, pp, mp));
    col_norms(c, Ux, m, (int64_t)p * B, m, s);
    col_scale(c, Ux, m, (int64_t)p * B, m, s, 2);
    check_status(c, "final_svd (batched)");
}

// copy the leading k of every p-long vector: out[b*k + i] = in[b*p + i]
void copy_lead(Ctx& c, const double* in, int p, int k, int B, double* out) {
    TNR_CUDA(cudaMemcpy2DAsync(out, k * sizeof(double), in, p * sizeof(double), k * sizeof(double), B,
                               cudaMemcpyDeviceToDevice, c.stream));
}

}  // namespace

// Split precision: the final Rayleigh-Ritz step of B lockstep instances.  Uq [B][m x r] comes
// from CholeskyQR3 with split Grams and FP32 Cholesky factors; the orthonormal basis Q' = Uq P,
// P = L^-T with Uq^T Uq = L L^T (FP64), is never formed: P is folded into the r x r problems.
// With Z = M^T Uq (the projection, on the tensor cores with chunked accumulation),
// Z' = M^T Q' = Z P and Z'^T Z' = P^T (Z^T Z) P = Vb S^2 Vb^T, so U = Uq (P Vb_k),
// S_k = the column norms of Z (P Vb_k) and Vt = (Z P Vb_k / S_k)^T.
// The eigenvectors of the r x r Gram come from an FP32 Jacobi alignment (polar-corrected
// in FP64) and a mixed-precision Jacobi cleanup.  FP64 GEMM work: two Grams over the long dimension
// and two rank-k products, against the plain path's polar step and one-sided final SVD
// (four long-dimension products more).  A Gram of Z loses relative accuracy of singular
// values below ~1e-8 of the largest (FP64 rounding of the squares), which is the noise floor
// of the split products anyway.  Returns the B x k kept values (host).
std::vector<double> final_rr_split(Ctx& c, const SplitA& PMt, const double* M, int64_t m, int64_t n, int r, int k,
                                   int B, const double* Uq, double* U, double* s, double* Vt) {
    const int64_t mn = m * n, mr = m * r, nr = n * r, rr = (int64_t)r * r, rk = (int64_t)r * k;
    Buf P(c.pool.get(), (size_t)B * rr * sizeof(double));
    Buf E(c.pool.get(), (size_t)B * rr * sizeof(double));
    Buf E2(c.pool.get(), (size_t)B * rr * sizeof(double));
    // P with (Uq P)^T (Uq P) = I: P = L^-T from the FP64 Cholesky of the exact Gram Uq^T Uq (a
    // tiny shift only if it breaks down: numerically dependent noise columns).  It holds for any
    // departure from orthonormality, which matters: on a numerically rank-deficient M the split
    // CholeskyQR3 leaves the noise directions of Uq far from orthonormal (||Uq^T Uq - I|| ~ 0.2
    // was seen), where a polar series in Uq^T Uq - I inflated sigma_1 by 1%.  P holds L^-1.
    gemm_f64(c, true, false, r, r, m, 1.0, Uq, m, Uq, m, 0.0, E.d(), r, strided(B, mr, mr, rr));
    double shift = 0.0;
    for (int attempt = 0;; ++attempt) {
        copy_f64(c, P.d(), E.d(), rr * B);
        chol_inv(c, P.d(), r, shift, B);
        int st = c.read_status_and_clear();
        if (!(st & ST_CHOL_BREAKDOWN)) break;
        TNR_REQUIRE(attempt < 8, TNR_ERR_NOT_CONVERGED, "final Rayleigh-Ritz: basis Gram not positive definite");
        shift = std::max(shift * 30.0, 1e-14);
    }
    // the projection Z = M^T Uq (n x r)
    Buf Z(c.pool.get(), (size_t)B * nr * sizeof(double));
    gemm_bulk_a(c, PMt, true, false, n, r, m, 1.0, M, m, Uq, m, 0.0, Z.d(), n, strided(B, mn, mr, nr), true);
    // Gp = P^T (Z^T Z) P = L^-1 (Z^T Z) L^-T
    Buf G(c.pool.get(), (size_t)B * rr * sizeof(double));
    gemm_f64(c, true, false, r, r, n, 1.0, Z.d(), n, Z.d(), n, 0.0, G.d(), r, strided(B, nr, nr, rr));
    gemm_f64(c, false, true, r, r, r, 1.0, G.d(), r, P.d(), r, 0.0, E.d(), r, strided(B, rr, rr, rr));
    gemm_f64(c, false, false, r, r, r, 1.0, P.d(), r, E.d(), r, 0.0, G.d(), r, strided(B, rr, rr, rr));
    // eigenvectors Vb of Gp: FP32 alignment W1 (made orthogonal in FP64), FP64 cleanup W2
    Buf W1(c.pool.get(), (size_t)B * rr * sizeof(double));
    Buf lam(c.pool.get(), (size_t)B * r * sizeof(double));
    jacobi_eigh_f32(c, G.d(), r, r, W1.d(), lam.d(), B, rr);
    polar_b(c, W1.d(), r, r, B);
    gemm_f64(c, false, false, r, r, r, 1.0, G.d(), r, W1.d(), r, 0.0, E.d(), r, strided(B, rr, rr, rr));
    gemm_f64(c, true, false, r, r, r, 1.0, W1.d(), r, E.d(), r, 0.0, E2.d(), r, strided(B, rr, rr, rr));
    // the cleanup resolves what the split products carry: rotations below 1e-10 of the pair's
    // diagonal scale or 1e-16 of |G| (eigenvalues below ~1e-16 of the largest, singular values
    // below ~1e-8 of the largest, lie under the split noise floor) are not worth a sweep; E2 is
    // nearly diagonal, so the mixed-precision Jacobi (FP64 diagonal) holds FP64 accuracy
    jacobi_eigh_mixed(c, E2.d(), r, r, G.d(), lam.d(), B, rr, 1e-10, 1e-16);   // W2 into G
    gemm_f64(c, false, false, r, r, r, 1.0, W1.d(), r, G.d(), r, 0.0, E.d(), r, strided(B, rr, rr, rr));   // Vb
    // PV = P Vb_k = L^-T Vb_k (r x k)
    Buf PV(c.pool.get(), (size_t)B * rk * sizeof(double));
    gemm_f64(c, true, false, r, k, r, 1.0, P.d(), r, E.d(), r, 0.0, PV.d(), r, strided(B, rr, rr, rk));
    // U = Uq PV; Ub = Z PV = Vt^T S
    gemm_f64(c, false, false, m, k, r, 1.0, Uq, m, PV.d(), r, 0.0, U, m, strided(B, mr, rk, m * k));
    Buf Ub(c.pool.get(), (size_t)B * n * k * sizeof(double));
    gemm_f64(c, false, false, n, k, r, 1.0, Z.d(), n, PV.d(), r, 0.0, Ub.d(), n, strided(B, nr, rk, n * k));
    col_norms(c, Ub.d(), n, (int64_t)k * B, n, s);
    col_scale(c, Ub.d(), n, (int64_t)k * B, n, s, 2);
    transpose_lead(c, Ub.d(), n, k, k, B, Vt);
    check_status(c, "final Rayleigh-Ritz (split)");
    return to_host(c, s, (int64_t)B * k);
}

static std::vector<TsvdOut> tsvd_batched_impl(Ctx& c, const double* M, int64_t m, int64_t n, int k, int B, double* U,
                                              double* s, double* Vt, std::vector<int>& flagged);

// M: B stacked m x n matrices (ld m, stride m*n).  U [B][m x k], s [B][k], Vt [B][k x n].
// A member whose gap at k is too small for the subspace iteration leaves the batch's
// iteration count alone and is decomposed again on its own by the FP64 gap fallback.
std::vector<TsvdOut> tsvd_batched(Ctx& c, const double* M, int64_t m, int64_t n, int k, int B, double* U, double* s,
                                  double* Vt) {
    std::vector<int> flagged;
    c.decompositions += (uint64_t)std::max(B, 0);
    std::vector<TsvdOut> outs = tsvd_batched_impl(c, M, m, n, k, B, U, s, Vt, flagged);
    const int64_t kk = outs.empty() ? 0 : outs[0].k;
    for (int b : flagged)
        outs[(size_t)b] = tsvd_gap_fallback(c, M + (size_t)b * m * n, m, n, (int)kk, U + (size_t)b * m * kk,
                                            s + (size_t)b * kk, Vt + (size_t)b * kk * n);
    for (auto& o : outs) c.max_iters = std::max(c.max_iters, o.iters);
    return outs;
}

static std::vector<TsvdOut> tsvd_batched_impl(Ctx& c, const double* M, int64_t m, int64_t n, int k, int B, double* U,
                                              double* s, double* Vt, std::vector<int>& flagged) {
    std::vector<TsvdOut> outs((size_t)B);
    const int64_t p = std::min(m, n);
    k = (int)std::min<int64_t>(k, p);
    for (auto& o : outs) o.k = k;
    if (k <= 0 || B <= 0) return outs;
    const int64_t mn = m * n;
    if (p <= RDIRECT) {
        const int pp = (int)p;
        const bool wide = m < n;
        const int64_t rows = wide ? n : m;
        Buf Ux(c.pool.get(), (size_t)B * rows * pp * sizeof(double));
        Buf V(c.pool.get(), (size_t)B * pp * pp * sizeof(double));
        Buf sv(c.pool.get(), (size_t)B * pp * sizeof(double));
        final_svd_b(c, M, wide, rows, pp, B, mn, Ux.d(), sv.d(), V.d());
        if (!wide) {
            // U[b] = Ux[b][:, :k] (m x k), Vt[b] = V[b][:, :k]^T
            TNR_CUDA(cudaMemcpy2DAsync(U, m * k * sizeof(double), Ux.d(), m * pp * sizeof(double),
                                       m * k * sizeof(double), B, cudaMemcpyDeviceToDevice, c.stream));
            transpose_lead(c, V.d(), pp, pp, k, B, Vt);
        } else {
            TNR_CUDA(cudaMemcpy2DAsync(U, m * k * sizeof(double), V.d(), (int64_t)pp * pp * sizeof(double),
                                       m * k * sizeof(double), B, cudaMemcpyDeviceToDevice, c.stream));
            transpose_lead(c, Ux.d(), n, pp, k, B, Vt);
        }
        copy_lead(c, sv.d(), pp, k, B, s);
        std::vector<double> vals = to_host(c, sv.d(), (int64_t)B * pp);
        for (int b = 0; b < B; ++b) outs[b].vals.assign(vals.begin() + (size_t)b * pp, vals.begin() + (size_t)b * pp + k);
        return outs;
    }
    int r = (int)std::min<int64_t>({p, (int64_t)RMAX, (int64_t)((3 * k + 7) / 8 * 8)});
    r = std::max(r, std::min((int)p, k + 8));
    const int64_t mr = m * r, nr = n * r, rr = (int64_t)r * r;
    Buf Om(c.pool.get(), (size_t)n * r * sizeof(double));
    Buf Y(c.pool.get(), (size_t)B * mr * sizeof(double));
    Buf Uq(c.pool.get(), (size_t)B * mr * sizeof(double));
    Buf Z(c.pool.get(), (size_t)B * nr * sizeof(double));
    Buf Vq(c.pool.get(), (size_t)B * nr * sizeof(double));
    Buf G(c.pool.get(), (size_t)B * rr * sizeof(double));
    Buf W(c.pool.get(), (size_t)B * rr * sizeof(double));
    Buf lam(c.pool.get(), (size_t)B * r * sizeof(double));
    fill_normal(c, Om.d(), n * (int64_t)r, c.seed + 0x1000193ull * (++c.call_counter));
    // the split precision splits every M[b] into BF16 planes once for every product of the iteration
    SplitA PM, PMt;
    split_a_prepare(c, PM, false, M, m, m, n, r, strided(B, mn, 0, 0));
    split_a_prepare(c, PMt, true, M, m, n, m, r, strided(B, mn, 0, 0));
    gemm_bulk_a(c, PM, false, false, m, r, n, 1.0, M, m, Om.d(), n, 0.0, Y.d(), m, strided(B, mn, 0, mr));
    orth_b(c, Y.d(), m, r, B, Uq.d());
    const double target = c.precision == TNR_PREC_F64 ? TNR_TARGET_F64 : 1e-9;
    int need = MAXIT, it = 0;
    for (; it < need; ++it) {
        gemm_bulk_a(c, PMt, true, false, n, r, m, 1.0, M, m, Uq.d(), m, 0.0, Z.d(), n, strided(B, mn, mr, nr));
        if (it == 0 || it == 2) sigma_estimates(c, Z.d(), n, r, B, G.d(), W.d(), Vq.d(), lam.d());
        orth_b(c, Z.d(), n, r, B, Vq.d());
        gemm_bulk_a(c, PM, false, false, m, r, n, 1.0, M, m, Vq.d(), n, 0.0, Y.d(), m, strided(B, mn, nr, mr));
        orth_b(c, Y.d(), m, r, B, Uq.d());
        if (it == 0 || it == 2) {
            std::vector<double> est = to_host(c, lam.d(), (int64_t)B * r);
            int mx = 2;
            for (int b = 0; b < B; ++b) {
                std::vector<double> eb(est.begin() + (size_t)b * r, est.begin() + (size_t)(b + 1) * r);
                if (it == 0 && gap_too_small(c, eb, k, r, 2, target, iteration_cap(c))) flagged.push_back(b);
                if (std::find(flagged.begin(), flagged.end(), b) != flagged.end()) continue;
                mx = std::max(mx, iterations_needed(eb, k, r, 2, target, iteration_cap(c)));
            }
            need = std::max(it + 1, mx);
            check_status(c, "tsvd (batched)");
        }
    }
    for (auto& o : outs) o.iters = it;
    if (c.precision == TNR_PREC_SPLIT) {
        std::vector<double> kept = final_rr_split(c, PMt, M, m, n, r, k, B, Uq.d(), U, s, Vt);
        for (int b = 0; b < B; ++b) outs[b].vals.assign(kept.begin() + (size_t)b * k, kept.begin() + (size_t)(b + 1) * k);
        return outs;
    }
    polar_b(c, Uq.d(), m, r, B);
    Buf Ub(c.pool.get(), (size_t)B * nr * sizeof(double));
    Buf Vb(c.pool.get(), (size_t)B * rr * sizeof(double));
    Buf sb(c.pool.get(), (size_t)B * r * sizeof(double));
    // split precision: the projection on the tensor cores with chunked (unbiased) accumulation
    gemm_bulk_a(c, PMt, true, false, n, r, m, 1.0, M, m, Uq.d(), m, 0.0, Z.d(), n, strided(B, mn, mr, nr), true);
    final_svd_b(c, Z.d(), false, n, r, B, nr, Ub.d(), sb.d(), Vb.d());
    gemm_f64(c, false, false, m, k, r, 1.0, Uq.d(), m, Vb.d(), r, 0.0, U, m, strided(B, mr, rr, m * k));
    copy_lead(c, sb.d(), r, k, B, s);
    transpose_lead(c, Ub.d(), n, r, k, B, Vt);
    std::vector<double> cur = to_host(c, sb.d(), (int64_t)B * r);
    for (int b = 0; b < B; ++b) outs[b].vals.assign(cur.begin() + (size_t)b * r, cur.begin() + (size_t)b * r + k);
    return outs;
}

}  // namespace tnr
