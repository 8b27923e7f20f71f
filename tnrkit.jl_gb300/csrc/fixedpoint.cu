// Finalizers on the fixed-point tensor of a 2D scheme (src/utility/cft.jl,
// src/utility/finalize.jl:17-41): the column transfer matrix and its eigenvalues (cft_data,
// ground_state_degeneracy), the Gu-Wen traces, the central charge's largest singular value and
// the 2 x 2 plaquette norm.  All of it runs once per call on small objects (chi x chi matrices,
// one pass over T), so the kernels are single-CTA reductions with a fixed summation order.
#include "schemes.cuh"
#include "hqr.cuh"

#include <cmath>
#include <cstring>

namespace tnr {

namespace {

// block-wide sum of one value per thread (blockDim.x a multiple of 32, at most 1024)
__device__ double block_sum(double acc) {
    __shared__ double sh[32];
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
        r = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;   // valid in thread 0
}

// M[b, c] = inv * wb[b] wc[c] sum_a T[a, b, c, a] wa[a]  (T: d0 x d1 x d2 x d0; null weight = 1)
__global__ void k_transfer(const double* __restrict__ T, int64_t d0, int64_t d1, int64_t d2,
                           const double* __restrict__ wa, const double* __restrict__ wb,
                           const double* __restrict__ wc, double inv, double* __restrict__ M) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d1 * d2) return;
    const int64_t b = e % d1, c = e / d1;
    double acc = 0.0;
    for (int64_t a = 0; a < d0; ++a) {
        double t = T[a + d0 * (b + d1 * (c + d2 * a))];
        if (wa) t *= wa[a];
        acc += t;
    }
    if (wb) acc *= wb[b];
    if (wc) acc *= wc[c];
    M[e] = acc * inv;
}

// eigenvalues of the n x n matrix M (overwritten), one thread; flag[0] = 1 if the QR
// iteration ran out of its budget
__global__ void k_real_eigvals(double* M, int n, double* wr, double* wi, double* work, int* flag) {
    if (blockIdx.x == 0 && threadIdx.x == 0) flag[0] = real_eigvals(M, n, wr, wi, work);
}

// out[0] = |sum_{a,b} Tu[a,b,b,a]|, out[1] = |sum_{a,c} P[a,c] P[c,a]| with P[a,c] =
// sum_b Tu[a,b,b,c], out[2] = |sum Tu[a,b,c,d] Tu[d,c,b,a]|, where Tu[a,b,c,d] =
// T[a,b,c,d] wa[a] wb[b] (T: d0 x d1 x d1 x d0).  P (d0 x d0) is scratch.
__global__ void k_gu_wen_partial(const double* __restrict__ T, int64_t d0, int64_t d1, const double* __restrict__ wa,
                                 const double* __restrict__ wb, double* __restrict__ P) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d0 * d0) return;
    const int64_t a = e % d0, c = e / d0;
    double acc = 0.0;
    for (int64_t b = 0; b < d1; ++b) {
        double t = T[a + d0 * (b + d1 * (b + d1 * c))];
        if (wb) t *= wb[b];
        acc += t;
    }
    P[e] = wa ? acc * wa[a] : acc;
}

__global__ void k_gu_wen_sums(const double* __restrict__ T, int64_t d0, int64_t d1, const double* __restrict__ wa,
                              const double* __restrict__ wb, const double* __restrict__ P, double* __restrict__ out) {
    double one = 0.0, x1 = 0.0, x2 = 0.0;
    for (int64_t e = threadIdx.x; e < d0 * d1; e += blockDim.x) {
        const int64_t a = e % d0, b = e / d0;
        double t = T[a + d0 * (b + d1 * (b + d1 * a))];
        if (wa) t *= wa[a];
        if (wb) t *= wb[b];
        one += t;
    }
    for (int64_t e = threadIdx.x; e < d0 * d0; e += blockDim.x) {
        const int64_t a = e % d0, c = e / d0;
        x1 += P[a + d0 * c] * P[c + d0 * a];
    }
    const int64_t n = d0 * d1 * d1 * d0;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
        const int64_t a = e % d0, b = (e / d0) % d1, c = (e / (d0 * d1)) % d1, d = e / (d0 * d1 * d1);
        double t = T[e] * T[d + d0 * (c + d1 * (b + d1 * a))];
        if (wa) t *= wa[a] * wa[d];
        if (wb) t *= wb[b] * wb[c];
        x2 += t;
    }
    one = block_sum(one);
    x1 = block_sum(x1);
    x2 = block_sum(x2);
    if (threadIdx.x == 0) {
        out[0] = fabs(one);
        out[1] = fabs(x1);
        out[2] = fabs(x2);
    }
}

// out[i] = sum_a P[a, i, a] for P of dims (da, inner, da): closes the ring of transfer tensors
__global__ void k_ring_close(const double* __restrict__ P, int64_t da, int64_t inner, double* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= inner) return;
    double acc = 0.0;
    for (int64_t a = 0; a < da; ++a) acc += P[a + da * (i + inner * a)];
    out[i] = acc;
}

// dst[0] = |src[0]|^(1/4)
__global__ void k_root4_abs(double* dst, const double* src) { dst[0] = pow(fabs(src[0]), 0.25); }

}  // namespace

// the bond weights of BTRG's unit tensor: S1 on leg 2 (dim d2), S2 on leg 1 (dim d1)
static void btrg_weights(const Scheme& s, const double** s1, const double** s2) {
    const bool btrg = s.kind == TNR_BTRG;
    *s1 = btrg ? s.S1.p() : nullptr;
    *s2 = btrg ? s.S2.p() : nullptr;
}

static DT copy_of_dt(Ctx& c, const DT& t) {
    DT o = make_dt(c.pool.get(), t.dims());
    copy_f64(c, o.p(), t.p(), t.size());
    return o;
}

static void require_2d(const Scheme& s, const char* what) {
    TNR_REQUIRE(s.kind == TNR_TRG || s.kind == TNR_BTRG || s.kind == TNR_HOTRG || s.kind == TNR_ATRG,
                TNR_ERR_INVALID_ARG, std::string(what) + " needs a TRG, BTRG, HOTRG or ATRG scheme");
    TNR_REQUIRE(s.T.rank == 4 && s.T.d[0] == s.T.d[3] && s.T.d[1] == s.T.d[2], TNR_ERR_INVALID_ARG,
                std::string(what) + " needs d1 == d4 and d2 == d3");
}

// finalize_two_by_two! (src/utility/finalize.jl:17-41): n = |T[7 1; 5 4] T[4 2; 6 7] T[3 6; 2 8]
// T[8 5; 1 3]|, for BTRG with S1 on the bonds (1, 6) and S2 on (8, 4): T1 carries S1 on leg 2 and
// S2 on leg 4, T2 S1 on leg 2, T4 S2 on leg 4.  d_norm = n^(1/4), T /= n^(1/4).
void Scheme::finalize_two_by_two_async(double* d_norm) {
    Ctx& c = *ctx;
    TNR_REQUIRE(kind == TNR_TRG || kind == TNR_BTRG || kind == TNR_HOTRG || kind == TNR_ATRG, TNR_ERR_INVALID_ARG,
                "the 2 x 2 finalizer needs a TRG, BTRG, HOTRG or ATRG scheme");
    const DT* t1 = &T;
    const DT* t2 = &T;
    const DT* t4 = &T;
    DT w1, w2, w4;
    if (kind == TNR_BTRG) {
        auto weighted = [&](DT& w, const double* leg2, const double* leg4) {
            w = make_dt(c.pool.get(), T.dims());
            copy_f64(c, w.p(), T.p(), T.size());
            if (leg2) scale_leg(c, w, 1, leg2);
            if (leg4) scale_leg(c, w, 3, leg4);
        };
        weighted(w1, S1.p(), S2.p());
        weighted(w2, S1.p(), nullptr);
        weighted(w4, nullptr, S2.p());
        t1 = &w1;
        t2 = &w2;
        t4 = &w4;
    }
    // labels 1..8 -> a..h: X[1,5,2,6] = T1[7,1,5,4] T2[4,2,6,7]; Y[6,2,5,1] = T3[3,6,2,8] T4[8,5,1,3]
    DT X = contract(c, *t1, {Lg, La, Le, Ld}, *t2, {Ld, Lb, Lf, Lg}, {La, Le, Lb, Lf});
    DT Y = contract(c, T, {Lc, Lf, Lb, Lh}, *t4, {Lh, Le, La, Lc}, {Lf, Lb, Le, La});
    std::vector<int64_t> dx = X.dims(), dy = Y.dims();
    dx.push_back(1);
    dy.push_back(1);
    DT Z = contract(c, X.p(), dx, {La, Le, Lb, Lf, Lx}, Y.p(), dy, {Lf, Lb, Le, La, Ly}, {Lx, Ly}, false);
    k_root4_abs<<<1, 1, 0, c.stream>>>(d_norm, Z.p());
    check_launch("root4_abs");
    scale_inplace(c, T.p(), T.size(), d_norm);
}

// eig_full of the unit-cell-1 column transfer matrix (src/utility/cft.jl:7-16, 41-50, 280-296):
// M[b, c] = sum_a T_unit[a, b, c, a], T_unit = T with BTRG's S1 on leg 2 and S2 on leg 1
// unitcell u > 1: u copies of T_unit on a ring, indices [i, -i, -(i+u), i+1] with the last leg
// closing on the first (cft.jl:7-15): the chain T_unit[a1, b1, c1, a2] T_unit[a2, b2, c2, a3] ... is
// contracted leg by leg, the ring closed by tracing a1 against a_{u+1}, and the (b, c) legs
// ordered as rows (b1..bu), columns (c1..cu)
static DT ring_transfer(Scheme& s, int unitcell) {
    Ctx& c = *s.ctx;
    DT Tu = copy_of_dt(c, s.T);
    if (s.kind == TNR_BTRG) {
        scale_leg(c, Tu, 1, s.S1.p());
        scale_leg(c, Tu, 0, s.S2.p());
    }
    const int64_t da = Tu.d[0], db = Tu.d[1], dc = Tu.d[2];
    // chain[a1, (b1 c1) ... (bi ci), a_{i+1}]
    DT chain = copy_of_dt(c, Tu);
    for (int i = 1; i < unitcell; ++i) {
        const int64_t inner = chain.size() / (da * da);
        DT next = contract(c, chain.p(), {da, inner, da}, {La, Lb, Lx}, Tu.p(), {da, db, dc, da}, {Lx, Lc, Ld, Le},
                           {La, Lb, Lc, Ld, Le});
        chain = std::move(next);
    }
    const int64_t inner = chain.size() / (da * da);
    DT ring = make_dt(c.pool.get(), {inner});
    k_ring_close<<<(unsigned)((inner + 255) / 256), 256, 0, c.stream>>>(chain.p(), da, inner, ring.p());
    check_launch("ring_close");
    // ring legs (b1, c1, b2, c2, ...) -> (b1, ..., bu, c1, ..., cu)
    std::vector<int64_t> dims;
    std::vector<int> perm;
    for (int i = 0; i < unitcell; ++i) {
        dims.push_back(db);
        dims.push_back(dc);
    }
    for (int i = 0; i < unitcell; ++i) perm.push_back(2 * i);
    for (int i = 0; i < unitcell; ++i) perm.push_back(2 * i + 1);
    ring.rank = (int)dims.size();
    for (int i = 0; i < ring.rank; ++i) ring.d[i] = dims[i];
    return permuted(c, ring, perm);
}

void Scheme::transfer_eigvals(int unitcell, std::vector<double>& re, std::vector<double>& im) {
    Ctx& c = *ctx;
    require_2d(*this, "the transfer matrix");
    TNR_REQUIRE(unitcell >= 1 && unitcell <= 4, TNR_ERR_INVALID_ARG, "unitcell must be 1..4");
    int64_t n = 1;
    for (int i = 0; i < unitcell; ++i) n *= T.d[1];
    TNR_REQUIRE(n <= 256, TNR_ERR_UNSUPPORTED, "transfer matrix above 256 x 256");
    const double *s1, *s2;
    btrg_weights(*this, &s1, &s2);
    Buf M(c.pool.get(), (size_t)n * n * sizeof(double)), w(c.pool.get(), (size_t)(3 * n + 1) * sizeof(double));
    if (unitcell == 1) {
        k_transfer<<<(unsigned)((n * n + 255) / 256), 256, 0, c.stream>>>(T.p(), T.d[0], T.d[1], T.d[2], s2, s1,
                                                                          nullptr, 1.0, M.d());
        check_launch("transfer");
    } else {
        DT R = ring_transfer(*this, unitcell);
        copy_f64(c, M.d(), R.p(), n * n);
    }
    double* wr = w.d();
    double* wi = wr + n;
    double* work = wi + n;
    int* flag = reinterpret_cast<int*>(work + n);
    k_real_eigvals<<<1, 1, 0, c.stream>>>(M.d(), (int)n, wr, wi, work, flag);
    check_launch("real_eigvals");
    std::vector<double> h = dvec_to_host(c, wr, 3 * n + 1);
    int f = 0;
    std::memcpy(&f, h.data() + 3 * n, sizeof(int));
    TNR_REQUIRE(f == 0, TNR_ERR_NOT_CONVERGED, "eig_full: the QR iteration did not converge");
    re.assign(h.begin(), h.begin() + n);
    im.assign(h.begin() + n, h.begin() + 2 * n);
}

// gu_wen_ratio (src/utility/cft.jl:374-396): X1 = one^2 / two_X1, X2 = one^2 / two_X2
void Scheme::gu_wen(double* x1, double* x2) {
    Ctx& c = *ctx;
    require_2d(*this, "gu_wen_ratio");
    const double *s1, *s2;
    btrg_weights(*this, &s1, &s2);
    const int64_t d0 = T.d[0], d1 = T.d[1];
    Buf P(c.pool.get(), (size_t)d0 * d0 * sizeof(double)), out(c.pool.get(), 3 * sizeof(double));
    k_gu_wen_partial<<<(unsigned)((d0 * d0 + 255) / 256), 256, 0, c.stream>>>(T.p(), d0, d1, s2, s1, P.d());
    check_launch("gu_wen_partial");
    k_gu_wen_sums<<<1, 1024, 0, c.stream>>>(T.p(), d0, d1, s2, s1, P.d(), out.d());
    check_launch("gu_wen_sums");
    std::vector<double> h = dvec_to_host(c, out.d(), 3);
    TNR_REQUIRE(std::isfinite(h[0]) && std::isfinite(h[1]) && std::isfinite(h[2]) && h[1] > 0 && h[2] > 0,
                TNR_ERR_NONFINITE, "gu_wen_ratio: non-finite or zero trace");
    *x1 = h[0] * h[0] / h[1];
    *x2 = h[0] * h[0] / h[2];
}

// central_charge (src/utility/cft.jl:256-269): log(sigma_1) 6 / pi of M = T[1 -1; -2 1] / n (BTRG:
// sum_a T[a, b, c, a] S1[c] S2[a] / n); sigma_1^2 is the largest eigenvalue of M^T M
double Scheme::central_charge(double n) {
    Ctx& c = *ctx;
    require_2d(*this, "central_charge");
    TNR_REQUIRE(std::isfinite(n) && n != 0.0, TNR_ERR_INVALID_ARG, "central_charge: n must be finite and nonzero");
    const int64_t m = T.d[1];
    TNR_REQUIRE(m <= 160, TNR_ERR_UNSUPPORTED, "central_charge: matrix above 160 x 160");
    const bool btrg = kind == TNR_BTRG;
    Buf M(c.pool.get(), (size_t)m * m * sizeof(double)), G(c.pool.get(), (size_t)m * m * sizeof(double));
    Buf W(c.pool.get(), (size_t)m * m * sizeof(double)), lam(c.pool.get(), (size_t)m * sizeof(double));
    k_transfer<<<(unsigned)((m * m + 255) / 256), 256, 0, c.stream>>>(T.p(), T.d[0], T.d[1], T.d[2],
                                                                      btrg ? S2.p() : nullptr, nullptr,
                                                                      btrg ? S1.p() : nullptr, 1.0 / n, M.d());
    check_launch("transfer");
    gemm_f64(c, true, false, m, m, m, 1.0, M.d(), m, 0, M.d(), m, 0, 0.0, G.d(), m, 0);
    jacobi_eigh(c, G.d(), m, (int)m, W.d(), lam.d());
    const int st = c.read_status_and_clear();
    TNR_REQUIRE(!(st & ST_JACOBI_NOCONV), TNR_ERR_NOT_CONVERGED, "central_charge: eigensolver did not converge");
    std::vector<double> l0 = dvec_to_host(c, lam.d(), 1);
    TNR_REQUIRE(std::isfinite(l0[0]) && l0[0] > 0, TNR_ERR_NONFINITE, "central_charge: zero or non-finite M");
    return std::log(std::sqrt(l0[0])) * 6.0 / 3.141592653589793;
}

}  // namespace tnr
