// Coarse-graining steps and normalisation of TRG, BTRG, HOTRG and HOTRG_3D on
// device-resident tensors (column-major, first leg fastest).
#include "schemes.cuh"

#include <algorithm>
#include <cmath>

namespace tnr {

std::vector<double> dvec_to_host(Ctx& c, const double* d, int64_t n) {
    std::vector<double> h((size_t)n);
    if (n) TNR_CUDA(cudaMemcpyAsync(h.data(), d, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    return h;
}

// T[..., i_leg, ...] *= v[i_leg]
__global__ void k_scale_leg(double* T, int64_t total, int64_t stride, int64_t dim, const double* v) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
        T[e] *= v[(e / stride) % dim];
}

void scale_leg(Ctx& c, DT& T, int leg, const double* v) {
    int64_t stride = 1;
    for (int i = 0; i < leg; ++i) stride *= T.d[i];
    int64_t total = T.size();
    if (!total) return;
    int g = (int)std::min<int64_t>((total + 255) / 256, (int64_t)sm_count() * 8);
    k_scale_leg<<<g, 256, 0, c.stream>>>(T.p(), total, stride, T.d[leg], v);
    check_launch("scale_leg");
}

void Scheme::record(const TsvdOut& r) {
    last_vals.insert(last_vals.end(), r.vals.begin(), r.vals.end());
    last_counts.push_back((int)r.vals.size());
}

// SVD12 (src/utility/projectors.jl:211-217): M4 as (d1 d2) x (d3 d4) -> A = U sqrt(s), B = sqrt(s) V
// sectors: decompose block by block over the sectors of M4's exact zeros (tsvd_sectors), so
// that every kept vector lies in one symmetry sector, as LAPACK's vectors of these
// block-structured matrices do
static void svd12(Scheme& s, const DT& M4, int chi, DT& A, DT& B, bool sectors = false) {
    Ctx& c = *s.ctx;
    int64_t m = M4.d[0] * M4.d[1], n = M4.d[2] * M4.d[3];
    if (M4.charged()) {
        // block by block over the charge sectors; A and B carry the new leg's charges
        DecompDT d = svd_dt(c, M4, 2, chi);
        A = std::move(d.U);
        B = std::move(d.Vt);
        if (s.pending) scale_inplace(c, d.s.d(), d.k, s.pending);   // T's folded normalisation
        col_scale(c, A.p(), m, d.k, m, d.s.d(), 1);
        row_scale(c, B.p(), d.k, n, d.k, d.s.d(), 1);
        s.record(d.info);
        return;
    }
    int k = (int)std::min<int64_t>(chi, std::min(m, n));
    A = make_dt(c.pool.get(), {M4.d[0], M4.d[1], (int64_t)k});
    B = make_dt(c.pool.get(), {(int64_t)k, M4.d[2], M4.d[3]});
    Buf sv(c.pool.get(), (size_t)k * sizeof(double));
    TsvdOut r = sectors ? tsvd_sectors(c, M4.p(), m, n, k, A.p(), sv.d(), B.p()) : tsvd(c, M4.p(), m, n, k, A.p(), sv.d(), B.p());
    if (s.pending) scale_inplace(c, sv.d(), k, s.pending);        // T's folded normalisation
    col_scale(c, A.p(), m, k, m, sv.d(), 1);
    row_scale(c, B.p(), k, n, k, sv.d(), 1);
    s.record(r);
}

// T[-1 -2;-3 -4] = D[-2;1 2] B[-1;4 1] C[4 3;-3] A[3 2;-4]  (src/schemes/trg.jl:39)
//   D[b,p,q] B[a,r,p] C[r,s,c] A[s,q,d]
static DT trg_contract(Ctx& c, const DT& D, const DT& B, const DT& C, const DT& A) {
    DT X = contract(c, D, {Lb, Lp, Lq}, B, {La, Lr, Lp}, {La, Lb, Lq, Lr});
    DT Y = contract(c, C, {Lr, Ls, Lc}, A, {Ls, Lq, Ld}, {Lq, Lr, Lc, Ld});
    return contract(c, X, {La, Lb, Lq, Lr}, Y, {Lq, Lr, Lc, Ld}, {La, Lb, Lc, Ld});
}

// step!(::TRG) (src/schemes/trg.jl:35-41)
static void step_trg(Scheme& s, int chi) {
    Ctx& c = *s.ctx;
    DT& T = s.T;
    TNR_REQUIRE(T.d[0] == T.d[3] && T.d[1] == T.d[2], TNR_ERR_INVALID_ARG, "TRG needs d1 == d4 and d2 == d3");
    DT A, B, C, D;
    svd12(s, T, chi, A, B);                         // A[i1,i2,k], B[k,i3,i4]
    DT Tp = permuted(c, T, {1, 3, 0, 2});           // transpose(T, ((2,4),(1,3)))
    svd12(s, Tp, chi, C, D);                        // C[i2,i4,k'], D[k',i1,i3]
    Tp = DT();
    s.T = trg_contract(c, D, B, C, A);
}

// svd_trunc of a (2, 2) tensor, unscaled: U[i1, i2; k], sv (k, device), Vt[k; i3, i4]
static void svd22(Scheme& s, const DT& M4, int chi, DT& U, Buf& sv, DT& Vt) {
    Ctx& c = *s.ctx;
    const int64_t m = M4.d[0] * M4.d[1], n = M4.d[2] * M4.d[3];
    const int k = (int)std::min<int64_t>(chi, std::min(m, n));
    U = make_dt(c.pool.get(), {M4.d[0], M4.d[1], (int64_t)k});
    Vt = make_dt(c.pool.get(), {(int64_t)k, M4.d[2], M4.d[3]});
    sv = Buf(c.pool.get(), (size_t)k * sizeof(double));
    TsvdOut r = tsvd(c, M4.p(), m, n, k, U.p(), sv.d(), Vt.p());
    s.record(r);
}

static DT copy_of(Ctx& c, const DT& t) {
    DT o = make_dt(c.pool.get(), t.dims());
    copy_f64(c, o.p(), t.p(), t.size());
    return o;
}

// _step!(::ATRG) (src/schemes/atrg.jl:47-81): SVD of T as (1,3) x (2,4) into A S D; the
// swapped pair M = (S D)(A S) is SVD'd into X Y (sqrt(S) on both); Q = A D X Y is SVD'd into
// H G (sqrt(S) on both) and T[-1 -2; -3 -4] = G[-1; -3 1] H[1 -2; -4]
static DT atrg_half(Scheme& s, const DT& T, int chi) {
    Ctx& c = *s.ctx;
    DT A, D, X, Y, H, G;
    Buf s1, s2, s3;
    {
        DT Tp = permuted(c, T, {0, 2, 1, 3});
        svd22(s, Tp, chi, A, s1, D);
    }
    {
        const int64_t k1 = A.d[2], mA = A.d[0] * A.d[1], nD = D.d[1] * D.d[2];
        DT C = copy_of(c, A), B = copy_of(c, D);
        col_scale(c, C.p(), mA, k1, mA, s1.d(), 0);      // C = A S
        row_scale(c, B.p(), k1, nD, k1, s1.d(), 0);      // B = S D
        // M[-1 -2; -3 -4] := B[-3; 1 -4] C[-1 1; -2]:  B[c,x,d] C[a,x,b] -> M[a,b,c,d]
        DT M = contract(c, B, {Lc, Lx, Ld}, C, {La, Lx, Lb}, {La, Lb, Lc, Ld});
        DT Mp = permuted(c, M, {0, 2, 1, 3});
        svd22(s, Mp, chi, X, s2, Y);
    }
    {
        const int64_t k2 = X.d[2], mX = X.d[0] * X.d[1], nY = Y.d[1] * Y.d[2];
        col_scale(c, X.p(), mX, k2, mX, s2.d(), 1);
        row_scale(c, Y.p(), k2, nY, k2, s2.d(), 1);
        // Q[-1 -2; -3 -4] := A[3 -3; 2] D[1; -2 4] X[4 2; -4] Y[-1 1; 3]
        //   A[c,z,b] X[d,b,w] -> AX[c,z,d,w];  Y[x,a,c] D[a,y,d] -> YD[x,c,y,d];  YD AX -> Q[x,y,z,w]
        DT AX = contract(c, A, {Lc, Lz, Lb}, X, {Ld, Lb, Lw}, {Lc, Lz, Ld, Lw});
        DT YD = contract(c, Y, {Lx, La, Lc}, D, {La, Ly, Ld}, {Lx, Lc, Ly, Ld});
        A = DT(); D = DT(); X = DT(); Y = DT();
        DT Q = contract(c, YD, {Lx, Lc, Ly, Ld}, AX, {Lc, Lz, Ld, Lw}, {Lx, Ly, Lz, Lw});
        svd22(s, Q, chi, H, s3, G);
    }
    const int64_t k3 = H.d[2], mH = H.d[0] * H.d[1], nG = G.d[1] * G.d[2];
    col_scale(c, H.p(), mH, k3, mH, s3.d(), 1);
    row_scale(c, G.p(), k3, nG, k3, s3.d(), 1);
    // T[-1 -2; -3 -4] := G[-1; -3 1] H[1 -2; -4]:  G[a,c,x] H[x,b,d] -> T[a,b,c,d]
    return contract(c, G, {La, Lc, Lx}, H, {Lx, Lb, Ld}, {La, Lb, Lc, Ld});
}

// step!(::ATRG) (src/schemes/atrg.jl:38-45): a half step, permute ((2,4),(1,3)), a half step,
// permute ((3,1),(4,2))
static void step_atrg(Scheme& s, int chi) {
    Ctx& c = *s.ctx;
    TNR_REQUIRE(s.T.d[0] == s.T.d[3] && s.T.d[1] == s.T.d[2], TNR_ERR_INVALID_ARG, "ATRG needs d1 == d4 and d2 == d3");
    DT T = atrg_half(s, s.T, chi);
    T = atrg_half(s, permuted(c, T, {1, 3, 0, 2}), chi);
    s.T = permuted(c, T, {2, 0, 3, 1});
}

// R of a QR decomposition Mat = Q R of a column-major m x n matrix (m >= n), up to an orthogonal
// factor on its rows: R' = diag(s) V^T from Mat's SVD.  The oblique projectors of ATRG_3D see R
// only through products whose SVD absorbs that factor (temp = R1 R2^T -> W1 temp W2^T), so they
// are unchanged.  At truncrank(12) these matrices can be exactly rank-deficient (the reference's
// LAPACK QR returns zero rows of R there); the SVD form needs no Cholesky of their Gram matrix.
static Buf qr_r(Ctx& c, const double* Mat, int64_t m, int64_t n) {
    TNR_REQUIRE(m >= n && n <= 160, TNR_ERR_UNSUPPORTED, "ATRG_3D: QR of a wide matrix or above 160 columns");
    Buf R(c.pool.get(), (size_t)n * n * sizeof(double));
    svd_r_factor(c, Mat, m, (int)n, R.d());
    return R;
}

// the oblique projector pair of atrg3d.jl:59-69 from Rl (left_orth R, r x n) and Rrt (the
// transpose of right_orth's L, r' x n): temp = Rl Rrt^T = U s V^T truncated to chi,
// Pa[pq; k] = Rrt^T V s^-1/2 (n x k), Pb[k; pq] = s^-1/2 U^T Rl (k x n), pseudopow for s^-1/2
static void oblique_projectors(Scheme& s, const Buf& Rl, const Buf& Rrt, int64_t n, int chi, Buf& Pa, Buf& Pb, int& k) {
    Ctx& c = *s.ctx;
    Buf tmp(c.pool.get(), (size_t)n * n * sizeof(double));
    gemm_f64(c, false, true, n, n, n, 1.0, Rl.d(), n, 0, Rrt.d(), n, 0, 0.0, tmp.d(), n, 0);
    k = (int)std::min<int64_t>(chi, n);
    Buf U(c.pool.get(), (size_t)n * k * sizeof(double)), sv(c.pool.get(), (size_t)k * sizeof(double));
    Buf Vt(c.pool.get(), (size_t)k * n * sizeof(double)), inv(c.pool.get(), (size_t)k * sizeof(double));
    TsvdOut r = tsvd(c, tmp.d(), n, n, k, U.d(), sv.d(), Vt.d());
    s.record(r);
    pseudopow(c, sv.d(), k, -0.5, inv.d());
    Pa = Buf(c.pool.get(), (size_t)n * k * sizeof(double));
    Pb = Buf(c.pool.get(), (size_t)k * n * sizeof(double));
    gemm_f64(c, true, true, n, k, n, 1.0, Rrt.d(), n, 0, Vt.d(), k, 0, 0.0, Pa.d(), n, 0);
    col_scale(c, Pa.d(), n, k, n, inv.d(), 0);
    gemm_f64(c, true, false, k, n, n, 1.0, U.d(), n, 0, Rl.d(), n, 0, 0.0, Pb.d(), k, 0);
    row_scale(c, Pb.d(), k, n, k, inv.d(), 0);
}

// _step!(::ATRG_3D) (src/schemes/atrg3d.jl:35-78) on T[t0..t5] (column-major, first leg fastest)
static DT atrg3d_half(Scheme& s, const DT& T, int chi) {
    Ctx& c = *s.ctx;
    DT A, B, C, D, X, Y;
    {
        // U, S, V = svd_trunc(permute(T, ((2,5,6), (3,4,1))))
        DT Tp = permuted(c, T, {1, 4, 5, 2, 3, 0});
        const int64_t m = Tp.d[0] * Tp.d[1] * Tp.d[2], n = Tp.d[3] * Tp.d[4] * Tp.d[5];
        const int k = (int)std::min<int64_t>(chi, std::min(m, n));
        DT U = make_dt(c.pool.get(), {Tp.d[0], Tp.d[1], Tp.d[2], (int64_t)k});
        DT V = make_dt(c.pool.get(), {(int64_t)k, Tp.d[3], Tp.d[4], Tp.d[5]});
        Buf sv(c.pool.get(), (size_t)k * sizeof(double));
        TsvdOut r = tsvd(c, Tp.p(), m, n, k, U.p(), sv.d(), V.p());
        s.record(r);
        A = permuted(c, U, {3, 0, 1, 2});            // A[k, t2; t5, t6]
        D = permuted(c, V, {3, 0, 1, 2});            // D[t1, k; t3, t4]
        C = copy_of(c, A);
        B = copy_of(c, D);
        scale_leg(c, C, 0, sv.d());                  // permute(U S)
        scale_leg(c, B, 1, sv.d());                  // permute(S V)
    }
    {
        // M[-1 -2; -3 -4 -5 -6] := B[1 -2; -3 -4] C[-1 1; -5 -6]
        DT M = contract(c, B, {Lx, Lb, Lc, Ld}, C, {La, Lx, Le, Lf}, {La, Lb, Lc, Ld, Le, Lf});
        B = DT();
        C = DT();
        DT Mp = permuted(c, M, {1, 4, 5, 2, 3, 0});
        M = DT();
        const int64_t m = Mp.d[0] * Mp.d[1] * Mp.d[2], n = Mp.d[3] * Mp.d[4] * Mp.d[5];
        const int k = (int)std::min<int64_t>(chi, std::min(m, n));
        DT U = make_dt(c.pool.get(), {Mp.d[0], Mp.d[1], Mp.d[2], (int64_t)k});
        DT V = make_dt(c.pool.get(), {(int64_t)k, Mp.d[3], Mp.d[4], Mp.d[5]});
        Buf sv(c.pool.get(), (size_t)k * sizeof(double));
        TsvdOut r = tsvd(c, Mp.p(), m, n, k, U.p(), sv.d(), V.p());
        s.record(r);
        col_scale(c, U.p(), m, k, m, sv.d(), 1);
        row_scale(c, V.p(), k, n, k, sv.d(), 1);
        X = permuted(c, U, {3, 0, 1, 2});            // X[k2, m2; m5, m6]
        Y = permuted(c, V, {3, 0, 1, 2});            // Y[m1, k2; m3, m4]
    }
    // AX[-1 -2; -3 -4 -5 -6] := A[1 -2; -3 -5] X[-1 1; -4 -6], YD likewise from Y and D
    DT AX = contract(c, A, {Lx, Lb, Lc, Le}, X, {La, Lx, Ld, Lf}, {La, Lb, Lc, Ld, Le, Lf});
    DT YD = contract(c, Y, {Lx, Lb, Lc, Le}, D, {La, Lx, Ld, Lf}, {La, Lb, Lc, Ld, Le, Lf});
    A = DT(); D = DT(); X = DT(); Y = DT();
    const int64_t y0 = YD.d[0], y1 = YD.d[1], x0 = AX.d[0], x1 = AX.d[1];
    const int64_t ab_y = y0 * y1, ab_x = x0 * x1;
    const int64_t n1 = YD.d[4] * YD.d[5], n3 = YD.d[2] * YD.d[3];
    TNR_REQUIRE(n1 == AX.d[4] * AX.d[5] && n3 == AX.d[2] * AX.d[3], TNR_ERR_INVALID_ARG, "ATRG_3D: leg mismatch");
    Buf P1, P2, P3, P4;
    int k1 = 0, k3 = 0;
    {
        // R1 = left_orth R of YD as (1,2,3,4) x (5,6); R2 = right_orth L of AX as (5,6) x (1,2,3,4),
        // whose transpose is the R of AX's natural (1,2,3,4) x (5,6) layout
        Buf R1 = qr_r(c, YD.p(), ab_y * n3, n1);
        Buf R2t = qr_r(c, AX.p(), ab_x * n3, n1);
        oblique_projectors(s, R1, R2t, n1, chi, P1, P2, k1);
    }
    {
        // R3 of YD as (1,2,5,6) x (3,4); R4 = right_orth L of AX as (3,4) x (1,2,5,6)
        DT YDp = permuted(c, YD, {0, 1, 4, 5, 2, 3});
        DT AXp = permuted(c, AX, {0, 1, 4, 5, 2, 3});
        Buf R3 = qr_r(c, YDp.p(), ab_y * n1, n3);
        Buf R4t = qr_r(c, AXp.p(), ab_x * n1, n3);
        oblique_projectors(s, R3, R4t, n3, chi, P3, P4, k3);
    }
    // H[-1 -2; -3 -4] := YD[-1 -2; 1 2 3 4] Proj_3[1 2; -3] Proj_1[3 4; -4]
    DT Z = contract(c, YD.p(), {ab_y, n3, n1}, {La, Lp, Lq}, P1.d(), {n1, (int64_t)k1}, {Lq, Lb}, {La, Lp, Lb});
    DT H = contract(c, Z.p(), Z.dims(), {La, Lp, Lb}, P3.d(), {n3, (int64_t)k3}, {Lp, Lc}, {La, Lc, Lb});
    YD = DT();
    // G[-1 -2; -3 -4] := AX[-1 -2; 1 2 3 4] Proj_4[-3; 1 2] Proj_2[-4; 3 4]
    Z = contract(c, AX.p(), {ab_x, n3, n1}, {La, Lp, Lq}, P2.d(), {(int64_t)k1, n1}, {Lb, Lq}, {La, Lp, Lb});
    DT G = contract(c, Z.p(), Z.dims(), {La, Lp, Lb}, P4.d(), {(int64_t)k3, n3}, {Lc, Lp}, {La, Lc, Lb});
    Z = DT();
    // (ab, k3, k1) read as the 4-leg H[y1, y2; k3, k1] and G[x1, x2; k3, k1]
    H.rank = 4;
    H.d[0] = y0; H.d[1] = y1; H.d[2] = k3; H.d[3] = k1;
    G.rank = 4;
    G.d[0] = x0; G.d[1] = x1; G.d[2] = k3; G.d[3] = k1;
    // T[-1 -2; -3 -4 -5 -6] := G[1 -2; -5 -6] H[-1 1; -3 -4]
    return contract(c, G, {Lx, Lb, Le, Lf}, H, {La, Lx, Lc, Ld}, {La, Lb, Lc, Ld, Le, Lf});
}

// step!(::ATRG_3D) (src/schemes/atrg3d.jl:80-90): three half steps, each followed by
// permute(T, ((4, 6), (2, 5, 1, 3)))
static void step_atrg3d(Scheme& s, int chi) {
    Ctx& c = *s.ctx;
    for (int i = 0; i < 3; ++i) s.T = permuted(c, atrg3d_half(s, s.T, chi), {3, 5, 1, 4, 0, 2});
}

// step!(::ImpurityTRG) (src/schemes/impuritytrg.jl:63-91): SVD12 of sites 1 and 3 and of the
// pure tensor, and of sites 2 and 4 and the pure tensor transposed ((2,4),(1,3)); the new
// pure and site tensors are five TRG contractions of those factors.  The contractions pair
// factors of different SVDs, so the result depends on the basis each SVD picks inside a
// degenerate group; decomposing over the sectors of the exact zeros keeps the vectors of a
// Z2-odd impurity's degenerate pairs in one sector each (the choice LAPACK makes on such
// block-structured matrices)
static void step_impurity_trg(Scheme& s, int chi) {
    Ctx& c = *s.ctx;
    TNR_REQUIRE(s.T.d[0] == s.T.d[3] && s.T.d[1] == s.T.d[2], TNR_ERR_INVALID_ARG,
                "ImpurityTRG needs d1 == d4 and d2 == d3");
    auto svd_t = [&](const DT& t, DT& C, DT& D) {
        DT tp = permuted(c, t, {1, 3, 0, 2});
        svd12(s, tp, chi, C, D, true);
    };
    DT A1, B1, C2, D2, A3, B3, C4, D4, Ap, Bp, Cp, Dp;
    svd12(s, s.site[0], chi, A1, B1, true);
    svd_t(s.site[1], C2, D2);
    svd12(s, s.site[2], chi, A3, B3, true);
    svd_t(s.site[3], C4, D4);
    svd12(s, s.T, chi, Ap, Bp, true);
    svd_t(s.T, Cp, Dp);
    DT T = trg_contract(c, Dp, Bp, Cp, Ap);
    DT N1 = trg_contract(c, Dp, B1, C2, Ap);
    DT N2 = trg_contract(c, D2, B3, Cp, Ap);
    DT N3 = trg_contract(c, D4, Bp, Cp, A3);
    DT N4 = trg_contract(c, Dp, Bp, C4, A1);
    s.T = std::move(T);
    s.site[0] = std::move(N1);
    s.site[1] = std::move(N2);
    s.site[2] = std::move(N3);
    s.site[3] = std::move(N4);
}

// step!(::BTRG) on a charged tensor: the two SVDs block by block over the charge sectors (the
// kept counts can be below chi), the 8-tensor network as blocked pairwise contractions
static void step_btrg_charged(Scheme& s, int chi) {
    Ctx& c = *s.ctx;
    DT& T = s.T;
    const double kexp = s.btrg_k;
    auto half = [&](const DT& M, DT& U, DT& V, DT& Sn) {
        DecompDT d = svd_dt(c, M, 2, chi);
        const int64_t m = M.d[0] * M.d[1], n = M.d[2] * M.d[3];
        if (s.pending) scale_inplace(c, d.s.d(), d.k, s.pending);   // T's folded normalisation
        Buf sa(c.pool.get(), (size_t)d.k * sizeof(double));
        Sn = make_dt(c.pool.get(), {(int64_t)d.k});
        pseudopow(c, d.s.d(), d.k, (1.0 - kexp) / 2.0, sa.d());
        pseudopow(c, d.s.d(), d.k, kexp, Sn.p());
        U = std::move(d.U);
        V = std::move(d.Vt);
        col_scale(c, U.p(), m, d.k, m, sa.d(), 0);
        row_scale(c, V.p(), d.k, n, d.k, sa.d(), 0);
        s.record(d.info);
    };
    DT A, B, C, D, S1n, S2n;
    half(T, A, B, S1n);
    half(permuted(c, T, {2, 0, 3, 1}), C, D, S2n);
    scale_leg(c, D, 2, s.S1.p());
    scale_leg(c, D, 1, s.S2.p());
    scale_leg(c, B, 2, s.S2.p());
    scale_leg(c, C, 0, s.S1.p());
    DT X = contract(c, D, {La, Lx, Lp}, B, {Lb, Lp, Ly}, {La, Lb, Lx, Ly});
    DT Y = contract(c, C, {Lz, Ly, Ld}, A, {Lx, Lz, Lc}, {Lx, Ly, Lc, Ld});
    A = DT(); B = DT(); C = DT(); D = DT();
    s.T = contract(c, X, {La, Lb, Lx, Ly}, Y, {Lx, Ly, Lc, Ld}, {La, Lb, Lc, Ld});
    s.S1 = std::move(S1n);
    s.S2 = std::move(S2n);
}

// step!(::BTRG) (src/schemes/btrg.jl:60-94)
static void step_btrg(Scheme& s, int chi) {
    Ctx& c = *s.ctx;
    DT& T = s.T;
    TNR_REQUIRE(T.d[0] == T.d[3] && T.d[1] == T.d[2], TNR_ERR_INVALID_ARG, "BTRG needs d1 == d4 and d2 == d3");
    const double kexp = s.btrg_k;
    const int64_t d1 = T.d[0], d2 = T.d[1], d3 = T.d[2], d4 = T.d[3];
    if (T.charged()) {
        step_btrg_charged(s, chi);
        return;
    }
    // first SVD: T as (d1 d2) x (d3 d4)
    int64_t m = d1 * d2, n = d3 * d4;
    int k1 = (int)std::min<int64_t>(chi, std::min(m, n));
    DT A = make_dt(c.pool.get(), {d1, d2, (int64_t)k1});
    DT B = make_dt(c.pool.get(), {(int64_t)k1, d3, d4});
    DT S1n = make_dt(c.pool.get(), {(int64_t)k1});
    {
        Buf sv(c.pool.get(), (size_t)k1 * sizeof(double)), sa(c.pool.get(), (size_t)k1 * sizeof(double));
        TsvdOut r = tsvd(c, T.p(), m, n, k1, A.p(), sv.d(), B.p());
        if (s.pending) scale_inplace(c, sv.d(), k1, s.pending);   // T's folded normalisation
        pseudopow(c, sv.d(), k1, (1.0 - kexp) / 2.0, sa.d());
        pseudopow(c, sv.d(), k1, kexp, S1n.p());
        col_scale(c, A.p(), m, k1, m, sa.d(), 0);
        row_scale(c, B.p(), k1, n, k1, sa.d(), 0);
        s.record(r);
    }
    // second SVD: permute(T, ((3,1),(4,2))) as (d3 d1) x (d4 d2)
    DT P = permuted(c, T, {2, 0, 3, 1});
    int64_t m2 = d3 * d1, n2 = d4 * d2;
    int k2 = (int)std::min<int64_t>(chi, std::min(m2, n2));
    DT C = make_dt(c.pool.get(), {d3, d1, (int64_t)k2});
    DT D = make_dt(c.pool.get(), {(int64_t)k2, d4, d2});
    DT S2n = make_dt(c.pool.get(), {(int64_t)k2});
    {
        Buf sv(c.pool.get(), (size_t)k2 * sizeof(double)), sa(c.pool.get(), (size_t)k2 * sizeof(double));
        TsvdOut r = tsvd(c, P.p(), m2, n2, k2, C.p(), sv.d(), D.p());
        if (s.pending) scale_inplace(c, sv.d(), k2, s.pending);
        pseudopow(c, sv.d(), k2, (1.0 - kexp) / 2.0, sa.d());
        pseudopow(c, sv.d(), k2, kexp, S2n.p());
        col_scale(c, C.p(), m2, k2, m2, sa.d(), 0);
        row_scale(c, D.p(), k2, n2, k2, sa.d(), 0);
        s.record(r);
    }
    P = DT();
    // T[-1 -2;-3 -4] = D[-1;4 7] S1[1;7] B[-2;1 3] S2[3;2] C[8 2;-4] S1[8;5] A[6 5;-3] S2[4;6]
    // with diagonal S1 (dim d2) and S2 (dim d1):  D[a,x,p] S1[p] S2[x], B[b,p,y] S2[y], C[z,y,d] S1[z], A[x,z,c]
    scale_leg(c, D, 2, s.S1.p());
    scale_leg(c, D, 1, s.S2.p());
    scale_leg(c, B, 2, s.S2.p());
    scale_leg(c, C, 0, s.S1.p());
    DT X = contract(c, D, {La, Lx, Lp}, B, {Lb, Lp, Ly}, {La, Lb, Lx, Ly});
    DT Y = contract(c, C, {Lz, Ly, Ld}, A, {Lx, Lz, Lc}, {Lx, Ly, Lc, Ld});
    A = DT(); B = DT(); C = DT(); D = DT();
    s.T = contract(c, X, {La, Lb, Lx, Ly}, Y, {Lx, Ly, Lc, Ld}, {La, Lb, Lc, Ld});
    s.S1 = std::move(S1n);
    s.S2 = std::move(S2n);
}

// eigh_trunc!(project_hermitian!(MM)) of a (rows x rows) Gram tensor -> U[r1, r2, k]
static DT eig_proj(Scheme& s, const DT& MM, int chi, TsvdOut& out) {
    Ctx& c = *s.ctx;
    if (MM.charged()) {
        DecompDT d = eigh_dt(c, MM, 2, chi);
        out = d.info;
        return std::move(d.U);
    }
    int64_t n = MM.d[0] * MM.d[1];
    int k = (int)std::min<int64_t>(chi, n);
    DT U = make_dt(c.pool.get(), {MM.d[0], MM.d[1], (int64_t)k});
    Buf lam(c.pool.get(), (size_t)k * sizeof(double));
    out = teigh(c, MM.p(), n, k, U.p(), lam.d());
    return U;
}

// choose between the two projectors: keep U unless eps > eps' (hotrg.jl:112-114)
static DT choose_proj(Scheme& s, DT&& U, TsvdOut& r, DT&& U2, TsvdOut& r2) {
    s.last_eps.push_back(r.err);
    s.last_eps.push_back(r2.err);
    if (r.err > r2.err) {
        s.record(r2);
        return std::move(U2);
    }
    s.record(r);
    return std::move(U);
}

// A copy of U with every charge negated: for real data the adjoint U' of TensorKit's network
// has the same entries and dual legs.
static DT dual_copy(Ctx& c, const DT& U) {
    DT o = make_dt(c.pool.get(), U.dims());
    copy_f64(c, o.p(), U.p(), U.size());
    o.N = U.N;
    for (const auto& q : U.q) {
        std::vector<int> nq(q.size());
        for (size_t i = 0; i < q.size(); ++i) nq[i] = (U.N - q[i] % U.N) % U.N;
        o.q.push_back(nq);
    }
    return o;
}

// _get_hotrg_xproj (src/schemes/hotrg.jl:82-116) with A1 = A2 = T
static DT hotrg_xproj(Scheme& s, const DT& T, int chi) {
    Ctx& c = *s.ctx;
    TsvdOut r1, r2;
    DT U1, U2;
    // conj(A): the same entries; a charged tensor's conjugate carries the dual charges
    DT Tdual;
    if (T.charged()) Tdual = dual_copy(c, T);
    const DT& Tc = T.charged() ? Tdual : T;
    {
        // MM[-1 -2;-3 -4] = A2[-1 5;1 2] A1[-2 3;5 4] conj(A2[-3 6;1 2]) conj(A1[-4 3;6 4])
        DT X = contract(c, T, {La, Le, Li, Lj}, Tc, {Lc, Lf, Li, Lj}, {La, Le, Lc, Lf}, false);
        DT Y = contract(c, T, {Lb, Lk, Le, Ll}, Tc, {Ld, Lk, Lf, Ll}, {Lb, Le, Ld, Lf}, false);
        DT MM = contract(c, X, {La, Le, Lc, Lf}, Y, {Lb, Le, Ld, Lf}, {La, Lb, Lc, Ld}, false);
        U1 = eig_proj(s, MM, chi, r1);
    }
    {
        // MM = conj(A2[2 5;1 -1]) conj(A1[4 3;5 -2]) A2[2 6;1 -3] A1[4 3;6 -4]
        DT X = contract(c, Tc, {Lj, Le, Li, La}, T, {Lj, Lf, Li, Lc}, {Le, La, Lf, Lc}, false);
        DT Y = contract(c, Tc, {Ll, Lk, Le, Lb}, T, {Ll, Lk, Lf, Ld}, {Le, Lb, Lf, Ld}, false);
        DT MM = contract(c, X, {Le, La, Lf, Lc}, Y, {Le, Lb, Lf, Ld}, {La, Lb, Lc, Ld}, false);
        U2 = eig_proj(s, MM, chi, r2);
    }
    return choose_proj(s, std::move(U1), r1, std::move(U2), r2);
}

// _get_hotrg_yproj (src/schemes/hotrg.jl:118-152)
static DT hotrg_yproj(Scheme& s, const DT& T, int chi) {
    Ctx& c = *s.ctx;
    TsvdOut r1, r2;
    DT U1, U2;
    DT Tdual;
    if (T.charged()) Tdual = dual_copy(c, T);
    const DT& Tc = T.charged() ? Tdual : T;
    {
        // MM = A1[1 -1;2 5] A2[5 -2;4 3] conj(A1[1 -3;2 6]) conj(A2[6 -4;4 3])
        DT X = contract(c, T, {Li, La, Lj, Lp}, Tc, {Li, Lc, Lj, Lr}, {La, Lp, Lc, Lr}, false);
        DT Y = contract(c, T, {Lp, Lb, Ll, Lk}, Tc, {Lr, Ld, Ll, Lk}, {Lp, Lb, Lr, Ld}, false);
        DT MM = contract(c, X, {La, Lp, Lc, Lr}, Y, {Lp, Lb, Lr, Ld}, {La, Lb, Lc, Ld}, false);
        U1 = eig_proj(s, MM, chi, r1);
    }
    {
        // MM = conj(A1[1 2;-1 5]) conj(A2[5 4;-2 3]) A1[1 2;-3 6] A2[6 4;-4 3]
        DT X = contract(c, Tc, {Li, Lj, La, Lp}, T, {Li, Lj, Lc, Lr}, {La, Lp, Lc, Lr}, false);
        DT Y = contract(c, Tc, {Lp, Ll, Lb, Lk}, T, {Lr, Ll, Ld, Lk}, {Lp, Lb, Lr, Ld}, false);
        DT MM = contract(c, X, {La, Lp, Lc, Lr}, Y, {Lp, Lb, Lr, Ld}, {La, Lb, Lc, Ld}, false);
        U2 = eig_proj(s, MM, chi, r2);
    }
    return choose_proj(s, std::move(U1), r1, std::move(U2), r2);
}

// The HOTRG half steps on charged tensors, as blocked pairwise contractions in the same
// order as the dense plans below (chi^6, chi^7, chi^6 flops); the projector on the
// incoming side is the adjoint (dual charges).
//   y: T'[a,b,g,d] = Ux'[i,j,a] Ux[k,l,d] A2[i,e,g,k] A1[j,b,e,l]
//   x: T'[a,b,c,d] = A1[a,i,k,e] A2[e,j,l,d] Uy'[i,j,b] Uy[k,l,c]
static DT hotrg_step_y_charged(Ctx& c, const DT& A1, const DT& A2, const DT& Ux) {
    DT Ud = dual_copy(c, Ux);
    DT W = contract(c, A1, {Lj, Lb, Le, Ll}, Ud, {Li, Lj, La}, {Lb, Le, Ll, Li, La});
    Ud = DT();
    DT V = contract(c, W, {Lb, Le, Ll, Li, La}, A2, {Li, Le, Lg, Lk}, {Lb, Ll, La, Lg, Lk});
    W = DT();
    return contract(c, V, {Lb, Ll, La, Lg, Lk}, Ux, {Lk, Ll, Ld}, {La, Lb, Lg, Ld});
}
static DT hotrg_step_x_charged(Ctx& c, const DT& A1, const DT& A2, const DT& Uy) {
    DT Ud = dual_copy(c, Uy);
    DT W = contract(c, A1, {La, Li, Lk, Le}, Ud, {Li, Lj, Lb}, {La, Lk, Le, Lj, Lb});
    Ud = DT();
    DT V = contract(c, W, {La, Lk, Le, Lj, Lb}, A2, {Le, Lj, Ll, Ld}, {La, Lk, Lb, Ll, Ld});
    W = DT();
    return contract(c, V, {La, Lk, Lb, Ll, Ld}, Uy, {Lk, Ll, Lc}, {La, Lb, Lc, Ld});
}

// _step_hotrg_y (src/schemes/hotrg.jl:42-60), A1 = A2 = T (dims dL, dD, dU, dR):
//   T'[a,b,g,d] = Ux[i,j,a] Ux[k,l,d] A2[i,e,g,k] A1[j,b,e,l]
// as W2[b,l,e,i,a] = A1p[j,(b,l,e)] Uxp[j,(i,a)];  V[b,l,k,g,a] = W2[(b,l),(e,i)] A2p[(e,i),(k,g)] per a;
//    O[b,d,g,a] = V[b,(l,k)] Uxq[(l,k),d] per (g,a);  T' = O permuted (a,b,g,d).
// (A1 and A2 of equal dims: the pure tensor twice for HOTRG, impurity pairs for ImpurityHOTRG)
// in_scale: A1 and A2 are read divided by |*in_scale| (a folded normalisation), or NULL
static DT hotrg_step_y2(Ctx& c, const DT& A1, const DT& A2, const DT& Ux, const double* in_scale = nullptr) {
    if (A1.charged() && A2.charged() && Ux.charged()) {
        TNR_REQUIRE(!in_scale, TNR_ERR_INVALID_ARG, "HOTRG: a folded normalisation on the charged path");
        return hotrg_step_y_charged(c, A1, A2, Ux);
    }
    const int64_t dL = A1.d[0], dD = A1.d[1], dU = A1.d[2], dR = A1.d[3], kx = Ux.d[2];
    TNR_REQUIRE(Ux.d[0] == dL && Ux.d[1] == dL && dL == dR && dD == dU, TNR_ERR_INVALID_ARG, "HOTRG y-step dims");
    for (int l = 0; l < 4; ++l) TNR_REQUIRE(A2.d[l] == A1.d[l], TNR_ERR_INVALID_ARG, "HOTRG y-step: A1/A2 dims differ");
    DT A1p = permuted_scaled(c, A1, {0, 1, 3, 2}, in_scale);         // [j,b,l,e]
    DT Uxp = permuted(c, Ux, {1, 0, 2});            // [j,i,a]
    const int64_t mW = dD * dR * dU, nW = dL * kx;
    DT W2 = make_dt(c.pool.get(), {dD, dR, dU, dL, kx});
    gemm_bulk(c, true, false, mW, nW, dL, 1.0, A1p.p(), dL, 0, Uxp.p(), dL, 0, 0.0, W2.p(), mW, 0, 1, true);
    A1p = DT(); Uxp = DT();
    DT A2p = permuted_scaled(c, A2, {1, 0, 3, 2}, in_scale);         // [e,i,k,g]
    DT V = make_dt(c.pool.get(), {dD, dR, dR, dU, kx});
    {
        Batch2 bt;
        bt.n1 = (int)kx;
        bt.sA1 = dD * dR * dU * dL;
        bt.sB1 = 0;
        bt.sC1 = dD * dR * dR * dU;
        gemm_bulk(c, false, false, dD * dR, dR * dU, dU * dL, 1.0, W2.p(), dD * dR, A2p.p(), dU * dL, 0.0, V.p(),
                  dD * dR, bt, true);
    }
    W2 = DT(); A2p = DT();
    DT Uxq = permuted(c, Ux, {1, 0, 2});            // [l,k,d]
    DT O = make_dt(c.pool.get(), {dD, kx, dU, kx});
    {
        Batch2 bt;
        bt.n1 = (int)(dU * kx);
        bt.sA1 = dD * dR * dR;
        bt.sC1 = dD * kx;
        gemm_bulk(c, false, false, dD, kx, dR * dR, 1.0, V.p(), dD, Uxq.p(), dR * dR, 0.0, O.p(), dD, bt, true);
    }
    V = DT();
    return permuted(c, O, {3, 0, 2, 1});
}

static void hotrg_step_y(Scheme& s, const DT& Ux) { s.T = hotrg_step_y2(*s.ctx, s.T, s.T, Ux, s.pending); }

// _step_hotrg_x (src/schemes/hotrg.jl:62-80):
//   T'[a,b,c,d] = A1[a,i,k,e] A2[e,j,l,d] Uy[i,j,b] Uy[k,l,c]
// as W[a,k,e,j,b] = A1p[(a,k,e),i] Uy[i,(j,b)];  V[a,k,l,d,b] = W[(a,k),(e,j)] A2[(e,j),(l,d)] per b;
//    T'[a,b,c,d] = V[a,(k,l)] Uy[(k,l),c] per (d,b), written in place (ldc = dL*ky).
static DT hotrg_step_x2(Ctx& c, const DT& A1, const DT& A2, const DT& Uy) {
    if (A1.charged() && A2.charged() && Uy.charged()) return hotrg_step_x_charged(c, A1, A2, Uy);
    const int64_t dL = A1.d[0], dD = A1.d[1], dU = A1.d[2], dR = A1.d[3], ky = Uy.d[2];
    TNR_REQUIRE(Uy.d[0] == dD && Uy.d[1] == dD && dL == dR && dD == dU, TNR_ERR_INVALID_ARG, "HOTRG x-step dims");
    for (int l = 0; l < 4; ++l) TNR_REQUIRE(A2.d[l] == A1.d[l], TNR_ERR_INVALID_ARG, "HOTRG x-step: A1/A2 dims differ");
    DT A1p = permuted(c, A1, {0, 2, 3, 1});         // [a,k,e,i]
    const int64_t mW = dL * dU * dR;
    DT W = make_dt(c.pool.get(), {dL, dU, dR, dD, ky});
    gemm_bulk(c, false, false, mW, dD * ky, dD, 1.0, A1p.p(), mW, 0, Uy.p(), dD, 0, 0.0, W.p(), mW, 0, 1, true);
    A1p = DT();
    DT V = make_dt(c.pool.get(), {dL, dU, dU, dR, ky});
    {
        Batch2 bt;
        bt.n1 = (int)ky;
        bt.sA1 = dL * dU * dR * dD;
        bt.sC1 = dL * dU * dU * dR;
        gemm_bulk(c, false, false, dL * dU, dU * dR, dR * dD, 1.0, W.p(), dL * dU, A2.p(), dR * dD, 0.0, V.p(),
                  dL * dU, bt, true);
    }
    W = DT();
    DT Tn = make_dt(c.pool.get(), {dL, ky, ky, dR});
    {
        Batch2 bt;
        bt.n1 = (int)dR;                 // d
        bt.sA1 = dL * dU * dU;
        bt.sC1 = dL * ky * ky;
        bt.n2 = (int)ky;                 // b
        bt.sA2 = dL * dU * dU * dR;
        bt.sC2 = dL;
        gemm_bulk(c, false, false, dL, ky, dU * dU, 1.0, V.p(), dL, Uy.p(), dU * dU, 0.0, Tn.p(), dL * ky, bt, true);
    }
    return Tn;
}

static void hotrg_step_x(Scheme& s, const DT& Uy) { s.T = hotrg_step_x2(*s.ctx, s.T, s.T, Uy); }

// step!(::HOTRG) (src/schemes/hotrg.jl:154-160)
static void step_hotrg(Scheme& s, int chi) {
    DT Ux = hotrg_xproj(s, s.T, chi);
    hotrg_step_y(s, Ux);
    DT Uy = hotrg_yproj(s, s.T, chi);
    hotrg_step_x(s, Uy);
}

// step!(::ImpurityHOTRG) (src/schemes/impurityhotrg.jl:48-84): the y projector of the pure
// tensor with x-steps of the pure / impurity pairs, then the x projector with y-steps;
// first-order impurities average the two placements, the second order the four
static void step_impurity_hotrg(Scheme& s, int chi) {
    Ctx& c = *s.ctx;
    for (int half = 0; half < 2; ++half) {
        const DT U = half == 0 ? hotrg_yproj(s, s.T, chi) : hotrg_xproj(s, s.T, chi);
        auto st = [&](const DT& A1, const DT& A2) {
            return half == 0 ? hotrg_step_x2(c, A1, A2, U) : hotrg_step_y2(c, A1, A2, U);
        };
        auto mix = [&](DT a, const DT& b, double w) {     // w a + w b, into a
            lincomb2(c, a.p(), a.size(), w, a.p(), w, b.p());
            return a;
        };
        DT T = st(s.T, s.T);
        DT I11 = mix(st(s.I11, s.T), st(s.T, s.I11), 0.5);
        DT I12 = mix(st(s.I12, s.T), st(s.T, s.I12), 0.5);
        DT I2 = mix(st(s.I2, s.T), st(s.T, s.I2), 0.25);
        {
            DT cross = mix(st(s.I11, s.I12), st(s.I12, s.I11), 0.25);
            lincomb2(c, I2.p(), I2.size(), 1.0, I2.p(), 1.0, cross.p());
        }
        s.T = std::move(T);
        s.I11 = std::move(I11);
        s.I12 = std::move(I12);
        s.I2 = std::move(I2);
    }
}

// ---------------------------------------------------------------------------
// HOTRG_3D (src/schemes/hotrg3d.jl); legs (1..6) = (D, U', N, E, S', W'), bosonic
// ---------------------------------------------------------------------------
// _get_MMdag_3d / _get_MdagM_3d (hotrg3d.jl:48-84); xleg = 5 (W) or 3 (E), 0-based
static DT gram3d(Scheme& s, const DT& T, bool mdagm) {
    Ctx& c = *s.ctx;
    // labels of the six legs of A2 / A1 copies
    // MMdag: A2[z w Y X y x] A2[v w Y X y u] -> P[x,z,v,u];  A1[p z Y X y r] A1[p v Y X y s] -> N[z,r,v,s]
    // MdagM: A2[z w Y x y X] A2[v w Y u y X] -> P[x,z,v,u];  A1[p z Y r y X] A1[p v Y s y X] -> N[z,r,v,s]
    const int Y = Lh, X = Lg, y = Ly, w = Lw;
    std::vector<int> a2 = mdagm ? std::vector<int>{Lz, w, Y, Lx, y, X} : std::vector<int>{Lz, w, Y, X, y, Lx};
    std::vector<int> a2c = mdagm ? std::vector<int>{Lv, w, Y, Lu, y, X} : std::vector<int>{Lv, w, Y, X, y, Lu};
    // the adjoint copies: the same entries; a charged tensor's adjoint carries the dual charges
    DT Tdual;
    if (T.charged()) Tdual = dual_copy(c, T);
    const DT& Tc = T.charged() ? Tdual : T;
    DT P = contract(c, T, a2, Tc, a2c, {Lx, Lz, Lv, Lu}, false);
    std::vector<int> a1 = mdagm ? std::vector<int>{Lp, Lz, Y, Lr, y, X} : std::vector<int>{Lp, Lz, Y, X, y, Lr};
    std::vector<int> a1c = mdagm ? std::vector<int>{Lp, Lv, Y, Ls, y, X} : std::vector<int>{Lp, Lv, Y, X, y, Ls};
    DT N = contract(c, T, a1, Tc, a1c, {Lz, Lr, Lv, Ls}, false);
    return contract(c, P, {Lx, Lz, Lv, Lu}, N, {Lz, Lr, Lv, Ls}, {Lr, Lx, Ls, Lu}, false);
}

// _get_hotrg3d_xproj (hotrg3d.jl:86-98)
static DT hotrg3d_xproj(Scheme& s, const DT& T, int chi) {
    TsvdOut r1, r2;
    DT U1, U2;
    {
        DT MM = gram3d(s, T, false);
        U1 = eig_proj(s, MM, chi, r1);
    }
    {
        DT MM = gram3d(s, T, true);
        U2 = eig_proj(s, MM, chi, r2);
    }
    return choose_proj(s, std::move(U1), r1, std::move(U2), r2);
}

// _step_hotrg3d (hotrg3d.jl:108-117):
//   T[a,b,c,d,e,f] = Ux[x1,x2,f] Ux[x1',x2',d] Uy[y1,y2,e] Uy[y1',y2',c] A1[a,z,y1',x1',y1,x1] A2[z,b,y2',x2',y2,x2]
// contracted leg by leg (largest intermediate chi^8), sliced over the open leg a.
// The same network on a Z2-charged tensor (Z2 charges are self-dual, so the network's adjoint
// legs need no separate charges): each slice of A1 over the open leg a is copied into a
// charged tensor and every pairwise contraction runs block by block over the charge sectors.
static void hotrg3d_contract_charged(Scheme& s, const DT& Ux, const DT& Uy, int64_t max_entries) {
    Ctx& c = *s.ctx;
    const DT& T = s.T;
    DT A1s = permuted(c, T, {1, 2, 3, 4, 5, 0});
    const int64_t da = T.d[0];
    int64_t per_a = 1;
    for (int i = 1; i < 6; ++i) per_a *= T.d[i];
    int64_t inter = (per_a / (T.d[2] * T.d[3])) * Ux.d[1] * Ux.d[2] * Uy.d[1] * Uy.d[2];
    int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(da, max_entries / std::max<int64_t>(inter, 1)));
    const int P_ = Lp, Q_ = Lq, R_ = Lr, S_ = Ls;
    std::vector<int64_t> od = {T.d[1], Uy.d[2], Ux.d[2], Uy.d[2], Ux.d[2], da};
    DT Out = make_dt(c.pool.get(), od);
    const int64_t slab = od[0] * od[1] * od[2] * od[3] * od[4];
    for (int64_t a0 = 0; a0 < da; a0 += chunk) {
        const int64_t na = std::min(chunk, da - a0);
        DT A1 = make_dt(c.pool.get(), {T.d[1], T.d[2], T.d[3], T.d[4], T.d[5], na});
        copy_f64(c, A1.p(), A1s.p() + a0 * per_a, per_a * na);
        A1.N = T.N;
        for (int l = 0; l < 5; ++l) A1.q.push_back(A1s.q[l]);
        A1.q.push_back(std::vector<int>(A1s.q[5].begin() + a0, A1s.q[5].begin() + a0 + na));
        DT X = contract(c, A1, {Lz, P_, Q_, Ly, Lx, La}, Ux, {Q_, R_, Ld}, {Lz, P_, Ly, Lx, La, R_, Ld});
        A1 = DT();
        DT Yt = contract(c, X, {Lz, P_, Ly, Lx, La, R_, Ld}, Uy, {P_, S_, Lc}, {Lz, Ly, Lx, La, R_, Ld, S_, Lc});
        X = DT();
        DT Z = contract(c, Yt, {Lz, Ly, Lx, La, R_, Ld, S_, Lc}, T, {Lz, Lb, S_, R_, Lu, Lv},
                        {Ly, Lx, La, Ld, Lc, Lb, Lu, Lv});
        Yt = DT();
        DT W = contract(c, Z, {Ly, Lx, La, Ld, Lc, Lb, Lu, Lv}, Ux, {Lx, Lv, Lf}, {Ly, La, Ld, Lc, Lb, Lu, Lf});
        Z = DT();
        DT O = contract(c, W, {Ly, La, Ld, Lc, Lb, Lu, Lf}, Uy, {Ly, Lu, Le}, {Lb, Lc, Ld, Le, Lf, La});
        copy_f64(c, Out.p() + a0 * slab, O.p(), slab * na);
        if (a0 == 0) {
            Out.N = O.N;
            for (int l = 0; l < 5; ++l) Out.q.push_back(O.q[l]);
            Out.q.push_back(T.q[0]);
        }
    }
    s.T = permuted(c, Out, {5, 0, 1, 2, 3, 4});
}

static void hotrg3d_contract(Scheme& s, const DT& Ux, const DT& Uy, int64_t max_entries) {
    Ctx& c = *s.ctx;
    const DT& T = s.T;
    if (T.charged() && Ux.charged() && Uy.charged()) {
        hotrg3d_contract_charged(s, Ux, Uy, max_entries);
        return;
    }
    // A1 with the open leg a moved last so slices are contiguous: A1s[z,P,Q,y,x,a]
    DT A1s = permuted(c, T, {1, 2, 3, 4, 5, 0});
    const int64_t da = T.d[0];
    int64_t per_a = 1;
    for (int i = 1; i < 6; ++i) per_a *= T.d[i];
    // largest intermediate per unit of a: the N and E legs of A1 replaced by (S, c) and (R, d)
    int64_t inter = (per_a / (T.d[2] * T.d[3])) * Ux.d[1] * Ux.d[2] * Uy.d[1] * Uy.d[2];
    int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(da, max_entries / std::max<int64_t>(inter, 1)));
    const int P_ = Lp, Q_ = Lq, R_ = Lr, S_ = Ls;
    // output collected as [b,c,d,e,f,a]
    std::vector<int64_t> od = {T.d[1], Uy.d[2], Ux.d[2], Uy.d[2], Ux.d[2], da};
    DT Out = make_dt(c.pool.get(), od);
    const int64_t slab = od[0] * od[1] * od[2] * od[3] * od[4];
    for (int64_t a0 = 0; a0 < da; a0 += chunk) {
        int64_t na = std::min(chunk, da - a0);
        std::vector<int64_t> ds = {T.d[1], T.d[2], T.d[3], T.d[4], T.d[5], na};
        const double* A1p = A1s.p() + a0 * per_a;
        // X[z,P,y,x,a,R,d] = A1[z,P,Q,y,x,a] Ux[Q,R,d]
        DT X = contract(c, A1p, ds, {Lz, P_, Q_, Ly, Lx, La}, Ux.p(), Ux.dims(), {Q_, R_, Ld},
                        {Lz, P_, Ly, Lx, La, R_, Ld});
        // Y = X Uy[P,S,c]
        DT Yt = contract(c, X, {Lz, P_, Ly, Lx, La, R_, Ld}, Uy, {P_, S_, Lc}, {Lz, Ly, Lx, La, R_, Ld, S_, Lc});
        X = DT();
        // Z = Y A2[z,b,S,R,u,v]
        DT Z = contract(c, Yt, {Lz, Ly, Lx, La, R_, Ld, S_, Lc}, T, {Lz, Lb, S_, R_, Lu, Lv},
                        {Ly, Lx, La, Ld, Lc, Lb, Lu, Lv});
        Yt = DT();
        // W = Z conj(Ux[x,v,f])
        DT W = contract(c, Z, {Ly, Lx, La, Ld, Lc, Lb, Lu, Lv}, Ux, {Lx, Lv, Lf}, {Ly, La, Ld, Lc, Lb, Lu, Lf});
        Z = DT();
        // out = W conj(Uy[y,u,e]) -> [b,c,d,e,f,a]
        DT O = contract(c, W, {Ly, La, Ld, Lc, Lb, Lu, Lf}, Uy, {Ly, Lu, Le}, {Lb, Lc, Ld, Le, Lf, La});
        copy_f64(c, Out.p() + a0 * slab, O.p(), slab * na);
    }
    s.T = permuted(c, Out, {5, 0, 1, 2, 3, 4});
}

// step!(::HOTRG_3D) (hotrg3d.jl:120-135)
static void step_hotrg3d(Scheme& s, int chi) {
    Ctx& c = *s.ctx;
    for (int sub = 0; sub < 3; ++sub) {
        DT Ux = hotrg3d_xproj(s, s.T, chi);
        DT Ty = permuted(c, s.T, {0, 1, 3, 2, 5, 4});   // _get_hotrg3d_yproj: perm ((1,2),(4,3,6,5))
        DT Uy = hotrg3d_xproj(s, Ty, chi);
        Ty = DT();
        hotrg3d_contract(s, Ux, Uy, s.max_slice_entries);
        s.T = permuted(c, s.T, {5, 3, 1, 2, 0, 4});      // permute(T, ((6,4),(2,3,1,5)))
    }
}

int split_fp64_steps(int kind) {
    return kind == TNR_HOTRG_3D || kind == TNR_ATRG_3D ? TNR_SPLIT_FP64_STEPS_3D : TNR_SPLIT_FP64_STEPS_2D;
}

// A split-precision solve runs a step in FP64 (a) while the bond dimension still grows in its
// first steps, whose norms carry the largest weights in the free energy, and (b) for every
// step of a 2D scheme at chi <= TNR_SPLIT_MIN_CHI: those problems are too small for the tensor
// cores to pay (a 256^3 contraction), and their split products moved f by up to 2.2e-7 on a
// high-temperature Ising instance (chi = 16, beta = 0.304), above the 1e-7 contract.
bool split_step_in_fp64(int kind, int64_t step, const int64_t* dims, int nlegs, int chi) {
    const bool three_d = kind == TNR_HOTRG_3D || kind == TNR_ATRG_3D;
    if (!three_d && chi <= TNR_SPLIT_MIN_CHI) return true;
    if (step >= split_fp64_steps(kind)) return false;
    for (int l = 0; l < nlegs; ++l)
        if (dims[l] >= chi) return false;   // the bond has reached chi: a full-size step
    return true;
}

// step!(::CorrelationHOTRG) with its finalizer (src/schemes/correlationhotrg.jl:94-135,177-250;
// src/utility/finalize.jl:104-124).  Phase 1 (the first dist steps) carries both impurities, phase
// 2 merges them in its x-step, phase 3 carries the merged one; each half step is the y projector
// of the pure tensor and x-steps, then the x projector and y-steps, an impurity step being the
// average of the (impurity, pure) and (pure, impurity) steps.  d3: (n, n_1, n_2) or (n, n_imp, n_imp).
static void step_correlation_hotrg(Scheme& s, int chi, double* d3) {
    Ctx& c = *s.ctx;
    const int phase = s.steps < s.corr_dist ? 1 : (s.steps == s.corr_dist ? 2 : 3);
    for (int half = 0; half < 2; ++half) {
        const DT U = half == 0 ? hotrg_yproj(s, s.T, chi) : hotrg_xproj(s, s.T, chi);
        auto st = [&](const DT& A1, const DT& A2) {
            return half == 0 ? hotrg_step_x2(c, A1, A2, U) : hotrg_step_y2(c, A1, A2, U);
        };
        auto sym = [&](const DT& a, const DT& b) {       // (st(a, b) + st(b, a)) / 2
            DT x = st(a, b);
            DT y = st(b, a);
            lincomb2(c, x.p(), x.size(), 0.5, x.p(), 0.5, y.p());
            return x;
        };
        DT T = st(s.T, s.T);
        if (phase == 1) {
            DT a = sym(s.C1, s.T);
            DT b = sym(s.C2, s.T);
            s.C1 = std::move(a);
            s.C2 = std::move(b);
        } else if (phase == 2 && half == 0) {
            s.Cf = sym(s.C1, s.C2);
        } else {
            s.Cf = sym(s.Cf, s.T);
        }
        s.T = std::move(T);
    }
    trace2d(c, s.T.p(), s.T.d, d3);
    if (phase == 1) {
        trace2d(c, s.C1.p(), s.C1.d, d3 + 1);
        trace2d(c, s.C2.p(), s.C2.d, d3 + 2);
        for (DT* t : {&s.T, &s.C1, &s.C2}) scale_inplace(c, t->p(), t->size(), d3);
    } else {
        trace2d(c, s.Cf.p(), s.Cf.d, d3 + 1);
        copy_f64(c, d3 + 2, d3 + 1, 1);
        for (DT* t : {&s.T, &s.Cf}) scale_inplace(c, t->p(), t->size(), d3);
        if (phase == 2) {
            s.C1 = DT();
            s.C2 = DT();
        }
    }
}

std::vector<double> Scheme::run_correlation(int chi, int maxiter) {
    Ctx& c = *ctx;
    TNR_REQUIRE(kind == TNR_CORRELATION_HOTRG, TNR_ERR_INVALID_ARG, "run_correlation needs a CorrelationHOTRG handle");
    TNR_REQUIRE(maxiter > corr_dist, TNR_ERR_INVALID_ARG, "run!: maxiter must be larger than dist");
    Buf norms(c.pool.get(), (size_t)maxiter * 3 * sizeof(double));
    for (int i = 0; i < maxiter; ++i) step(chi, norms.d() + 3 * i);
    check_finite(c, norms.d(), 3 * (int64_t)maxiter);
    return dvec_to_host(c, norms.d(), 3 * (int64_t)maxiter);
}

void Scheme::step(int chi, double* d_corr) {
    TNR_REQUIRE(chi >= 1, TNR_ERR_INVALID_ARG, "truncrank(chi) needs chi >= 1");
    last_vals.clear();
    last_counts.clear();
    last_eps.clear();
    // the split precision computes the leading steps exactly as the FP64 path does
    PrecisionScope scope(*ctx, split_step_in_fp64(kind, steps, T.d, T.rank, chi));
    switch (kind) {
        case TNR_TRG: step_trg(*this, chi); break;
        case TNR_BTRG: step_btrg(*this, chi); break;
        case TNR_HOTRG: step_hotrg(*this, chi); break;
        case TNR_HOTRG_3D: step_hotrg3d(*this, chi); break;
        case TNR_ATRG: step_atrg(*this, chi); break;
        case TNR_ATRG_3D: step_atrg3d(*this, chi); break;
        case TNR_IMPURITY_HOTRG: step_impurity_hotrg(*this, chi); break;
        case TNR_IMPURITY_TRG: step_impurity_trg(*this, chi); break;
        case TNR_CORRELATION_HOTRG: {
            Buf scratch(ctx->pool.get(), d_corr ? 0 : 3 * sizeof(double));
            step_correlation_hotrg(*this, chi, d_corr ? d_corr : scratch.d());
            break;
        }
        default: throw Error(TNR_ERR_INVALID_ARG, "unknown scheme kind");
    }
    ++steps;
}

// finalize! (src/utility/finalize.jl:4-14,62-66): norm into *d_norm, T /= norm
// TRG and BTRG fold T's normalisation into the next step's singular values; HOTRG (dense)
// into the permutes of its y half step (its projector Grams see T unscaled, which changes
// their eigenvalues by |n|^-4 and not their eigenvectors)
bool Scheme::folds_normalisation() const {
    if (finalizer != FINALIZER_DEFAULT) return false;
    return kind == TNR_TRG || kind == TNR_BTRG || (kind == TNR_HOTRG && !T.charged());
}

void Scheme::finalize_async(double* d_norm, bool scale) {
    Ctx& c = *ctx;
    TNR_REQUIRE(kind != TNR_CORRELATION_HOTRG, TNR_ERR_INVALID_ARG,
                "CorrelationHOTRG finalizes inside step!: run it with tnr_run_correlation");
    if (finalizer == FINALIZER_TWO_BY_TWO) {
        finalize_two_by_two_async(d_norm);
        return;
    }
    if (kind == TNR_IMPURITY_HOTRG || kind == TNR_IMPURITY_TRG) {
        // the pure norm; the impurity norms go to scratch (run_impurity reads them all)
        Buf d4(c.pool.get(), 4 * sizeof(double));
        finalize_multi_async(d4.d());
        copy_f64(c, d_norm, d4.d(), 1);
        return;
    }
    switch (kind) {
        case TNR_TRG:
        case TNR_HOTRG:
        case TNR_ATRG: trace2d(c, T.p(), T.d, d_norm); break;
        case TNR_BTRG: trace_btrg(c, T.p(), T.d, S1.p(), S2.p(), d_norm); break;
        case TNR_HOTRG_3D:
        case TNR_ATRG_3D: trace3d(c, T.p(), T.d, d_norm); break;
        default: throw Error(TNR_ERR_INVALID_ARG, "unknown scheme kind");
    }
    if (scale) scale_inplace(c, T.p(), T.size(), d_norm);
}

// finalize!(::ImpurityHOTRG) (src/utility/finalize.jl:91-101)
void Scheme::finalize_impurity_async(double* d4) {
    Ctx& c = *ctx;
    const DT* ts[4] = {&T, &I11, &I12, &I2};
    for (int i = 0; i < 4; ++i) trace2d(c, ts[i]->p(), ts[i]->d, d4 + i);
    for (int i = 0; i < 4; ++i) scale_inplace(c, ts[i]->p(), ts[i]->size(), d4);
}

// finalize!(::ImpurityTRG) (src/utility/finalize.jl:75-88): every tensor /= the pure trace
// norm, then |T_imp1[5 4;6 1] T_imp2[1 2;7 5] T_imp3[3 7;2 8] T_imp4[8 6;4 3]|
void Scheme::finalize_impurity_trg_async(double* d2) {
    Ctx& c = *ctx;
    trace2d(c, T.p(), T.d, d2);
    scale_inplace(c, T.p(), T.size(), d2);
    for (int i = 0; i < 4; ++i) scale_inplace(c, site[i].p(), site[i].size(), d2);
    // labels 1..8 -> a..h; X[4,6,2,7] = T1[5,4,6,1] T2[1,2,7,5]; Y[7,2,6,4] = T3[3,7,2,8] T4[8,6,4,3]
    DT X = contract(c, site[0], {Le, Ld, Lf, La}, site[1], {La, Lb, Lg, Le}, {Ld, Lf, Lb, Lg});
    DT Y = contract(c, site[2], {Lc, Lg, Lb, Lh}, site[3], {Lh, Lf, Ld, Lc}, {Lg, Lb, Lf, Ld});
    // the closing contraction over all four legs, as a 1 x 1 product (a unit leg on each side)
    std::vector<int64_t> dx = X.dims(), dy = Y.dims();
    dx.push_back(1);
    dy.push_back(1);
    DT Z = contract(c, X.p(), dx, {Ld, Lf, Lb, Lg, Lx}, Y.p(), dy, {Lg, Lb, Lf, Ld, Ly}, {Lx, Ly}, false);
    abs_copy(c, d2 + 1, Z.p());
}

void Scheme::finalize_multi_async(double* d) {
    if (kind == TNR_IMPURITY_HOTRG) finalize_impurity_async(d);
    else if (kind == TNR_IMPURITY_TRG) finalize_impurity_trg_async(d);
    else throw Error(TNR_ERR_INVALID_ARG, "not an impurity scheme");
}

std::vector<double> Scheme::run_impurity(int chi, int maxiter, bool finalize_beginning) {
    Ctx& c = *ctx;
    const int np = norms_per_entry();
    TNR_REQUIRE(np > 1, TNR_ERR_INVALID_ARG, "run_impurity needs an impurity scheme handle");
    const int nsteps = std::max(maxiter, 1);
    const int nn = nsteps + (finalize_beginning ? 1 : 0);
    Buf norms(c.pool.get(), (size_t)nn * np * sizeof(double));
    int at = 0;
    if (finalize_beginning) finalize_multi_async(norms.d() + np * (at++));
    for (int i = 0; i < nsteps; ++i) {
        step(chi);
        finalize_multi_async(norms.d() + np * (at++));
    }
    check_finite(c, norms.d(), (int64_t)np * nn);
    std::vector<double> h = dvec_to_host(c, norms.d(), (int64_t)np * nn);
    int st = c.read_status_and_clear();
    TNR_REQUIRE(!(st & ST_NONFINITE), TNR_ERR_NONFINITE, "run!: non-finite norm");
    return h;
}

double Scheme::finalize() {
    finalize_async(ctx->d_scalar + 8);
    std::vector<double> n = dvec_to_host(*ctx, ctx->d_scalar + 8, 1);
    return n[0];
}

std::vector<double> Scheme::run(int chi, int maxiter, bool finalize_beginning) {
    Ctx& c = *ctx;
    const int nsteps = std::max(maxiter, 1);       // the loop body runs before the first check
    const int nn = nsteps + (finalize_beginning ? 1 : 0);
    Buf norms(c.pool.get(), (size_t)nn * sizeof(double));
    const bool fold = folds_normalisation();
    int at = 0, last_in = -1;                      // last_in: the norm folded into the last step
    if (finalize_beginning) {
        finalize_async(norms.d() + at, !fold);
        if (fold) pending = norms.d() + at;
        ++at;
    }
    try {
        for (int i = 0; i < nsteps; ++i) {
            last_in = pending ? at - 1 : -1;
            step(chi);
            pending = nullptr;
            finalize_async(norms.d() + at, !fold);
            if (fold) pending = norms.d() + at;
            ++at;
        }
        if (pending) scale_inplace(c, T.p(), T.size(), pending);   // T normalised when run!() returns
    } catch (...) {
        pending = nullptr;
        throw;
    }
    pending = nullptr;
    check_finite(c, norms.d(), nn);
    std::vector<double> h = dvec_to_host(c, norms.d(), nn);
    int st = c.read_status_and_clear();
    TNR_REQUIRE(!(st & ST_NONFINITE), TNR_ERR_NONFINITE, "run!: non-finite norm");
    if (last_in >= 0) {
        // the last step decomposed T before its normalisation: its recorded values are in T's
        // unnormalised scale (singular values |n| times, HOTRG's x-projector Gram |n|^4 times)
        const double n = std::fabs(h[last_in]);
        if (kind == TNR_HOTRG) {
            const double n4 = n * n * n * n;
            const int k0 = last_counts.empty() ? 0 : last_counts[0];
            for (int i = 0; i < k0 && i < (int)last_vals.size(); ++i) last_vals[i] /= n4;
            for (int i = 0; i < 2 && i < (int)last_eps.size(); ++i) last_eps[i] /= n4;
        } else {
            for (double& v : last_vals) v /= n;
        }
    }
    return h;
}

}  // namespace tnr
