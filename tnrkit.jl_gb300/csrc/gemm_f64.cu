// FP64 GEMM on the CUDA cores (DFMA): the plain path of every contraction and the
// FP64 pieces of the truncated decompositions.  Column-major, op(A)/op(B) in {N,T},
// strided batch, deterministic split-K for skinny outputs (Gram matrices).
#include "common.cuh"

#include <algorithm>

namespace tnr {

constexpr int BM = 64, BN = 64, BK = 16;

// one CTA: 64x64 tile of C, 256 threads, 4x4 outputs per thread.  sym: C = op(A) op(B) is a Gram
// (A == B, one of them transposed, beta = 0): tiles above the diagonal are skipped and those
// below it also write their transpose (c_ij and c_ji are the same products in the same order,
// so the result is the one of the full product bit for bit)
__global__ void __launch_bounds__(256)
k_dgemm(bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* __restrict__ A,
        int64_t lda, const double* __restrict__ B, int64_t ldb, double beta,
        double* __restrict__ C, int64_t ldc, Batch2 bt, int ksplit, int64_t kchunk, double* __restrict__ part,
        bool sym) {
    if (sym && blockIdx.x < blockIdx.y) return;
    const bool mirror = sym && blockIdx.x > blockIdx.y;
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int64_t i0 = blockIdx.x * (int64_t)BM, j0 = blockIdx.y * (int64_t)BN;
    int bz = blockIdx.z;
    int ks = bz % ksplit;
    int b = bz / ksplit;
    int b1 = b % bt.n1, b2 = b / bt.n1;
    A += b1 * bt.sA1 + b2 * bt.sA2;
    B += b1 * bt.sB1 + b2 * bt.sB2;
    const int64_t kbeg = ks * kchunk, kend = min(k, kbeg + kchunk);

    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

    for (int64_t kk0 = kbeg; kk0 < kend; kk0 += BK) {
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            int e = threadIdx.x + 256 * l;
            int ii, kk;
            double v = 0.0;
            if (!ta) { ii = e % BM; kk = e / BM; } else { kk = e % BK; ii = e / BK; }
            int64_t gi = i0 + ii, gk = kk0 + kk;
            if (gi < m && gk < kend) v = ta ? A[gk + gi * lda] : A[gi + gk * lda];
            As[kk][ii] = v;
            int jj;
            double w = 0.0;
            if (!tb) { kk = e % BK; jj = e / BK; } else { jj = e % BN; kk = e / BN; }
            int64_t gj = j0 + jj;
            gk = kk0 + kk;
            if (gj < n && gk < kend) w = tb ? B[gj + gk * ldb] : B[gk + gj * ldb];
            Bs[kk][jj] = w;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            double a[4], bb[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][tx + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bb[j] = Bs[kk][ty + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], bb[j], acc[i][j]);
        }
        __syncthreads();
    }
    if (ksplit > 1) {
        double* P = part + ((int64_t)b * ksplit + ks) * m * n;
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int64_t gi = i0 + tx + 16 * i, gj = j0 + ty + 16 * j;
                if (gi < m && gj < n) {
                    P[gi + gj * m] = acc[i][j];
                    if (mirror) P[gj + gi * m] = acc[i][j];
                }
            }
        return;
    }
    C += b1 * bt.sC1 + b2 * bt.sC2;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int64_t gi = i0 + tx + 16 * i, gj = j0 + ty + 16 * j;
            if (gi < m && gj < n) {
                double v = alpha * acc[i][j];
                if (beta != 0.0) v = fma(beta, C[gi + gj * ldc], v);
                C[gi + gj * ldc] = v;
                if (mirror) C[gj + gi * ldc] = v;
            }
        }
}

// C_b = alpha * sum_s P[b][s] + beta * C_b for every batch entry b (fixed summation order:
// deterministic); P holds ks partial m x n products per batch entry
__global__ void k_splitk_reduce(const double* __restrict__ P, int ks, int64_t m, int64_t n, double alpha,
                                double beta, double* C, int64_t ldc, Batch2 bt) {
    const int64_t mn = m * n, total = mn * bt.n1 * bt.n2;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = e / mn, r = e % mn;
        const double* Pb = P + b * ks * mn;
        double s = 0.0;
        for (int i = 0; i < ks; ++i) s += Pb[r + (int64_t)i * mn];
        const int b1 = (int)(b % bt.n1), b2 = (int)(b / bt.n1);
        double* Cb = C + b1 * bt.sC1 + b2 * bt.sC2;
        int64_t gi = r % m, gj = r / m;
        double v = alpha * s;
        if (beta != 0.0) v = fma(beta, Cb[gi + gj * ldc], v);
        Cb[gi + gj * ldc] = v;
    }
}

void gemm_f64(Ctx& c, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
              int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, const Batch2& bt) {
    const int batch = bt.n1 * bt.n2;
    if (m <= 0 || n <= 0 || batch <= 0) return;
    TNR_REQUIRE(k > 0, TNR_ERR_INVALID_ARG, "gemm with k = 0");
    int64_t gm = (m + BM - 1) / BM, gn = (n + BN - 1) / BN;
    TNR_REQUIRE(gn <= 65535, TNR_ERR_UNSUPPORTED, "gemm: n too large for the grid");
    int ksplit = 1;
    int64_t tiles = gm * gn * batch;
    if (tiles < 2 * sm_count() && k >= 256) {
        // small outputs (Gram matrices, r x r products, also in lockstep batches): spread K so
        // that every SM's FP64 pipe gets work (GB300 runs FP64 at ~2 DFMA/clk/SM, so an idle
        // SM is lost throughput)
        ksplit = (int)std::min<int64_t>({k / 128, (4 * sm_count() + tiles - 1) / tiles, 64});
        if (ksplit < 2) ksplit = 1;
    }
    int64_t kchunk = ksplit > 1 ? ((k + ksplit - 1) / ksplit + BK - 1) / BK * BK : k;
    if (ksplit > 1) ksplit = (int)((k + kchunk - 1) / kchunk);
    TNR_REQUIRE((int64_t)batch * ksplit <= 65535, TNR_ERR_UNSUPPORTED, "gemm: batch too large");
    Buf part;
    if (ksplit > 1) part = Buf(c.pool.get(), (size_t)ksplit * batch * m * n * sizeof(double));
    dim3 grid((unsigned)gm, (unsigned)gn, (unsigned)(batch * ksplit));
    const bool sym = A == B && lda == ldb && ta != tb && m == n && beta == 0.0 && bt.sA1 == bt.sB1 &&
                     bt.sA2 == bt.sB2 && gm > 1;
    int rec = prof_start(c.stream);
    k_dgemm<<<grid, 256, 0, c.stream>>>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, bt, ksplit,
                                        kchunk, part.d(), sym);
    check_launch("dgemm");
    if (ksplit > 1) {
        int g = (int)std::min<int64_t>((m * n * batch + 255) / 256, (int64_t)sm_count() * 8);
        k_splitk_reduce<<<g, 256, 0, c.stream>>>(part.d(), ksplit, m, n, alpha, beta, C, ldc, bt);
        check_launch("splitk_reduce");
    }
    prof_stop(rec, c.stream, c.bulk_call ? PROF_GEMM_BULK : PROF_GEMM_F64, 2.0 * m * n * k * batch);
}

void gemm_f64(Ctx& c, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
              int64_t lda, int64_t sA, const double* B, int64_t ldb, int64_t sB, double beta, double* C,
              int64_t ldc, int64_t sC, int batch) {
    Batch2 bt;
    bt.n1 = batch; bt.sA1 = sA; bt.sB1 = sB; bt.sC1 = sC;
    gemm_f64(c, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, bt);
}

#ifndef TNR_SPLIT_MIN_MNK
#define TNR_SPLIT_MIN_MNK 4194304.0   // m n k summed over the batch below which a bulk product stays FP64
#endif
#ifndef TNR_SPLIT_CHUNK_KB
#define TNR_SPLIT_CHUNK_KB 1          // K blocks of 64 per FP32 accumulation chunk of a contraction
#endif

int split_chunk_kb() { return TNR_SPLIT_CHUNK_KB; }

void gemm_bulk(Ctx& c, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
               int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, const Batch2& bt,
               bool exact_sum) {
    // a product whose whole batch is too small to fill the tensor cores stays on the FP64 path
    // (the split kernel's launch and plane pass would cost more than the FP64 GEMM); the
    // early coarse-graining steps and 2D problems at chi <= 16, whose split products would
    // move the free energy beyond the contract, run in FP64 through PrecisionScope
    const double work = (double)m * n * k * bt.n1 * bt.n2;
    if (c.precision == TNR_PREC_SPLIT && work >= TNR_SPLIT_MIN_MNK &&
        gemm_split_tc(c, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, bt, exact_sum ? TNR_SPLIT_CHUNK_KB : 0))
        return;
    c.bulk_call = true;
    gemm_f64(c, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, bt);
    c.bulk_call = false;
}

void split_a_prepare(Ctx& c, SplitA& P, bool ta, const double* A, int64_t lda, int64_t m, int64_t k,
                     int64_t n_hint, const Batch2& bt) {
    P.active = false;
    if (c.precision != TNR_PREC_SPLIT || (double)m * n_hint * k * bt.n1 * bt.n2 < TNR_SPLIT_MIN_MNK || n_hint < 16)
        return;
    split_a_build(c, P, ta, A, lda, m, k, bt);
}

void gemm_bulk_a(Ctx& c, const SplitA& P, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha,
                 const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                 const Batch2& bt, bool exact_sum) {
    if (P.active && P.m == m && P.k == k &&
        gemm_split_tc_a(c, P, tb, n, B, ldb, alpha, beta, C, ldc, bt, exact_sum ? TNR_SPLIT_CHUNK_KB : 0))
        return;
    gemm_bulk(c, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, bt, exact_sum);
}

void gemm_bulk(Ctx& c, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
               int64_t lda, int64_t sA, const double* B, int64_t ldb, int64_t sB, double beta, double* C,
               int64_t ldc, int64_t sC, int batch, bool exact_sum) {
    Batch2 bt;
    bt.n1 = batch; bt.sA1 = sA; bt.sB1 = sB; bt.sC1 = sC;
    gemm_bulk(c, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, bt, exact_sum);
}

}  // namespace tnr
