// Small dense FP64 linear algebra on one CTA: parallel-ordering (round-robin)
// two-sided Jacobi eigensolver and Cholesky factor + triangular inverse.
// Both keep the matrix in shared memory; every loop has a fixed iteration cap
// and reports failure through the context status word (no trap, no spin).
#include "common.cuh"

#include <algorithm>
#include <cmath>
#include <mutex>

namespace tnr {

constexpr int JMAX = 160;           // largest matrix held in shared memory
constexpr int JTHREADS = 512;
constexpr int JMAX_SWEEPS = 60;          // FP64 cleanup
constexpr int JMAX_SWEEPS_F32 = 16;      // FP32 alignment (converged or cycling on noise by then)

template <class T>
__device__ __forceinline__ T& SG(T* G, int ld, int i, int j) { return G[i + j * ld]; }

// Rotation thresholds: rotate (p, q) iff |g_pq| > max(rel * sqrt|g_pp g_qq|, floor * |G|_F).
// FP64 cleans up matrices already aligned by the FP32 pass: rel = 1e-12 leaves
// orthogonality errors of 1e-12; the floor 1e-22 keeps graded values down to 1e-11 of the
// largest singular value resolved while rounding noise (~1e-32) is left alone.
// FP32 (alignment only) cannot resolve entries below ~1e-7 |G|: below the floor 1e-9 |G|
// rotations would only stir rounding noise, so they are skipped (the FP64 stage resolves
// those directions).
#ifndef TNR_JACOBI64_REL
#define TNR_JACOBI64_REL 1e-12
#endif
#ifndef TNR_JACOBI64_FLOOR
#define TNR_JACOBI64_FLOOR 1e-22
#endif
#ifndef TNR_JACOBI32_FLOOR
#define TNR_JACOBI32_FLOOR 1e-9
#endif
template <class T> struct JTol;
template <> struct JTol<double> { static constexpr double rel = TNR_JACOBI64_REL, floor = TNR_JACOBI64_FLOOR; };
template <> struct JTol<float> { static constexpr double rel = 2e-7, floor = TNR_JACOBI32_FLOOR; };

// Parallel (round-robin ordering) two-sided Jacobi in shared memory, arithmetic type T.
// Input G is FP64 (symmetrised on load); W (FP64, r x r) and lam (FP64) are sorted by |lambda|.
template <class T>
__global__ void __launch_bounds__(JTHREADS)
k_jacobi(const double* __restrict__ Gin, int64_t ldg, int64_t strideG, int r, double* __restrict__ Wout,
         double* __restrict__ lam, T* __restrict__ Ww, int* status) {
    // one CTA per matrix of a batch
    Gin += (int64_t)blockIdx.x * strideG;
    Wout += (int64_t)blockIdx.x * r * r;
    lam += (int64_t)blockIdx.x * r;
    if (sizeof(T) == 8) Ww += (int64_t)blockIdx.x * r * r;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ld = r + 1;
    T* G = reinterpret_cast<T*>(smem_raw);  // r x r, leading dim r+1
    T* cs = G + (size_t)ld * r;             // JMAX/2 + 1 each
    T* sn = cs + (JMAX / 2 + 1);
    int* pp = (int*)(sn + (JMAX / 2 + 1));
    int* qq = pp + (JMAX / 2 + 1);
    // FP32: the eigenvector matrix lives in shared memory too (two r x r FP32 arrays fit);
    // FP64 keeps it in global memory (L1/L2 resident)
    if (sizeof(T) == 4) Ww = reinterpret_cast<T*>(qq + (JMAX / 2 + 1));
    __shared__ int rot_count;
    __shared__ T fro;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int R = r + (r & 1), n = R - 1, npair = R / 2;

    // load (symmetrised) and W = I
    for (int e = tid; e < r * r; e += nt) {
        int i = e % r, j = e / r;
        SG(G, ld, i, j) = (T)(0.5 * (Gin[i + j * ldg] + Gin[j + i * ldg]));
        Ww[e] = (i == j) ? T(1) : T(0);
    }
    __syncthreads();
    if (tid < 32) {
        T acc = 0;
        for (int e = tid; e < r * r; e += 32) {
            T v = SG(G, ld, e % r, e / r);
            acc = fma(v, v, acc);
        }
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (tid == 0) fro = sqrt(acc);
    }
    __syncthreads();
    const T abs_floor = (T)JTol<T>::floor * fro;
    const T reltol = (T)JTol<T>::rel;
    int sweep = 0;
    bool converged = (r <= 1);
    const int max_sweeps = sizeof(T) == 4 ? JMAX_SWEEPS_F32 : JMAX_SWEEPS;
    for (; sweep < max_sweeps && !converged; ++sweep) {
        if (tid == 0) rot_count = 0;
        __syncthreads();
        for (int t = 0; t < n; ++t) {
            // pair schedule: player n (the even fill-in) meets t; (t+i, t-i) mod n for i >= 1
            for (int i = tid; i < npair; i += nt) {
                int p, q;
                if (i == 0) { p = n; q = t; }
                else { p = (t + i) % n; q = (t - i + n) % n; }
                if (p > q) { int tmp = p; p = q; q = tmp; }
                T c = 1, s = 0;
                if (q < r) {
                    T apq = SG(G, ld, p, q), app = SG(G, ld, p, p), aqq = SG(G, ld, q, q);
                    if (fabs(apq) > fmax(reltol * sqrt(fabs(app * aqq)), abs_floor)) {
                        T tau = (aqq - app) / (T(2) * apq);
                        T tt;
                        if (fabs(tau) > (T)1e18) tt = T(0.5) / tau;
                        else tt = (tau >= T(0) ? T(1) : T(-1)) / (fabs(tau) + sqrt(T(1) + tau * tau));
                        c = rsqrt(T(1) + tt * tt);
                        s = tt * c;
                        atomicAdd(&rot_count, 1);
                    }
                }
                pp[i] = p; qq[i] = (q < r) ? q : -1; cs[i] = c; sn[i] = s;
            }
            __syncthreads();
            // G <- G J (columns p, q) and W <- W J
            for (int e = tid; e < npair * r; e += nt) {
                int i = e / r, j = e % r;
                int q = qq[i];
                T s = sn[i];
                if (q < 0 || s == T(0)) continue;
                int p = pp[i];
                T c = cs[i];
                T gp = SG(G, ld, j, p), gq = SG(G, ld, j, q);
                SG(G, ld, j, p) = c * gp - s * gq;
                SG(G, ld, j, q) = s * gp + c * gq;
                T wp = Ww[j + p * r], wq = Ww[j + q * r];
                Ww[j + p * r] = c * wp - s * wq;
                Ww[j + q * r] = s * wp + c * wq;
            }
            __syncthreads();
            // G <- J^T G (rows p, q)
            for (int e = tid; e < npair * r; e += nt) {
                int i = e / r, j = e % r;
                int q = qq[i];
                T s = sn[i];
                if (q < 0 || s == T(0)) continue;
                int p = pp[i];
                T c = cs[i];
                T gp = SG(G, ld, p, j), gq = SG(G, ld, q, j);
                SG(G, ld, p, j) = c * gp - s * gq;
                SG(G, ld, q, j) = s * gp + c * gq;
            }
            __syncthreads();
            for (int i = tid; i < npair; i += nt) {
                int q = qq[i];
                if (q >= 0 && sn[i] != T(0)) { SG(G, ld, pp[i], q) = T(0); SG(G, ld, q, pp[i]) = T(0); }
            }
            __syncthreads();
        }
        converged = (rot_count == 0);
        __syncthreads();
    }
    // The FP32 pass only aligns a basis for the FP64 stage: no convergence requirement.
    // FP64: after the cap, only a remaining off-diagonal above 1e-9 of its diagonal scale
    // (not rounding noise in a numerically zero block) is reported.
    if (!converged && sizeof(T) == 8) {
        __shared__ int bad;
        if (tid == 0) bad = 0;
        __syncthreads();
        for (int e = tid; e < r * r; e += nt) {
            int i = e % r, j = e / r;
            if (i < j) {
                T g = SG(G, ld, i, j);
                if (fabs(g) > (T)1e-9 * sqrt(fabs(SG(G, ld, i, i) * SG(G, ld, j, j))) && fabs(g) > (T)1e-16 * fro)
                    bad = 1;
            }
        }
        __syncthreads();
        if (tid == 0 && bad) atomicOr(status, ST_JACOBI_NOCONV);
    }
    // sort by |lambda| descending (stable by index)
    for (int i = tid; i < r; i += nt) {
        T li = SG(G, ld, i, i);
        if (!isfinite(li)) atomicOr(status, ST_NONFINITE);
        int rank = 0;
        for (int j = 0; j < r; ++j) {
            T lj = fabs(SG(G, ld, j, j));
            rank += (lj > fabs(li)) || (lj == fabs(li) && j < i);
        }
        lam[rank] = (double)li;
        for (int j = 0; j < r; ++j) Wout[j + (int64_t)rank * r] = (double)Ww[j + (int64_t)i * r];
    }
}

template <class T>
static void launch_jacobi(Ctx& c, const double* G, int64_t ldg, int r, double* W, double* lam, int batch,
                          int64_t strideG) {
    TNR_REQUIRE(r >= 1 && r <= JMAX, TNR_ERR_UNSUPPORTED, "jacobi_eigh: r out of range");
    const size_t aux = 2 * (JMAX / 2 + 1) * (sizeof(T) + sizeof(int));
    const bool w_in_smem = sizeof(T) == 4;      // FP32: eigenvectors in shared memory as well
    size_t smem = (size_t)(r + 1) * r * sizeof(T) + aux + (w_in_smem ? (size_t)r * r * sizeof(T) : 0);
    static std::atomic<uint64_t> attr_set{0};
    const size_t maxs = (size_t)(JMAX + 1) * JMAX * sizeof(T) + aux + (w_in_smem ? (size_t)JMAX * JMAX * sizeof(T) : 0);
    ensure_smem_attr(attr_set, (const void*)k_jacobi<T>, (int)maxs);
    Buf ww(c.pool.get(), w_in_smem ? sizeof(T) : (size_t)batch * r * r * sizeof(T));
    int nt = r <= 32 ? 128 : (r <= 64 ? 256 : JTHREADS);
    int rec = prof_start(c.stream);
    k_jacobi<T><<<batch, nt, smem, c.stream>>>(G, ldg, strideG, r, W, lam, ww.as<T>(), c.d_status);
    check_launch("jacobi");
    prof_stop(rec, c.stream, sizeof(T) == 8 ? PROF_JACOBI : PROF_JACOBI32, (double)r * r * r * batch);
}

void jacobi_eigh(Ctx& c, const double* G, int64_t ldg, int r, double* W, double* lam, int batch, int64_t strideG) {
    launch_jacobi<double>(c, G, ldg, r, W, lam, batch, strideG);
}

void jacobi_eigh_f32(Ctx& c, const double* G, int64_t ldg, int r, double* W, double* lam, int batch,
                     int64_t strideG) {
    launch_jacobi<float>(c, G, ldg, r, W, lam, batch, strideG);
}

// Cholesky of (G + shift I) = L L^T in shared memory, then L^{-1} (lower) written over G.
template <class T>
__global__ void __launch_bounds__(512)
k_chol_inv(double* G, int r, double shift, int* status) {
    G += (int64_t)blockIdx.x * r * r;     // one CTA per matrix of a batch
    extern __shared__ __align__(16) unsigned char smem_c[];
    T* S = reinterpret_cast<T*>(smem_c);
    const int ld = r + 1;
    const int tid = threadIdx.x, nt = blockDim.x;
    __shared__ int bad;
    if (tid == 0) bad = 0;
    for (int e = tid; e < r * r; e += nt) {
        int i = e % r, j = e / r;
        S[i + j * ld] = (T)((i >= j) ? G[e] + (i == j ? shift : 0.0) : 0.0);
    }
    __syncthreads();
    // right-looking Cholesky, two barriers per column: the square root of the next pivot
    // is taken by the lane that finishes its update (warp 0, lane 0 owns column k+1's
    // diagonal) and published in `pivot` for the next iteration
    const int warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
    __shared__ T pivot;
    if (tid == 0) {
        T d = S[0];
        if (!(d > T(0)) || !isfinite(d)) { bad = 1; d = (T)1e-30; }
        pivot = sqrt(d);
    }
    __syncthreads();
    for (int k = 0; k < r; ++k) {
        const T dk = pivot;
        for (int i = k + 1 + tid; i < r; i += nt) S[i + k * ld] /= dk;
        __syncthreads();
        if (tid == 0) S[k + k * ld] = dk;
        // trailing update of the lower triangle: one warp per column j, lanes over rows i >= j
        for (int j = k + 1 + warp; j < r; j += nw) {
            const T sj = S[j + k * ld];
            for (int i = j + lane; i < r; i += 32) S[i + j * ld] -= S[i + k * ld] * sj;
            if (j == k + 1 && lane == 0) {
                T d = S[j + j * ld];
                if (!(d > T(0)) || !isfinite(d)) { bad = 1; d = (T)1e-30; }
                pivot = sqrt(d);
            }
        }
        __syncthreads();
    }
    // inverse X = L^{-1} of the lower-triangular L, row by row: row i needs only the rows
    // above it, so thread j < i computes X[i,j] = -(sum_{kk=j}^{i-1} L[i,kk] X[kk,j]) / L[i,i].  X shares S's storage: X[i,j], i > j, sits at the transposed
    // position S[j + i*ld] (strict upper triangle, free once L is done) and X[j,j] = 1/L[j,j]
    // in the spare row S[r + j*ld]; L stays in the lower triangle.
    for (int i = tid; i < r; i += nt) S[r + i * ld] = T(1) / S[i + i * ld];
    __syncthreads();
    for (int i = 1; i < r; ++i) {
        for (int j = tid; j < i; j += nt) {
            // four partial sums: eight independent shared-memory loads per trip
            T a0 = S[i + j * ld] * S[r + j * ld], a1 = T(0), a2 = T(0), a3 = T(0);
            int kk = j + 1;
            for (; kk + 3 < i; kk += 4) {
                a0 += S[i + kk * ld] * S[j + kk * ld];
                a1 += S[i + (kk + 1) * ld] * S[j + (kk + 1) * ld];
                a2 += S[i + (kk + 2) * ld] * S[j + (kk + 2) * ld];
                a3 += S[i + (kk + 3) * ld] * S[j + (kk + 3) * ld];
            }
            for (; kk < i; ++kk) a0 += S[i + kk * ld] * S[j + kk * ld];
            S[j + i * ld] = -((a0 + a1) + (a2 + a3)) * S[r + i * ld];
        }
        __syncthreads();
    }
    __syncthreads();
    for (int e = tid; e < r * r; e += nt) {
        int i = e % r, j = e / r;
        G[e] = i > j ? (double)S[j + i * ld] : (i == j ? (double)S[r + j * ld] : 0.0);
    }
    if (tid == 0 && bad) atomicOr(status, ST_CHOL_BREAKDOWN);
}

template <class T>
static void launch_chol(Ctx& c, double* G, int r, double shift, int batch) {
    TNR_REQUIRE(r >= 1 && r <= JMAX, TNR_ERR_UNSUPPORTED, "chol_inv: r out of range");
    size_t smem = (size_t)(r + 1) * r * sizeof(T);
    TNR_REQUIRE(smem <= 227 * 1024, TNR_ERR_UNSUPPORTED, "chol_inv: matrix too large for shared memory");
    static std::atomic<uint64_t> attr_set{0};
    ensure_smem_attr(attr_set, (const void*)k_chol_inv<T>,
                     (int)std::min<size_t>((size_t)(JMAX + 1) * JMAX * sizeof(T), 227 * 1024));
    int rec = prof_start(c.stream);
    k_chol_inv<T><<<batch, 512, smem, c.stream>>>(G, r, shift, c.d_status);
    check_launch("chol_inv");
    prof_stop(rec, c.stream, PROF_CHOL, (double)r * r * r * batch);
}

void chol_inv(Ctx& c, double* G, int r, double shift, int batch) { launch_chol<double>(c, G, r, shift, batch); }
void chol_inv_f32(Ctx& c, double* G, int r, double shift, int batch) { launch_chol<float>(c, G, r, shift, batch); }

}  // namespace tnr
