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
         double* __restrict__ lam, T* __restrict__ Ww, int* status, double rel_tol, double floor_tol) {
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
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
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
    const T abs_floor = (T)floor_tol * fro;
    const T reltol = (T)rel_tol;
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
            // G <- G J (columns p, q) and W <- W J: a warp per pair, lanes along the column
            for (int i = warp; i < npair; i += nwarp) {
                const int q = qq[i];
                const T s = sn[i];
                if (q < 0 || s == T(0)) continue;
                const int p = pp[i];
                const T c = cs[i];
                for (int j = lane; j < r; j += 32) {
                    T gp = SG(G, ld, j, p), gq = SG(G, ld, j, q);
                    SG(G, ld, j, p) = c * gp - s * gq;
                    SG(G, ld, j, q) = s * gp + c * gq;
                    T wp = Ww[j + p * r], wq = Ww[j + q * r];
                    Ww[j + p * r] = c * wp - s * wq;
                    Ww[j + q * r] = s * wp + c * wq;
                }
            }
            __syncthreads();
            // G <- J^T G (rows p, q)
            for (int i = warp; i < npair; i += nwarp) {
                const int q = qq[i];
                const T s = sn[i];
                if (q < 0 || s == T(0)) continue;
                const int p = pp[i];
                const T c = cs[i];
                for (int j = lane; j < r; j += 32) {
                    T gp = SG(G, ld, p, j), gq = SG(G, ld, q, j);
                    SG(G, ld, p, j) = c * gp - s * gq;
                    SG(G, ld, q, j) = s * gp + c * gq;
                }
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

// Jacobi cleanup of a nearly diagonal symmetric G (an eigenbasis already aligned to FP32
// level), in mixed precision: the diagonal is FP64, the off-diagonal part and W - I are FP32.
// Both stay small against the diagonal scale (~1e-7 of it after the alignment), so FP32 holds
// them to ~1e-14 of that scale, as FP64 Jacobi on the full matrix would; each rotation costs
// three FP64 operations (the diagonal updates a_pp -= t a_pq, a_qq += t a_pq and the difference
// a_qq - a_pp of its angle), everything else is FP32.  Rotation (p, q): tau = (a_qq - a_pp) /
// (2 a_pq), t = sign(tau) / (|tau| + sqrt(1 + tau^2)), c = 1 / sqrt(1 + t^2), s = t c; columns
// p, q of A and W take c x_p - s x_q, s x_p + c x_q, and W - I is updated with the identity's
// share: (c - 1) on (p, p), (q, q), -s on (q, p), s on (p, q).  Same schedule, thresholds and
// outputs as k_jacobi (W FP64 sorted by |lambda| descending).
constexpr int JMW = JTHREADS / 32;    // warps of the mixed kernel

__global__ void __launch_bounds__(JTHREADS)
k_jacobi_mixed(const double* __restrict__ Gin, int64_t ldg, int64_t strideG, int r, double* __restrict__ Wout,
               double* __restrict__ lam, int* status, float rel_tol, float floor_tol) {
    Gin += (int64_t)blockIdx.x * strideG;
    Wout += (int64_t)blockIdx.x * r * r;
    lam += (int64_t)blockIdx.x * r;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ld = r + 1;
    double* dg = reinterpret_cast<double*>(smem_raw);       // r: the FP64 diagonal
    float* A = reinterpret_cast<float*>(dg + JMAX);          // r x r off-diagonal part, ld r + 1
    float* D = A + (size_t)ld * r;                           // W - I, r x r
    float* cs = D + (size_t)r * r;                           // per pair: c, s, c - 1
    float* sn = cs + (JMAX / 2 + 1);
    float* cm = sn + (JMAX / 2 + 1);
    int* pp = reinterpret_cast<int*>(cm + (JMAX / 2 + 1));
    int* qq = pp + (JMAX / 2 + 1);
    __shared__ int rot_count;
    __shared__ float fro;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int R = r + (r & 1), n = R - 1, npair = R / 2;

    // load: symmetrised off-diagonal part in FP32, the diagonal in FP64; W - I = 0
    for (int j = warp; j < r; j += JMW)
        for (int i = lane; i < r; i += 32) {
            const double g = 0.5 * (Gin[i + j * ldg] + Gin[j + i * ldg]);
            if (i == j) dg[i] = g;
            A[i + j * ld] = i == j ? 0.0f : f64_to_f32_rn(g);
            D[i + j * r] = 0.0f;
        }
    __syncthreads();
    if (warp == 0) {
        float acc = 0.0f;
        for (int j = 0; j < r; ++j)
            for (int i = lane; i < r; i += 32) {
                const float v = i == j ? f64_to_f32_rn(dg[i]) : A[i + j * ld];
                acc = fmaf(v, v, acc);
            }
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) fro = sqrtf(acc);
    }
    __syncthreads();
    const float abs_floor = floor_tol * fro;
    bool converged = (r <= 1);
    for (int sweep = 0; sweep < JMAX_SWEEPS && !converged; ++sweep) {
        if (tid == 0) rot_count = 0;
        __syncthreads();
        for (int t = 0; t < n; ++t) {
            // pair schedule of k_jacobi; each pair's thread also updates its two diagonal entries
            for (int i = tid; i < npair; i += JTHREADS) {
                int p, q;
                if (i == 0) { p = n; q = t; }
                else { p = (t + i) % n; q = (t - i + n) % n; }
                if (p > q) { int tmp = p; p = q; q = tmp; }
                float c = 1.0f, s = 0.0f, cm1 = 0.0f;
                if (q < r) {
                    const float apq = A[p + q * ld];
                    const double app = dg[p], aqq = dg[q];
                    const float thr = fmaxf(rel_tol * sqrtf(fabsf(f64_to_f32_rn(app))) * sqrtf(fabsf(f64_to_f32_rn(aqq))),
                                            abs_floor);
                    if (fabsf(apq) > thr) {
                        const float tau = f64_to_f32_rn(aqq - app) / (2.0f * apq);
                        const float tt = fabsf(tau) > 1e18f ? 0.5f / tau
                                                            : copysignf(1.0f, tau) / (fabsf(tau) + sqrtf(1.0f + tau * tau));
                        c = rsqrtf(1.0f + tt * tt);
                        s = tt * c;
                        cm1 = -(tt * tt) * c * c / (1.0f + c);
                        const double dlt = f32_to_f64(tt * apq);
                        dg[p] = app - dlt;
                        dg[q] = aqq + dlt;
                        atomicAdd(&rot_count, 1);
                    }
                }
                pp[i] = p; qq[i] = (q < r) ? q : -1; cs[i] = c; sn[i] = s; cm[i] = cm1;
            }
            __syncthreads();
            // A <- A J (columns p, q, rows other than p, q) and W - I <- (W - I) J + (J - I)
            for (int i = warp; i < npair; i += JMW) {
                const int q = qq[i];
                const float s = sn[i];
                if (q < 0 || s == 0.0f) continue;
                const int p = pp[i];
                const float c = cs[i], cm1 = cm[i];
                for (int j = lane; j < r; j += 32) {
                    if (j != p && j != q) {
                        const float gp = A[j + p * ld], gq = A[j + q * ld];
                        A[j + p * ld] = c * gp - s * gq;
                        A[j + q * ld] = s * gp + c * gq;
                    }
                    const float wp = D[j + p * r], wq = D[j + q * r];
                    D[j + p * r] = c * wp - s * wq + (j == p ? cm1 : (j == q ? -s : 0.0f));
                    D[j + q * r] = s * wp + c * wq + (j == p ? s : (j == q ? cm1 : 0.0f));
                }
            }
            __syncthreads();
            // A <- J^T A (rows p, q, columns other than p, q); the 2 x 2 block is diagonal now
            for (int i = warp; i < npair; i += JMW) {
                const int q = qq[i];
                const float s = sn[i];
                if (q < 0 || s == 0.0f) continue;
                const int p = pp[i];
                const float c = cs[i];
                for (int j = lane; j < r; j += 32) {
                    if (j != p && j != q) {
                        const float gp = A[p + j * ld], gq = A[q + j * ld];
                        A[p + j * ld] = c * gp - s * gq;
                        A[q + j * ld] = s * gp + c * gq;
                    } else {
                        A[p + j * ld] = 0.0f;
                        A[q + j * ld] = 0.0f;
                    }
                }
            }
            __syncthreads();
        }
        converged = (rot_count == 0);
        __syncthreads();
    }
    if (!converged) {
        __shared__ int bad;
        if (tid == 0) bad = 0;
        __syncthreads();
        for (int j = warp; j < r; j += JMW)
            for (int i = lane; i < j; i += 32) {
                const float g = A[i + j * ld];
                if (fabsf(g) > 1e-9f * sqrtf(fabsf(f64_to_f32_rn(dg[i]))) * sqrtf(fabsf(f64_to_f32_rn(dg[j]))) &&
                    fabsf(g) > 1e-16f * fro)
                    bad = 1;
            }
        __syncthreads();
        if (tid == 0 && bad) atomicOr(status, ST_JACOBI_NOCONV);
    }
    // sort by |lambda| descending (stable by index); W = I + (W - I) in FP64
    for (int i = tid; i < r; i += JTHREADS) {
        const double li = dg[i];
        if (!isfinite(li)) atomicOr(status, ST_NONFINITE);
        int rank = 0;
        for (int j = 0; j < r; ++j) {
            const double lj = fabs(dg[j]);
            rank += (lj > fabs(li)) || (lj == fabs(li) && j < i);
        }
        lam[rank] = li;
        for (int j = 0; j < r; ++j) {
            const double d = f32_to_f64(D[j + (int64_t)i * r]);
            Wout[j + (int64_t)rank * r] = j == i ? 1.0 + d : d;
        }
    }
}

void jacobi_eigh_mixed(Ctx& c, const double* G, int64_t ldg, int r, double* W, double* lam, int batch,
                       int64_t strideG, double rel, double floor) {
    TNR_REQUIRE(r >= 1 && r <= JMAX, TNR_ERR_UNSUPPORTED, "jacobi_eigh_mixed: r out of range");
    auto bytes = [](int rr) {
        return (size_t)JMAX * sizeof(double) + ((size_t)(rr + 1) * rr + (size_t)rr * rr) * sizeof(float) +
               3 * (JMAX / 2 + 1) * sizeof(float) + 2 * (JMAX / 2 + 1) * sizeof(int);
    };
    static std::atomic<uint64_t> attr_set{0};
    ensure_smem_attr(attr_set, (const void*)k_jacobi_mixed, (int)bytes(JMAX));
    int rec = prof_start(c.stream);
    k_jacobi_mixed<<<batch, JTHREADS, bytes(r), c.stream>>>(G, ldg, strideG, r, W, lam, c.d_status, (float)rel,
                                                            (float)floor);
    check_launch("jacobi_mixed");
    prof_stop(rec, c.stream, PROF_JACOBI, (double)r * r * r * batch);
}

template <class T>
static void launch_jacobi(Ctx& c, const double* G, int64_t ldg, int r, double* W, double* lam, int batch,
                          int64_t strideG, double rel = JTol<T>::rel, double floor = JTol<T>::floor) {
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
    k_jacobi<T><<<batch, nt, smem, c.stream>>>(G, ldg, strideG, r, W, lam, ww.as<T>(), c.d_status, rel, floor);
    check_launch("jacobi");
    prof_stop(rec, c.stream, sizeof(T) == 8 ? PROF_JACOBI : PROF_JACOBI32, (double)r * r * r * batch);
}

void jacobi_eigh(Ctx& c, const double* G, int64_t ldg, int r, double* W, double* lam, int batch, int64_t strideG) {
    launch_jacobi<double>(c, G, ldg, r, W, lam, batch, strideG);
}

void jacobi_eigh_tol(Ctx& c, const double* G, int64_t ldg, int r, double* W, double* lam, int batch, int64_t strideG,
                     double rel, double floor) {
    launch_jacobi<double>(c, G, ldg, r, W, lam, batch, strideG, rel, floor);
}

void jacobi_eigh_f32(Ctx& c, const double* G, int64_t ldg, int r, double* W, double* lam, int batch,
                     int64_t strideG) {
    launch_jacobi<float>(c, G, ldg, r, W, lam, batch, strideG);
}

// Cholesky of (G + shift I) = L L^T in shared memory, then L^{-1} (lower) written over G.
// Blocked by CB = 32 columns so that the CTA meets about 30 barriers instead of one or two per
// column:
//  * per panel: the 32 x 32 diagonal block is factored by one warp (lane l owns row l,
//    __syncwarp only); the rows below it solve against it (one thread per row, forward
//    substitution); the trailing lower triangle takes the rank-32 update (one warp per column);
//  * inverse: each diagonal block is inverted by one warp (lane j owns column j); the blocks
//    below the diagonal follow by block distance, X_ij = -X_ii (sum_t L_it X_tj), through one
//    32 x 32 scratch block.
// Storage in S (column-major, ld = r + 1): L in the lower triangle; X[i,j] (i > j) at the
// transposed position S[j + i ld] (strict upper triangle, free once L is done); X[j,j] in the
// spare row S[r + j ld].
constexpr int CB = 32;
constexpr int CHOL_THREADS = 256;

template <class T>
__global__ void __launch_bounds__(CHOL_THREADS)
k_chol_inv(double* G, int r, double shift, int* status) {
    G += (int64_t)blockIdx.x * r * r;     // one CTA per matrix of a batch
    extern __shared__ __align__(16) unsigned char smem_c[];
    T* S = reinterpret_cast<T*>(smem_c);
    const int ld = r + 1;
    T* Y = S + (size_t)ld * r;            // CB x CB scratch block, leading dimension CB + 1
    constexpr int ldy = CB + 1;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = CHOL_THREADS / 32;
    __shared__ int bad;
    if (tid == 0) bad = 0;
    for (int e = tid; e < r * r; e += CHOL_THREADS) {
        int i = e % r, j = e / r;
        if (sizeof(T) == 4) {
            // FP32: convert with integer operations, shift in FP32 (no FP64 arithmetic)
            const float v = i >= j ? f64_to_f32_rn(G[e]) : 0.0f;
            S[i + j * ld] = (T)(i == j ? v + (float)shift : v);
        } else {
            S[i + j * ld] = (T)((i >= j) ? G[e] + (i == j ? shift : 0.0) : 0.0);
        }
    }
    __syncthreads();
    const int nblk = (r + CB - 1) / CB;
    for (int pb = 0; pb < nblk; ++pb) {
        const int p = pb * CB, nb = min(CB, r - p);
        // (1) diagonal block, one warp, right-looking, in registers: lane l holds row p + l; the
        // column of the pivot comes from the other lanes by shuffles
        if (warp == 0) {
            T a[CB];
#pragma unroll
            for (int jj = 0; jj < CB; ++jj)
                a[jj] = (jj <= lane && lane < nb && jj < nb) ? S[(p + lane) + (p + jj) * ld] : T(0);
#pragma unroll
            for (int j = 0; j < CB; ++j) {
                if (j < nb) {                                   // warp-uniform
                    T d = __shfl_sync(0xffffffffu, a[j], j);
                    if (!(d > T(0)) || !isfinite(d)) {
                        if (lane == 0) bad = 1;
                        d = (T)1e-30;
                    }
                    const T piv = sqrt(d);
                    if (lane == j) a[j] = piv;
                    else if (lane > j) a[j] = a[j] / piv;      // L[l][j]
                    const T x = a[j];
#pragma unroll
                    for (int jj = j + 1; jj < CB; ++jj) {
                        const T v = __shfl_sync(0xffffffffu, a[j], jj);   // L[jj][j]
                        if (lane >= jj) a[jj] -= x * v;
                    }
                }
            }
#pragma unroll
            for (int jj = 0; jj < CB; ++jj)
                if (jj <= lane && lane < nb && jj < nb) S[(p + lane) + (p + jj) * ld] = a[jj];
        }
        __syncthreads();
        // (2) rows below the block: L21 = A21 L11^-T, one thread per row, the row in registers
        for (int i = p + nb + tid; i < r; i += CHOL_THREADS) {
            T x[CB];
#pragma unroll
            for (int j = 0; j < CB; ++j) {
                if (j < nb) {
                    T acc = S[i + (p + j) * ld];
#pragma unroll
                    for (int t = 0; t < j; ++t) acc -= x[t] * S[(p + j) + (p + t) * ld];
                    x[j] = acc / S[(p + j) + (p + j) * ld];
                }
            }
#pragma unroll
            for (int j = 0; j < CB; ++j)
                if (j < nb) S[i + (p + j) * ld] = x[j];
        }
        __syncthreads();
        // (3) trailing lower triangle: A22 -= L21 L21^T, one warp per column
        for (int j = p + nb + warp; j < r; j += NW) {
            for (int i = j + lane; i < r; i += 32) {
                T acc = T(0);
                for (int t = 0; t < nb; ++t) acc += S[i + (p + t) * ld] * S[j + (p + t) * ld];
                S[i + j * ld] -= acc;
            }
        }
        __syncthreads();
    }
    // (4) diagonal blocks of X = L^-1, one warp per block, lane j owns column j of the block in
    // registers (x[t] = X[p + t][p + j]); rows of L are read as shared-memory broadcasts
    for (int pb = warp; pb < nblk; pb += NW) {
        const int p = pb * CB, nb = min(CB, r - p);
        const int j = lane;
        T x[CB];
#pragma unroll
        for (int i = 0; i < CB; ++i) {
            if (i < nb) {
                T v = T(0);
                if (i == j) {
                    v = T(1) / S[(p + j) + (p + j) * ld];
                } else if (i > j) {
                    T acc = T(0);
#pragma unroll
                    for (int t = 0; t < i; ++t)
                        if (t >= j) acc += S[(p + i) + (p + t) * ld] * x[t];
                    v = -acc / S[(p + i) + (p + i) * ld];
                }
                x[i] = v;
            }
        }
        if (j < nb) {
#pragma unroll
            for (int i = 0; i < CB; ++i) {
                if (i == j) S[r + (p + j) * ld] = x[i];
                else if (i > j && i < nb) S[(p + j) + (p + i) * ld] = x[i];
            }
        }
    }
    __syncthreads();
    // (5) blocks below the diagonal, by block distance: X_ij = -X_ii Y, Y = sum_{t=j}^{i-1} L_it X_tj
    for (int dist = 1; dist < nblk; ++dist) {
        for (int bj = 0; bj + dist < nblk; ++bj) {
            const int bi = bj + dist;
            const int pi = bi * CB, ni = min(CB, r - pi), pj = bj * CB, nj = min(CB, r - pj);
            for (int e = tid; e < ni * nj; e += CHOL_THREADS) {
                const int ii = e % ni, jj = e / ni;
                const int i = pi + ii, j = pj + jj;
                // t = j: X[j,j] on the spare row; t in (j, pi): X[t,j] at S[j + t ld]
                T acc = S[i + j * ld] * S[r + j * ld];
                for (int t = j + 1; t < pi; ++t) acc += S[i + t * ld] * S[j + t * ld];
                Y[ii + jj * ldy] = acc;
            }
            __syncthreads();
            for (int e = tid; e < ni * nj; e += CHOL_THREADS) {
                const int ii = e % ni, jj = e / ni;
                const int i = pi + ii, j = pj + jj;
                // (X_ii Y)[ii, jj] = X[i,i] Y[ii,jj] + sum_{s < ii} X[i, pi + s] Y[s, jj]
                T acc = S[r + i * ld] * Y[ii + jj * ldy];
                for (int s2 = 0; s2 < ii; ++s2) acc += S[(pi + s2) + i * ld] * Y[s2 + jj * ldy];
                S[j + i * ld] = -acc;
            }
            __syncthreads();
        }
    }
    for (int e = tid; e < r * r; e += CHOL_THREADS) {
        int i = e % r, j = e / r;
        const T v = i > j ? S[j + i * ld] : (i == j ? S[r + j * ld] : T(0));
        G[e] = sizeof(T) == 4 ? f32_to_f64((float)v) : (double)v;
    }
    if (tid == 0 && bad) atomicOr(status, ST_CHOL_BREAKDOWN);
}

// shared memory of k_chol_inv: the r x r matrix (ld r + 1) and the CB x CB scratch block
template <class T>
static size_t chol_smem(int r) { return ((size_t)(r + 1) * r + (size_t)CB * (CB + 1)) * sizeof(T); }

template <class T>
static void launch_chol(Ctx& c, double* G, int r, double shift, int batch) {
    TNR_REQUIRE(r >= 1 && r <= JMAX, TNR_ERR_UNSUPPORTED, "chol_inv: r out of range");
    const size_t smem = chol_smem<T>(r);
    TNR_REQUIRE(smem <= 227 * 1024, TNR_ERR_UNSUPPORTED, "chol_inv: matrix too large for shared memory");
    static std::atomic<uint64_t> attr_set{0};
    ensure_smem_attr(attr_set, (const void*)k_chol_inv<T>, (int)std::min<size_t>(chol_smem<T>(JMAX), 227 * 1024));
    int rec = prof_start(c.stream);
    k_chol_inv<T><<<batch, CHOL_THREADS, smem, c.stream>>>(G, r, shift, c.d_status);
    check_launch("chol_inv");
    prof_stop(rec, c.stream, sizeof(T) == 8 ? PROF_CHOL : PROF_CHOL32, (double)r * r * r * batch);
}

void chol_inv(Ctx& c, double* G, int r, double shift, int batch) { launch_chol<double>(c, G, r, shift, batch); }
// FP32 Cholesky + inverse of CholeskyQR in split precision: the storage and the result of
// k_chol_inv<float>, with the work of each phase spread over the eight warps:
//  * diagonal block: one warp in registers, reciprocal square roots (1 / L_jj kept for later);
//  * rows below it (L21 = A21 L11^-T): one thread per row, two partial sums per dot product;
//  * trailing update A22 -= L21 L21^T: per warp strips of 4 columns x 128 rows (lane owns
//    rows lane + 32k), 4 x 4 register tiles, rows broadcast-free and columns broadcast;
//  * diagonal blocks of X = L^-1: one warp per block, lane j owns column j;
//  * blocks below the diagonal by block distance, X_ij = -X_ii sum_t L_it X_tj, every block of
//    a distance at once: lanes own rows, warps take (block, column) units.
constexpr int C32_NW = CHOL_THREADS / 32;
constexpr int C32_MAXBLK = (JMAX + CB - 1) / CB;

__global__ void __launch_bounds__(CHOL_THREADS, 1)
k_chol_inv_f32(double* G, int r, double shift, int* status) {
    G += (int64_t)blockIdx.x * r * r;
    extern __shared__ __align__(16) unsigned char smem_c32[];
    float* S = reinterpret_cast<float*>(smem_c32);
    const int ld = r + 1;
    float* inv = S + (size_t)ld * r;                 // 1 / L_jj
    float* Yb = inv + JMAX;                          // per block pair: CB x CB, ld CB + 1
    constexpr int ldy = CB + 1;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __shared__ int bad;
    if (tid == 0) bad = 0;
    const float fshift = (float)shift;
    for (int j = warp; j < r; j += C32_NW)
        for (int i = lane; i < r; i += 32) {
            const float v = i >= j ? f64_to_f32_rn(G[i + (int64_t)j * r]) : 0.0f;
            S[i + j * ld] = i == j ? v + fshift : v;
        }
    __syncthreads();
    const int nblk = (r + CB - 1) / CB;
    for (int pb = 0; pb < nblk; ++pb) {
        const int p = pb * CB, nb = min(CB, r - p);
        if (warp == 0) {
            float a[CB];
#pragma unroll
            for (int jj = 0; jj < CB; ++jj)
                a[jj] = (jj <= lane && lane < nb && jj < nb) ? S[(p + lane) + (p + jj) * ld] : 0.0f;
            float myinv = 0.0f;
#pragma unroll
            for (int j = 0; j < CB; ++j) {
                if (j < nb) {                                   // warp-uniform
                    float d = __shfl_sync(0xffffffffu, a[j], j);
                    if (!(d > 0.0f) || !isfinite(d)) {
                        if (lane == 0) bad = 1;
                        d = 1e-30f;
                    }
                    const float rs = rsqrtf(d);
                    if (lane == j) {
                        a[j] = d * rs;
                        myinv = rs;
                    } else if (lane > j) {
                        a[j] *= rs;                             // L[l][j]
                    }
                    const float x = a[j];
#pragma unroll
                    for (int jj = j + 1; jj < CB; ++jj) {
                        const float v = __shfl_sync(0xffffffffu, a[j], jj);   // L[jj][j]
                        if (lane >= jj) a[jj] = fmaf(-x, v, a[jj]);
                    }
                }
            }
#pragma unroll
            for (int jj = 0; jj < CB; ++jj)
                if (jj <= lane && lane < nb && jj < nb) S[(p + lane) + (p + jj) * ld] = a[jj];
            if (lane < nb) inv[p + lane] = myinv;
        }
        __syncthreads();
        const int m2 = r - p - CB;           // rows below the block (the block is full if any)
        if (m2 <= 0) continue;
        for (int i = p + CB + tid; i < r; i += CHOL_THREADS) {
            float x[CB];
#pragma unroll
            for (int j = 0; j < CB; ++j) {
                float a0 = S[i + (p + j) * ld], a1 = 0.0f;
#pragma unroll
                for (int t = 0; t < j; t += 2) {
                    a0 = fmaf(-x[t], S[(p + j) + (p + t) * ld], a0);
                    if (t + 1 < j) a1 = fmaf(-x[t + 1], S[(p + j) + (p + t + 1) * ld], a1);
                }
                x[j] = (a0 + a1) * inv[p + j];
            }
#pragma unroll
            for (int j = 0; j < CB; ++j) S[i + (p + j) * ld] = x[j];
        }
        __syncthreads();
        const int q0 = p + CB, ncg = (m2 + 3) / 4;
        for (int cg = warp; cg < ncg; cg += C32_NW) {
            const int j0 = q0 + 4 * cg;
            for (int i0 = j0; i0 < r; i0 += 128) {
                float acc[4][4];
#pragma unroll
                for (int k = 0; k < 4; ++k)
#pragma unroll
                    for (int l = 0; l < 4; ++l) acc[k][l] = 0.0f;
#pragma unroll 4
                for (int t = 0; t < CB; ++t) {
                    const float* col = S + (p + t) * ld;
                    float a[4], b[4];
#pragma unroll
                    for (int l = 0; l < 4; ++l) b[l] = (j0 + l < r) ? col[j0 + l] : 0.0f;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const int i = i0 + lane + 32 * k;
                        a[k] = i < r ? col[i] : 0.0f;
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k)
#pragma unroll
                        for (int l = 0; l < 4; ++l) acc[k][l] = fmaf(a[k], b[l], acc[k][l]);
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int i = i0 + lane + 32 * k;
#pragma unroll
                    for (int l = 0; l < 4; ++l)
                        if (i < r && j0 + l < r && i >= j0 + l) S[i + (j0 + l) * ld] -= acc[k][l];
                }
            }
        }
        __syncthreads();
    }
    // diagonal blocks of X: X[p+i][p+j] (i > j) at S[(p+j) + (p+i) ld], X[p+j][p+j] at S[r + (p+j) ld]
    if (warp < nblk) {
        const int p = warp * CB, nb = min(CB, r - p);
        const int j = lane;
        float x[CB];
#pragma unroll
        for (int i = 0; i < CB; ++i) {
            float v = 0.0f;
            if (i < nb && j < nb) {
                if (i == j) {
                    v = inv[p + j];
                } else if (i > j) {
                    float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
                    for (int t = 0; t < i; t += 2) {           // x[t] = 0 for t < j
                        a0 = fmaf(S[(p + i) + (p + t) * ld], x[t], a0);
                        if (t + 1 < i) a1 = fmaf(S[(p + i) + (p + t + 1) * ld], x[t + 1], a1);
                    }
                    v = -(a0 + a1) * inv[p + i];
                }
            }
            x[i] = v;
        }
        if (j < nb) {
#pragma unroll
            for (int i = 0; i < CB; ++i) {
                if (i == j) S[r + (p + j) * ld] = x[i];
                else if (i > j && i < nb) S[(p + j) + (p + i) * ld] = x[i];
            }
        }
    }
    __syncthreads();
    for (int dist = 1; dist < nblk; ++dist) {
        const int nbp = nblk - dist, units = nbp * CB;
        // Y_b[ii][jj] = sum_{t = pj + jj}^{pi - 1} L[pi + ii][t] X[t][pj + jj]   (block pair b = bj)
        for (int u = warp; u < units; u += C32_NW) {
            const int bj = u / CB, jj = u % CB, bi = bj + dist;
            const int pi = bi * CB, pj = bj * CB, ni = min(CB, r - pi), j = pj + jj;
            const int ii = lane;
            float a0 = 0.0f, a1 = 0.0f;
            if (ii < ni) {
                const float* Li = S + pi + ii;                 // L[pi + ii][t] = Li[t * ld]
                a0 = Li[j * ld] * S[r + j * ld];               // t = j: X[j][j]
                int t = j + 1;
                for (; t + 1 < pi; t += 2) {
                    a0 = fmaf(Li[t * ld], S[j + t * ld], a0);
                    a1 = fmaf(Li[(t + 1) * ld], S[j + (t + 1) * ld], a1);
                }
                if (t < pi) a0 = fmaf(Li[t * ld], S[j + t * ld], a0);
            }
            Yb[bj * CB * ldy + ii + jj * ldy] = a0 + a1;
        }
        __syncthreads();
        // X[pi + ii][pj + jj] = -sum_{s <= ii} X[pi + ii][pi + s] Y_b[s][jj]
        for (int u = warp; u < units; u += C32_NW) {
            const int bj = u / CB, jj = u % CB, bi = bj + dist;
            const int pi = bi * CB, pj = bj * CB, ni = min(CB, r - pi);
            const int ii = lane;
            if (ii < ni) {
                const float* Y = Yb + bj * CB * ldy + jj * ldy;
                float a0 = S[r + (pi + ii) * ld] * Y[ii], a1 = 0.0f;
                int s2 = 0;
                for (; s2 + 1 < ii; s2 += 2) {
                    a0 = fmaf(S[(pi + s2) + (pi + ii) * ld], Y[s2], a0);
                    a1 = fmaf(S[(pi + s2 + 1) + (pi + ii) * ld], Y[s2 + 1], a1);
                }
                if (s2 < ii) a0 = fmaf(S[(pi + s2) + (pi + ii) * ld], Y[s2], a0);
                S[(pj + jj) + (pi + ii) * ld] = -(a0 + a1);
            }
        }
        __syncthreads();
    }
    for (int j = warp; j < r; j += C32_NW)
        for (int i = lane; i < r; i += 32) {
            const float v = i > j ? S[j + i * ld] : (i == j ? S[r + j * ld] : 0.0f);
            G[i + (int64_t)j * r] = f32_to_f64(v);
        }
    if (tid == 0 && bad) atomicOr(status, ST_CHOL_BREAKDOWN);
}

static size_t chol32_smem(int r) {
    return ((size_t)(r + 1) * r + JMAX + (size_t)C32_MAXBLK * CB * (CB + 1)) * sizeof(float);
}

void chol_inv_f32(Ctx& c, double* G, int r, double shift, int batch) {
    TNR_REQUIRE(r >= 1 && r <= JMAX, TNR_ERR_UNSUPPORTED, "chol_inv: r out of range");
    static std::atomic<uint64_t> attr_set{0};
    ensure_smem_attr(attr_set, (const void*)k_chol_inv_f32, (int)chol32_smem(JMAX));
    int rec = prof_start(c.stream);
    k_chol_inv_f32<<<batch, CHOL_THREADS, chol32_smem(r), c.stream>>>(G, r, shift, c.d_status);
    check_launch("chol_inv_f32");
    prof_stop(rec, c.stream, PROF_CHOL32, (double)r * r * r * batch);
}

}  // namespace tnr
