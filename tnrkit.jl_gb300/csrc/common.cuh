// Shared declarations of the GB300 coarse-graining engine (internal).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <map>
#include <string>
#include <vector>
#include <stdexcept>
#include <atomic>
#include <memory>

#include "../../include/tnr_gb300.h"

namespace tnr {

#ifdef __CUDACC__
// FP32 <-> FP64 conversions with integer operations only: FP64 arithmetic, conversions
// included, runs at a small fraction of the FP32 rate on this part.
// FP32 -> FP64: exponent rebias and mantissa shift; FP32 subnormals (below 2^-126) become
// signed zero, infinities and NaNs keep their class.
__device__ __forceinline__ double f32_to_f64(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xFFu, mant = u & 0x7FFFFFu, sign = u & 0x80000000u;
    const uint32_t e64 = e == 255u ? 2047u : e + 896u;
    const uint32_t hi = e == 0u ? sign : (sign | (e64 << 20) | (mant >> 3));
    const uint32_t lo = e == 0u ? 0u : (mant << 29);
    return __hiloint2double((int)hi, (int)lo);
}

// FP64 -> FP32, rounded to nearest (ties to even) on the 29 dropped mantissa bits; |x| below
// 2^-126 becomes signed zero, |x| beyond the FP32 range infinity, NaN stays NaN.
__device__ __forceinline__ float f64_to_f32_rn(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const uint32_t hi = (uint32_t)(u >> 32), lo = (uint32_t)u;
    const uint32_t sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7FFu);
    if (e <= 896) return __uint_as_float(sign);
    if (e >= 1151) {
        const bool nan = e == 2047 && (((hi & 0xFFFFFu) | lo) != 0u);
        return __uint_as_float(sign | 0x7F800000u | (nan ? 0x00400000u : 0u));
    }
    const uint32_t m23 = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const uint32_t rem = lo & 0x1FFFFFFFu;
    uint32_t bits = ((uint32_t)(e - 896) << 23) | m23;
    if (rem > 0x10000000u || (rem == 0x10000000u && (m23 & 1u))) bits += 1u;   // a carry moves the exponent
    return __uint_as_float(sign | bits);
}
#endif

// ---------------------------------------------------------------------------
// errors: C++ exceptions inside the library, status codes at the C ABI
// ---------------------------------------------------------------------------
struct Error : public std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define TNR_CUDA(call)                                                              \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            throw ::tnr::Error(e_ == cudaErrorMemoryAllocation ? TNR_ERR_OOM        \
                                                               : TNR_ERR_CUDA,      \
                               std::string(#call) + ": " + cudaGetErrorString(e_)); \
        }                                                                           \
    } while (0)

#define TNR_REQUIRE(cond, code, msg)                 \
    do {                                             \
        if (!(cond)) throw ::tnr::Error((code), (msg)); \
    } while (0)

// every kernel launch goes through this counter (reported by tnr_kernel_launches)
extern std::atomic<uint64_t> g_launches;

// Per-device one-time setup: `done` holds one bit per device index (0..63).  A kernel's
// dynamic shared-memory limit and a memory pool's attributes belong to the current device's
// context, so a process that uses several devices sets them on each.  Two threads that race
// on the same device both set the same value, which is harmless.
inline bool device_once(std::atomic<uint64_t>& done, int* dev_out = nullptr) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev > 63) {
        cudaGetLastError();
        throw ::tnr::Error(TNR_ERR_CUDA, "no current CUDA device (or device index above 63)");
    }
    if (dev_out) *dev_out = dev;
    return !(done.load(std::memory_order_acquire) & (1ull << dev));
}
inline void device_done(std::atomic<uint64_t>& done, int dev) { done.fetch_or(1ull << dev, std::memory_order_release); }
inline void ensure_smem_attr(std::atomic<uint64_t>& done, const void* func, int bytes) {
    int dev = 0;
    if (!device_once(done, &dev)) return;
    TNR_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    device_done(done, dev);
}
inline void count_launch(int n = 1) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }

inline void check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        throw Error(TNR_ERR_CUDA, std::string("launch ") + what + ": " + cudaGetErrorString(e));
    count_launch();
}

// device status word bits written by iterative kernels (never trap, never spin forever)
enum : int {
    ST_JACOBI_NOCONV = 1,
    ST_CHOL_BREAKDOWN = 2,
    ST_NONFINITE = 4,
    ST_TC_TIMEOUT = 8,    // a tcgen05 pipeline wait gave up: the call's results are invalid
};

int sm_count();

// ---------------------------------------------------------------------------
// per-kernel-class profiler: CUDA events around launches, algorithmic work units
// ---------------------------------------------------------------------------
enum ProfClass : int {
    PROF_GEMM_BULK = 0,   // bulk contraction / projection GEMMs run in FP64, work = flops
    PROF_GEMM_F64 = 1,    // FP64 GEMMs of the decompositions, work = flops
    PROF_JACOBI = 2,      // small Jacobi eigensolver, work = r^3
    PROF_CHOL = 3,        // Cholesky + inverse, work = r^3
    PROF_PERMUTE = 4,     // leg permutes, work = bytes moved
    PROF_SPLIT = 5,       // FP64 -> BF16 split conversion, work = bytes moved
    PROF_JACOBI32 = 6,    // FP32 Jacobi (alignment), work = r^3
    PROF_TC = 7,          // split 3xBF16 tcgen05 GEMMs, work = 2 m n k flops
    PROF_CHOL32 = 8,      // FP32 Cholesky + inverse (split-precision CholeskyQR), work = r^3
    PROF_NCLASS = 9
};
extern std::atomic<bool> g_prof_on;
int prof_start(cudaStream_t s);
void prof_stop(int rec, cudaStream_t s, int cls, double work);
void prof_reset();
void prof_read(int cls, uint64_t* launches, double* ms, double* work);

// ---------------------------------------------------------------------------
// caching device allocator (stream-ordered reuse on one stream)
// ---------------------------------------------------------------------------
class Pool {
  public:
    explicit Pool(cudaStream_t s) : stream_(s) {}
    ~Pool();
    void* get(size_t bytes);
    void put(void* p);
    size_t held_bytes() const { return held_; }
    void trim();

  private:
    cudaStream_t stream_;
    std::multimap<size_t, void*> free_;
    std::map<void*, size_t> size_of_;
    size_t held_ = 0;
};

// RAII handle on a pool block
class Buf {
  public:
    Buf() = default;
    Buf(Pool* pool, size_t bytes) : pool_(pool), bytes_(bytes) { p_ = bytes ? pool->get(bytes) : nullptr; }
    Buf(const Buf&) = delete;
    Buf& operator=(const Buf&) = delete;
    Buf(Buf&& o) noexcept { *this = std::move(o); }
    Buf& operator=(Buf&& o) noexcept {
        release();
        pool_ = o.pool_; p_ = o.p_; bytes_ = o.bytes_;
        o.p_ = nullptr; o.bytes_ = 0;
        return *this;
    }
    ~Buf() { release(); }
    void release() {
        if (p_ && pool_) pool_->put(p_);
        p_ = nullptr; bytes_ = 0;
    }
    template <class T> T* as() const { return static_cast<T*>(p_); }
    double* d() const { return static_cast<double*>(p_); }
    size_t bytes() const { return bytes_; }

  private:
    Pool* pool_ = nullptr;
    void* p_ = nullptr;
    size_t bytes_ = 0;
};

// ---------------------------------------------------------------------------
// dense FP64 device tensor, column-major (first leg fastest)
// ---------------------------------------------------------------------------
constexpr int MAXR = 8;

struct DT {
    Buf buf;
    int rank = 0;
    int64_t d[MAXR] = {0};
    // Z_N charges (N > 1): q[l][i] is the signed charge that basis index i of leg l contributes
    // to the conservation law sum_l q[l][i_l] = 0 (mod N) obeyed by every nonzero entry
    // (codomain legs carry +charge, domain legs -charge).  The data stay the dense embedding;
    // contractions and decompositions of charged tensors run block by block over the sectors.
    int N = 1;
    std::vector<std::vector<int>> q;
    bool charged() const { return N > 1 && (int)q.size() == rank; }
    double* p() const { return buf.d(); }
    int64_t size() const {
        int64_t s = 1;
        for (int i = 0; i < rank; ++i) s *= d[i];
        return rank ? s : 0;
    }
    std::vector<int64_t> dims() const { return std::vector<int64_t>(d, d + rank); }
};

DT make_dt(Pool* pool, const std::vector<int64_t>& dims);

// ---------------------------------------------------------------------------
// per-handle execution context
// ---------------------------------------------------------------------------
struct Ctx {
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int precision = TNR_PREC_F64;
    uint64_t seed = 0x9e3779b97f4a7c15ull;
    uint64_t call_counter = 0;     // varies the random sketch between calls
    std::unique_ptr<Pool> pool;
    int* d_status = nullptr;       // device status word
    double* d_scalar = nullptr;    // small device scratch (norms, reductions)
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // statistics of the decompositions
    int last_iters = 0;
    uint64_t decompositions = 0;   // truncated SVDs / eigendecompositions run
    uint64_t gap_fallbacks = 0;    // of them, decomposed in full FP64 for a too small gap
    int max_iters = 0;             // most subspace iterations of one of them
    bool exact_jacobi = false;     // the gap fallback: FP64 Jacobi converged to 1e-15
    bool bulk_call = false;        // the FP64 GEMM in flight serves a bulk contraction
    Ctx(cudaStream_t s, int prec, uint64_t seed_);
    ~Ctx();
    void sync();
    int read_status_and_clear();
};

// ---------------------------------------------------------------------------
// kernels / primitives (launch wrappers)
// ---------------------------------------------------------------------------
// out = alpha * permute(in) with out.d[k] = in.d[perm[k]]; alpha from *scale_ptr if given
void permute(Ctx& c, const double* in, const int64_t* in_dims, int rank, const int* perm,
             double* out, const double* scale_ptr = nullptr);

// two-level strided batch: batch index b = b1 + n1 * b2, offsets b1*s*1 + b2*s*2
struct Batch2 {
    int n1 = 1, n2 = 1;
    int64_t sA1 = 0, sB1 = 0, sC1 = 0, sA2 = 0, sB2 = 0, sC2 = 0;
};

// C = alpha * op(A) op(B) + beta * C  (column-major, strided batch)
void gemm_f64(Ctx& c, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
              int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, const Batch2& bt);
// exact_sum: a contraction of the coarse-graining step, whose split-precision products
// accumulate K in chunks summed in FP64 (see gemm_split_tc_a)
void gemm_bulk(Ctx& c, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
               int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, const Batch2& bt,
               bool exact_sum = false);
void gemm_f64(Ctx& c, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha,
              const double* A, int64_t lda, int64_t sA, const double* B, int64_t ldb, int64_t sB,
              double beta, double* C, int64_t ldc, int64_t sC, int batch = 1);

// bulk-contraction GEMM in the context's precision (FP64 or split 3xBF16 on tcgen05)
void gemm_bulk(Ctx& c, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha,
               const double* A, int64_t lda, int64_t sA, const double* B, int64_t ldb, int64_t sB,
               double beta, double* C, int64_t ldc, int64_t sC, int batch = 1, bool exact_sum = false);

// CholeskyQR passes of the split-precision orthonormalisation (the FP64 path always runs three)
#ifndef TNR_SPLIT_ORTH_PASSES
#define TNR_SPLIT_ORTH_PASSES 3
#endif

// subspace iterations of the truncated SVD / eigensolver from sigma estimates (tsvd.cu)
int iterations_needed(std::vector<double> v, int k, int r, int power, double target, int cap);
int iteration_cap(const Ctx& c);
// the estimates say the gap at k is too small for the subspace iteration (tsvd.cu)
bool gap_too_small(const Ctx& c, std::vector<double> v, int k, int r, int power, double target, int cap);

void sigma_estimates(Ctx& c, const double* X, int64_t n, int r, int B, double* G, double* W, double* Xa, double* lam);

// K blocks per accumulation chunk of the contraction GEMMs in split precision
int split_chunk_kb();

// split 3xBF16 tcgen05 GEMM (FP32 accumulate in TMEM); returns false if the shape is unsupported
bool gemm_split_tc(Ctx& c, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha,
                   const double* A, int64_t lda, const double* B, int64_t ldb,
                   double beta, double* C, int64_t ldc, const Batch2& bt, int chunk_kb = 0);

// BF16 planes of one FP64 A operand, split once and reused by every product with it
// (the matrix of a truncated SVD meets many thin right-hand sides); inactive unless the
// context runs the split precision and the products qualify for the tcgen05 kernel.
struct SplitA {
    bool active = false;
    bool batched = false;
    int nb = 0;
    int64_t m = 0, k = 0, Kp = 0;
    Buf planes;
    CUtensorMap map;
};
// prepare op(A) (m x k; batch from bt.n1/bt.sA1) for products with about n_hint columns
void split_a_prepare(Ctx& c, SplitA& P, bool ta, const double* A, int64_t lda, int64_t m, int64_t k,
                     int64_t n_hint, const Batch2& bt);
// gemm_bulk with a prepared A (falls back to gemm_bulk when P is inactive)
void gemm_bulk_a(Ctx& c, const SplitA& P, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha,
                 const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                 const Batch2& bt, bool exact_sum = false);
bool gemm_split_tc_a(Ctx& c, const SplitA& P, bool tb, int64_t n, const double* B, int64_t ldb, double alpha,
                     double beta, double* C, int64_t ldc, const Batch2& bt, int chunk_kb = 0);
bool split_a_build(Ctx& c, SplitA& P, bool ta, const double* A, int64_t lda, int64_t m, int64_t k,
                   const Batch2& bt);

// symmetric eigendecomposition of an r x r matrix (r <= 128), eigenvalues sorted by |lambda| desc
// batch > 1: `batch` matrices strideG apart; W (r x r) and lam (r) outputs packed per matrix
void jacobi_eigh(Ctx& c, const double* G, int64_t ldg, int r, double* W, double* lam, int batch = 1,
                 int64_t strideG = 0);
// the same with the FP64 rotation thresholds given: rotate (p, q) while |g_pq| > max(rel sqrt|g_pp g_qq|,
// floor |G|_F) (jacobi_eigh: rel 1e-12, floor 1e-22)
void jacobi_eigh_tol(Ctx& c, const double* G, int64_t ldg, int r, double* W, double* lam, int batch,
                     int64_t strideG, double rel, double floor);
// G <- Cholesky factor inverse: on exit Linv (lower) with (G + shift I) = L L^T; returns via status
void chol_inv(Ctx& c, double* G, int r, double shift, int batch = 1);
// FP32 versions (one SM runs FP32 at 64x its FP64 rate): results returned in FP64 buffers
// the FP64 cleanup of an FP32-aligned (nearly diagonal) G with the diagonal in FP64 and the
// off-diagonal part and W - I in FP32: same outputs and thresholds as jacobi_eigh_tol
void jacobi_eigh_mixed(Ctx& c, const double* G, int64_t ldg, int r, double* W, double* lam, int batch,
                       int64_t strideG, double rel, double floor);
void jacobi_eigh_f32(Ctx& c, const double* G, int64_t ldg, int r, double* W, double* lam, int batch = 1,
                     int64_t strideG = 0);
void chol_inv_f32(Ctx& c, double* G, int r, double shift, int batch = 1);
void add_identity(Ctx& c, double* X, int r, double alpha, int batch = 1);
void polar_coeff(Ctx& c, const double* E, const double* E2, double* C, int r, int batch = 1);
// X (k x n_total, ld k) rows scaled per batch: X[i, j] *= f(s[(j / n_per) * k + i])
void row_scale_batched(Ctx& c, double* X, int64_t k, int64_t n_total, const double* s, int mode, int64_t n_per);
// T (per = elements per instance, batch instances): T[e] *= v[b * dim + (e % per / stride) % dim]
void scale_leg_batched(Ctx& c, double* T, int64_t per, int batch, int64_t stride, int64_t dim, const double* v);
// out[b] (k x n) = transpose of the leading k columns of in[b] (n x p, ld n)
void transpose_lead(Ctx& c, const double* in, int64_t n, int64_t p, int k, int batch, double* out);
// trace norms of a batch: out[b] = |trace(T_b)|; then T_b /= out[b]
void trace2d_batched(Ctx& c, const double* T, const int64_t* d, int batch, const double* S1, const double* S2,
                     double* out);
void scale_batched(Ctx& c, double* T, int64_t per, int batch, const double* norms);
void fill_normal(Ctx& c, double* x, int64_t n, uint64_t seed);
void col_scale(Ctx& c, double* X, int64_t m, int64_t n, int64_t ldx, const double* s, int mode);
void row_scale(Ctx& c, double* X, int64_t m, int64_t n, int64_t ldx, const double* s, int mode);
void col_norms(Ctx& c, const double* X, int64_t m, int64_t n, int64_t ldx, double* out);
void gram_unit_diag(Ctx& c, double* G, int r, double* dscale, int batch = 1);
void sum_squares(Ctx& c, const double* x, int64_t n, double* out);
void scale_inplace(Ctx& c, double* x, int64_t n, const double* inv_scale_ptr);
void copy_f64(Ctx& c, double* dst, const double* src, int64_t n);
// Q (m x r, orthonormal columns spanning those of Y) by shifted CholeskyQR3; Y is overwritten
void orth_scaled(Ctx& c, double* Y, int64_t m, int r, double* Q);
// dst[0] = |src[0]|
void abs_copy(Ctx& c, double* dst, const double* src);
// out[i] = a x[i] + b y[i] (out may alias x or y)
void lincomb2(Ctx& c, double* out, int64_t n, double a, const double* x, double b, const double* y);

// trace norms (finalize.jl:4-14,62-66): writes |trace| into *out
void trace2d(Ctx& c, const double* T, const int64_t* d, double* out);
void trace_btrg(Ctx& c, const double* T, const int64_t* d, const double* S1, const double* S2, double* out);
void trace3d(Ctx& c, const double* T, const int64_t* d, double* out);
// pseudopow of a diagonal (btrg.jl:50-58): out = s >= tol ? s^a : s
void pseudopow(Ctx& c, const double* s, int n, double a, double* out);
void check_finite(Ctx& c, const double* x, int64_t n);

// ---------------------------------------------------------------------------
// truncated decompositions
// ---------------------------------------------------------------------------
struct TsvdOut {
    int k = 0;
    double fro2 = 0;        // ||M||_F^2
    double err = 0;         // 2-norm of the discarded values
    int iters = 0;
    std::vector<double> vals;  // kept values (host copy)
};

// the gap fallback of one m x n matrix: decomposed exactly in FP64 (min(m, n) <= 160) or
// iterated in FP64 on a 160-wide subspace; outputs as tsvd's
TsvdOut tsvd_gap_fallback(Ctx& c, const double* M, int64_t m, int64_t n, int k, double* U, double* s, double* Vt);

// M (m x n, ld = m, column-major): U (m x k), s (k), Vt (k x n)
// direct_max: largest min(m, n) decomposed directly (one-CTA solvers on the whole matrix) rather
// than by subspace iteration; at most 128
TsvdOut tsvd(Ctx& c, const double* M, int64_t m, int64_t n, int k, double* U, double* s, double* Vt,
             int direct_max = 128);
// R' = diag(s) V^T (n x n) from the SVD M = U diag(s) V^T of a column-major m x n matrix (m >= n,
// n <= 160).  R' equals the R of any QR decomposition M = Q R up to an orthogonal factor on its
// rows (R = W R'), for every rank of M: exactly rank-deficient M, which breaks CholeskyQR, is fine.
void svd_r_factor(Ctx& c, const double* M, int64_t m, int n, double* R);
// symmetric M (n x n): U (n x k) eigenvectors of the k largest |eigenvalues|, lam (k)
TsvdOut teigh(Ctx& c, const double* M, int64_t n, int k, double* U, double* lam, int direct_max = 128);
// The truncated SVD of M over the sectors its exact zeros reveal (connected components of the
// bipartite graph row r -- column c iff M[r, c] != 0): one SVD per sector block, the k largest
// values over all blocks kept, every singular vector supported on one sector (zero elsewhere).
// A matrix without such structure is one sector: then it is tsvd itself.
TsvdOut tsvd_sectors(Ctx& c, const double* M, int64_t m, int64_t n, int k, double* U, double* s, double* Vt);
// split precision: the final Rayleigh-Ritz step of tsvd / tsvd_batched for B instances (B = 1
// for one matrix) from the iteration's basis Uq [B][m x r]; writes U [B][m x k], s [B][k],
// Vt [B][k x n] and returns the B x k kept values on the host
std::vector<double> final_rr_split(Ctx& c, const SplitA& PMt, const double* M, int64_t m, int64_t n, int r, int k,
                                   int B, const double* Uq, double* U, double* s, double* Vt);
// Truncated SVD / eigh of a tensor's (row legs <- column legs) matrix, nrow row legs.  An
// uncharged tensor goes through tsvd / teigh.  A charged one decomposes sector by sector
// (rows of class c = sum of row-leg charges, columns whose charges sum to -c), keeps the chi
// largest values over all sectors (ties: lower sector, then lower index, first; descending
// order), and gives the new leg the charge -c on the U side and +c on the Vt side
// (MatrixAlgebraKit's svd_trunc / eigh_trunc! with truncrank on TensorKit's block layout).
// The kept count can be below min(chi, m, n) when the sectors hold fewer values.
struct DecompDT {
    DT U;       // row legs + new leg
    DT Vt;      // new leg + column legs (SVD only)
    Buf s;      // kept values (|eigenvalue| order for eigh), k doubles
    int k = 0;
    TsvdOut info;
};
DecompDT svd_dt(Ctx& c, const DT& M, int nrow, int chi);
DecompDT eigh_dt(Ctx& c, const DT& MM, int nrow, int chi);
// B stacked m x n matrices (stride m*n), decomposed in lockstep: U [B][m x k], s [B][k], Vt [B][k x n]
std::vector<TsvdOut> tsvd_batched(Ctx& c, const double* M, int64_t m, int64_t n, int k, int B, double* U, double* s,
                                  double* Vt);

// ---------------------------------------------------------------------------
// generic pairwise contraction (permute + GEMM + permute)
// ---------------------------------------------------------------------------
// labels are small ints; out_labels gives the output leg order
// batch > 1: A, B and the result carry `batch` instances (an implicit trailing leg); the
// dims / labels name the per-instance legs and the result's dims end with `batch`
DT contract(Ctx& c, const double* A, const std::vector<int64_t>& dA, const std::vector<int>& lA,
            const double* B, const std::vector<int64_t>& dB, const std::vector<int>& lB,
            const std::vector<int>& lOut, bool bulk = true, int batch = 1);
// A pairwise contraction of two charged tensors (the same Z_N), one GEMM per charge sector:
// the rows (free legs of A) of class c meet the contracted index combinations of class -c and
// the columns (free legs of B) of class -c.  Each sector block is gathered from the dense
// embedding, multiplied (tensor cores in split precision) and scattered into the zeroed
// result, which carries the free legs' charges.  The work is sum_c m_c k_c n_c instead of
// m k n: about N^2 times less for balanced sectors.
DT contract_blocked(Ctx& c, const DT& A, const std::vector<int>& lA, const DT& B, const std::vector<int>& lB,
                    const std::vector<int>& lOut, bool bulk);
inline DT contract(Ctx& c, const DT& A, const std::vector<int>& lA, const DT& B,
                   const std::vector<int>& lB, const std::vector<int>& lOut, bool bulk = true) {
    if (A.charged() && B.charged()) return contract_blocked(c, A, lA, B, lB, lOut, bulk);
    return contract(c, A.p(), A.dims(), lA, B.p(), B.dims(), lB, lOut, bulk);
}
DT permuted(Ctx& c, const DT& A, const std::vector<int>& perm);
// the same, every entry divided by |*scale| (a device scalar) on the way
DT permuted_scaled(Ctx& c, const DT& A, const std::vector<int>& perm, const double* scale);

}  // namespace tnr
