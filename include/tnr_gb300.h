/*
 * tnr_gb300.h -- C ABI of the GB300 (sm_103a) coarse-graining engine.
 *
 * Drop-in boundary for the hot path of TNRKit.jl v0.5.1: the scheme structs
 * TRG / BTRG / HOTRG / HOTRG_3D, step!(scheme, truncrank(chi)),
 * finalize!(scheme), run!(scheme, truncrank(chi), maxiter(n)) and
 * free_energy(data, beta).  A Julia `ccall` layer (or Python ctypes) holds an
 * opaque handle in place of the scheme's tensors; the tensors stay resident in
 * GPU memory between calls.  Plain pointers and sizes only.
 *
 * Tensor layout: column-major, first leg fastest, exactly TensorKit's dense
 * storage of a TensorMap V1 (x) V2 <- V3 (x) V4 (the array T[i1,i2,i3,i4]).
 * Leg order: 2D = (left, down, up, right); 3D = (D, U', N, E, S', W').
 *
 * Status codes: every function returns TNR_OK (0) or a TNR_ERR_* code and
 * never aborts the process; tnr_last_error() gives the message.
 * Threading: a handle is single-owner and bound to one CUDA stream; calls on
 * different handles may come from different threads.
 */
#ifndef TNR_GB300_H
#define TNR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define TNR_OK                 0
#define TNR_ERR_INVALID_ARG    1  /* bad argument (reference: ArgumentError / SpaceMismatch) */
#define TNR_ERR_OOM            2  /* device allocation failed                                */
#define TNR_ERR_NOT_CONVERGED  3  /* an iterative solver hit its iteration cap               */
#define TNR_ERR_CUDA           4  /* CUDA runtime error                                      */
#define TNR_ERR_ADMISSION      5  /* request refused: HBM footprint above the admission cap  */
#define TNR_ERR_NONFINITE      6  /* NaN/Inf in inputs or produced by a step                 */
#define TNR_ERR_UNSUPPORTED    7  /* configuration not supported by this build               */
#define TNR_ERR_NO_DEVICE      8  /* no usable sm_103 GPU                                    */

/* ---- scheme kinds (reference: src/schemes/{trg,btrg,hotrg,hotrg3d}.jl) --- */
#define TNR_TRG       1   /* trg.jl:26-41     */
#define TNR_BTRG      2   /* btrg.jl:26-94   */
#define TNR_HOTRG     3   /* hotrg.jl:27-160   */
#define TNR_HOTRG_3D  4   /* hotrg3d.jl:27-135 */
#define TNR_IMPURITY_HOTRG 5 /* impurityhotrg.jl:26-84; created by tnr_create_impurity_hotrg */
#define TNR_IMPURITY_TRG   6 /* impuritytrg.jl:38-91; created by tnr_create_impurity_trg */
#define TNR_CORRELATION_HOTRG 7 /* correlationhotrg.jl:29-250; created by tnr_create_correlation_hotrg */
#define TNR_ATRG           8 /* atrg.jl:26-81; tnr_create with a 4-leg tensor */
#define TNR_ATRG_3D        9 /* atrg3d.jl:26-90; tnr_create with a 6-leg tensor */

/* ---- arithmetic of the bulk contractions -------------------------------- */
#define TNR_PREC_F64    0  /* plain path: every operation in FP64                      */
#define TNR_PREC_SPLIT  1  /* contractions as 3xBF16 tcgen05 products, FP32 accumulate;
                              FP64 small Jacobi, re-orthonormalisation and log-norms  */

typedef struct tnr_handle_s* tnr_handle;

typedef struct tnr_options {
    int    precision;      /* TNR_PREC_F64 or TNR_PREC_SPLIT                          */
    double btrg_k;         /* BTRG bond-weight exponent k (btrg.jl:48 default -0.5)   */
    int    symmetry_n;     /* 1 = Trivial, N = Z_N charges given in leg_charges         */
    const int32_t* leg_charges; /* sum(dims) ints: charge of each basis index per leg,
                                   or NULL.  Used to validate charge conservation.     */
    uint64_t seed;         /* seed of the randomized range finder (0 = default)        */
    void*  stream;         /* cudaStream_t to run on, or NULL for a private stream      */
} tnr_options;

/* Fill *opts with defaults (FP64, k=-0.5, Trivial, private stream). */
void tnr_default_options(tnr_options* opts);

/* Create a scheme from a host tensor.
 *   kind  : TNR_TRG | TNR_BTRG | TNR_HOTRG (nlegs = 4) or TNR_HOTRG_3D (nlegs = 6)
 *   dims  : leg dimensions; data: prod(dims) doubles, column-major.
 * Replaces the constructors TRG(T) (trg.jl:30), BTRG(T, k) (btrg.jl:39-48),
 * HOTRG(T) (hotrg.jl:31), HOTRG_3D(T) (hotrg3d.jl:31). */
int tnr_create(tnr_handle* out, int kind, int nlegs, const int64_t* dims,
               const double* data, const tnr_options* opts);

/* Same, from a device pointer (column-major FP64) already in GPU memory. */
int tnr_create_device(tnr_handle* out, int kind, int nlegs, const int64_t* dims,
                      const double* device_data, const tnr_options* opts);

/* ImpurityHOTRG(T, T_imp_order1_1, T_imp_order1_2, T_imp_order2)
 * (impurityhotrg.jl:26-46): four host tensors of the same dims (4 legs, column-major).
 * tnr_step steps all four (impurityhotrg.jl:48-84); tnr_finalize returns the pure norm and
 * tnr_finalize_impurity the four norms of finalize!(::ImpurityHOTRG) (finalize.jl:91-101). */
int tnr_create_impurity_hotrg(tnr_handle* out, const int64_t* dims, const double* T,
                              const double* T_imp_order1_1, const double* T_imp_order1_2,
                              const double* T_imp_order2, const tnr_options* opts);
/* ImpurityTRG(T, T_imp1, T_imp2, T_imp3, T_imp4) (impuritytrg.jl:38-61): five host tensors
 * of the same dims; tnr_step steps all five (impuritytrg.jl:63-91). */
int tnr_create_impurity_trg(tnr_handle* out, const int64_t* dims, const double* T, const double* T_imp1,
                            const double* T_imp2, const double* T_imp3, const double* T_imp4,
                            const tnr_options* opts);
/* CorrelationHOTRG(Tpure, Timp1, Timp2, dist) (correlationhotrg.jl:51-68): two first-order
 * impurities 2^dist sites apart, merged into one at step dist (dist >= 0).  tnr_step runs
 * step! with its phase finalizer (correlationhotrg.jl:94-135); tnr_finalize and tnr_run do not
 * apply to it. */
int tnr_create_correlation_hotrg(tnr_handle* out, const int64_t* dims, const double* Tpure, const double* Timp1,
                                 const double* Timp2, int dist, const tnr_options* opts);
/* run!(::CorrelationHOTRG) (correlationhotrg.jl:138-162): maxiter steps (maxiter > dist), three
 * norms per step into norms_out (cap doubles): (n, n_1, n_2) before the merge, (n, n_imp, n_imp)
 * from it on (finalize.jl:104-124); *n_out = steps written. */
int tnr_run_correlation(tnr_handle h, int chi, int maxiter, double* norms_out, size_t cap, size_t* n_out);
/* |tr Timp_final| / |tr Tpure| of a CorrelationHOTRG handle after the merge: the correlation
 * the reference's tests read (test/schemes.jl:506,517,530). */
int tnr_correlation_ratio(tnr_handle h, double* out);
/* Finalizers (src/utility/finalize.jl): TNR_FINALIZER_DEFAULT is finalize! (the trace norm),
 * TNR_FINALIZER_TWO_BY_TWO is two_by_two_Finalizer (finalize.jl:17-41,151: the 2 x 2 plaquette
 * norm n, T /= n^(1/4), entry n^(1/4); TRG, BTRG and HOTRG).  tnr_set_finalizer selects the one
 * tnr_finalize and tnr_run use, as run!(scheme, trunc, crit, finalizer) does. */
#define TNR_FINALIZER_DEFAULT    0
#define TNR_FINALIZER_TWO_BY_TWO 1
int tnr_set_finalizer(tnr_handle h, int finalizer);
/* eig_full of the column transfer matrix M[b, c] = sum_a T_unit[a, b, c, a] of a 2D scheme
 * (TRG, BTRG with its bond weights, HOTRG; cft.jl:5-73, 278-340): the eigenvalues, re + i im, in
 * no particular order (the caller sorts and filters as cft_data / ground_state_degeneracy do).
 * unitcell 1..4 copies of T_unit on the ring (cft.jl:7-15); M above 256 x 256 is refused. */
int tnr_transfer_eigvals(tnr_handle h, int unitcell, double* re, double* im, size_t cap, size_t* n_out);
/* gu_wen_ratio (cft.jl:374-396): X1 = |T[1 2;2 1]|^2 / |T[1 2;2 3] T[3 4;4 1]|,
 * X2 = |T[1 2;2 1]|^2 / |T[1 2;3 4] T[4 3;2 1]| of T_unit. */
int tnr_gu_wen_ratio(tnr_handle h, double* x1, double* x2);
/* central_charge(scheme, n) (cft.jl:256-269): log(sigma_1) 6 / pi of M[-1;-2] = T[1 -1;-2 1] / n. */
int tnr_central_charge(tnr_handle h, double n, double* c_out);
/* finalize! of an impurity scheme: ImpurityHOTRG writes 4 norms (pure, +1, -1, second order;
 * finalize.jl:91-101), ImpurityTRG 2 (pure, plaquette of the four impurities; finalize.jl:75-88). */
int tnr_finalize_impurity(tnr_handle h, double* norms_out);
/* run! with ImpurityHOTRG_Finalizer / ImpurityTRG_Finalizer (tnrscheme.jl:27-28): 4 or 2 norms
 * per entry into norms_out (cap doubles); *n_out = entries written. */
int tnr_run_impurity(tnr_handle h, int chi, int maxiter, int finalize_beginning,
                     double* norms_out, size_t cap, size_t* n_out);

/* One coarse-graining step with truncrank(chi).
 * Replaces step!(scheme, trunc) (tnrscheme.jl:2; trg.jl:35, btrg.jl:60,
 * hotrg.jl:154, hotrg3d.jl:127). */
int tnr_step(tnr_handle h, int chi);

/* Trace-normalise the tensor and return the norm (synchronises).
 * Replaces finalize!(scheme) (finalize.jl:4-14,62-66). */
int tnr_finalize(tnr_handle h, double* norm_out);

/* run!(scheme, truncrank(chi), maxiter(maxiter); finalize_beginning)
 * (tnrscheme.jl:33-59 with the default Finalizer).  Writes maxiter (+1 when
 * finalize_beginning) norms into norms_out; *n_out = count written. */
int tnr_run(tnr_handle h, int chi, int maxiter, int finalize_beginning,
            double* norms_out, size_t cap, size_t* n_out);

/* free_energy(data, beta; scalefactor, initial_size) (free_energy.jl:13-20). */
double tnr_free_energy(const double* norms, size_t n, double beta,
                       double scalefactor, double initial_size);

/* Copy the current tensor to host (column-major); dims_out gets nlegs entries. */
int tnr_get_tensor(tnr_handle h, double* host_out, size_t cap, int64_t* dims_out, int* nlegs_out);
/* The impurity tensors of an impurity scheme, as tnr_get_tensor copies T: ImpurityHOTRG which =
 * 0, 1, 2 -> T_imp_order1_1, T_imp_order1_2, T_imp_order2 (impurityhotrg.jl:26-46); ImpurityTRG
 * 0..3 -> T_imp1..T_imp4 (impuritytrg.jl:38-61); CorrelationHOTRG 0, 1, 2 -> Timp1, Timp2 (before
 * the merge), Timp_final (from it on; correlationhotrg.jl:29-71). */
int tnr_get_impurity_tensor(tnr_handle h, int which, double* host_out, size_t cap, int64_t* dims_out, int* nlegs_out);

/* Kept singular values (TRG/BTRG) or kept eigenvalues of the chosen Gram
 * matrices (HOTRG/HOTRG_3D) of the most recent step, concatenated in the order
 * the reference computes them; counts[i] = length of decomposition i. */
int tnr_singular_values(tnr_handle h, double* out, size_t cap, size_t* n_out,
                        int32_t* counts, size_t counts_cap, size_t* ndec_out);

/* Truncation errors (eps, eps') of the projector choices of the last step
 * (HOTRG: hotrg.jl:112,148; HOTRG_3D: hotrg3d.jl:97). */
int tnr_truncation_errors(tnr_handle h, double* out, size_t cap, size_t* n_out);

/* BTRG bond tensors S1 / S2 (diagonals) of the current state. */
int tnr_btrg_bonds(tnr_handle h, double* s1, size_t cap1, size_t* n1,
                   double* s2, size_t cap2, size_t* n2);

/* Bytes of device memory the scheme holds now (tensor + workspace). */
int tnr_device_bytes(tnr_handle h, size_t* bytes_out);

/* Statistics of the truncated decompositions run on this handle since it was created:
 * how many, how many of them the spectral-gap fallback decomposed in full FP64 (the
 * subspace iteration could not resolve the gap at chi), and the most subspace iterations
 * one of them took.  Any pointer may be NULL.  No reference counterpart (diagnostic). */
int tnr_decomposition_stats(tnr_handle h, uint64_t* decompositions, uint64_t* gap_fallbacks, int* max_iters);

int  tnr_destroy(tnr_handle h);
int  tnr_last_error(tnr_handle h, char* buf, size_t cap); /* h may be NULL: global */
const char* tnr_status_string(int status);

/* Device-time measurement on the handle's stream (CUDA events).  No reference counterpart
 * (the reference times run!() with @elapsed on the host, tnrscheme.jl:46). */
int tnr_timer_start(tnr_handle h);
int tnr_timer_stop(tnr_handle h, double* ms_out);

/* ---- batched runs: many independent (model, beta, chi) instances --------- */
/* Runs run!() on n handles.  Fresh TRG/BTRG handles with equal kind, precision,
 * k, initial legs, chi and maxiter form lockstep groups (one batched GEMM per
 * contraction, one CTA per member in the small solvers); groups and the other
 * handles run concurrently, one CUDA stream each, from up to 32 host workers
 * (environment variable TNR_BATCH_WORKERS, 1..32).  norms_out is n*stride doubles; n_out[i] = norms written for
 * instance i.  device_ms_out (nullable) = device time from the first launch of
 * the batch to the last completion (CUDA events); latency_ms_out (nullable, n
 * entries) = host wall time from batch start to completion of instance i.
 * No reference counterpart: the reference runs one run!() at a time
 * (tnrscheme.jl:33); this is the batched form of that call. */
int tnr_run_batch(tnr_handle* hs, int n, const int* chi, const int* maxiter,
                  int finalize_beginning, double* norms_out, size_t stride,
                  size_t* n_out, double* device_ms_out, double* latency_ms_out);

/* ---- serving loop: run!() requests admitted by HBM footprint ------------- */
/* No reference counterpart (the reference runs one run!() per call,
 * tnrscheme.jl:33).  A server owns max_active host workers; a request is admitted
 * when a worker is free and its estimated footprint (tnr_footprint_bytes: chi^4
 * tensors for TRG/BTRG, two chi^5 intermediates for HOTRG, chi^6 tensors plus a
 * sliced chi^8 intermediate for HOTRG_3D) fits the unused part of the budget.
 * Admitted requests keep their tensor resident and iterate concurrently, one
 * CUDA stream each; requests that arrive meanwhile wait in FIFO order and are
 * admitted as slots and memory free up.  A request that can never fit is refused
 * at submission with TNR_ERR_ADMISSION. */
typedef struct tnr_server_s* tnr_server;
int tnr_server_create(tnr_server* out, size_t hbm_budget_bytes, int max_active, int precision);
int tnr_server_submit(tnr_server s, int kind, int nlegs, const int64_t* dims, const double* data,
                      int chi, int maxiter, double btrg_k, uint64_t* id_out);
/* The same for a Z_N-symmetric tensor (TRG, BTRG, HOTRG): symmetry_n and leg_charges as in
 * tnr_options (sum(dims) ints, codomain legs 1-2 +charge, domain legs -charge).  The request
 * then runs block by block over the charge sectors (contractions as one GEMM per sector,
 * decompositions per sector with the global truncrank cut), as TensorKit's block-sparse
 * tensors do in the reference's run!(). */
int tnr_server_submit_sym(tnr_server s, int kind, int nlegs, const int64_t* dims, const double* data,
                          int symmetry_n, const int32_t* leg_charges, int chi, int maxiter, double btrg_k,
                          uint64_t* id_out);
/* wait != 0 blocks until request `id` finishes.  Returns the request's status;
 * latency_ms = submission to completion, queue_ms = submission to admission. */
int tnr_server_poll(tnr_server s, uint64_t id, int wait, int* done, double* norms, size_t cap,
                    size_t* n_out, double* latency_ms, double* queue_ms);
int tnr_server_stats(tnr_server s, int* active, int* queued, size_t* bytes_in_use);
int tnr_server_destroy(tnr_server s);
/* Device bytes a run!() of this kind, chi and initial legs needs (the admission estimate). */
size_t tnr_footprint_bytes(int kind, int chi, int nlegs, const int64_t* dims);

/* ---- profiling: CUDA events around every launch of a kernel class -------- */
/* No reference counterpart: per-class launch counts, device time and algorithmic work
 * for the roofline of the benchmark. */
#define TNR_PROF_GEMM_BULK 0  /* bulk contraction / projection GEMMs run in FP64; work = flops */
#define TNR_PROF_GEMM_F64  1  /* FP64 GEMMs inside the decompositions; work = flops */
#define TNR_PROF_JACOBI    2  /* Jacobi eigensolver; work = r^3                     */
#define TNR_PROF_CHOL      3  /* FP64 Cholesky + inverse; work = r^3                */
#define TNR_PROF_PERMUTE   4  /* leg permutes; work = bytes read + written          */
#define TNR_PROF_SPLIT     5  /* FP64 -> 3xBF16 operand split; work = bytes         */
#define TNR_PROF_JACOBI32  6  /* FP32 Jacobi (basis alignment); work = r^3          */
#define TNR_PROF_TC        7  /* split 3xBF16 tcgen05 GEMMs; work = 2 m n k flops   */
#define TNR_PROF_CHOL32    8  /* FP32 Cholesky + inverse (split CholeskyQR); r^3    */
int tnr_profile_enable(int on);
int tnr_profile_reset(void);
int tnr_profile_read(int cls, uint64_t* launches, double* total_ms, double* work);

/* ---- diagnostics: one bulk GEMM through the engine's kernels ------------- */
/* C (m x n) = op(A) op(B) for `batch` strided problems, host buffers,
 * column-major.  precision TNR_PREC_SPLIT runs the tcgen05 3xBF16 kernel as the
 * contractions of a coarse-graining step do (K accumulated in chunks of 64 on
 * fresh FP32 accumulators, chunks summed with round-to-nearest) and returns TNR_ERR_UNSUPPORTED
 * when that kernel declines the shape; TNR_PREC_F64 runs the FP64 kernel.  No reference counterpart (parity test of the
 * contraction kernels). */
int tnr_debug_gemm(int precision, int ta, int tb, int64_t m, int64_t n, int64_t k,
                   const double* A, int64_t lda, int64_t strideA,
                   const double* B, int64_t ldb, int64_t strideB,
                   double* C, int64_t ldc, int64_t strideC, int batch);

/* Inverse Cholesky factors through the engine's one-CTA kernel: for each of `batch`
 * symmetric r x r matrices G (column-major, host, lower triangle read), Linv =
 * L^-1 with (G + shift I) = L L^T, lower triangular, zero above.  precision
 * TNR_PREC_SPLIT runs the FP32 kernel of the split path's orthonormalisation,
 * TNR_PREC_F64 the FP64 one; *breakdown = 1 when a pivot was not positive.
 * No reference counterpart (parity test of the CholeskyQR kernels). */
int tnr_debug_chol(int precision, int r, double shift, int batch, const double* G, double* Linv, int* breakdown);

/* Device time of one batched GEMM of that shape on seeded N(0,1) device operands
 * (contiguous column-major, strides m*k, k*n, m*n): *ms_out = the CUDA-event time
 * of `reps` back-to-back calls / reps, after one untimed call.  For the split
 * precision the time includes the FP64 -> BF16 plane pass; contraction = 1 times
 * the contraction path (K accumulated in chunks), 0 the single-accumulation kernel
 * of the truncated SVD's products.  No reference counterpart (kernel measurements). */
int tnr_gemm_time(int precision, int ta, int tb, int64_t m, int64_t n, int64_t k, int batch, int reps,
                  int contraction, double* ms_out);

/* ---- allocation-free split GEMM ------------------------------------------ */
/* No counterpart in the reference.  C = alpha * op(A) op(B) + beta * C on device
 * pointers (column-major FP64), computed by the split 3xBF16 tensor-core kernel
 * without allocating: its BF16 plane scratch is a 16 MiB file-scope device array
 * that every GPU loading the library holds until exit.  For callers that cannot
 * call cudaMalloc (code running inside another allocator's arena, such as a
 * CUDA.jl pool or a server that reserves all free HBM, and latency-critical paths
 * where cudaMalloc's implicit device synchronisation stalls other streams).
 *   - limits: m >= 64, n >= 16, k >= 16 and 6 * (m + n) * ceil8(k) bytes <= 16 MiB;
 *     larger operands are rejected with TNR_ERR_INVALID_ARG and a message in err;
 *   - the first call on a device resolves the scratch's device address and sets the
 *     kernel's shared-memory limit with that device current;
 *   - every call shares the one scratch array: calls that overlap on the GPU
 *     (different streams, different host threads) race; serialise them;
 *   - runs on `stream` (NULL = legacy default stream) and returns after
 *     synchronising it; calls no cudaMalloc, cudaFree or allocating routine. */
int tnr_gemm_split_noalloc(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                           const double* A, int64_t lda, const double* B, int64_t ldb,
                           double beta, double* C, int64_t ldc, void* stream,
                           char* err, size_t err_cap);

/* ---- library info (no reference counterpart) ----------------------------- */
int tnr_device_info(int* sm_count, int* cc_major, int* cc_minor, size_t* hbm_bytes);
const char* tnr_version(void);

/* Kernel-launch counter of this process (every kernel the library launched). */
uint64_t tnr_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif /* TNR_GB300_H */
