// Core runtime: caching allocator, execution context, leg permutes, elementwise
// kernels, trace norms and the seeded Gaussian sketch.
#include "common.cuh"

#include <algorithm>
#include <cmath>
#include <mutex>

namespace tnr {

std::atomic<uint64_t> g_launches{0};
std::atomic<bool> g_prof_on{false};

namespace {
struct ProfRec {
    cudaEvent_t a = nullptr, b = nullptr;
    int cls = -1;
    double work = 0;
};
std::mutex g_prof_mu;
std::vector<ProfRec> g_prof;
std::vector<cudaEvent_t> g_ev_free;

cudaEvent_t ev_get() {
    if (!g_ev_free.empty()) {
        cudaEvent_t e = g_ev_free.back();
        g_ev_free.pop_back();
        return e;
    }
    cudaEvent_t e;
    TNR_CUDA(cudaEventCreate(&e));
    return e;
}
}  // namespace

int prof_start(cudaStream_t s) {
    if (!g_prof_on.load(std::memory_order_relaxed)) return -1;
    std::lock_guard<std::mutex> g(g_prof_mu);
    ProfRec r;
    r.a = ev_get();
    r.b = ev_get();
    TNR_CUDA(cudaEventRecord(r.a, s));
    g_prof.push_back(r);
    return (int)g_prof.size() - 1;
}

void prof_stop(int rec, cudaStream_t s, int cls, double work) {
    if (rec < 0) return;
    std::lock_guard<std::mutex> g(g_prof_mu);
    if (rec >= (int)g_prof.size()) return;
    ProfRec& r = g_prof[rec];
    r.cls = cls;
    r.work = work;
    TNR_CUDA(cudaEventRecord(r.b, s));
}

void prof_reset() {
    std::lock_guard<std::mutex> g(g_prof_mu);
    for (auto& r : g_prof) {
        cudaEventSynchronize(r.b);
        g_ev_free.push_back(r.a);
        g_ev_free.push_back(r.b);
    }
    g_prof.clear();
}

void prof_read(int cls, uint64_t* launches, double* ms, double* work) {
    std::lock_guard<std::mutex> g(g_prof_mu);
    uint64_t n = 0;
    double t = 0, w = 0;
    for (auto& r : g_prof) {
        if (r.cls != cls) continue;
        TNR_CUDA(cudaEventSynchronize(r.b));
        float x = 0;
        TNR_CUDA(cudaEventElapsedTime(&x, r.a, r.b));
        ++n;
        t += x;
        w += r.work;
    }
    if (launches) *launches = n;
    if (ms) *ms = t;
    if (work) *work = w;
}

int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// ---------------------------------------------------------------------------
// Pool
// ---------------------------------------------------------------------------
static size_t round_block(size_t b) {
    if (b <= (1u << 20)) return (b + 4095) & ~size_t(4095);
    size_t g = size_t(2) << 20;                 // 2 MiB granularity above 1 MiB
    return (b + g - 1) / g * g;
}

// Stream-ordered allocations: cudaMallocAsync / cudaFreeAsync never synchronise the device,
// so many handles on many streams allocate without stalling each other.  The device's
// default pool keeps freed memory cached (release threshold raised once per device).
static void keep_pool_memory() {
    static std::atomic<uint64_t> done{0};
    int dev = 0;
    if (!device_once(done, &dev)) return;
    cudaMemPool_t mp;
    if (cudaDeviceGetDefaultMemPool(&mp, dev) == cudaSuccess) {
        uint64_t thr = ~0ull;
        cudaMemPoolSetAttribute(mp, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    cudaGetLastError();
    device_done(done, dev);
}

Pool::~Pool() {
    for (auto& kv : size_of_) cudaFreeAsync(kv.first, stream_);
}

void* Pool::get(size_t bytes) {
    size_t b = round_block(bytes);
    auto it = free_.lower_bound(b);
    if (it != free_.end() && it->first <= b + b / 4 + (size_t(2) << 20)) {
        void* p = it->second;
        free_.erase(it);
        return p;
    }
    void* p = nullptr;
    keep_pool_memory();
    cudaError_t e = cudaMallocAsync(&p, b, stream_);
    if (e != cudaSuccess) {
        cudaGetLastError();
        trim();                                // give cached blocks back, then retry once
        e = cudaMallocAsync(&p, b, stream_);
        if (e != cudaSuccess) {
            cudaGetLastError();
            throw Error(TNR_ERR_OOM, "device allocation of " + std::to_string(b) + " bytes failed");
        }
    }
    size_of_[p] = b;
    held_ += b;
    return p;
}

void Pool::put(void* p) {
    auto it = size_of_.find(p);
    if (it == size_of_.end()) return;
    free_.emplace(it->second, p);
}

void Pool::trim() {
    cudaStreamSynchronize(stream_);
    for (auto& kv : free_) {
        auto it = size_of_.find(kv.second);
        if (it != size_of_.end()) {
            held_ -= it->second;
            size_of_.erase(it);
        }
        cudaFreeAsync(kv.second, stream_);
    }
    free_.clear();
    cudaStreamSynchronize(stream_);
}

DT make_dt(Pool* pool, const std::vector<int64_t>& dims) {
    DT t;
    t.rank = (int)dims.size();
    TNR_REQUIRE(t.rank <= MAXR, TNR_ERR_UNSUPPORTED, "rank > 8");
    for (int i = 0; i < t.rank; ++i) t.d[i] = dims[i];
    t.buf = Buf(pool, (size_t)std::max<int64_t>(t.size(), 1) * sizeof(double));
    return t;
}

// ---------------------------------------------------------------------------
// Ctx
// ---------------------------------------------------------------------------
Ctx::Ctx(cudaStream_t s, int prec, uint64_t seed_) : precision(prec) {
    if (seed_) seed = seed_;
    if (s) {
        stream = s;
    } else {
        TNR_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        own_stream = true;
    }
    pool.reset(new Pool(stream));
    keep_pool_memory();
    TNR_CUDA(cudaMallocAsync((void**)&d_status, 64, stream));
    TNR_CUDA(cudaMemsetAsync(d_status, 0, 64, stream));
    TNR_CUDA(cudaMallocAsync((void**)&d_scalar, 4096 * sizeof(double), stream));
    TNR_CUDA(cudaEventCreate(&ev0));
    TNR_CUDA(cudaEventCreate(&ev1));
}

Ctx::~Ctx() {
    if (stream) cudaStreamSynchronize(stream);
    pool.reset();
    if (d_status) cudaFreeAsync(d_status, stream);
    if (d_scalar) cudaFreeAsync(d_scalar, stream);
    if (stream) cudaStreamSynchronize(stream);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (own_stream && stream) cudaStreamDestroy(stream);
}

void Ctx::sync() { TNR_CUDA(cudaStreamSynchronize(stream)); }

// Every reader of the status word goes through here, so a tensor-core pipeline timeout
// (whose GEMM wrote zeros) fails the call whichever status bit the caller looks for.
int Ctx::read_status_and_clear() {
    int h = 0;
    TNR_CUDA(cudaMemcpyAsync(&h, d_status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    TNR_CUDA(cudaMemsetAsync(d_status, 0, sizeof(int), stream));
    TNR_CUDA(cudaStreamSynchronize(stream));
    TNR_REQUIRE(!(h & ST_TC_TIMEOUT), TNR_ERR_CUDA, "tensor-core pipeline wait timed out; the results are invalid");
    return h;
}

static inline int grid_for(int64_t n, int threads, int per_sm = 8) {
    int64_t g = (n + threads - 1) / threads;
    int64_t cap = (int64_t)sm_count() * per_sm;
    return (int)std::max<int64_t>(1, std::min(g, cap));
}

// ---------------------------------------------------------------------------
// permute: out[j0..j_{r-1}] = alpha * in[...], out.d[k] = in.d[perm[k]]
// ---------------------------------------------------------------------------
struct PermArgs {
    int rank;
    int64_t in_d[MAXR];
    int64_t in_s[MAXR];
    int64_t out_d[MAXR];
    int64_t out_s_of_in[MAXR];  // output stride of each INPUT axis
    int perm[MAXR];
};

// generic element-wise permute (degenerate axes): every thread writes consecutive output elements
__global__ void k_permute_rows(const double* __restrict__ in, double* __restrict__ out,
                               PermArgs a, int64_t total, const double* scale_ptr) {
    const double alpha = scale_ptr ? 1.0 / fabs(*scale_ptr) : 1.0;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < total;
         j += (int64_t)gridDim.x * blockDim.x) {
        int64_t rem = j, off = 0;
        for (int k = 0; k < a.rank; ++k) {
            int64_t ik = rem % a.out_d[k];
            rem /= a.out_d[k];
            off += ik * a.in_s[a.perm[k]];
        }
        out[j] = scale_ptr ? alpha * in[off] : in[off];
    }
}

// fastest axis kept in place (perm[0] == 0): the tensor is a list of contiguous rows of d0
// elements in both layouts; a warp copies one row, its input offset computed once by lane 0
// (the mixed-radix division chain runs per row, not per element)
__global__ void k_permute_rows0(const double* __restrict__ in, double* __restrict__ out,
                                PermArgs a, int64_t nrows, const double* scale_ptr) {
    const double alpha = scale_ptr ? 1.0 / fabs(*scale_ptr) : 1.0;
    const int64_t d0 = a.in_d[0];
    for (int64_t r = blockIdx.x * (int64_t)blockDim.y + threadIdx.y; r < nrows;
         r += (int64_t)gridDim.x * blockDim.y) {
        long long off = 0;
        if (threadIdx.x == 0) {
            int64_t rem = r;
            for (int k = 1; k < a.rank; ++k) {
                const int64_t ik = rem % a.out_d[k];
                rem /= a.out_d[k];
                off += ik * a.in_s[a.perm[k]];
            }
        }
        off = __shfl_sync(0xffffffffu, off, 0);
        const double* src = in + off;
        double* dst = out + r * d0;
        if (scale_ptr) {
            for (int64_t x = threadIdx.x; x < d0; x += 32) dst[x] = alpha * src[x];
        } else {
            for (int64_t x = threadIdx.x; x < d0; x += 32) dst[x] = src[x];
        }
    }
}

// input-fastest axis (0) and output-fastest axis (input axis B = perm[0]) differ:
// stage 32x32 tiles in shared memory so both the reads and the writes coalesce
__global__ void k_permute_tiled(const double* __restrict__ in, double* __restrict__ out,
                                PermArgs a, int axB, int64_t ntA, int64_t ntB, int64_t nbatch,
                                const double* scale_ptr) {
    __shared__ double tile[32][33];
    double alpha = scale_ptr ? 1.0 / fabs(*scale_ptr) : 1.0;
    const int64_t dA = a.in_d[0], dB = a.in_d[axB];
    const int64_t sB_in = a.in_s[axB];
    const int64_t sA_out = a.out_s_of_in[0];
    const int64_t ntiles = ntA * ntB * nbatch;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int64_t tA = t % ntA;
        int64_t r1 = t / ntA;
        int64_t tB = r1 % ntB;
        int64_t bt = r1 / ntB;
        // batch index over the remaining input axes (increasing order)
        int64_t in_off = 0, out_off = 0, rem = bt;
        for (int ax = 1; ax < a.rank; ++ax) {
            if (ax == axB) continue;
            int64_t i = rem % a.in_d[ax];
            rem /= a.in_d[ax];
            in_off += i * a.in_s[ax];
            out_off += i * a.out_s_of_in[ax];
        }
        const int64_t a0 = tA * 32, b0 = tB * 32;
        __syncthreads();
        for (int y = threadIdx.y; y < 32; y += blockDim.y) {
            int64_t ia = a0 + threadIdx.x, ib = b0 + y;
            if (ia < dA && ib < dB) tile[y][threadIdx.x] = in[in_off + ib * sB_in + ia];
        }
        __syncthreads();
        for (int y = threadIdx.y; y < 32; y += blockDim.y) {
            int64_t ia = a0 + y, ib = b0 + threadIdx.x;
            if (ia < dA && ib < dB)
                out[out_off + ia * sA_out + ib] = scale_ptr ? alpha * tile[threadIdx.x][y] : tile[threadIdx.x][y];
        }
    }
}

void permute(Ctx& c, const double* in, const int64_t* in_dims, int rank, const int* perm,
             double* out, const double* scale_ptr) {
    TNR_REQUIRE(rank >= 1 && rank <= MAXR, TNR_ERR_UNSUPPORTED, "permute rank");
    PermArgs a{};
    a.rank = rank;
    int64_t s = 1;
    for (int i = 0; i < rank; ++i) {
        a.in_d[i] = in_dims[i];
        a.in_s[i] = s;
        s *= in_dims[i];
    }
    const int64_t total = s;
    if (total == 0) return;
    int64_t os = 1;
    for (int k = 0; k < rank; ++k) {
        a.perm[k] = perm[k];
        a.out_d[k] = in_dims[perm[k]];
        a.out_s_of_in[perm[k]] = os;
        os *= a.out_d[k];
    }
    // squeeze: if the permutation is the identity, copy
    bool ident = true;
    for (int k = 0; k < rank; ++k) ident &= (perm[k] == k);
    if (ident && !scale_ptr) {
        TNR_CUDA(cudaMemcpyAsync(out, in, total * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
        return;
    }
    int axB = perm[0];
    int rec = prof_start(c.stream);
    if (axB == 0) {
        const int64_t nrows = total / in_dims[0];
        const int g = (int)std::min<int64_t>((nrows + 7) / 8, (int64_t)sm_count() * 16);
        k_permute_rows0<<<g, dim3(32, 8), 0, c.stream>>>(in, out, a, nrows, scale_ptr);
        check_launch("permute_rows0");
        prof_stop(rec, c.stream, PROF_PERMUTE, 16.0 * total);
        return;
    }
    if (in_dims[0] == 1 || in_dims[axB] == 1) {
        k_permute_rows<<<grid_for(total, 256), 256, 0, c.stream>>>(in, out, a, total, scale_ptr);
        check_launch("permute_rows");
        prof_stop(rec, c.stream, PROF_PERMUTE, 16.0 * total);
        return;
    }
    int64_t ntA = (in_dims[0] + 31) / 32, ntB = (in_dims[axB] + 31) / 32;
    int64_t nb = total / (in_dims[0] * in_dims[axB]);
    int64_t ntiles = ntA * ntB * nb;
    int g = (int)std::min<int64_t>(ntiles, (int64_t)sm_count() * 16);
    k_permute_tiled<<<g, dim3(32, 8), 0, c.stream>>>(in, out, a, axB, ntA, ntB, nb, scale_ptr);
    check_launch("permute_tiled");
    prof_stop(rec, c.stream, PROF_PERMUTE, 16.0 * total);
}

DT permuted_scaled(Ctx& c, const DT& A, const std::vector<int>& perm, const double* scale) {
    std::vector<int64_t> od(A.rank);
    for (int k = 0; k < A.rank; ++k) od[k] = A.d[perm[k]];
    DT o = make_dt(c.pool.get(), od);
    permute(c, A.p(), A.d, A.rank, perm.data(), o.p(), scale);
    if (A.charged()) {
        o.N = A.N;
        for (int k = 0; k < A.rank; ++k) o.q.push_back(A.q[perm[k]]);
    }
    return o;
}

DT permuted(Ctx& c, const DT& A, const std::vector<int>& perm) {
    std::vector<int64_t> od(A.rank);
    for (int k = 0; k < A.rank; ++k) od[k] = A.d[perm[k]];
    DT o = make_dt(c.pool.get(), od);
    permute(c, A.p(), A.d, A.rank, perm.data(), o.p());
    if (A.charged()) {
        o.N = A.N;
        for (int k = 0; k < A.rank; ++k) o.q.push_back(A.q[perm[k]]);
    }
    return o;
}

// ---------------------------------------------------------------------------
// elementwise helpers
// ---------------------------------------------------------------------------
// mode 0: X[:,j] *= s[j]; mode 1: *= sqrt(s[j]); mode 2: /= s[j] (0 -> 0); mode 3: *= 1/sqrt(s[j]) (0 -> 0)
__device__ __forceinline__ double scale_of(double v, int mode) {
    switch (mode) {
        case 0: return v;
        case 1: return sqrt(fmax(v, 0.0));
        case 2: return v != 0.0 ? 1.0 / v : 0.0;
        default: return v > 0.0 ? rsqrt(v) : 0.0;
    }
}

__global__ void k_col_scale(double* X, int64_t m, int64_t n, int64_t ldx, const double* s, int mode) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m * n;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = e % m, j = e / m;
        X[i + j * ldx] *= scale_of(s[j], mode);
    }
}
void col_scale(Ctx& c, double* X, int64_t m, int64_t n, int64_t ldx, const double* s, int mode) {
    if (m * n == 0) return;
    k_col_scale<<<grid_for(m * n, 256), 256, 0, c.stream>>>(X, m, n, ldx, s, mode);
    check_launch("col_scale");
}

__global__ void k_row_scale(double* X, int64_t m, int64_t n, int64_t ldx, const double* s, int mode) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m * n;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = e % m, j = e / m;
        X[i + j * ldx] *= scale_of(s[i], mode);
    }
}
void row_scale(Ctx& c, double* X, int64_t m, int64_t n, int64_t ldx, const double* s, int mode) {
    if (m * n == 0) return;
    k_row_scale<<<grid_for(m * n, 256), 256, 0, c.stream>>>(X, m, n, ldx, s, mode);
    check_launch("row_scale");
}

// column 2-norms, one warp per column
__global__ void k_col_norms(const double* X, int64_t m, int64_t n, int64_t ldx, double* out) {
    int64_t col = blockIdx.x * (int64_t)(blockDim.x / 32) + threadIdx.x / 32;
    int lane = threadIdx.x & 31;
    if (col >= n) return;
    double acc = 0.0;
    for (int64_t i = lane; i < m; i += 32) {
        double v = X[i + col * ldx];
        acc = fma(v, v, acc);
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) out[col] = sqrt(acc);
}
void col_norms(Ctx& c, const double* X, int64_t m, int64_t n, int64_t ldx, double* out) {
    if (n == 0) return;
    int wpb = 8;
    k_col_norms<<<(int)((n + wpb - 1) / wpb), 32 * wpb, 0, c.stream>>>(X, m, n, ldx, out);
    check_launch("col_norms");
}

// G <- D^{-1} G D^{-1} with D = sqrt(diag(G)); dscale <- 1/sqrt(diag) (0 for a zero column)
__global__ void k_gram_unit_diag(double* G, int r, double* dscale) {
    __shared__ double inv[256];
    G += (int64_t)blockIdx.x * r * r;     // one CTA per matrix of a batch
    dscale += (int64_t)blockIdx.x * r;
    for (int i = threadIdx.x; i < r; i += blockDim.x) {
        double v = G[i + (int64_t)i * r];
        inv[i] = v > 0.0 ? rsqrt(v) : 0.0;
        dscale[i] = inv[i];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < r * r; e += blockDim.x) {
        int i = e % r, j = e / r;
        double v = G[e] * inv[i] * inv[j];
        if (i == j) v = inv[i] > 0.0 ? 1.0 : 0.0;
        G[e] = v;
    }
}
void gram_unit_diag(Ctx& c, double* G, int r, double* dscale, int batch) {
    TNR_REQUIRE(r <= 256, TNR_ERR_UNSUPPORTED, "gram_unit_diag r > 256");
    k_gram_unit_diag<<<batch, 256, 0, c.stream>>>(G, r, dscale);
    check_launch("gram_unit_diag");
}

// sum of squares: deterministic two-level reduction into out[0]
__global__ void k_sumsq_partial(const double* x, int64_t n, double* part) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc = fma(x[i], x[i], acc);
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) part[blockIdx.x] = acc;
    }
}
__global__ void k_sum_final(const double* part, int n, double* out) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += part[i];
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) out[0] = acc;
    }
}
void sum_squares(Ctx& c, const double* x, int64_t n, double* out) {
    int g = grid_for(n, 256, 4);
    g = std::min(g, 1024);
    Buf part(c.pool.get(), g * sizeof(double));
    k_sumsq_partial<<<g, 256, 0, c.stream>>>(x, n, part.d());
    check_launch("sumsq_partial");
    k_sum_final<<<1, 1024, 0, c.stream>>>(part.d(), g, out);
    check_launch("sum_final");
}

__global__ void k_scale(double* x, int64_t n, const double* sp) {
    double a = 1.0 / fabs(*sp);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] *= a;
}
void scale_inplace(Ctx& c, double* x, int64_t n, const double* inv_scale_ptr) {
    if (!n) return;
    k_scale<<<grid_for(n, 256), 256, 0, c.stream>>>(x, n, inv_scale_ptr);
    check_launch("scale");
}


// X += alpha * I (r x r)
__global__ void k_add_identity(double* X, int r, double alpha) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    X += (int64_t)blockIdx.y * r * r;
    if (i < r) X[i + (int64_t)i * r] += alpha;
}
void add_identity(Ctx& c, double* X, int r, double alpha, int batch) {
    k_add_identity<<<dim3((r + 127) / 128, batch), 128, 0, c.stream>>>(X, r, alpha);
    check_launch("add_identity");
}

// C = I - E/2 + 3/8 E^2 (C may alias E)
__global__ void k_polar_coeff(const double* E, const double* E2, double* C, int r, int64_t total) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = e % r, j = (e / r) % r;
        C[e] = (i == j ? 1.0 : 0.0) - 0.5 * E[e] + 0.375 * E2[e];
    }
}
void polar_coeff(Ctx& c, const double* E, const double* E2, double* C, int r, int batch) {
    const int64_t total = (int64_t)r * r * batch;
    k_polar_coeff<<<grid_for(total, 256), 256, 0, c.stream>>>(E, E2, C, r, total);
    check_launch("polar_coeff");
}

__global__ void k_abs_copy(double* dst, const double* src) { dst[0] = fabs(src[0]); }
void abs_copy(Ctx& c, double* dst, const double* src) {
    k_abs_copy<<<1, 1, 0, c.stream>>>(dst, src);
    check_launch("abs_copy");
}

__global__ void k_lincomb2(double* out, int64_t n, double a, const double* x, double b, const double* y) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        out[e] = a * x[e] + b * y[e];
}
void lincomb2(Ctx& c, double* out, int64_t n, double a, const double* x, double b, const double* y) {
    if (!n) return;
    k_lincomb2<<<grid_for(n, 256), 256, 0, c.stream>>>(out, n, a, x, b, y);
    check_launch("lincomb2");
}

__global__ void k_row_scale_batched(double* X, int64_t k, int64_t n_total, const double* s, int mode, int64_t n_per) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < k * n_total;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = e % k, j = e / k;
        X[e] *= scale_of(s[(j / n_per) * k + i], mode);
    }
}
void row_scale_batched(Ctx& c, double* X, int64_t k, int64_t n_total, const double* s, int mode, int64_t n_per) {
    if (k * n_total == 0) return;
    k_row_scale_batched<<<grid_for(k * n_total, 256), 256, 0, c.stream>>>(X, k, n_total, s, mode, n_per);
    check_launch("row_scale_batched");
}

__global__ void k_scale_leg_batched(double* T, int64_t per, int64_t total, int64_t stride, int64_t dim,
                                    const double* v) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
        T[e] *= v[(e / per) * dim + ((e % per) / stride) % dim];
}
void scale_leg_batched(Ctx& c, double* T, int64_t per, int batch, int64_t stride, int64_t dim, const double* v) {
    const int64_t total = per * batch;
    if (!total) return;
    k_scale_leg_batched<<<grid_for(total, 256), 256, 0, c.stream>>>(T, per, total, stride, dim, v);
    check_launch("scale_leg_batched");
}

__global__ void k_transpose_lead(const double* in, int64_t n, int64_t p, int k, int64_t total, double* out) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        // out[b][i + k * j] = in[b][j + n * i],  i < k, j < n
        int64_t b = e / (k * n), rem = e % (k * n);
        int64_t i = rem % k, j = rem / k;
        out[e] = in[b * n * p + j + n * i];
    }
}
void transpose_lead(Ctx& c, const double* in, int64_t n, int64_t p, int k, int batch, double* out) {
    const int64_t total = (int64_t)k * n * batch;
    if (!total) return;
    k_transpose_lead<<<grid_for(total, 256), 256, 0, c.stream>>>(in, n, p, k, total, out);
    check_launch("transpose_lead");
}

// |sum_{a,b} T_b[a,b,b,a] w1[b] w2[a]| per instance (one CTA per instance)
__global__ void k_trace2d_batched(const double* T, int64_t d1, int64_t d2, int64_t d3, int64_t per,
                                  const double* S1, const double* S2, double* out) {
    __shared__ double sh[32];
    const int b = blockIdx.x;
    T += (int64_t)b * per;
    if (S1) S1 += (int64_t)b * d2;
    if (S2) S2 += (int64_t)b * d1;
    double acc = 0.0;
    for (int64_t e = threadIdx.x; e < d1 * d2; e += blockDim.x) {
        int64_t a = e % d1, bb = e / d1;
        double v = T[a + d1 * (bb + d2 * (bb + d3 * a))];
        if (S1) v *= S1[bb];
        if (S2) v *= S2[a];
        acc += v;
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) out[b] = fabs(acc);
    }
}
void trace2d_batched(Ctx& c, const double* T, const int64_t* d, int batch, const double* S1, const double* S2,
                     double* out) {
    TNR_REQUIRE(d[0] == d[3] && d[1] == d[2], TNR_ERR_INVALID_ARG, "trace T[1 2;2 1] needs d1==d4, d2==d3");
    k_trace2d_batched<<<batch, 256, 0, c.stream>>>(T, d[0], d[1], d[2], d[0] * d[1] * d[2] * d[3], S1, S2, out);
    check_launch("trace2d_batched");
}

__global__ void k_scale_batched(double* T, int64_t per, int64_t total, const double* norms) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
        T[e] /= fabs(norms[e / per]);
}
void scale_batched(Ctx& c, double* T, int64_t per, int batch, const double* norms) {
    const int64_t total = per * batch;
    if (!total) return;
    k_scale_batched<<<grid_for(total, 256), 256, 0, c.stream>>>(T, per, total, norms);
    check_launch("scale_batched");
}

void copy_f64(Ctx& c, double* dst, const double* src, int64_t n) {
    if (n) TNR_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
}

// seeded N(0,1) entries: splitmix64 counter hash -> two uniforms -> Box-Muller
__device__ __forceinline__ uint64_t splitmix(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__global__ void k_normal(double* x, int64_t n, uint64_t seed) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t h1 = splitmix(seed ^ (2 * (uint64_t)i));
        uint64_t h2 = splitmix(h1 ^ 0x5851f42d4c957f2dull);
        double u1 = ((h1 >> 11) + 1) * (1.0 / 9007199254740993.0);  // (0, 1]
        double u2 = (h2 >> 11) * (1.0 / 9007199254740992.0);        // [0, 1)
        x[i] = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
    }
}
void fill_normal(Ctx& c, double* x, int64_t n, uint64_t seed) {
    if (!n) return;
    k_normal<<<grid_for(n, 256), 256, 0, c.stream>>>(x, n, seed);
    check_launch("normal");
}

// ---------------------------------------------------------------------------
// trace norms (src/utility/finalize.jl:4-14, 62-66)
// ---------------------------------------------------------------------------
// |sum_{a,b} T[a,b,b,a] * w1[b] * w2[a]| with optional diagonal weights
__global__ void k_trace2d(const double* T, int64_t d1, int64_t d2, int64_t d3, const double* S1,
                          const double* S2, double* out) {
    __shared__ double sh[32];
    double acc = 0.0;
    const int64_t n = d1 * d2;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
        int64_t a = e % d1, b = e / d1;
        double v = T[a + d1 * (b + d2 * (b + d3 * a))];
        if (S1) v *= S1[b];
        if (S2) v *= S2[a];
        acc += v;
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) out[0] = fabs(acc);
    }
}
void trace2d(Ctx& c, const double* T, const int64_t* d, double* out) {
    TNR_REQUIRE(d[0] == d[3] && d[1] == d[2], TNR_ERR_INVALID_ARG, "trace T[1 2;2 1] needs d1==d4, d2==d3");
    k_trace2d<<<1, 1024, 0, c.stream>>>(T, d[0], d[1], d[2], nullptr, nullptr, out);
    check_launch("trace2d");
}
void trace_btrg(Ctx& c, const double* T, const int64_t* d, const double* S1, const double* S2, double* out) {
    TNR_REQUIRE(d[0] == d[3] && d[1] == d[2], TNR_ERR_INVALID_ARG, "BTRG trace needs d1==d4, d2==d3");
    k_trace2d<<<1, 1024, 0, c.stream>>>(T, d[0], d[1], d[2], S1, S2, out);
    check_launch("trace_btrg");
}

// |sum_{a,b,c} T[a,a,b,c,b,c]|
__global__ void k_trace3d(const double* T, int64_t d1, int64_t d3, int64_t d4, double* out) {
    __shared__ double sh[32];
    double acc = 0.0;
    const int64_t n = d1 * d3 * d4;
    const int64_t s2 = d1, s3 = d1 * d1, s4 = s3 * d3, s5 = s4 * d4, s6 = s5 * d3;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
        int64_t a = e % d1, r = e / d1, b = r % d3, cc = r / d3;
        acc += T[a + a * s2 + b * s3 + cc * s4 + b * s5 + cc * s6];
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) out[0] = fabs(acc);
    }
}
void trace3d(Ctx& c, const double* T, const int64_t* d, double* out) {
    TNR_REQUIRE(d[0] == d[1] && d[2] == d[4] && d[3] == d[5], TNR_ERR_INVALID_ARG,
                "trace T[1 1;2 3 2 3] needs d1==d2, d3==d5, d4==d6");
    k_trace3d<<<1, 1024, 0, c.stream>>>(T, d[0], d[2], d[3], out);
    check_launch("trace3d");
}

// pseudopow (src/schemes/btrg.jl:50-58), tol = eps(Float64)^(3/4)
__global__ void k_pseudopow(const double* s, int n, double a, double tol, double* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = s[i] < tol ? s[i] : pow(s[i], a);
}
void pseudopow(Ctx& c, const double* s, int n, double a, double* out) {
    if (!n) return;
    const double tol = pow(2.220446049250313e-16, 0.75);
    k_pseudopow<<<(n + 127) / 128, 128, 0, c.stream>>>(s, n, a, tol, out);
    check_launch("pseudopow");
}

__global__ void k_check_finite(const double* x, int64_t n, int* status) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (!isfinite(x[i])) { atomicOr(status, ST_NONFINITE); return; }
}
void check_finite(Ctx& c, const double* x, int64_t n) {
    if (!n) return;
    k_check_finite<<<grid_for(n, 256, 2), 256, 0, c.stream>>>(x, n, c.d_status);
    check_launch("check_finite");
}

}  // namespace tnr
