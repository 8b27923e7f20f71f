// Split-precision GEMM on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// C (FP64) = alpha * op(A) op(B) + beta * C with every FP64 operand split into three
// BF16 planes x = x0 + x1 + x2 (each the BF16 rounding of the previous residual).
// Six plane products x_i y_j with i + j <= 2 are accumulated in FP32 in tensor memory
// (TMEM): about 24 bits of each operand and FP32 accumulation, the five small products
// in one accumulator and the leading x0 y0 in another, added once at the end.  The contractions of a coarse-graining
// step use the chunked variant below (unbiased accumulation over long K).
//
//  * split pass: FP64 -> BF16 planes in a K-major [batch][plane][rows][Kp] layout
//    (shared-memory tiled transpose where the source is not K-contiguous);
//  * GEMM: 128 x BN tile per CTA.  A pipeline stage holds one K block of 32 of all
//    three planes of both operands (two TMA loads of 3 x 8 KB, 64-byte swizzle), so
//    every plane is fetched from L2 once for the six products that use it; a
//    STAGES-deep mbarrier ring, one thread issues tcgen05.mma (kind::f16, M=128,
//    K=16), tcgen05.commit frees stages, the four warps read the FP32 accumulators
//    with tcgen05.ld and write FP64 C (coalesced along the rows).
// Every wait is bounded by a 2-second global-timer limit and reports through the
// context status word instead of hanging.
#include "common.cuh"

#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>

namespace tnr {

namespace {

constexpr int BM = 128, BN = 128, BK = 32, STAGES = 4, NTHREADS = 128;
constexpr int PLANES = 3;
constexpr int TILE_A_BYTES = BM * BK * 2;                       // 8 KB: one plane of A
constexpr int TILE_B_BYTES = BN * BK * 2;                       // 8 KB: one plane of B
constexpr int STAGE_A_BYTES = PLANES * TILE_A_BYTES;            // 24 KB
constexpr int STAGE_BYTES = PLANES * (TILE_A_BYTES + TILE_B_BYTES);   // 48 KB
// tiles | barriers | slack: the slack keeps every shared-memory descriptor of the MMAs inside
// the CTA's allocation even past the last tile
constexpr int SMEM_TAIL = 256 /*barriers*/ + 8192 /*slack*/;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*align*/ + SMEM_TAIL;
constexpr int NTERMS = 6;

// plane pairs, smallest contributions first; the last (x0 y0) goes to its own accumulator
__host__ __device__ constexpr int term_pa(int t) { return t == 0 ? 2 : (t == 1 || t == 3) ? 1 : 0; }
__host__ __device__ constexpr int term_pb(int t) { return t == 2 ? 2 : (t == 1 || t == 4) ? 1 : 0; }

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait: gives up after 2 s, records the timeout and returns false
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* status) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > 2000000000ull) {
            atomicOr(status, ST_TC_TIMEOUT);
            return false;
        }
        __nanosleep(40);
    }
}

__device__ __forceinline__ void tma_load_4d(const CUtensorMap* map, uint64_t* bar, void* dst, int c0, int c1, int c2,
                                            int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

// tcgen05 shared-memory matrix descriptor: K-major, 64-byte swizzle (rows of BK = 32 BF16),
// 8-row groups 512 B apart; tiles start 1024-byte aligned (matrix base offset 0)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);          // start address
    d |= (uint64_t)1 << 16;                          // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(512 >> 4) << 32;                 // stride byte offset: 8 rows x 64 B
    d |= (uint64_t)1 << 46;                          // descriptor version (fixed 0b001)
    d |= (uint64_t)4 << 61;                          // swizzle: 64 B
    return d;
}

// instruction descriptor: kind::f16, A/B = BF16, D = F32, both K-major, M = 128, N = BN
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct TcArgs {
    int64_t m, n;
    int nkb;            // K blocks of BK = 32 in this launch
    int kb0;            // first K block
    double alpha, beta;
    double* C;
    int64_t ldc;
    int n1;             // batch level 1 size (b = b1 + n1 * b2)
    int64_t sC1, sC2;
    int a_batched, b_batched;
    int* status;
};

__global__ void __launch_bounds__(NTHREADS, 1)
k_gemm_split_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcArgs a) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t pad = ((raw + 1023) & ~1023u) - raw;
    unsigned char* tiles = smem_raw + pad;
    uint64_t* bars = reinterpret_cast<uint64_t*>(tiles + STAGES * STAGE_BYTES);
    uint64_t* full = bars;                   // STAGES
    uint64_t* empty = bars + STAGES;         // STAGES
    uint64_t* accum = bars + 2 * STAGES;     // 1
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile_m = blockIdx.x, tile_n = blockIdx.y, b = blockIdx.z;
    const int niter = a.nkb;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accum, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
    }
    if (warp == 0) {
        // two accumulators: the five small plane products, and x0 y0
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(2 * BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    bool ok = true;

    if (warp == 0 && lane == 0) {
        // TMA producer: one K block of all three planes of A and of B per stage
        const int ab = a.a_batched ? b : 0, bb = a.b_batched ? b : 0;
        for (int it = 0; it < niter && ok; ++it) {
            const int s = it % STAGES;
            const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
            ok = mbar_wait(&empty[s], ph ^ 1u, a.status);
            if (!ok) break;
            unsigned char* sa = tiles + s * STAGE_BYTES;
            unsigned char* sb = sa + STAGE_A_BYTES;
            mbar_expect_tx(&full[s], STAGE_BYTES);
            tma_load_4d(&tmA, &full[s], sa, (a.kb0 + it) * BK, tile_m * BM, 0, ab);
            tma_load_4d(&tmB, &full[s], sb, (a.kb0 + it) * BK, tile_n * BN, 0, bb);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer: per stage the six plane products, the small ones into columns [0, BN),
        // x0 y0 into [BN, 2 BN), so that the small terms never add into the large accumulator
        for (int it = 0; it < niter && ok; ++it) {
            const int s = it % STAGES;
            const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
            ok = mbar_wait(&full[s], ph, a.status);
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = smem_u32(tiles + s * STAGE_BYTES);
            const uint32_t sb = sa + STAGE_A_BYTES;
#pragma unroll
            for (int t = 0; t < NTERMS; ++t) {
                const uint32_t d = t < NTERMS - 1 ? tmem : tmem + BN;
                const uint32_t at = sa + term_pa(t) * TILE_A_BYTES, bt = sb + term_pb(t) * TILE_B_BYTES;
#pragma unroll
                for (int kk = 0; kk < BK / 16; ++kk) {
                    const bool first = it == 0 && kk == 0 && (t == 0 || t == NTERMS - 1);
                    mma_bf16(d, smem_desc(at + kk * 32), smem_desc(bt + kk * 32), first ? 0u : 1u);
                }
            }
            mma_commit(&empty[s]);
        }
        mma_commit(accum);
    }
    __syncwarp();
    // epilogue: all four warps, TMEM lanes 32w..32w+31 = tile rows
    ok = mbar_wait(accum, 0, a.status) && ok;
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int b1 = b % a.n1, b2 = b / a.n1;
    double* C = a.C + b1 * a.sC1 + b2 * a.sC2;
    const int64_t row = (int64_t)tile_m * BM + warp * 32 + lane;
    const bool plain = a.alpha == 1.0 && a.beta == 0.0;   // C = op(A) op(B): no FP64 arithmetic
    const bool add_c = a.alpha == 1.0 && a.beta == 1.0;   // C += op(A) op(B): one FP64 add
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
        float v[16], vb[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(BN + c0), vb);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = __fadd_rn(vb[j], v[j]);
        if (row < a.m) {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int64_t col = (int64_t)tile_n * BN + c0 + j;
                if (col < a.n) {
                    double* p = C + row + col * a.ldc;
                    double r = f32_to_f64(v[j]);
                    if (add_c) {
                        r += *p;
                    } else if (!plain) {
                        r *= a.alpha;
                        if (a.beta != 0.0) r = fma(a.beta, *p, r);
                    }
                    *p = ok ? r : 0.0;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN));
    }
}

// ---------------------------------------------------------------------------
// Chunked-accumulation variant for the contractions of a coarse-graining step.  The
// tensor cores truncate when they add into an FP32 accumulator (about 2^-25 of its
// value per K = 16 step, one sign for same-sign sums), so a long K builds a bias
// (-6e-6 relative at K = 2304).  Here K runs in chunks of `chunk` x 64, each chunk on
// a fresh pair of accumulators (the five small plane products, and x0 y0), so that only
// the few x0 y0 steps of one chunk truncate at the full magnitude; the stages of a chunk
// are released one by one.  Two accumulator pairs (all 512 TMEM columns) alternate so
// the MMA of chunk c+1 overlaps the drain of chunk c.  Eight drain warps (warp & 3 = TMEM lane quadrant, warp >> 2 =
// column half) add every chunk into register pairs (hi, lo) with FP32 TwoSum (round to
// nearest), and round hi + lo once at the end.  Warp 8 issues the TMA loads, warp 9
// the MMAs, warps 10-11 only fill the last warpgroup.  Every wait is bounded as in
// k_gemm_split_tc.
// ---------------------------------------------------------------------------
constexpr int ACC_STAGES = 4;                 // 192 KB: one CTA per SM
constexpr int SMEM_BYTES_ACC = ACC_STAGES * STAGE_BYTES + 1024 /*align*/ + SMEM_TAIL;
constexpr int MAX_CHUNK = 8;                      // chunks of at most 8 x 64
constexpr int ACC_WARPS = 8;
// drain warps + the TMA and MMA warps, rounded up to whole warpgroups (registers are
// granted per group of four warps, so ten warps cost as much as twelve)
constexpr int NT_ACC = 12 * 32;
constexpr int ACC_COLS = BN / 2;              // columns per drain warp

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// (hi, lo) += v with Knuth's TwoSum in round-to-nearest FP32
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float v) {
    const float s = __fadd_rn(hi, v);
    const float bp = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(v, bp));
    hi = s;
    lo = __fadd_rn(lo, e);
}

// every lane of the warp waits on lane 0's bounded wait
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity, int* status, int lane) {
    bool okw = true;
    if (lane == 0) okw = mbar_wait(bar, parity, status);
    okw = __shfl_sync(0xffffffffu, okw ? 1 : 0, 0) != 0;
    __syncwarp();
    return okw;
}

__global__ void __launch_bounds__(NT_ACC, 1)
k_gemm_split_tc_chunked(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcArgs a,
                        int chunk) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t pad = ((raw + 1023) & ~1023u) - raw;
    unsigned char* tiles = smem_raw + pad;
    uint64_t* bars = reinterpret_cast<uint64_t*>(tiles + ACC_STAGES * STAGE_BYTES);
    uint64_t* full = bars;                        // ACC_STAGES
    uint64_t* empty = bars + ACC_STAGES;              // ACC_STAGES
    uint64_t* acc_full = bars + 2 * ACC_STAGES;       // 2: chunk accumulated
    uint64_t* acc_empty = bars + 2 * ACC_STAGES + 2;  // 2: chunk drained
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * ACC_STAGES + 4);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile_m = blockIdx.x, tile_n = blockIdx.y, b = blockIdx.z;
    const int nkb = a.nkb;                    // stages (K blocks of BK = 32)
    const int cs = chunk * (64 / BK);         // stages per chunk
    const int nchunks = (nkb + cs - 1) / cs;

    if (threadIdx.x == 0) {
        for (int s = 0; s < ACC_STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&acc_full[i], 1);
            mbar_init(&acc_empty[i], ACC_WARPS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
    }
    if (warp == 0) {
        // accumulator pair of buffer u: small products at columns 2u BN, x0 y0 at (2u + 1) BN
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(4 * BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    bool ok = true;

    if (warp == ACC_WARPS && lane == 0) {
        // TMA producer: one K block of all three planes of A and of B per stage, in K order
        const int ab = a.a_batched ? b : 0, bb = a.b_batched ? b : 0;
        for (int it = 0; it < nkb && ok; ++it) {
            const int s = it % ACC_STAGES;
            const uint32_t ph = (uint32_t)(it / ACC_STAGES) & 1u;
            ok = mbar_wait(&empty[s], ph ^ 1u, a.status);
            if (!ok) break;
            unsigned char* sa = tiles + s * STAGE_BYTES;
            unsigned char* sb = sa + STAGE_A_BYTES;
            mbar_expect_tx(&full[s], STAGE_BYTES);
            tma_load_4d(&tmA, &full[s], sa, (a.kb0 + it) * BK, tile_m * BM, 0, ab);
            tma_load_4d(&tmB, &full[s], sb, (a.kb0 + it) * BK, tile_n * BN, 0, bb);
        }
    } else if (warp == ACC_WARPS + 1 && lane == 0) {
        // MMA issuer: chunk c into accumulator pair c & 1, once the drain of chunk c - 2 is
        // done; every stage's six products go out as soon as it lands, and the stage is freed
        for (int c = 0; c < nchunks && ok; ++c) {
            const int buf = c & 1;
            if (c >= 2) {
                ok = mbar_wait(&acc_empty[buf], (uint32_t)((c >> 1) - 1) & 1u, a.status);
                if (!ok) break;
            }
            const uint32_t d_small = tmem + (uint32_t)(2 * buf * BN), d_big = d_small + BN;
            const int ibeg = c * cs, iend = min(nkb, ibeg + cs);
            for (int it = ibeg; it < iend && ok; ++it) {
                const int s = it % ACC_STAGES;
                ok = mbar_wait(&full[s], (uint32_t)(it / ACC_STAGES) & 1u, a.status);
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t sa = smem_u32(tiles + s * STAGE_BYTES);
                const uint32_t sb = sa + STAGE_A_BYTES;
#pragma unroll
                for (int t = 0; t < NTERMS; ++t) {
                    const uint32_t d = t < NTERMS - 1 ? d_small : d_big;
                    const uint32_t at = sa + term_pa(t) * TILE_A_BYTES, bt = sb + term_pb(t) * TILE_B_BYTES;
#pragma unroll
                    for (int kk = 0; kk < BK / 16; ++kk) {
                        const bool first = it == ibeg && kk == 0 && (t == 0 || t == NTERMS - 1);
                        mma_bf16(d, smem_desc(at + kk * 32), smem_desc(bt + kk * 32), first ? 0u : 1u);
                    }
                }
                mma_commit(&empty[s]);
            }
            mma_commit(&acc_full[buf]);
        }
    } else if (warp < ACC_WARPS) {
        // drain: this warp's 32 rows (TMEM lanes) x 64 columns of the tile
        const int quad = warp & 3, half = warp >> 2;
        float hi[ACC_COLS], lo[ACC_COLS];
#pragma unroll
        for (int j = 0; j < ACC_COLS; ++j) hi[j] = lo[j] = 0.0f;
        for (int c = 0; c < nchunks && ok; ++c) {
            const int buf = c & 1;
            ok = warp_wait(&acc_full[buf], (uint32_t)(c >> 1) & 1u, a.status, lane);
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // x0 y0 into (hi, lo) by TwoSum; the small products (2^-8 of it) straight into lo
            const uint32_t base = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(2 * buf * BN + half * ACC_COLS);
#pragma unroll
            for (int q = 0; q < ACC_COLS / 16; ++q) {
                float v[16], w[16];
                tmem_ld16(base + (uint32_t)(BN + q * 16), v);
                tmem_ld16(base + (uint32_t)(q * 16), w);
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    two_sum_acc(hi[q * 16 + j], lo[q * 16 + j], v[j]);
                    lo[q * 16 + j] = __fadd_rn(lo[q * 16 + j], w[j]);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[buf]);
        }
        const int b1 = b % a.n1, b2 = b / a.n1;
        double* C = a.C + b1 * a.sC1 + b2 * a.sC2;
        const int64_t row = (int64_t)tile_m * BM + quad * 32 + lane;
        const int64_t col0 = (int64_t)tile_n * BN + half * ACC_COLS;
        const bool plain = a.alpha == 1.0 && a.beta == 0.0;
        const bool add_c = a.alpha == 1.0 && a.beta == 1.0;
        if (row < a.m) {
#pragma unroll
            for (int j = 0; j < ACC_COLS; ++j) {
                const int64_t col = col0 + j;
                if (col < a.n) {
                    double* p = C + row + col * a.ldc;
                    double r = f32_to_f64(__fadd_rn(hi[j], lo[j]));
                    if (add_c) {
                        r += *p;
                    } else if (!plain) {
                        r *= a.alpha;
                        if (a.beta != 0.0) r = fma(a.beta, *p, r);
                    }
                    *p = ok ? r : 0.0;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(4 * BN));
    }
}

// FP64 operand -> three BF16 planes, K-major: dst[b][plane][row][Kp] (Kp >= K, zero padded).
// Source element (row i, k) of batch (b1, b2) at src[b1*s1 + b2*s2 + i*si + k*sk].
struct SplitArgs {
    const double* src;
    int64_t rows, K, Kp, si, sk, s1, s2;
    int n1, nb;
    __nv_bfloat16* dst;
};

// x (FP64) -> three BF16 planes with integer and FP32 operations only (FP64 arithmetic is
// scarce on this part).  xh = x truncated to 24 significant bits (bit fields), xl = the
// next 23 bits of x as an FP32 value; p0 = rn(xh), p1 = rn(xh - p0), p2 = rn(xh - p0 - p1
// + xl) with both differences exact in FP32.  |x| below 2^-126 gives zero planes; |x| at
// or above 2^128 gives infinities, NaN gives NaN.
__device__ __forceinline__ void split3(double x, __nv_bfloat16& p0, __nv_bfloat16& p1, __nv_bfloat16& p2) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const uint32_t hi = (uint32_t)(bits >> 32), lo = (uint32_t)bits;
    const uint32_t sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7FF);   // biased FP64 exponent
    float xh, xl = 0.0f;
    if (e < 897) {                              // below the FP32 normal range (or zero)
        xh = __uint_as_float(sign);
    } else if (e > 1150) {                      // beyond the FP32 range: inf, or NaN
        const bool nan = e == 2047 && (((hi & 0xFFFFFu) | lo) != 0u);
        xh = __uint_as_float(sign | 0x7F800000u | (nan ? 0x00400000u : 0u));
    } else {
        xh = __uint_as_float(sign | ((uint32_t)(e - 896) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
        const int es = e - 1023 - 23 + 127;     // FP32 biased exponent of 2^(E - 23)
        if (es >= 1) {
            const uint32_t r23 = (lo & 0x1FFFFFFFu) >> 6;   // next 23 bits of the significand
            const float fr = __uint_as_float(0x4B000000u | r23) - 8388608.0f;   // exact integer
            xl = (fr * 1.1920928955078125e-07f) * __uint_as_float((uint32_t)es << 23);   // r23 2^-23 2^(E-23)
            if (sign) xl = -xl;
        }
    }
    p0 = __float2bfloat16_rn(xh);
    const float r1 = xh - __bfloat162float(p0);
    p1 = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(p1);
    p2 = __float2bfloat16_rn(r2 + xl);
}

__global__ void k_split_planes(SplitArgs a) {
    __shared__ double tile[32][33];
    const int64_t tr = (a.rows + 31) / 32, tk = (a.Kp + 31) / 32;
    const int64_t ntiles = tr * tk * a.nb;
    const bool kfast = (a.sk == 1);
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t bi = t / (tr * tk), rem = t % (tr * tk);
        const int64_t i0 = (rem / tk) * 32, k0 = (rem % tk) * 32;
        const int b1 = (int)(bi % a.n1), b2 = (int)(bi / a.n1);
        const double* S = a.src + b1 * a.s1 + b2 * a.s2;
        __syncthreads();
        for (int y = threadIdx.y; y < 32; y += blockDim.y) {
            // coalesced along whichever index is contiguous in the source
            int64_t i = kfast ? i0 + y : i0 + threadIdx.x;
            int64_t k = kfast ? k0 + threadIdx.x : k0 + y;
            double v = (i < a.rows && k < a.K) ? S[i * a.si + k * a.sk] : 0.0;
            if (kfast) tile[y][threadIdx.x] = v;       // tile[i][k]
            else tile[threadIdx.x][y] = v;
        }
        __syncthreads();
        // 4 consecutive k of one row per thread (8 threads per row): 8-byte plane stores
        // (Kp % 4 == 0, k0 % 32 == 0, so every group lies inside [0, Kp) or outside it)
        {
            const int tid = threadIdx.y * 32 + threadIdx.x;
            const int y = tid >> 3, kq = (tid & 7) * 4;
            const int64_t i = i0 + y, k = k0 + kq;
            if (i < a.rows && k < a.Kp) {
                __nv_bfloat16 p0[4], p1[4], p2[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) split3(tile[y][kq + e], p0[e], p1[e], p2[e]);
                const int64_t plane = a.rows * a.Kp;
                __nv_bfloat16* D = a.dst + bi * 3 * plane + i * a.Kp + k;
                uint2 u0, u1, u2;
                memcpy(&u0, p0, 8);
                memcpy(&u1, p1, 8);
                memcpy(&u2, p2, 8);
                *reinterpret_cast<uint2*>(D) = u0;
                *reinterpret_cast<uint2*>(D + plane) = u1;
                *reinterpret_cast<uint2*>(D + 2 * plane) = u2;
            }
        }
    }
}

// The same planes for a K-contiguous source (sk == 1): no transpose, so no shared memory;
// a thread splits 4 consecutive k of one row and writes 8 bytes per plane.  Needs Kp % 4 == 0
// and rows * Kp / 4 * nb below 4e9 (32-bit item index plus the grid stride).
__global__ void k_split_planes_kfast(SplitArgs a) {
    const uint32_t nk4 = (uint32_t)(a.Kp / 4);
    const uint32_t per_b = (uint32_t)a.rows * nk4;
    const uint32_t total = per_b * (uint32_t)a.nb;
    const int64_t plane = a.rows * a.Kp;
    for (uint32_t it = blockIdx.x * blockDim.x + threadIdx.x; it < total; it += gridDim.x * blockDim.x) {
        const uint32_t bi = it / per_b, rem = it - bi * per_b;
        const uint32_t i = rem / nk4;
        const int64_t k = (int64_t)(rem - i * nk4) * 4;
        const int b1 = (int)(bi % (uint32_t)a.n1), b2 = (int)(bi / (uint32_t)a.n1);
        const double* S = a.src + b1 * a.s1 + b2 * a.s2 + (int64_t)i * a.si;
        __nv_bfloat16 p0[4], p1[4], p2[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) split3(k + e < a.K ? S[k + e] : 0.0, p0[e], p1[e], p2[e]);
        __nv_bfloat16* D = a.dst + (int64_t)bi * 3 * plane + (int64_t)i * a.Kp + k;
        uint2 u0, u1, u2;
        memcpy(&u0, p0, 8);
        memcpy(&u1, p1, 8);
        memcpy(&u2, p2, 8);
        *reinterpret_cast<uint2*>(D) = u0;
        *reinterpret_cast<uint2*>(D + plane) = u1;
        *reinterpret_cast<uint2*>(D + 2 * plane) = u2;
    }
}

// planes of one operand on `st`: the K-contiguous kernel where it applies, else the tiled one
void launch_split(const SplitArgs& sa, cudaStream_t st) {
    if (sa.sk == 1 && sa.Kp % 4 == 0 && (double)sa.rows * (sa.Kp / 4) * sa.nb < 4.0e9) {   // index + stride < 2^32
        const int64_t items = sa.rows * (sa.Kp / 4) * sa.nb;
        const int g = (int)std::min<int64_t>((items + 255) / 256, (int64_t)sm_count() * 8);
        k_split_planes_kfast<<<g, 256, 0, st>>>(sa);
    } else {
        const int64_t ntiles = ((sa.rows + 31) / 32) * ((sa.Kp + 31) / 32) * sa.nb;
        const int g = (int)std::min<int64_t>(ntiles, (int64_t)sm_count() * 16);
        k_split_planes<<<g, dim3(32, 8), 0, st>>>(sa);
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// planes [nb][3][rows][Kp] bf16 -> 4D map {Kp, rows, 3, nb}, box {32, box_rows, 3, 1}
void make_map(CUtensorMap* m, const void* base, int64_t rows, int64_t Kp, int nb, int box_rows) {
    EncodeTiledFn fn = encode_fn();
    TNR_REQUIRE(fn, TNR_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[4] = {(cuuint64_t)Kp, (cuuint64_t)rows, 3, (cuuint64_t)nb};
    cuuint64_t strides[3] = {(cuuint64_t)Kp * 2, (cuuint64_t)Kp * 2 * rows, (cuuint64_t)Kp * 2 * rows * 3};
    cuuint32_t box[4] = {BK, (cuuint32_t)box_rows, PLANES, 1};   // all three planes of a K block
    cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    TNR_REQUIRE(r == CUDA_SUCCESS, TNR_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

void split_operand(Ctx& c, const double* src, int64_t rows, int64_t K, int64_t Kp, int64_t si, int64_t sk,
                   int64_t s1, int64_t s2, int n1, int nb, __nv_bfloat16* dst) {
    SplitArgs sa{src, rows, K, Kp, si, sk, s1, s2, n1, nb, dst};
    int rec = prof_start(c.stream);
    launch_split(sa, c.stream);
    check_launch("split_planes");
    prof_stop(rec, c.stream, PROF_SPLIT, (double)rows * K * nb * 8 + (double)rows * Kp * nb * 6);
}

}  // namespace

namespace {

// The kernels' dynamic shared-memory limits are attributes of the current device's context,
// so they are raised once per device (first tensor-core call with that device current).
std::atomic<uint64_t> g_tc_attr_set{0};

bool tc_ready() {
    if (!encode_fn()) return false;
    ensure_smem_attr(g_tc_attr_set, (const void*)k_gemm_split_tc, SMEM_BYTES);
    static std::atomic<uint64_t> acc_set{0};
    ensure_smem_attr(acc_set, (const void*)k_gemm_split_tc_chunked, SMEM_BYTES_ACC);
    return true;
}

bool tc_shape_ok(int64_t m, int64_t n, int64_t k, int batch) {
    if (m < 64 || n < 16 || k < 16) return false;
    return batch <= 65535 && (m + BM - 1) / BM <= 2147483647 && (n + BN - 1) / BN <= 65535;
}

void launch_tc(Ctx& c, const CUtensorMap& mA, const CUtensorMap& mB, int64_t m, int64_t n, int64_t k, int kb0,
               int nkb, double alpha, double beta, double* C, int64_t ldc, const Batch2& bt, bool a_b, bool b_b) {
    const int batch = bt.n1 * bt.n2;
    TcArgs args;
    args.m = m;
    args.n = n;
    args.nkb = nkb;
    args.kb0 = kb0;
    args.alpha = alpha;
    args.beta = beta;
    args.C = C;
    args.ldc = ldc;
    args.n1 = bt.n1;
    args.sC1 = bt.sC1;
    args.sC2 = bt.sC2;
    args.a_batched = a_b;
    args.b_batched = b_b;
    args.status = c.d_status;
    dim3 grid((unsigned)((m + BM - 1) / BM), (unsigned)((n + BN - 1) / BN), (unsigned)batch);
    int rec = prof_start(c.stream);
    k_gemm_split_tc<<<grid, NTHREADS, SMEM_BYTES, c.stream>>>(mA, mB, args);
    check_launch("gemm_split_tc");
    prof_stop(rec, c.stream, PROF_TC, 2.0 * m * n * std::min<int64_t>(k - (int64_t)kb0 * BK, (int64_t)nkb * BK) * batch);
}

void launch_tc_chunked(Ctx& c, const CUtensorMap& mA, const CUtensorMap& mB, int64_t m, int64_t n, int64_t k,
                       int nkb, int chunk, double alpha, double beta, double* C, int64_t ldc, const Batch2& bt,
                       bool a_b, bool b_b) {
    const int batch = bt.n1 * bt.n2;
    TNR_REQUIRE(chunk >= 1 && chunk <= MAX_CHUNK, TNR_ERR_UNSUPPORTED, "split chunk out of range");
    TcArgs args;
    args.m = m;
    args.n = n;
    args.nkb = nkb;
    args.kb0 = 0;
    args.alpha = alpha;
    args.beta = beta;
    args.C = C;
    args.ldc = ldc;
    args.n1 = bt.n1;
    args.sC1 = bt.sC1;
    args.sC2 = bt.sC2;
    args.a_batched = a_b;
    args.b_batched = b_b;
    args.status = c.d_status;
    dim3 grid((unsigned)((m + BM - 1) / BM), (unsigned)((n + BN - 1) / BN), (unsigned)batch);
    int rec = prof_start(c.stream);
    k_gemm_split_tc_chunked<<<grid, NT_ACC, SMEM_BYTES_ACC, c.stream>>>(mA, mB, args, chunk);
    check_launch("gemm_split_tc_chunked");
    prof_stop(rec, c.stream, PROF_TC, 2.0 * m * n * k * batch);
}

// op(B) (k x n) as n rows of K-major planes; returns whether B is batched
bool split_b(Ctx& c, bool tb, int64_t n, int64_t k, int64_t Kp, const double* B, int64_t ldb, const Batch2& bt,
             Buf& pb, CUtensorMap& mB) {
    const int batch = bt.n1 * bt.n2;
    const bool b_b = (bt.sB1 != 0 || bt.sB2 != 0) && batch > 1;
    const int nbB = b_b ? batch : 1;
    pb = Buf(c.pool.get(), (size_t)nbB * 3 * n * Kp * 2);
    // op(B)(kk, j) as rows j: tb ? B[j + kk*ldb] : B[kk + j*ldb]
    split_operand(c, B, n, k, Kp, tb ? 1 : ldb, tb ? ldb : 1, b_b ? bt.sB1 : 0, b_b ? bt.sB2 : 0, b_b ? bt.n1 : 1, nbB,
                  pb.as<__nv_bfloat16>());
    make_map(&mB, pb.as<void>(), n, Kp, nbB, BN);
    return b_b;
}

// the GEMM on planes already split: A's (P) and B's map
bool launch_planes(Ctx& c, const SplitA& P, const CUtensorMap& mB, bool b_b, int64_t n, double alpha, double beta,
                   double* C, int64_t ldc, const Batch2& bt, int chunk_kb) {
    const int nkb = (int)((P.Kp + BK - 1) / BK);      // K blocks of 32; chunk_kb counts blocks of 64
    if (chunk_kb > 0 && nkb > chunk_kb * (64 / BK))
        launch_tc_chunked(c, P.map, mB, P.m, n, P.k, nkb, chunk_kb, alpha, beta, C, ldc, bt, P.batched, b_b);
    else
        launch_tc(c, P.map, mB, P.m, n, P.k, 0, nkb, alpha, beta, C, ldc, bt, P.batched, b_b);
    return true;
}

}  // namespace

bool gemm_split_tc(Ctx& c, bool ta, bool tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                   int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, const Batch2& bt,
                   int chunk_kb) {
    const int batch = bt.n1 * bt.n2;
    if (!tc_shape_ok(m, n, k, batch) || !tc_ready()) return false;
    SplitA P;
    if (!split_a_build(c, P, ta, A, lda, m, k, bt)) return false;
    // a Gram X^T X (same matrices, same batch strides): op(B)'s rows are op(A)'s rows, so
    // B uses A's planes and map (BM == BN) and the plane pass runs once
    if (ta && !tb && A == B && lda == ldb && m == n && bt.sA1 == bt.sB1 && bt.sA2 == bt.sB2 && BM == BN)
        return launch_planes(c, P, P.map, P.batched, n, alpha, beta, C, ldc, bt, chunk_kb);
    return gemm_split_tc_a(c, P, tb, n, B, ldb, alpha, beta, C, ldc, bt, chunk_kb);
}

// planes of op(A) (m x k): op(A)(i, kk) = ta ? A[kk + i*lda] : A[i + kk*lda]
bool split_a_build(Ctx& c, SplitA& P, bool ta, const double* A, int64_t lda, int64_t m, int64_t k,
                   const Batch2& bt) {
    const int batch = bt.n1 * bt.n2;
    if (m < 64 || k < 16 || batch > 65535 || !tc_ready()) return false;
    P.m = m;
    P.k = k;
    P.Kp = (k + 7) / 8 * 8;
    P.batched = (bt.sA1 != 0 || bt.sA2 != 0) && batch > 1;
    P.nb = P.batched ? batch : 1;
    P.planes = Buf(c.pool.get(), (size_t)P.nb * 3 * m * P.Kp * 2);
    split_operand(c, A, m, k, P.Kp, ta ? lda : 1, ta ? 1 : lda, P.batched ? bt.sA1 : 0, P.batched ? bt.sA2 : 0,
                  P.batched ? bt.n1 : 1, P.nb, P.planes.as<__nv_bfloat16>());
    make_map(&P.map, P.planes.as<void>(), m, P.Kp, P.nb, BM);
    P.active = true;
    return true;
}

// chunk_kb > 0: the K blocks are accumulated chunk_kb at a time, each chunk on a fresh
// FP32 accumulator (k_gemm_split_tc_chunked).  The tensor cores truncate when they add
// into the FP32 accumulator, a loss of about 2^-25 of its value per K = 16 step and the
// same sign for same-sign sums (-6e-6 relative at K = 2304); chunks bound that bias by
// the chunk length, and the chunks are summed with round-to-nearest TwoSum.
bool gemm_split_tc_a(Ctx& c, const SplitA& P, bool tb, int64_t n, const double* B, int64_t ldb, double alpha,
                     double beta, double* C, int64_t ldc, const Batch2& bt, int chunk_kb) {
    const int batch = bt.n1 * bt.n2;
    if (!P.active || !tc_shape_ok(P.m, n, P.k, batch)) return false;
    if (P.batched && P.nb != batch) return false;
    Buf pb;
    CUtensorMap mB;
    const bool b_b = split_b(c, tb, n, P.k, P.Kp, B, ldb, bt, pb, mB);
    return launch_planes(c, P, mB, b_b, n, alpha, beta, C, ldc, bt, chunk_kb);
}

// ---------------------------------------------------------------------------
// Allocation-free entry point: the same split kernel with its BF16 plane scratch in a
// file-scope device array instead of the pool.  For callers that cannot call cudaMalloc:
// code running inside another allocator's arena (a Julia CUDA.jl pool, or a serving
// process that reserves all free HBM up front) and latency-critical paths where
// cudaMalloc's implicit device synchronisation would stall every other stream.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(16) << 20;   // 16 MiB of BF16 planes, held until exit
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];
static __device__ int g_noalloc_status;

struct NoAllocDevice {
    unsigned char* scratch = nullptr;
    int* status = nullptr;
    bool smem_attr = false;   // k_gemm_split_tc's dynamic shared-memory limit raised on this device
};
constexpr int NOALLOC_MAX_DEVICES = 64;
NoAllocDevice g_noalloc_dev[NOALLOC_MAX_DEVICES];
std::mutex g_noalloc_mu;

// First call on a device: resolve the device addresses of the file-scope arrays with that
// device current (a host-side use of the array name is not a device address).
const NoAllocDevice* noalloc_device(int dev) {
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    NoAllocDevice& d = g_noalloc_dev[dev];
    if (!d.scratch) {
        void* p = nullptr;
        void* q = nullptr;
        TNR_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        TNR_CUDA(cudaGetSymbolAddress(&q, g_noalloc_status));
        d.scratch = static_cast<unsigned char*>(p);
        d.status = static_cast<int*>(q);
    }
    if (!d.smem_attr) {
        // set here, with this device current, under the mutex (not through tc_ready's shared flag)
        TNR_CUDA(cudaFuncSetAttribute(k_gemm_split_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        d.smem_attr = true;
    }
    return &d;
}

}  // namespace

}  // namespace tnr

using tnr::Error;

extern "C" int tnr_gemm_split_noalloc(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                                      const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
                                      double* C, int64_t ldc, void* stream, char* err, size_t err_cap) {
    using namespace tnr;
    auto report = [&](int code, const std::string& msg) {
        if (err && err_cap) {
            size_t len = std::min(err_cap - 1, msg.size());
            std::memcpy(err, msg.data(), len);
            err[len] = 0;
        }
        return code;
    };
    if (!A || !B || !C) return report(TNR_ERR_INVALID_ARG, "NULL operand pointer");
    if (m < 64 || n < 16 || k < 16)
        return report(TNR_ERR_UNSUPPORTED, "split kernel shape limits: m >= 64, n >= 16, k >= 16");
    if (lda < (ta ? k : m) || ldb < (tb ? n : k) || ldc < m) return report(TNR_ERR_INVALID_ARG, "leading dimension too small");
    // each of m, n and ceil8(k) is at most the scratch size, so the byte counts below
    // cannot overflow (and the grid stays far inside its limits)
    if (m > (int64_t)NOALLOC_SCRATCH_BYTES || n > (int64_t)NOALLOC_SCRATCH_BYTES || k > (int64_t)NOALLOC_SCRATCH_BYTES)
        return report(TNR_ERR_INVALID_ARG, "operands exceed the allocation-free scratch of " +
                                               std::to_string(NOALLOC_SCRATCH_BYTES) + " bytes (6*(m+n)*ceil8(k) bytes)");
    if ((n + BN - 1) / BN > 65535) return report(TNR_ERR_UNSUPPORTED, "n too large for the grid");
    const int64_t Kp = (k + 7) / 8 * 8;
    const size_t bytesA = (size_t)3 * m * Kp * 2, bytesB = (size_t)3 * n * Kp * 2;
    const size_t offB = (bytesA + 255) / 256 * 256;
    if (offB + bytesB > NOALLOC_SCRATCH_BYTES)
        return report(TNR_ERR_INVALID_ARG, "operands need " + std::to_string(offB + bytesB) +
                                               " bytes of BF16 planes; the allocation-free scratch holds " +
                                               std::to_string(NOALLOC_SCRATCH_BYTES) + " (6*(m+n)*ceil8(k) bytes)");
    try {
        int dev = 0;
        TNR_CUDA(cudaGetDevice(&dev));
        TNR_REQUIRE(dev >= 0 && dev < NOALLOC_MAX_DEVICES, TNR_ERR_UNSUPPORTED, "device index out of range");
        const NoAllocDevice* d = noalloc_device(dev);
        TNR_REQUIRE(encode_fn(), TNR_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        // the status word keeps the previous call's value: clear it
        TNR_CUDA(cudaMemsetAsync(d->status, 0, sizeof(int), st));
        __nv_bfloat16* pa = reinterpret_cast<__nv_bfloat16*>(d->scratch);
        __nv_bfloat16* pb = reinterpret_cast<__nv_bfloat16*>(d->scratch + offB);
        SplitArgs sa{A, m, k, Kp, ta ? lda : 1, ta ? 1 : lda, 0, 0, 1, 1, pa};
        SplitArgs sb{B, n, k, Kp, tb ? 1 : ldb, tb ? ldb : 1, 0, 0, 1, 1, pb};
        for (const SplitArgs* s : {&sa, &sb}) {
            launch_split(*s, st);
            check_launch("split_planes (allocation-free)");
        }
        CUtensorMap mA, mB;
        make_map(&mA, pa, m, Kp, 1, BM);
        make_map(&mB, pb, n, Kp, 1, BN);
        TcArgs args;
        args.m = m;
        args.n = n;
        args.nkb = (int)((Kp + BK - 1) / BK);
        args.kb0 = 0;
        args.alpha = alpha;
        args.beta = beta;
        args.C = C;
        args.ldc = ldc;
        args.n1 = 1;
        args.sC1 = 0;
        args.sC2 = 0;
        args.a_batched = 0;
        args.b_batched = 0;
        args.status = d->status;
        dim3 grid((unsigned)((m + BM - 1) / BM), (unsigned)((n + BN - 1) / BN), 1);
        k_gemm_split_tc<<<grid, NTHREADS, SMEM_BYTES, st>>>(mA, mB, args);
        check_launch("gemm_split_tc (allocation-free)");
        int h = 0;
        TNR_CUDA(cudaMemcpyAsync(&h, d->status, sizeof(int), cudaMemcpyDeviceToHost, st));
        TNR_CUDA(cudaStreamSynchronize(st));
        TNR_REQUIRE(h == 0, TNR_ERR_CUDA, "tensor-core pipeline wait timed out (status " + std::to_string(h) + ")");
    } catch (const Error& e) {
        return report(e.code, e.what());
    } catch (const std::exception& e) {
        return report(TNR_ERR_CUDA, e.what());
    }
    return report(TNR_OK, "");
}
