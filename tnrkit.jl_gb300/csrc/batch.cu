// Lockstep batches of TRG / BTRG instances with equal shapes and bond dimension: every
// instance of a group has the same tensor dimensions at every step (they depend only on
// chi and the initial legs), so the whole group steps together.  Every contraction is
// one batched GEMM, every decomposition a batched truncated SVD whose one-CTA solvers
// run one CTA per instance, and the norms stay on the device until the run ends.
#include "schemes.cuh"

#include <algorithm>
#include <cmath>

namespace tnr {

namespace {
std::vector<int64_t> per_dims(const DT& t) { return std::vector<int64_t>(t.d, t.d + t.rank - 1); }
int64_t per_size(const DT& t) {
    int64_t s = 1;
    for (int i = 0; i + 1 < t.rank; ++i) s *= t.d[i];
    return s;
}
}  // namespace

struct BatchState {
    int kind = TNR_BTRG;
    int B = 0;
    double k = -0.5;
    DT T;        // (d1, d2, d3, d4, B)
    DT S1, S2;   // (d2, B), (d1, B) for BTRG
    // finalize! leaves T unscaled and points here at the B norms; the next step divides its
    // singular values by them (both SVDs decompose T or a permute of it), so the batch's
    // chi^4 tensors are not rescaled in a pass of their own
    const double* pending = nullptr;
};

// SVD12 of every instance of M4 (d1, d2, d3, d4, B): A = U sqrt(s), Bv = sqrt(s) V
static void svd12_b(Ctx& c, const DT& M4, int chi, int B, DT& A, DT& Bv, const double* pending) {
    const int64_t d1 = M4.d[0], d2 = M4.d[1], d3 = M4.d[2], d4 = M4.d[3];
    const int64_t m = d1 * d2, n = d3 * d4;
    const int k = (int)std::min<int64_t>(chi, std::min(m, n));
    A = make_dt(c.pool.get(), {d1, d2, (int64_t)k, (int64_t)B});
    Bv = make_dt(c.pool.get(), {(int64_t)k, d3, d4, (int64_t)B});
    Buf sv(c.pool.get(), (size_t)k * B * sizeof(double));
    tsvd_batched(c, M4.p(), m, n, k, B, A.p(), sv.d(), Bv.p());
    if (pending) scale_batched(c, sv.d(), k, B, pending);
    col_scale(c, A.p(), m, (int64_t)k * B, m, sv.d(), 1);
    row_scale_batched(c, Bv.p(), k, n * B, sv.d(), 1, n);
}

// step!(::TRG) for a batch (src/schemes/trg.jl:35-41)
static void step_trg_b(Ctx& c, BatchState& s, int chi) {
    const int B = s.B;
    DT A, Bv, C, D;
    svd12_b(c, s.T, chi, B, A, Bv, s.pending);
    DT Tp = permuted(c, s.T, {1, 3, 0, 2, 4});
    svd12_b(c, Tp, chi, B, C, D, s.pending);
    Tp = DT();
    DT X = contract(c, D.p(), per_dims(D), {Lb, Lp, Lq}, Bv.p(), per_dims(Bv), {La, Lr, Lp}, {La, Lb, Lq, Lr}, true, B);
    DT Y = contract(c, C.p(), per_dims(C), {Lr, Ls, Lc}, A.p(), per_dims(A), {Ls, Lq, Ld}, {Lq, Lr, Lc, Ld}, true, B);
    A = DT(); Bv = DT(); C = DT(); D = DT();
    s.T = contract(c, X.p(), per_dims(X), {La, Lb, Lq, Lr}, Y.p(), per_dims(Y), {Lq, Lr, Lc, Ld}, {La, Lb, Lc, Ld},
                   true, B);
}

// step!(::BTRG) for a batch (src/schemes/btrg.jl:60-94)
static void step_btrg_b(Ctx& c, BatchState& s, int chi) {
    const int B = s.B;
    const double kexp = s.k;
    const int64_t d1 = s.T.d[0], d2 = s.T.d[1], d3 = s.T.d[2], d4 = s.T.d[3];
    auto half = [&](const DT& M4, int64_t r1, int64_t r2, int64_t c1, int64_t c2, DT& U, DT& V, DT& Sn) {
        const int64_t m = r1 * r2, n = c1 * c2;
        const int k = (int)std::min<int64_t>(chi, std::min(m, n));
        U = make_dt(c.pool.get(), {r1, r2, (int64_t)k, (int64_t)B});
        V = make_dt(c.pool.get(), {(int64_t)k, c1, c2, (int64_t)B});
        Sn = make_dt(c.pool.get(), {(int64_t)k, (int64_t)B});
        Buf sv(c.pool.get(), (size_t)k * B * sizeof(double)), sa(c.pool.get(), (size_t)k * B * sizeof(double));
        tsvd_batched(c, M4.p(), m, n, k, B, U.p(), sv.d(), V.p());
        if (s.pending) scale_batched(c, sv.d(), k, B, s.pending);
        pseudopow(c, sv.d(), k * B, (1.0 - kexp) / 2.0, sa.d());
        pseudopow(c, sv.d(), k * B, kexp, Sn.p());
        col_scale(c, U.p(), m, (int64_t)k * B, m, sa.d(), 0);
        row_scale_batched(c, V.p(), k, n * B, sa.d(), 0, n);
    };
    DT A, Bv, S1n, C, D, S2n;
    half(s.T, d1, d2, d3, d4, A, Bv, S1n);
    DT P = permuted(c, s.T, {2, 0, 3, 1, 4});                // permute(T, ((3,1),(4,2))) per instance
    half(P, d3, d1, d4, d2, C, D, S2n);
    P = DT();
    // D[a,x,p] S1[p] S2[x], B[b,p,y] S2[y], C[z,y,d] S1[z]  (per-instance diagonal bond tensors)
    const int64_t kD = D.d[0], kB = Bv.d[0];
    scale_leg_batched(c, D.p(), per_size(D), B, kD * d4, d2, s.S1.p());
    scale_leg_batched(c, D.p(), per_size(D), B, kD, d4, s.S2.p());
    scale_leg_batched(c, Bv.p(), per_size(Bv), B, kB * d3, d4, s.S2.p());
    scale_leg_batched(c, C.p(), per_size(C), B, 1, d3, s.S1.p());
    DT X = contract(c, D.p(), per_dims(D), {La, Lx, Lp}, Bv.p(), per_dims(Bv), {Lb, Lp, Ly}, {La, Lb, Lx, Ly}, true, B);
    DT Y = contract(c, C.p(), per_dims(C), {Lz, Ly, Ld}, A.p(), per_dims(A), {Lx, Lz, Lc}, {Lx, Ly, Lc, Ld}, true, B);
    A = DT(); Bv = DT(); C = DT(); D = DT();
    s.T = contract(c, X.p(), per_dims(X), {La, Lb, Lx, Ly}, Y.p(), per_dims(Y), {Lx, Ly, Lc, Ld}, {La, Lb, Lc, Ld},
                   true, B);
    s.S1 = std::move(S1n);
    s.S2 = std::move(S2n);
}

// finalize! of every member: the norms, with T's scaling left to the next step (pending)
static void finalize_b(Ctx& c, BatchState& s, double* d_norms) {
    const bool btrg = s.kind == TNR_BTRG;
    trace2d_batched(c, s.T.p(), s.T.d, s.B, btrg ? s.S1.p() : nullptr, btrg ? s.S2.p() : nullptr, d_norms);
    s.pending = d_norms;
}

// run!() of every member in lockstep; members are fresh schemes with equal kind, dims, k
void run_group(Ctx& c, const std::vector<Scheme*>& mem, int chi, int maxiter, bool finalize_beginning,
               std::vector<std::vector<double>>& norms) {
    const int B = (int)mem.size();
    BatchState s;
    s.kind = mem[0]->kind;
    s.B = B;
    s.k = mem[0]->btrg_k;
    const DT& T0 = mem[0]->T;
    std::vector<int64_t> dims(T0.d, T0.d + T0.rank);
    const int64_t per = T0.size();
    dims.push_back(B);
    s.T = make_dt(c.pool.get(), dims);
    if (s.kind == TNR_BTRG) {
        s.S1 = make_dt(c.pool.get(), {T0.d[1], (int64_t)B});
        s.S2 = make_dt(c.pool.get(), {T0.d[0], (int64_t)B});
    }
    for (int b = 0; b < B; ++b) {
        mem[b]->ctx->sync();
        TNR_CUDA(cudaMemcpyAsync(s.T.p() + b * per, mem[b]->T.p(), per * sizeof(double), cudaMemcpyDeviceToDevice,
                                 c.stream));
        if (s.kind == TNR_BTRG) {
            TNR_CUDA(cudaMemcpyAsync(s.S1.p() + b * T0.d[1], mem[b]->S1.p(), T0.d[1] * sizeof(double),
                                     cudaMemcpyDeviceToDevice, c.stream));
            TNR_CUDA(cudaMemcpyAsync(s.S2.p() + b * T0.d[0], mem[b]->S2.p(), T0.d[0] * sizeof(double),
                                     cudaMemcpyDeviceToDevice, c.stream));
        }
    }
    const int nsteps = std::max(maxiter, 1);
    const int nn = nsteps + (finalize_beginning ? 1 : 0);
    Buf dn(c.pool.get(), (size_t)nn * B * sizeof(double));
    int at = 0;
    if (finalize_beginning) finalize_b(c, s, dn.d() + (at++) * B);
    const int64_t step0 = mem[0]->steps;
    for (int i = 0; i < nsteps; ++i) {
        {
            PrecisionScope scope(c, split_step_in_fp64(s.kind, step0 + i, s.T.d, s.T.rank - 1, chi));
            if (s.kind == TNR_TRG) step_trg_b(c, s, chi);
            else step_btrg_b(c, s, chi);
            s.pending = nullptr;
        }
        finalize_b(c, s, dn.d() + (at++) * B);
    }
    // the members get their tensors back normalised, as after run!()
    if (s.pending) scale_batched(c, s.T.p(), per_size(s.T), s.B, s.pending);
    s.pending = nullptr;
    check_finite(c, dn.d(), (int64_t)nn * B);
    std::vector<double> h((size_t)nn * B);
    TNR_CUDA(cudaMemcpyAsync(h.data(), dn.d(), h.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    int st = c.read_status_and_clear();
    TNR_REQUIRE(!(st & ST_NONFINITE), TNR_ERR_NONFINITE, "run! (batched): non-finite norm");
    norms.assign(B, std::vector<double>(nn));
    for (int b = 0; b < B; ++b)
        for (int i = 0; i < nn; ++i) norms[b][i] = h[(size_t)i * B + b];
    // hand every member its final tensor (and bond tensors) back
    const int64_t perT = per_size(s.T);
    for (int b = 0; b < B; ++b) {
        Scheme& m = *mem[b];
        m.T = make_dt(m.ctx->pool.get(), per_dims(s.T));
        if (s.kind == TNR_BTRG) {
            m.S1 = make_dt(m.ctx->pool.get(), {s.S1.d[0]});
            m.S2 = make_dt(m.ctx->pool.get(), {s.S2.d[0]});
        }
        m.ctx->sync();   // the member's stream-ordered allocations are complete before the copies
        TNR_CUDA(cudaMemcpyAsync(m.T.p(), s.T.p() + b * perT, perT * sizeof(double), cudaMemcpyDeviceToDevice,
                                 c.stream));
        if (s.kind == TNR_BTRG) {
            const int64_t k1 = s.S1.d[0], k2 = s.S2.d[0];
            TNR_CUDA(cudaMemcpyAsync(m.S1.p(), s.S1.p() + b * k1, k1 * sizeof(double), cudaMemcpyDeviceToDevice,
                                     c.stream));
            TNR_CUDA(cudaMemcpyAsync(m.S2.p(), s.S2.p() + b * k2, k2 * sizeof(double), cudaMemcpyDeviceToDevice,
                                     c.stream));
        }
        m.steps += nsteps;
        m.last_vals.clear();
        m.last_counts.clear();
        m.last_eps.clear();
    }
    c.sync();
}

}  // namespace tnr
