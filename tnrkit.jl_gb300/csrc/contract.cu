// Pairwise tensor contraction as permute -> GEMM -> permute (the @tensor /
// @plansor / @tensoropt pairwise steps of TensorOperations, restated).  The
// planner picks, among the layouts that need the fewest moved elements, one
// GEMM over the grouped legs; every permute is the shared-memory tiled kernel.
#include "common.cuh"

#include <algorithm>

namespace tnr {

namespace {

struct Plan {
    std::vector<int> K, FA, FB;   // label orders
    bool permA = false, permB = false, permOut = false;
    bool ta = false, tb = false, swap = false;
    double cost = 1e300;
};

int idx_of(const std::vector<int>& v, int x) {
    for (size_t i = 0; i < v.size(); ++i)
        if (v[i] == x) return (int)i;
    return -1;
}

std::vector<int> concat(const std::vector<int>& a, const std::vector<int>& b) {
    std::vector<int> r(a);
    r.insert(r.end(), b.begin(), b.end());
    return r;
}

}  // namespace

DT contract(Ctx& c, const double* A, const std::vector<int64_t>& dA, const std::vector<int>& lA,
            const double* B, const std::vector<int64_t>& dB, const std::vector<int>& lB,
            const std::vector<int>& lOut, bool bulk, int batch) {
    TNR_REQUIRE(batch >= 1, TNR_ERR_INVALID_ARG, "contract: batch < 1");
    TNR_REQUIRE(dA.size() == lA.size() && dB.size() == lB.size(), TNR_ERR_INVALID_ARG, "contract: rank/labels");
    std::vector<int> K, FA, FB;
    for (int x : lA) {
        if (idx_of(lB, x) >= 0) K.push_back(x);
        else FA.push_back(x);
    }
    for (int x : lB)
        if (idx_of(lA, x) < 0) FB.push_back(x);
    TNR_REQUIRE(FA.size() + FB.size() == lOut.size(), TNR_ERR_INVALID_ARG, "contract: output labels");
    auto dim_of = [&](int x) -> int64_t {
        int i = idx_of(lA, x);
        if (i >= 0) return dA[i];
        return dB[idx_of(lB, x)];
    };
    for (int x : K) TNR_REQUIRE(dA[idx_of(lA, x)] == dB[idx_of(lB, x)], TNR_ERR_INVALID_ARG, "contract: dim mismatch");
    for (int x : lOut) TNR_REQUIRE(idx_of(FA, x) >= 0 || idx_of(FB, x) >= 0, TNR_ERR_INVALID_ARG, "contract: stray output label");
    int64_t sizeA = 1, sizeB = 1, sizeC = 1, m = 1, n = 1, kk = 1;
    for (auto d : dA) sizeA *= d;
    for (auto d : dB) sizeB *= d;
    for (int x : FA) m *= dim_of(x);
    for (int x : FB) n *= dim_of(x);
    for (int x : K) kk *= dim_of(x);
    sizeC = m * n;

    // candidate label orders
    std::vector<int> KB;
    for (int x : lB)
        if (idx_of(K, x) >= 0) KB.push_back(x);
    std::vector<int> FAo, FBo;   // FA / FB in output order
    for (int x : lOut) {
        if (idx_of(FA, x) >= 0) FAo.push_back(x);
        else FBo.push_back(x);
    }
    Plan best;
    for (const auto& Kc : {K, KB})
        for (const auto& FAc : {FA, FAo})
            for (const auto& FBc : {FB, FBo})
                for (int swap = 0; swap < 2; ++swap) {
                    Plan p;
                    p.K = Kc; p.FA = FAc; p.FB = FBc; p.swap = swap;
                    double cost = 0;
                    // A as [FA|K] (N) or [K|FA] (T)
                    if (lA == concat(FAc, Kc)) { p.ta = false; }
                    else if (lA == concat(Kc, FAc)) { p.ta = true; }
                    else { p.permA = true; p.ta = false; cost += 2.0 * sizeA; }
                    if (lB == concat(Kc, FBc)) { p.tb = false; }
                    else if (lB == concat(FBc, Kc)) { p.tb = true; }
                    else { p.permB = true; p.tb = false; cost += 2.0 * sizeB; }
                    std::vector<int> nat = swap ? concat(FBc, FAc) : concat(FAc, FBc);
                    if (nat != lOut) { p.permOut = true; cost += 2.0 * sizeC; }
                    cost += 1e-3 * swap;   // tie-break towards the plain orientation
                    p.cost = cost;
                    if (cost < best.cost) best = p;
                }
    Pool* pool = c.pool.get();
    Buf bufA, bufB;
    const double* pa = A;
    const double* pb = B;
    // a batch is a trailing leg that every operand and the output carry unchanged
    auto permute_b = [&](const double* in, const std::vector<int64_t>& d, std::vector<int> perm, double* out) {
        std::vector<int64_t> dd(d);
        if (batch > 1) {
            perm.push_back((int)d.size());
            dd.push_back(batch);
        }
        permute(c, in, dd.data(), (int)dd.size(), perm.data(), out);
    };
    if (best.permA) {
        std::vector<int> target = concat(best.FA, best.K);
        std::vector<int> perm(target.size());
        for (size_t i = 0; i < target.size(); ++i) perm[i] = idx_of(lA, target[i]);
        bufA = Buf(pool, (size_t)sizeA * batch * sizeof(double));
        permute_b(A, dA, perm, bufA.d());
        pa = bufA.d();
    }
    if (best.permB) {
        std::vector<int> target = concat(best.K, best.FB);
        std::vector<int> perm(target.size());
        for (size_t i = 0; i < target.size(); ++i) perm[i] = idx_of(lB, target[i]);
        bufB = Buf(pool, (size_t)sizeB * batch * sizeof(double));
        permute_b(B, dB, perm, bufB.d());
        pb = bufB.d();
    }
    // result in natural order
    std::vector<int> nat = best.swap ? concat(best.FB, best.FA) : concat(best.FA, best.FB);
    std::vector<int64_t> natd;
    for (int x : nat) natd.push_back(dim_of(x));
    if (batch > 1) natd.push_back(batch);
    DT Cn = make_dt(pool, natd);
    const int64_t lda = best.ta ? kk : m;   // A matrix: [FA|K] (m x kk) or [K|FA] (kk x m)
    const int64_t ldb = best.tb ? n : kk;   // B matrix: [K|FB] (kk x n) or [FB|K] (n x kk)
    auto run = [&](bool ta, bool tb, int64_t M_, int64_t N_, const double* X, int64_t ldx, int64_t sX,
                   const double* Yp, int64_t ldy, int64_t sY) {
        Batch2 bt;
        bt.n1 = batch;
        bt.sA1 = sX;
        bt.sB1 = sY;
        bt.sC1 = M_ * N_;
        if (bulk) gemm_bulk(c, ta, tb, M_, N_, kk, 1.0, X, ldx, Yp, ldy, 0.0, Cn.p(), M_, bt, true);
        else gemm_f64(c, ta, tb, M_, N_, kk, 1.0, X, ldx, Yp, ldy, 0.0, Cn.p(), M_, bt);
    };
    if (!best.swap) run(best.ta, best.tb, m, n, pa, lda, sizeA, pb, ldb, sizeB);
    else run(!best.tb, !best.ta, n, m, pb, ldb, sizeB, pa, lda, sizeA);   // C^T = op(B)^T op(A)^T
    bufA.release();
    bufB.release();
    if (!best.permOut) {
        // labels already in output order
        return Cn;
    }
    std::vector<int> perm(lOut.size());
    for (size_t i = 0; i < lOut.size(); ++i) perm[i] = idx_of(nat, lOut[i]);
    if (batch > 1) perm.push_back((int)lOut.size());
    return permuted(c, Cn, perm);
}

namespace {

// out[i + j mr] = X[ro[i] + co[j]]
__global__ void k_gather_offsets(const double* __restrict__ X, const int64_t* __restrict__ ro, int64_t mr,
                                 const int64_t* __restrict__ co, int64_t nc, double* __restrict__ out) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < mr * nc; e += (int64_t)gridDim.x * blockDim.x)
        out[e] = X[ro[e % mr] + co[e / mr]];
}

// X[ro[i] + co[j]] = in[i + j mr]
__global__ void k_scatter_offsets(const double* __restrict__ in, const int64_t* __restrict__ ro, int64_t mr,
                                  const int64_t* __restrict__ co, int64_t nc, double* __restrict__ X) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < mr * nc; e += (int64_t)gridDim.x * blockDim.x)
        X[ro[e % mr] + co[e / mr]] = in[e];
}

unsigned grid_of(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

// Every combination of a group of legs (first leg fastest): its offsets under two stride sets
// and its charge sum mod N (charges from `qs`, one vector per leg).
struct Combos {
    std::vector<int64_t> off1, off2;
    std::vector<int> q;
};
Combos enumerate(const std::vector<int64_t>& dims, const std::vector<int64_t>& st1, const std::vector<int64_t>& st2,
                 const std::vector<const std::vector<int>*>& qs, int N) {
    Combos c;
    int64_t total = 1;
    for (auto d : dims) total *= d;
    c.off1.assign(total, 0);
    c.off2.assign(total, 0);
    c.q.assign(total, 0);
    for (int64_t e = 0; e < total; ++e) {
        int64_t rem = e, o1 = 0, o2 = 0;
        int q = 0;
        for (size_t l = 0; l < dims.size(); ++l) {
            const int64_t i = rem % dims[l];
            rem /= dims[l];
            o1 += i * st1[l];
            o2 += i * st2[l];
            q += (*qs[l])[i];
        }
        c.off1[e] = o1;
        c.off2[e] = o2;
        c.q[e] = ((q % N) + N) % N;
    }
    return c;
}

std::vector<int64_t> col_major_strides(const DT& t) {
    std::vector<int64_t> st(t.rank);
    int64_t s = 1;
    for (int l = 0; l < t.rank; ++l) {
        st[l] = s;
        s *= t.d[l];
    }
    return st;
}

}  // namespace

DT contract_blocked(Ctx& c, const DT& A, const std::vector<int>& lA, const DT& B, const std::vector<int>& lB,
                    const std::vector<int>& lOut, bool bulk) {
    TNR_REQUIRE(A.N == B.N, TNR_ERR_INVALID_ARG, "contract: operands of different Z_N");
    TNR_REQUIRE((int)lA.size() == A.rank && (int)lB.size() == B.rank, TNR_ERR_INVALID_ARG, "contract: rank/labels");
    const int N = A.N;
    std::vector<int> K, FA, FB;
    for (int x : lA) (idx_of(lB, x) >= 0 ? K : FA).push_back(x);
    for (int x : lB)
        if (idx_of(lA, x) < 0) FB.push_back(x);
    TNR_REQUIRE(FA.size() + FB.size() == lOut.size(), TNR_ERR_INVALID_ARG, "contract: output labels");
    const std::vector<int64_t> sA = col_major_strides(A), sB = col_major_strides(B);
    // output layout (lOut order)
    std::vector<int64_t> od;
    std::vector<const std::vector<int>*> oq;
    for (int x : lOut) {
        const int ia = idx_of(lA, x), ib = idx_of(lB, x);
        TNR_REQUIRE((ia >= 0) != (ib >= 0), TNR_ERR_INVALID_ARG, "contract: stray output label");
        od.push_back(ia >= 0 ? A.d[ia] : B.d[ib]);
        oq.push_back(ia >= 0 ? &A.q[ia] : &B.q[ib]);
    }
    DT O = make_dt(c.pool.get(), od);
    O.N = N;
    for (auto* q : oq) O.q.push_back(*q);
    std::vector<int64_t> sO(od.size());
    {
        int64_t st = 1;
        for (size_t l = 0; l < od.size(); ++l) {
            sO[l] = st;
            st *= od[l];
        }
    }
    TNR_CUDA(cudaMemsetAsync(O.p(), 0, (size_t)O.size() * sizeof(double), c.stream));
    // free legs of A: (offset in A, offset in O, charge); contracted: (offset in A, offset in B,
    // charge on A's side); free legs of B: (offset in B, offset in O, charge)
    std::vector<int64_t> dFA, s1FA, s2FA, dK, s1K, s2K, dFB, s1FB, s2FB;
    std::vector<const std::vector<int>*> qFA, qK, qFB;
    for (int x : FA) {
        const int ia = idx_of(lA, x);
        dFA.push_back(A.d[ia]); s1FA.push_back(sA[ia]); s2FA.push_back(sO[idx_of(lOut, x)]); qFA.push_back(&A.q[ia]);
    }
    for (int x : K) {
        const int ia = idx_of(lA, x), ib = idx_of(lB, x);
        TNR_REQUIRE(A.d[ia] == B.d[ib], TNR_ERR_INVALID_ARG, "contract: dim mismatch");
        for (int64_t i = 0; i < A.d[ia]; ++i)
            TNR_REQUIRE(((A.q[ia][i] + B.q[ib][i]) % N + N) % N == 0, TNR_ERR_INVALID_ARG,
                        "contract: contracted legs are not dual (their charges do not cancel)");
        dK.push_back(A.d[ia]); s1K.push_back(sA[ia]); s2K.push_back(sB[ib]); qK.push_back(&A.q[ia]);
    }
    for (int x : FB) {
        const int ib = idx_of(lB, x);
        dFB.push_back(B.d[ib]); s1FB.push_back(sB[ib]); s2FB.push_back(sO[idx_of(lOut, x)]); qFB.push_back(&B.q[ib]);
    }
    const Combos cFA = enumerate(dFA, s1FA, s2FA, qFA, N), cK = enumerate(dK, s1K, s2K, qK, N),
                 cFB = enumerate(dFB, s1FB, s2FB, qFB, N);
    for (int cl = 0; cl < N; ++cl) {
        const int ncl = (N - cl) % N;
        std::vector<int64_t> rA, rO, kA, kB, cB, cO;
        for (size_t e = 0; e < cFA.q.size(); ++e)
            if (cFA.q[e] == cl) { rA.push_back(cFA.off1[e]); rO.push_back(cFA.off2[e]); }
        for (size_t e = 0; e < cK.q.size(); ++e)
            if (cK.q[e] == ncl) { kA.push_back(cK.off1[e]); kB.push_back(cK.off2[e]); }
        for (size_t e = 0; e < cFB.q.size(); ++e)
            if (cFB.q[e] == ncl) { cB.push_back(cFB.off1[e]); cO.push_back(cFB.off2[e]); }
        const int64_t mc = (int64_t)rA.size(), kc = (int64_t)kA.size(), nc = (int64_t)cB.size();
        if (!mc || !kc || !nc) continue;   // an empty sector contributes nothing (O is zero there)
        Buf ofs(c.pool.get(), (size_t)(2 * mc + 2 * kc + 2 * nc) * sizeof(int64_t));
        int64_t* d = ofs.as<int64_t>();
        std::vector<int64_t> all;
        all.reserve(2 * (mc + kc + nc));
        for (auto* v : {&rA, &rO, &kA, &kB, &cB, &cO}) all.insert(all.end(), v->begin(), v->end());
        TNR_CUDA(cudaMemcpyAsync(d, all.data(), all.size() * sizeof(int64_t), cudaMemcpyHostToDevice, c.stream));
        const int64_t *d_rA = d, *d_rO = d + mc, *d_kA = d + 2 * mc, *d_kB = d + 2 * mc + kc,
                      *d_cB = d + 2 * mc + 2 * kc, *d_cO = d + 2 * mc + 2 * kc + nc;
        Buf Ab(c.pool.get(), (size_t)mc * kc * sizeof(double)), Bb(c.pool.get(), (size_t)kc * nc * sizeof(double));
        Buf Cb(c.pool.get(), (size_t)mc * nc * sizeof(double));
        k_gather_offsets<<<grid_of(mc * kc), 256, 0, c.stream>>>(A.p(), d_rA, mc, d_kA, kc, Ab.d());
        check_launch("gather_offsets");
        k_gather_offsets<<<grid_of(kc * nc), 256, 0, c.stream>>>(B.p(), d_kB, kc, d_cB, nc, Bb.d());
        check_launch("gather_offsets");
        if (bulk) gemm_bulk(c, false, false, mc, nc, kc, 1.0, Ab.d(), mc, Bb.d(), kc, 0.0, Cb.d(), mc, Batch2(), true);
        else gemm_f64(c, false, false, mc, nc, kc, 1.0, Ab.d(), mc, Bb.d(), kc, 0.0, Cb.d(), mc, Batch2());
        k_scatter_offsets<<<grid_of(mc * nc), 256, 0, c.stream>>>(Cb.d(), d_rO, mc, d_cO, nc, O.p());
        check_launch("scatter_offsets");
        // (a host-to-device copy from pageable memory has read `all` when it returns)
    }
    return O;
}

}  // namespace tnr
