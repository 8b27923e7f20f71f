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

}  // namespace tnr
