// Pairwise tensor contraction as permute -> GEMM -> permute (the @tensor /
// @plansor / @tensoropt pairwise steps of TensorOperations, restated).  The
// planner picks, among the layouts that need the fewest moved elements, one
// GEMM over the grouped legs; every permute is the shared-memory tiled kernel.
#include "common.cuh"

#include <algorithm>
#include <cstring>

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

// out[i + j ld] = X[ro[i] + co[j]], i < mr, j < nc
__global__ void k_gather_offsets(const double* __restrict__ X, const int64_t* __restrict__ ro, int64_t mr,
                                 const int64_t* __restrict__ co, int64_t nc, double* __restrict__ out, int64_t ld) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < mr * nc; e += (int64_t)gridDim.x * blockDim.x)
        out[e % mr + (e / mr) * ld] = X[ro[e % mr] + co[e / mr]];
}

// X[ro[i] + co[j]] = in[i + j ld], i < mr, j < nc
__global__ void k_scatter_offsets(const double* __restrict__ in, int64_t ld, const int64_t* __restrict__ ro,
                                  int64_t mr, const int64_t* __restrict__ co, int64_t nc, double* __restrict__ X) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < mr * nc; e += (int64_t)gridDim.x * blockDim.x)
        X[ro[e % mr] + co[e / mr]] = in[e % mr + (e / mr) * ld];
}

unsigned grid_of(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

// A group of legs (first leg fastest) split by charge class.  Every leg's basis indices are
// listed class by class on the host (O(sum of dims)); a class of the group is the union of the
// products of per-leg lists whose classes sum to it ("tuples", at most N^L of them), and the
// device expands the tuples into the combinations' offsets under two stride sets.  Nothing of
// size O(combinations) is built or copied on the host.
constexpr int MAXL = MAXR;
struct TupleDesc {
    int64_t start, size;          // position of the tuple in its class's list, its combinations
    int off[MAXL], len[MAXL];     // per leg: the class list's offset in `lists` and its length
};

__global__ void k_expand_offsets(const TupleDesc* __restrict__ tup, int ntup, const int* __restrict__ lists, int L,
                                 const int64_t* __restrict__ st, int64_t total, int64_t* __restrict__ o1,
                                 int64_t* __restrict__ o2) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = ntup - 1;             // the last tuple whose start is <= e
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (tup[mid].start <= e) lo = mid;
            else hi = mid - 1;
        }
        const int t = lo;
        int64_t j = e - tup[t].start, a = 0, b = 0;
        for (int l = 0; l < L; ++l) {
            const int n = tup[t].len[l];
            const int i = lists[tup[t].off[l] + (int)(j % n)];
            j /= n;
            a += (int64_t)i * st[l];
            b += (int64_t)i * st[MAXL + l];
        }
        o1[e] = a;
        o2[e] = b;
    }
}

struct GroupPlan {
    std::vector<int> lists;                      // per leg, per class: the basis indices
    std::vector<std::vector<TupleDesc>> tuples;  // per class of the group
    std::vector<int64_t> count;                  // per class: combinations
};

GroupPlan plan_group(const std::vector<int64_t>& dims, const std::vector<const std::vector<int>*>& qs, int N) {
    const int L = (int)dims.size();
    TNR_REQUIRE(L <= MAXL, TNR_ERR_UNSUPPORTED, "contract: too many legs in a group");
    GroupPlan g;
    std::vector<std::vector<int>> off(L, std::vector<int>(N, 0)), len(L, std::vector<int>(N, 0));
    for (int l = 0; l < L; ++l)
        for (int cl = 0; cl < N; ++cl) {
            off[l][cl] = (int)g.lists.size();
            for (int64_t i = 0; i < dims[l]; ++i)
                if ((*qs[l])[i] == cl) g.lists.push_back((int)i);
            len[l][cl] = (int)g.lists.size() - off[l][cl];
        }
    g.tuples.assign(N, {});
    g.count.assign(N, 0);
    int64_t ntuples = 1;
    for (int l = 0; l < L; ++l) ntuples *= N;
    for (int64_t t = 0; t < ntuples; ++t) {
        int64_t r = t, size = 1;
        int sum = 0;
        TupleDesc d{};
        for (int l = 0; l < L; ++l) {
            const int cl = (int)(r % N);
            r /= N;
            sum += cl;
            d.off[l] = off[l][cl];
            d.len[l] = len[l][cl];
            size *= d.len[l];
        }
        if (size == 0) continue;
        const int cl = sum % N;
        d.start = g.count[cl];
        d.size = size;
        g.count[cl] += size;
        g.tuples[cl].push_back(d);
    }
    return g;
}

// device offsets of one class of a group (tuples `d_t`, `ntup` of them; lists and strides on the
// device): o1 / o2 under the two stride sets.  An empty group (L = 0) is the single
// combination with offset 0.
void expand_class(Ctx& c, const TupleDesc* d_t, int ntup, int64_t total, const int* d_lists, int L,
                  const int64_t* d_st, int64_t* o1, int64_t* o2) {
    if (!ntup || !total) return;
    k_expand_offsets<<<grid_of(total), 256, 0, c.stream>>>(d_t, ntup, d_lists, L, d_st, total, o1, o2);
    check_launch("expand_offsets");
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
    const GroupPlan g[3] = {plan_group(dFA, qFA, N), plan_group(dK, qK, N), plan_group(dFB, qFB, N)};
    const std::vector<int64_t>* st[3][2] = {{&s1FA, &s2FA}, {&s1K, &s2K}, {&s1FB, &s2FB}};
    // everything the device needs in one upload: per group its strides, per-leg class lists and
    // tuples of every class (one host-to-device copy per contraction)
    std::vector<unsigned char> blob;
    auto put = [&](const void* p, size_t bytes) {
        const size_t at = (blob.size() + 15) / 16 * 16;
        blob.resize(at + bytes);
        if (bytes) std::memcpy(blob.data() + at, p, bytes);
        return at;
    };
    size_t at_st[3], at_lists[3];
    std::vector<size_t> at_tup[3];
    for (int q = 0; q < 3; ++q) {
        at_tup[q].assign(N, 0);
        int64_t sv[2 * MAXL] = {};
        for (size_t l = 0; l < st[q][0]->size(); ++l) {
            sv[l] = (*st[q][0])[l];
            sv[MAXL + l] = (*st[q][1])[l];
        }
        at_st[q] = put(sv, sizeof sv);
        at_lists[q] = put(g[q].lists.data(), g[q].lists.size() * sizeof(int));
        for (int cl = 0; cl < N; ++cl)
            at_tup[q][cl] = put(g[q].tuples[cl].data(), g[q].tuples[cl].size() * sizeof(TupleDesc));
    }
    Buf dblob(c.pool.get(), std::max<size_t>(blob.size(), 16));
    TNR_CUDA(cudaMemcpyAsync(dblob.d(), blob.data(), blob.size(), cudaMemcpyHostToDevice, c.stream));
    const unsigned char* base = dblob.as<unsigned char>();
    auto expand = [&](int q, int cl, int64_t* o1, int64_t* o2) {
        expand_class(c, reinterpret_cast<const TupleDesc*>(base + at_tup[q][cl]), (int)g[q].tuples[cl].size(),
                     g[q].count[cl], reinterpret_cast<const int*>(base + at_lists[q]), (int)st[q][0]->size(),
                     reinterpret_cast<const int64_t*>(base + at_st[q]), o1, o2);
    };
    for (int cl = 0; cl < N; ++cl) {
        const int ncl = (N - cl) % N;
        const int64_t mc = g[0].count[cl], kc = g[1].count[ncl], nc = g[2].count[ncl];
        if (!mc || !kc || !nc) continue;   // an empty sector contributes nothing (O is zero there)
        Buf ofs(c.pool.get(), (size_t)(2 * mc + 2 * kc + 2 * nc) * sizeof(int64_t));
        int64_t* d = ofs.as<int64_t>();
        int64_t *d_rA = d, *d_rO = d + mc, *d_kA = d + 2 * mc, *d_kB = d + 2 * mc + kc,
                *d_cB = d + 2 * mc + 2 * kc, *d_cO = d + 2 * mc + 2 * kc + nc;
        expand(0, cl, d_rA, d_rO);
        expand(1, ncl, d_kA, d_kB);
        expand(2, ncl, d_cB, d_cO);
        // The sector GEMM C_c = A_c B_c (mc x kc by kc x nc).  Sector blocks can be thin (a
        // single Z2 leg of chi = 16 leaves 8 columns), below the tensor-core kernel's limits
        // (rows >= 64, columns >= 16, K >= 16): in split precision a thin block is computed
        // transposed when that gives it 64 rows (C_c^T = B_c^T A_c^T), and its columns and K
        // are zero-padded to 16, rather than falling back to the FP64 pipe.
        const bool split = bulk && c.precision == TNR_PREC_SPLIT;
        const bool swap = split && mc < 64 && nc >= 64;
        const int64_t M = swap ? nc : mc, Nn = swap ? mc : nc;
        const int64_t *gA_r = swap ? d_cB : d_rA, *gA_c = swap ? d_kB : d_kA;    // rows / K offsets of op "A"
        const int64_t *gB_r = swap ? d_kA : d_kB, *gB_c = swap ? d_rA : d_cB;    // K / column offsets of op "B"
        const int64_t *sO_r = swap ? d_cO : d_rO, *sO_c = swap ? d_rO : d_cO;
        const double* XA = swap ? B.p() : A.p();
        const double* XB = swap ? A.p() : B.p();
        const bool pad = split && M >= 64 && (Nn < 16 || kc < 16);
        const int64_t Np = pad ? std::max<int64_t>(Nn, 16) : Nn, Kp = pad ? std::max<int64_t>(kc, 16) : kc;
        Buf Ab(c.pool.get(), (size_t)M * Kp * sizeof(double)), Bb(c.pool.get(), (size_t)Kp * Np * sizeof(double));
        Buf Cb(c.pool.get(), (size_t)M * Np * sizeof(double));
        if (Kp > kc) TNR_CUDA(cudaMemsetAsync(Ab.d(), 0, (size_t)M * Kp * sizeof(double), c.stream));
        if (Kp > kc || Np > Nn) TNR_CUDA(cudaMemsetAsync(Bb.d(), 0, (size_t)Kp * Np * sizeof(double), c.stream));
        k_gather_offsets<<<grid_of(M * kc), 256, 0, c.stream>>>(XA, gA_r, M, gA_c, kc, Ab.d(), M);
        check_launch("gather_offsets");
        k_gather_offsets<<<grid_of(kc * Nn), 256, 0, c.stream>>>(XB, gB_r, kc, gB_c, Nn, Bb.d(), Kp);
        check_launch("gather_offsets");
        if (bulk) gemm_bulk(c, false, false, M, Np, Kp, 1.0, Ab.d(), M, Bb.d(), Kp, 0.0, Cb.d(), M, Batch2(), true);
        else gemm_f64(c, false, false, M, Np, Kp, 1.0, Ab.d(), M, Bb.d(), Kp, 0.0, Cb.d(), M, Batch2());
        k_scatter_offsets<<<grid_of(M * Nn), 256, 0, c.stream>>>(Cb.d(), M, sO_r, M, sO_c, Nn, O.p());
        check_launch("scatter_offsets");
    }
    return O;
}

}  // namespace tnr
