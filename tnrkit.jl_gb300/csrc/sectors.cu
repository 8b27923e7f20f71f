// Truncated SVD over the sectors a matrix's zero pattern reveals.
//
// A tensor with an abelian (Z2) symmetry stored as its dense embedding has exact zeros
// wherever the charges do not match: reshaped to a matrix, its rows and columns split into
// sectors, and every nonzero entry joins a row sector to its column sector.  The sectors are
// the connected components of the bipartite graph "row r -- column c iff M[r, c] != 0".  The
// SVD of such a matrix is the union of the SVDs of its sector blocks, and truncation keeps
// the k largest values over all blocks (MatrixAlgebraKit's global truncrank).  Computing it
// block by block gives singular vectors that are exactly supported on one sector: the basis
// LAPACK's dense SVD returns for these block-structured matrices, and the one ImpurityTRG's
// network needs (its step contracts factors of different SVDs, impuritytrg.jl:84-88, so a
// vector that mixes the sectors of a degenerate pair mixes a Z2-odd impurity into the even
// sector).  The zeros survive every later step exactly: each forbidden entry of a
// contraction is a sum of products that each hold an exact zero factor.
//
// A matrix without exact zeros (a field h != 0, or no symmetry) is one sector, and the call
// is the plain truncated SVD.
#include "common.cuh"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace tnr {

namespace {

// bits[r * words + w] bit b = (M[r, 32 w + b] != 0), M column-major m x n
__global__ void k_nz_bitmap(const double* __restrict__ M, int64_t m, int64_t n, int words, uint32_t* __restrict__ bits) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= m * words) return;
    const int64_t r = e % m;
    const int w = (int)(e / m);
    uint32_t v = 0;
    for (int b = 0; b < 32; ++b) {
        const int64_t c = (int64_t)w * 32 + b;
        if (c < n && M[r + c * m] != 0.0) v |= 1u << b;
    }
    bits[r * words + w] = v;
}

// B[i + j mr] = M[rows[i] + cols[j] m]
__global__ void k_gather_block(const double* __restrict__ M, int64_t m, const int* __restrict__ rows, int mr,
                               const int* __restrict__ cols, int nc, double* __restrict__ B) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= (int64_t)mr * nc) return;
    const int i = (int)(e % mr), j = (int)(e / mr);
    B[e] = M[rows[i] + (int64_t)cols[j] * m];
}

// U[rows[i] + dst[t] m] = Ub[i + src[t] mr]  (cnt kept columns of one sector)
__global__ void k_scatter_cols(const double* __restrict__ Ub, int mr, const int* __restrict__ rows,
                               const int* __restrict__ src, const int* __restrict__ dst, int cnt,
                               double* __restrict__ U, int64_t m) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= (int64_t)mr * cnt) return;
    const int i = (int)(e % mr), t = (int)(e / mr);
    U[rows[i] + (int64_t)dst[t] * m] = Ub[i + (int64_t)src[t] * mr];
}

// Vt[dst[t] + cols[j] k] = Vb[src[t] + j kb]  (Vb: kb x nc, Vt: k x n)
__global__ void k_scatter_rows(const double* __restrict__ Vb, int kb, const int* __restrict__ cols, int nc,
                               const int* __restrict__ src, const int* __restrict__ dst, int cnt,
                               double* __restrict__ Vt, int k) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= (int64_t)cnt * nc) return;
    const int t = (int)(e % cnt), j = (int)(e / cnt);
    Vt[dst[t] + (int64_t)cols[j] * k] = Vb[src[t] + (int64_t)j * kb];
}

unsigned blocks_for(int64_t n) { return (unsigned)std::max<int64_t>(1, (n + 255) / 256); }

struct Sector {
    std::vector<int> rows, cols;
};

// connected components of the bipartite nonzero graph (union-find over m + n nodes)
std::vector<Sector> find_sectors(const std::vector<uint32_t>& bits, int64_t m, int64_t n, int words) {
    std::vector<int> parent(m + n);
    std::iota(parent.begin(), parent.end(), 0);
    auto find = [&](int x) {
        while (parent[x] != x) {
            parent[x] = parent[parent[x]];
            x = parent[x];
        }
        return x;
    };
    for (int64_t r = 0; r < m; ++r)
        for (int w = 0; w < words; ++w) {
            uint32_t v = bits[r * words + w];
            while (v) {
                const int b = __builtin_ctz(v);
                v &= v - 1;
                const int a = find((int)r), c = find((int)(m + (int64_t)w * 32 + b));
                if (a != c) parent[std::max(a, c)] = std::min(a, c);
            }
        }
    std::vector<int> id(m + n, -1);
    std::vector<Sector> out;
    for (int64_t x = 0; x < m + n; ++x) {
        const int root = find((int)x);
        if (id[root] < 0) {
            id[root] = (int)out.size();
            out.emplace_back();
        }
        Sector& s = out[id[root]];
        if (x < m) s.rows.push_back((int)x);
        else s.cols.push_back((int)(x - m));
    }
    return out;
}

}  // namespace

TsvdOut tsvd_sectors(Ctx& c, const double* M, int64_t m, int64_t n, int k, double* U, double* s, double* Vt) {
    const int64_t p = std::min(m, n);
    k = (int)std::min<int64_t>(k, p);
    TNR_REQUIRE(m <= (1 << 30) && n <= (1 << 30), TNR_ERR_UNSUPPORTED, "tsvd_sectors: matrix too large");
    const int words = (int)((n + 31) / 32);
    Buf bitsd(c.pool.get(), (size_t)m * words * sizeof(uint32_t));
    k_nz_bitmap<<<blocks_for(m * words), 256, 0, c.stream>>>(M, m, n, words, bitsd.as<uint32_t>());
    check_launch("nz_bitmap");
    std::vector<uint32_t> bits((size_t)m * words);
    TNR_CUDA(cudaMemcpyAsync(bits.data(), bitsd.d(), bits.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                             c.stream));
    c.sync();
    std::vector<Sector> sec = find_sectors(bits, m, n, words);
    // sectors that hold both rows and columns carry singular values; the rest are zero rows /
    // columns, whose (zero) values only pad the kept set
    std::vector<int> live;
    for (int i = 0; i < (int)sec.size(); ++i)
        if (!sec[i].rows.empty() && !sec[i].cols.empty()) live.push_back(i);
    if (live.size() == 1 && (int64_t)sec[live[0]].rows.size() == m && (int64_t)sec[live[0]].cols.size() == n)
        return tsvd(c, M, m, n, k, U, s, Vt);

    struct Part {
        int sector = 0, kb = 0;
        Buf Ub, Vb;
        std::vector<double> vals;
    };
    std::vector<Part> parts;
    TsvdOut out;
    out.k = k;
    double fro2 = 0;
    for (int id : live) {
        const Sector& S = sec[id];
        const int mr = (int)S.rows.size(), nc = (int)S.cols.size();
        const int kb = std::min({k, mr, nc});
        Buf rows(c.pool.get(), (size_t)mr * sizeof(int)), cols(c.pool.get(), (size_t)nc * sizeof(int));
        TNR_CUDA(cudaMemcpyAsync(rows.d(), S.rows.data(), (size_t)mr * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        TNR_CUDA(cudaMemcpyAsync(cols.d(), S.cols.data(), (size_t)nc * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        Buf B(c.pool.get(), (size_t)mr * nc * sizeof(double));
        k_gather_block<<<blocks_for((int64_t)mr * nc), 256, 0, c.stream>>>(M, m, rows.as<int>(), mr, cols.as<int>(), nc,
                                                                           B.d());
        check_launch("gather_block");
        Part P;
        P.sector = id;
        P.kb = kb;
        P.Ub = Buf(c.pool.get(), (size_t)mr * kb * sizeof(double));
        P.Vb = Buf(c.pool.get(), (size_t)kb * nc * sizeof(double));
        Buf sb(c.pool.get(), (size_t)kb * sizeof(double));
        TsvdOut r = tsvd(c, B.d(), mr, nc, kb, P.Ub.d(), sb.d(), P.Vb.d());
        P.vals = r.vals;
        fro2 += r.fro2;
        c.sync();      // the host index arrays above are copied before they go out of scope
        parts.push_back(std::move(P));
    }
    // global truncation: the k largest values over all sectors, descending (ties keep the
    // lower sector first)
    struct Pick {
        double v;
        int part, idx;
    };
    std::vector<Pick> all;
    for (int q = 0; q < (int)parts.size(); ++q)
        for (int i = 0; i < (int)parts[q].vals.size(); ++i) all.push_back({parts[q].vals[i], q, i});
    std::stable_sort(all.begin(), all.end(), [](const Pick& a, const Pick& b) { return a.v > b.v; });
    const int kept = std::min<int>(k, (int)all.size());
    TNR_CUDA(cudaMemsetAsync(U, 0, (size_t)m * k * sizeof(double), c.stream));
    TNR_CUDA(cudaMemsetAsync(Vt, 0, (size_t)k * n * sizeof(double), c.stream));
    std::vector<double> sv(k, 0.0);
    double kept2 = 0;
    for (int t = 0; t < kept; ++t) {
        sv[t] = all[t].v;
        kept2 += all[t].v * all[t].v;
    }
    TNR_CUDA(cudaMemcpyAsync(s, sv.data(), (size_t)k * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    for (int q = 0; q < (int)parts.size(); ++q) {
        std::vector<int> src, dst;
        for (int t = 0; t < kept; ++t)
            if (all[t].part == q) {
                src.push_back(all[t].idx);
                dst.push_back(t);
            }
        if (src.empty()) continue;
        const Sector& S = sec[parts[q].sector];
        const int mr = (int)S.rows.size(), nc = (int)S.cols.size(), cnt = (int)src.size();
        Buf rows(c.pool.get(), (size_t)mr * sizeof(int)), cols(c.pool.get(), (size_t)nc * sizeof(int));
        Buf srcd(c.pool.get(), (size_t)cnt * sizeof(int)), dstd(c.pool.get(), (size_t)cnt * sizeof(int));
        TNR_CUDA(cudaMemcpyAsync(rows.d(), S.rows.data(), (size_t)mr * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        TNR_CUDA(cudaMemcpyAsync(cols.d(), S.cols.data(), (size_t)nc * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        TNR_CUDA(cudaMemcpyAsync(srcd.d(), src.data(), (size_t)cnt * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        TNR_CUDA(cudaMemcpyAsync(dstd.d(), dst.data(), (size_t)cnt * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        k_scatter_cols<<<blocks_for((int64_t)mr * cnt), 256, 0, c.stream>>>(parts[q].Ub.d(), mr, rows.as<int>(),
                                                                            srcd.as<int>(), dstd.as<int>(), cnt, U, m);
        check_launch("scatter_cols");
        k_scatter_rows<<<blocks_for((int64_t)cnt * nc), 256, 0, c.stream>>>(parts[q].Vb.d(), parts[q].kb,
                                                                            cols.as<int>(), nc, srcd.as<int>(),
                                                                            dstd.as<int>(), cnt, Vt, k);
        check_launch("scatter_rows");
        c.sync();
    }
    out.fro2 = fro2;
    out.err = std::sqrt(std::max(fro2 - kept2, 0.0));
    out.vals = sv;
    return out;
}

namespace {

// Row and column classes of a charged tensor's (row legs <- column legs) matrix, first leg
// fastest: row class = (sum of the row legs' charges) mod N, column class = -(sum of the column
// legs' charges) mod N; every nonzero entry joins a row and a column of the same class.
void matrix_classes(const DT& M, int nrow, std::vector<int>& rc, std::vector<int>& cc) {
    const int N = M.N;
    auto classes = [&](int l0, int l1, int sign, std::vector<int>& out) {
        int64_t total = 1;
        for (int l = l0; l < l1; ++l) total *= M.d[l];
        out.assign(total, 0);
        for (int64_t e = 0; e < total; ++e) {
            int64_t rem = e;
            int q = 0;
            for (int l = l0; l < l1; ++l) {
                q += M.q[l][rem % M.d[l]];
                rem /= M.d[l];
            }
            out[e] = (((sign * q) % N) + N) % N;
        }
    };
    classes(0, nrow, 1, rc);
    classes(nrow, M.rank, -1, cc);
}

DecompDT decompose_charged(Ctx& c, const DT& M, int nrow, int chi, bool eigh) {
    const int N = M.N;
    std::vector<int> rc, cc;
    matrix_classes(M, nrow, rc, cc);
    const int64_t m = (int64_t)rc.size(), n = (int64_t)cc.size();
    struct Part {
        int cls = 0, kb = 0;
        std::vector<int> rows, cols;
        Buf Ub, Vb;
        std::vector<double> vals;
    };
    std::vector<Part> parts;
    double fro2 = 0;
    for (int cl = 0; cl < N; ++cl) {
        Part P;
        P.cls = cl;
        for (int64_t i = 0; i < m; ++i)
            if (rc[i] == cl) P.rows.push_back((int)i);
        for (int64_t j = 0; j < n; ++j)
            if (cc[j] == cl) P.cols.push_back((int)j);
        if (P.rows.empty() || P.cols.empty()) continue;
        if (eigh)
            TNR_REQUIRE(P.rows == P.cols, TNR_ERR_INVALID_ARG,
                        "eigh of a charged tensor: row and column sectors differ (not a Gram matrix)");
        const int mr = (int)P.rows.size(), nc = (int)P.cols.size();
        P.kb = std::min({chi, mr, nc});
        if (P.kb <= 0) continue;
        Buf rows(c.pool.get(), (size_t)mr * sizeof(int)), cols(c.pool.get(), (size_t)nc * sizeof(int));
        TNR_CUDA(cudaMemcpyAsync(rows.d(), P.rows.data(), (size_t)mr * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        TNR_CUDA(cudaMemcpyAsync(cols.d(), P.cols.data(), (size_t)nc * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        Buf Bm(c.pool.get(), (size_t)mr * nc * sizeof(double));
        k_gather_block<<<blocks_for((int64_t)mr * nc), 256, 0, c.stream>>>(M.p(), m, rows.as<int>(), mr,
                                                                            cols.as<int>(), nc, Bm.d());
        check_launch("gather_block");
        P.Ub = Buf(c.pool.get(), (size_t)mr * P.kb * sizeof(double));
        Buf sb(c.pool.get(), (size_t)P.kb * sizeof(double));
        TsvdOut r;
        // a sector block far wider than the values it keeps goes through subspace iteration:
        // the direct path would run the one-CTA solvers on the whole block
        const int p = std::min(mr, nc), direct_max = (3 * P.kb + 8 >= p) ? 128 : 64;
        if (eigh) {
            r = teigh(c, Bm.d(), mr, P.kb, P.Ub.d(), sb.d(), direct_max);
        } else {
            P.Vb = Buf(c.pool.get(), (size_t)P.kb * nc * sizeof(double));
            r = tsvd(c, Bm.d(), mr, nc, P.kb, P.Ub.d(), sb.d(), P.Vb.d(), direct_max);
        }
        P.vals = r.vals;
        fro2 += r.fro2;
        parts.push_back(std::move(P));
    }
    // global truncation over the sectors: the chi largest |values|, descending; ties keep the
    // lower sector, then the lower index, first
    struct Pick {
        double a;
        int part, idx;
    };
    std::vector<Pick> all;
    for (int p = 0; p < (int)parts.size(); ++p)
        for (int i = 0; i < (int)parts[p].vals.size(); ++i) all.push_back({std::fabs(parts[p].vals[i]), p, i});
    std::stable_sort(all.begin(), all.end(), [](const Pick& a, const Pick& b) { return a.a > b.a; });
    const int k = std::min<int>(chi, (int)all.size());
    TNR_REQUIRE(k >= 1, TNR_ERR_INVALID_ARG, "decomposition of a charged tensor with no nonzero sector");
    DecompDT out;
    out.k = k;
    std::vector<int64_t> ud(M.d, M.d + nrow), vd{(int64_t)k};
    ud.push_back(k);
    for (int l = nrow; l < M.rank; ++l) vd.push_back(M.d[l]);
    out.U = make_dt(c.pool.get(), ud);
    TNR_CUDA(cudaMemsetAsync(out.U.p(), 0, (size_t)out.U.size() * sizeof(double), c.stream));
    if (!eigh) {
        out.Vt = make_dt(c.pool.get(), vd);
        TNR_CUDA(cudaMemsetAsync(out.Vt.p(), 0, (size_t)out.Vt.size() * sizeof(double), c.stream));
    }
    std::vector<double> sv(k);
    std::vector<int> bond(k);
    double kept2 = 0;
    for (int t = 0; t < k; ++t) {
        sv[t] = parts[all[t].part].vals[all[t].idx];
        bond[t] = parts[all[t].part].cls;
        kept2 += sv[t] * sv[t];
    }
    out.s = Buf(c.pool.get(), (size_t)k * sizeof(double));
    TNR_CUDA(cudaMemcpyAsync(out.s.d(), sv.data(), (size_t)k * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    for (int p = 0; p < (int)parts.size(); ++p) {
        std::vector<int> src, dst;
        for (int t = 0; t < k; ++t)
            if (all[t].part == p) {
                src.push_back(all[t].idx);
                dst.push_back(t);
            }
        if (src.empty()) continue;
        const Part& P = parts[p];
        const int mr = (int)P.rows.size(), nc = (int)P.cols.size(), cnt = (int)src.size();
        Buf rows(c.pool.get(), (size_t)mr * sizeof(int)), cols(c.pool.get(), (size_t)nc * sizeof(int));
        Buf srcd(c.pool.get(), (size_t)cnt * sizeof(int)), dstd(c.pool.get(), (size_t)cnt * sizeof(int));
        TNR_CUDA(cudaMemcpyAsync(rows.d(), P.rows.data(), (size_t)mr * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        TNR_CUDA(cudaMemcpyAsync(cols.d(), P.cols.data(), (size_t)nc * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        TNR_CUDA(cudaMemcpyAsync(srcd.d(), src.data(), (size_t)cnt * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        TNR_CUDA(cudaMemcpyAsync(dstd.d(), dst.data(), (size_t)cnt * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        k_scatter_cols<<<blocks_for((int64_t)mr * cnt), 256, 0, c.stream>>>(P.Ub.d(), mr, rows.as<int>(),
                                                                            srcd.as<int>(), dstd.as<int>(), cnt,
                                                                            out.U.p(), m);
        check_launch("scatter_cols");
        if (!eigh) {
            k_scatter_rows<<<blocks_for((int64_t)cnt * nc), 256, 0, c.stream>>>(P.Vb.d(), P.kb, cols.as<int>(), nc,
                                                                                srcd.as<int>(), dstd.as<int>(), cnt,
                                                                                out.Vt.p(), k);
            check_launch("scatter_rows");
        }
    }
    out.U.N = N;
    for (int l = 0; l < nrow; ++l) out.U.q.push_back(M.q[l]);
    std::vector<int> qu(k), qv(k);
    for (int t = 0; t < k; ++t) {
        qu[t] = (N - bond[t]) % N;
        qv[t] = bond[t];
    }
    out.U.q.push_back(qu);
    if (!eigh) {
        out.Vt.N = N;
        out.Vt.q.push_back(qv);
        for (int l = nrow; l < M.rank; ++l) out.Vt.q.push_back(M.q[l]);
    }
    out.info.k = k;
    out.info.fro2 = fro2;
    out.info.err = std::sqrt(std::max(fro2 - kept2, 0.0));
    out.info.vals = sv;
    c.sync();      // every host index vector above outlives its copies
    return out;
}

DecompDT decompose_plain(Ctx& c, const DT& M, int nrow, int chi, bool eigh) {
    int64_t m = 1, n = 1;
    for (int l = 0; l < nrow; ++l) m *= M.d[l];
    for (int l = nrow; l < M.rank; ++l) n *= M.d[l];
    const int k = (int)std::min<int64_t>(chi, std::min(m, n));
    DecompDT out;
    out.k = k;
    std::vector<int64_t> ud(M.d, M.d + nrow), vd{(int64_t)k};
    ud.push_back(k);
    for (int l = nrow; l < M.rank; ++l) vd.push_back(M.d[l]);
    out.U = make_dt(c.pool.get(), ud);
    out.s = Buf(c.pool.get(), (size_t)k * sizeof(double));
    if (eigh) {
        out.info = teigh(c, M.p(), m, k, out.U.p(), out.s.d());
    } else {
        out.Vt = make_dt(c.pool.get(), vd);
        out.info = tsvd(c, M.p(), m, n, k, out.U.p(), out.s.d(), out.Vt.p());
    }
    return out;
}

}  // namespace

DecompDT svd_dt(Ctx& c, const DT& M, int nrow, int chi) {
    return M.charged() ? decompose_charged(c, M, nrow, chi, false) : decompose_plain(c, M, nrow, chi, false);
}

DecompDT eigh_dt(Ctx& c, const DT& MM, int nrow, int chi) {
    return MM.charged() ? decompose_charged(c, MM, nrow, chi, true) : decompose_plain(c, MM, nrow, chi, true);
}

}  // namespace tnr
