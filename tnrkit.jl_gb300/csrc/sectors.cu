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

}  // namespace tnr
