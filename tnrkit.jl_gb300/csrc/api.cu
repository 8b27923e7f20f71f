// C ABI of the engine (include/tnr_gb300.h).  Every entry point catches
// exceptions and returns a status code; nothing aborts the process.
#include "schemes.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <map>
#include <mutex>
#include <thread>

using namespace tnr;

struct tnr_handle_s {
    Scheme s;
};

namespace {
thread_local std::string g_err;

int fail(tnr_handle h, int code, const std::string& msg) {
    g_err = msg;
    if (h) h->s.err = msg;
    return code;
}

template <class F>
int guarded(tnr_handle h, F&& f) {
    try {
        f();
        return TNR_OK;
    } catch (const Error& e) {
        return fail(h, e.code, e.what());
    } catch (const std::bad_alloc&) {
        return fail(h, TNR_ERR_OOM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(h, TNR_ERR_CUDA, e.what());
    }
}

void require_device() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        throw Error(TNR_ERR_NO_DEVICE, "no CUDA device available");
    }
}

void validate_charges(int kind, int nlegs, const int64_t* dims, const double* host, const tnr_options* o) {
    if (!o || o->symmetry_n <= 1 || !o->leg_charges || !host) return;
    // signed charges: codomain legs (2 for every scheme here) +q, domain legs -q
    const int N = o->symmetry_n;
    const int nout = 2;
    std::vector<int64_t> off(nlegs + 1, 0);
    for (int l = 0; l < nlegs; ++l) off[l + 1] = off[l] + dims[l];
    int64_t total = 1;
    for (int l = 0; l < nlegs; ++l) total *= dims[l];
    double maxabs = 0;
    for (int64_t e = 0; e < total; ++e) maxabs = std::max(maxabs, std::fabs(host[e]));
    for (int64_t e = 0; e < total; ++e) {
        int64_t rem = e;
        int q = 0;
        for (int l = 0; l < nlegs; ++l) {
            int64_t i = rem % dims[l];
            rem /= dims[l];
            int ch = o->leg_charges[off[l] + i];
            q += (l < nout) ? ch : -ch;
        }
        q = ((q % N) + N) % N;
        if (q != 0 && std::fabs(host[e]) > 1e-12 * maxabs)
            throw Error(TNR_ERR_INVALID_ARG, "tensor violates Z_N charge conservation of the given leg charges");
    }
    (void)kind;
}

int create_common(tnr_handle* out, int kind, int nlegs, const int64_t* dims, const double* data, bool device,
                  const tnr_options* opts) {
    tnr_options o;
    tnr_default_options(&o);
    if (opts) o = *opts;
    if (!out) return fail(nullptr, TNR_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if ((kind < TNR_TRG || kind > TNR_HOTRG_3D) && kind != TNR_ATRG && kind != TNR_ATRG_3D)
        return fail(nullptr, TNR_ERR_INVALID_ARG, "unknown scheme kind");
    int want = kind == TNR_HOTRG_3D || kind == TNR_ATRG_3D ? 6 : 4;
    if (nlegs != want || !dims || !data)
        return fail(nullptr, TNR_ERR_INVALID_ARG, "scheme needs a " + std::to_string(want) + "-leg tensor");
    for (int l = 0; l < nlegs; ++l)
        if (dims[l] < 1) return fail(nullptr, TNR_ERR_INVALID_ARG, "leg dimension < 1");
    if (o.precision != TNR_PREC_F64 && o.precision != TNR_PREC_SPLIT)
        return fail(nullptr, TNR_ERR_INVALID_ARG, "unknown precision");
    tnr_handle h = new (std::nothrow) tnr_handle_s();
    if (!h) return fail(nullptr, TNR_ERR_OOM, "host allocation failed");
    int st = guarded(h, [&] {
        require_device();
        if (!device) {
            for (int64_t e = 0, t = [&] { int64_t p = 1; for (int l = 0; l < nlegs; ++l) p *= dims[l]; return p; }();
                 e < t; ++e)
                TNR_REQUIRE(std::isfinite(data[e]), TNR_ERR_NONFINITE, "non-finite entry in the input tensor");
            validate_charges(kind, nlegs, dims, data, &o);
        }
        Scheme& s = h->s;
        s.kind = kind;
        s.btrg_k = o.btrg_k;
        s.ctx.reset(new Ctx((cudaStream_t)o.stream, o.precision, o.seed));
        std::vector<int64_t> dv(dims, dims + nlegs);
        s.T = make_dt(s.ctx->pool.get(), dv);
        if (o.symmetry_n > 1 && o.leg_charges &&
            (kind == TNR_TRG || kind == TNR_BTRG || kind == TNR_HOTRG || (kind == TNR_HOTRG_3D && o.symmetry_n == 2))) {
            // Z_N tensors run block by block over the charge sectors: signed charges, +q on
            // the two codomain legs and -q on the domain legs (HOTRG_3D: Z2, whose charges are
            // self-dual, as its network's adjoint legs assume)
            const int N = o.symmetry_n;
            s.T.N = N;
            int64_t off = 0;
            for (int l = 0; l < nlegs; ++l) {
                std::vector<int> q((size_t)dims[l]);
                for (int64_t i = 0; i < dims[l]; ++i) {
                    const int ch = o.leg_charges[off + i];
                    q[i] = (((l < 2 ? ch : -ch) % N) + N) % N;
                }
                off += dims[l];
                s.T.q.push_back(q);
            }
        }
        TNR_CUDA(cudaMemcpyAsync(s.T.p(), data, s.T.size() * sizeof(double),
                                 device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s.ctx->stream));
        if (kind == TNR_BTRG) {
            // S1 = id(space(T, 2)), S2 = id(space(T, 1))  (btrg.jl:39-44)
            s.S1 = make_dt(s.ctx->pool.get(), {dims[1]});
            s.S2 = make_dt(s.ctx->pool.get(), {dims[0]});
            std::vector<double> ones((size_t)std::max(dims[0], dims[1]), 1.0);
            TNR_CUDA(cudaMemcpyAsync(s.S1.p(), ones.data(), dims[1] * sizeof(double), cudaMemcpyHostToDevice, s.ctx->stream));
            TNR_CUDA(cudaMemcpyAsync(s.S2.p(), ones.data(), dims[0] * sizeof(double), cudaMemcpyHostToDevice, s.ctx->stream));
        }
        s.ctx->sync();
    });
    if (st != TNR_OK) {
        delete h;
        return st;
    }
    *out = h;
    return TNR_OK;
}
}  // namespace

extern "C" {

void tnr_default_options(tnr_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->precision = TNR_PREC_F64;
    o->btrg_k = -0.5;
    o->symmetry_n = 1;
}

int tnr_create(tnr_handle* out, int kind, int nlegs, const int64_t* dims, const double* data, const tnr_options* opts) {
    return create_common(out, kind, nlegs, dims, data, false, opts);
}

int tnr_create_device(tnr_handle* out, int kind, int nlegs, const int64_t* dims, const double* data,
                      const tnr_options* opts) {
    return create_common(out, kind, nlegs, dims, data, true, opts);
}

// A scheme holding impurity tensors beside the pure one: all share the pure tensor's dims
static int create_impurity(tnr_handle* out, int kind, const char* name, const int64_t* dims, const double* T,
                           std::initializer_list<const double*> imps, const tnr_options* opts, int dist = 0) {
    if (!out) return fail(nullptr, TNR_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    bool null_arg = !dims || !T;
    for (const double* p : imps) null_arg = null_arg || !p;
    if (null_arg) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL tensor or dims");
    for (int l = 0; l < 4; ++l)
        if (dims[l] < 1) return fail(nullptr, TNR_ERR_INVALID_ARG, "leg dimension < 1");
    if (dims[0] != dims[3] || dims[1] != dims[2])
        return fail(nullptr, TNR_ERR_INVALID_ARG, std::string(name) + " needs d1 == d4 and d2 == d3");
    if (dist < 0) return fail(nullptr, TNR_ERR_INVALID_ARG, "Distance must be non-negative");
    tnr_handle h = nullptr;
    int st = create_common(&h, kind == TNR_IMPURITY_TRG ? TNR_TRG : TNR_HOTRG, 4, dims, T, false, opts);
    if (st != TNR_OK) return st;
    st = guarded(h, [&] {
        Scheme& s = h->s;
        const int64_t n = dims[0] * dims[1] * dims[2] * dims[3];
        DT* hotrg_dst[3] = {&s.I11, &s.I12, &s.I2};
        DT* corr_dst[2] = {&s.C1, &s.C2};
        int i = 0;
        for (const double* src : imps) {
            for (int64_t e = 0; e < n; ++e)
                TNR_REQUIRE(std::isfinite(src[e]), TNR_ERR_NONFINITE, "non-finite entry in an impurity tensor");
            DT& dst = kind == TNR_IMPURITY_HOTRG ? *hotrg_dst[i] : kind == TNR_CORRELATION_HOTRG ? *corr_dst[i] : s.site[i];
            dst = make_dt(s.ctx->pool.get(), {dims[0], dims[1], dims[2], dims[3]});
            TNR_CUDA(cudaMemcpyAsync(dst.p(), src, n * sizeof(double), cudaMemcpyHostToDevice, s.ctx->stream));
            ++i;
        }
        s.kind = kind;
        s.corr_dist = dist;
        s.ctx->sync();
    });
    if (st != TNR_OK) {
        tnr_destroy(h);
        return st;
    }
    *out = h;
    return TNR_OK;
}

int tnr_create_impurity_hotrg(tnr_handle* out, const int64_t* dims, const double* T, const double* T11,
                              const double* T12, const double* T2, const tnr_options* opts) {
    return create_impurity(out, TNR_IMPURITY_HOTRG, "ImpurityHOTRG", dims, T, {T11, T12, T2}, opts);
}

int tnr_create_impurity_trg(tnr_handle* out, const int64_t* dims, const double* T, const double* T_imp1,
                            const double* T_imp2, const double* T_imp3, const double* T_imp4,
                            const tnr_options* opts) {
    return create_impurity(out, TNR_IMPURITY_TRG, "ImpurityTRG", dims, T, {T_imp1, T_imp2, T_imp3, T_imp4}, opts);
}

int tnr_create_correlation_hotrg(tnr_handle* out, const int64_t* dims, const double* Tpure, const double* Timp1,
                                 const double* Timp2, int dist, const tnr_options* opts) {
    return create_impurity(out, TNR_CORRELATION_HOTRG, "CorrelationHOTRG", dims, Tpure, {Timp1, Timp2}, opts, dist);
}

int tnr_run_correlation(tnr_handle h, int chi, int maxiter, double* norms_out, size_t cap, size_t* n_out) {
    if (!h) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL handle");
    return guarded(h, [&] {
        TNR_REQUIRE(h->s.kind == TNR_CORRELATION_HOTRG, TNR_ERR_INVALID_ARG, "not a CorrelationHOTRG handle");
        TNR_REQUIRE(maxiter > h->s.corr_dist, TNR_ERR_INVALID_ARG, "run!: maxiter must be larger than dist");
        TNR_REQUIRE(norms_out && cap >= 3 * (size_t)maxiter, TNR_ERR_INVALID_ARG, "norms_out too small for run!");
        std::vector<double> v = h->s.run_correlation(chi, maxiter);
        std::memcpy(norms_out, v.data(), v.size() * sizeof(double));
        if (n_out) *n_out = v.size() / 3;
    });
}

int tnr_correlation_ratio(tnr_handle h, double* out) {
    if (!h || !out) return fail(h, TNR_ERR_INVALID_ARG, "NULL argument");
    return guarded(h, [&] {
        Scheme& s = h->s;
        TNR_REQUIRE(s.kind == TNR_CORRELATION_HOTRG, TNR_ERR_INVALID_ARG, "not a CorrelationHOTRG handle");
        TNR_REQUIRE(s.Cf.size() > 0, TNR_ERR_INVALID_ARG, "the impurities have not merged yet (steps <= dist)");
        Buf d2(s.ctx->pool.get(), 2 * sizeof(double));
        trace2d(*s.ctx, s.T.p(), s.T.d, d2.d());
        trace2d(*s.ctx, s.Cf.p(), s.Cf.d, d2.d() + 1);
        double tr[2];
        TNR_CUDA(cudaMemcpyAsync(tr, d2.d(), sizeof tr, cudaMemcpyDeviceToHost, s.ctx->stream));
        s.ctx->sync();
        TNR_REQUIRE(std::isfinite(tr[0]) && std::isfinite(tr[1]) && tr[0] > 0, TNR_ERR_NONFINITE,
                    "correlation: non-finite or zero trace");
        *out = tr[1] / tr[0];
    });
}

int tnr_set_finalizer(tnr_handle h, int finalizer) {
    if (!h) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL handle");
    return guarded(h, [&] {
        Scheme& s = h->s;
        TNR_REQUIRE(finalizer == TNR_FINALIZER_DEFAULT || finalizer == TNR_FINALIZER_TWO_BY_TWO,
                    TNR_ERR_INVALID_ARG, "unknown finalizer");
        TNR_REQUIRE(finalizer == TNR_FINALIZER_DEFAULT || s.kind == TNR_TRG || s.kind == TNR_BTRG ||
                        s.kind == TNR_HOTRG || s.kind == TNR_ATRG,
                    TNR_ERR_INVALID_ARG, "the 2 x 2 finalizer needs a TRG, BTRG, HOTRG or ATRG scheme");
        s.finalizer = finalizer == TNR_FINALIZER_TWO_BY_TWO ? FINALIZER_TWO_BY_TWO : FINALIZER_DEFAULT;
    });
}

int tnr_transfer_eigvals(tnr_handle h, int unitcell, double* re, double* im, size_t cap, size_t* n_out) {
    if (!h || !re || !im) return fail(h, TNR_ERR_INVALID_ARG, "NULL argument");
    return guarded(h, [&] {
        std::vector<double> wr, wi;
        h->s.transfer_eigvals(unitcell, wr, wi);
        TNR_REQUIRE(cap >= wr.size(), TNR_ERR_INVALID_ARG, "eigenvalue buffers too small");
        std::memcpy(re, wr.data(), wr.size() * sizeof(double));
        std::memcpy(im, wi.data(), wi.size() * sizeof(double));
        if (n_out) *n_out = wr.size();
    });
}

int tnr_gu_wen_ratio(tnr_handle h, double* x1, double* x2) {
    if (!h || !x1 || !x2) return fail(h, TNR_ERR_INVALID_ARG, "NULL argument");
    return guarded(h, [&] { h->s.gu_wen(x1, x2); });
}

int tnr_central_charge(tnr_handle h, double n, double* c_out) {
    if (!h || !c_out) return fail(h, TNR_ERR_INVALID_ARG, "NULL argument");
    return guarded(h, [&] { *c_out = h->s.central_charge(n); });
}

int tnr_finalize_impurity(tnr_handle h, double* norms_out) {
    if (!h || !norms_out) return fail(h, TNR_ERR_INVALID_ARG, "NULL argument");
    return guarded(h, [&] {
        Scheme& s = h->s;
        const int np = s.norms_per_entry();
        TNR_REQUIRE(np > 1, TNR_ERR_INVALID_ARG, "not an impurity scheme handle");
        Buf d(s.ctx->pool.get(), 4 * sizeof(double));
        s.finalize_multi_async(d.d());
        TNR_CUDA(cudaMemcpyAsync(norms_out, d.d(), np * sizeof(double), cudaMemcpyDeviceToHost, s.ctx->stream));
        s.ctx->sync();
        for (int i = 0; i < np; ++i)
            TNR_REQUIRE(std::isfinite(norms_out[i]), TNR_ERR_NONFINITE, "finalize!: non-finite norm");
    });
}

int tnr_run_impurity(tnr_handle h, int chi, int maxiter, int finalize_beginning, double* norms_out, size_t cap,
                     size_t* n_out) {
    if (!h) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL handle");
    return guarded(h, [&] {
        const size_t np = (size_t)h->s.norms_per_entry();
        TNR_REQUIRE(np > 1, TNR_ERR_INVALID_ARG, "not an impurity scheme handle");
        const size_t need = np * ((size_t)std::max(maxiter, 1) + (finalize_beginning ? 1 : 0));
        TNR_REQUIRE(norms_out && cap >= need, TNR_ERR_INVALID_ARG, "norms_out too small for run!");
        std::vector<double> v = h->s.run_impurity(chi, maxiter, finalize_beginning != 0);
        std::memcpy(norms_out, v.data(), v.size() * sizeof(double));
        if (n_out) *n_out = v.size() / np;
    });
}

int tnr_step(tnr_handle h, int chi) {
    if (!h) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL handle");
    return guarded(h, [&] { h->s.step(chi); });
}

int tnr_finalize(tnr_handle h, double* norm_out) {
    if (!h) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL handle");
    return guarded(h, [&] {
        double n = h->s.finalize();
        TNR_REQUIRE(std::isfinite(n), TNR_ERR_NONFINITE, "finalize!: non-finite norm");
        if (norm_out) *norm_out = n;
    });
}

int tnr_run(tnr_handle h, int chi, int maxiter, int finalize_beginning, double* norms_out, size_t cap, size_t* n_out) {
    if (!h) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL handle");
    return guarded(h, [&] {
        const size_t need = (size_t)std::max(maxiter, 1) + (finalize_beginning ? 1 : 0);
        TNR_REQUIRE(norms_out && cap >= need, TNR_ERR_INVALID_ARG, "norms_out too small for run!");
        std::vector<double> v = h->s.run(chi, maxiter, finalize_beginning != 0);
        std::memcpy(norms_out, v.data(), v.size() * sizeof(double));
        if (n_out) *n_out = v.size();
    });
}

double tnr_free_energy(const double* norms, size_t n, double beta, double scalefactor, double initial_size) {
    // free_energy.jl:13-20
    double lnz = 0.0;
    const double x = 1.0 - std::log(initial_size) / std::log(scalefactor);
    for (size_t i = 0; i < n; ++i) lnz += std::log(norms[i]) * std::pow(scalefactor, x - (double)(i + 1));
    return -lnz / beta;
}

int tnr_get_tensor(tnr_handle h, double* host_out, size_t cap, int64_t* dims_out, int* nlegs_out) {
    if (!h) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL handle");
    return guarded(h, [&] {
        Scheme& s = h->s;
        if (nlegs_out) *nlegs_out = s.T.rank;
        if (dims_out)
            for (int i = 0; i < s.T.rank; ++i) dims_out[i] = s.T.d[i];
        if (host_out) {
            TNR_REQUIRE(cap >= (size_t)s.T.size(), TNR_ERR_INVALID_ARG, "host_out too small");
            TNR_CUDA(cudaMemcpyAsync(host_out, s.T.p(), s.T.size() * sizeof(double), cudaMemcpyDeviceToHost, s.ctx->stream));
            s.ctx->sync();
        }
    });
}

int tnr_get_impurity_tensor(tnr_handle h, int which, double* host_out, size_t cap, int64_t* dims_out, int* nlegs_out) {
    if (!h) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL handle");
    return guarded(h, [&] {
        Scheme& s = h->s;
        const DT* t = nullptr;
        if (s.kind == TNR_IMPURITY_HOTRG && which >= 0 && which < 3) t = which == 0 ? &s.I11 : which == 1 ? &s.I12 : &s.I2;
        if (s.kind == TNR_IMPURITY_TRG && which >= 0 && which < 4) t = &s.site[which];
        if (s.kind == TNR_CORRELATION_HOTRG && which >= 0 && which < 3) t = which == 0 ? &s.C1 : which == 1 ? &s.C2 : &s.Cf;
        TNR_REQUIRE(t != nullptr, TNR_ERR_INVALID_ARG, "no impurity tensor with that index in this scheme");
        TNR_REQUIRE(t->rank > 0, TNR_ERR_INVALID_ARG, "that impurity tensor is not present at this step");
        if (nlegs_out) *nlegs_out = t->rank;
        if (dims_out)
            for (int i = 0; i < t->rank; ++i) dims_out[i] = t->d[i];
        if (host_out) {
            TNR_REQUIRE(cap >= (size_t)t->size(), TNR_ERR_INVALID_ARG, "host_out too small");
            TNR_CUDA(cudaMemcpyAsync(host_out, t->p(), t->size() * sizeof(double), cudaMemcpyDeviceToHost, s.ctx->stream));
            s.ctx->sync();
        }
    });
}

int tnr_singular_values(tnr_handle h, double* out, size_t cap, size_t* n_out, int32_t* counts, size_t counts_cap,
                        size_t* ndec_out) {
    if (!h) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL handle");
    return guarded(h, [&] {
        Scheme& s = h->s;
        if (n_out) *n_out = s.last_vals.size();
        if (ndec_out) *ndec_out = s.last_counts.size();
        if (out) {
            TNR_REQUIRE(cap >= s.last_vals.size(), TNR_ERR_INVALID_ARG, "out too small");
            std::memcpy(out, s.last_vals.data(), s.last_vals.size() * sizeof(double));
        }
        if (counts) {
            TNR_REQUIRE(counts_cap >= s.last_counts.size(), TNR_ERR_INVALID_ARG, "counts too small");
            for (size_t i = 0; i < s.last_counts.size(); ++i) counts[i] = s.last_counts[i];
        }
    });
}

int tnr_truncation_errors(tnr_handle h, double* out, size_t cap, size_t* n_out) {
    if (!h) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL handle");
    return guarded(h, [&] {
        Scheme& s = h->s;
        if (n_out) *n_out = s.last_eps.size();
        if (out) {
            TNR_REQUIRE(cap >= s.last_eps.size(), TNR_ERR_INVALID_ARG, "out too small");
            std::memcpy(out, s.last_eps.data(), s.last_eps.size() * sizeof(double));
        }
    });
}

int tnr_btrg_bonds(tnr_handle h, double* s1, size_t cap1, size_t* n1, double* s2, size_t cap2, size_t* n2) {
    if (!h) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL handle");
    return guarded(h, [&] {
        Scheme& s = h->s;
        TNR_REQUIRE(s.kind == TNR_BTRG, TNR_ERR_INVALID_ARG, "not a BTRG scheme");
        if (n1) *n1 = (size_t)s.S1.size();
        if (n2) *n2 = (size_t)s.S2.size();
        if (s1) {
            TNR_REQUIRE(cap1 >= (size_t)s.S1.size(), TNR_ERR_INVALID_ARG, "s1 too small");
            TNR_CUDA(cudaMemcpyAsync(s1, s.S1.p(), s.S1.size() * sizeof(double), cudaMemcpyDeviceToHost, s.ctx->stream));
        }
        if (s2) {
            TNR_REQUIRE(cap2 >= (size_t)s.S2.size(), TNR_ERR_INVALID_ARG, "s2 too small");
            TNR_CUDA(cudaMemcpyAsync(s2, s.S2.p(), s.S2.size() * sizeof(double), cudaMemcpyDeviceToHost, s.ctx->stream));
        }
        s.ctx->sync();
    });
}

int tnr_device_bytes(tnr_handle h, size_t* bytes_out) {
    if (!h || !bytes_out) return fail(h, TNR_ERR_INVALID_ARG, "NULL argument");
    *bytes_out = h->s.ctx->pool->held_bytes();
    return TNR_OK;
}

int tnr_decomposition_stats(tnr_handle h, uint64_t* decompositions, uint64_t* gap_fallbacks, int* max_iters) {
    if (!h) return fail(h, TNR_ERR_INVALID_ARG, "NULL handle");
    const Ctx& c = *h->s.ctx;
    if (decompositions) *decompositions = c.decompositions;
    if (gap_fallbacks) *gap_fallbacks = c.gap_fallbacks;
    if (max_iters) *max_iters = c.max_iters;
    return TNR_OK;
}

int tnr_destroy(tnr_handle h) {
    if (!h) return TNR_OK;
    int st = guarded(nullptr, [&] { h->s.ctx->sync(); });
    delete h;
    return st;
}

int tnr_last_error(tnr_handle h, char* buf, size_t cap) {
    const std::string& m = h ? h->s.err : g_err;
    if (buf && cap) {
        size_t n = std::min(cap - 1, m.size());
        std::memcpy(buf, m.data(), n);
        buf[n] = 0;
    }
    return TNR_OK;
}

const char* tnr_status_string(int st) {
    switch (st) {
        case TNR_OK: return "ok";
        case TNR_ERR_INVALID_ARG: return "invalid argument";
        case TNR_ERR_OOM: return "out of device memory";
        case TNR_ERR_NOT_CONVERGED: return "iteration cap reached";
        case TNR_ERR_CUDA: return "CUDA error";
        case TNR_ERR_ADMISSION: return "admission refused";
        case TNR_ERR_NONFINITE: return "non-finite value";
        case TNR_ERR_UNSUPPORTED: return "unsupported";
        case TNR_ERR_NO_DEVICE: return "no device";
        default: return "unknown status";
    }
}

int tnr_timer_start(tnr_handle h) {
    if (!h) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL handle");
    return guarded(h, [&] { TNR_CUDA(cudaEventRecord(h->s.ctx->ev0, h->s.ctx->stream)); });
}

int tnr_timer_stop(tnr_handle h, double* ms_out) {
    if (!h) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL handle");
    return guarded(h, [&] {
        TNR_CUDA(cudaEventRecord(h->s.ctx->ev1, h->s.ctx->stream));
        TNR_CUDA(cudaEventSynchronize(h->s.ctx->ev1));
        float ms = 0;
        TNR_CUDA(cudaEventElapsedTime(&ms, h->s.ctx->ev0, h->s.ctx->ev1));
        if (ms_out) *ms_out = ms;
    });
}

int tnr_run_batch(tnr_handle* hs, int n, const int* chi, const int* maxiter, int finalize_beginning, double* norms_out,
                  size_t stride, size_t* n_out, double* device_ms_out, double* latency_ms_out) {
    if (!hs || n < 0 || !chi || !maxiter || !norms_out || !n_out)
        return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL argument");
    for (int i = 0; i < n; ++i) {
        if (!hs[i]) return fail(nullptr, TNR_ERR_INVALID_ARG, "NULL handle in batch");
        size_t need = (size_t)std::max(maxiter[i], 1) + (finalize_beginning ? 1 : 0);
        if (need > stride) return fail(nullptr, TNR_ERR_INVALID_ARG, "stride too small for run!");
    }
    {
        // a handle is single-owner: the same handle twice would be driven by two workers at once
        std::vector<tnr_handle> sorted(hs, hs + n);
        std::sort(sorted.begin(), sorted.end());
        if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
            return fail(nullptr, TNR_ERR_INVALID_ARG, "the same handle appears twice in the batch");
    }
    // lockstep groups: fresh TRG/BTRG schemes with equal kind, precision, k, dims, chi, maxiter
    struct Task {
        std::vector<int> idx;
        std::unique_ptr<Ctx> ctx;   // group context (null: run the single handle on its own)
    };
    std::vector<Task> tasks;
    {
        std::map<std::string, int> key_to_task;
        for (int i = 0; i < n; ++i) {
            Scheme& sc = hs[i]->s;
            bool groupable = (sc.kind == TNR_TRG || sc.kind == TNR_BTRG) && sc.steps == 0 &&
                             sc.finalizer == FINALIZER_DEFAULT && !sc.T.charged();
            std::string key;
            if (groupable) {
                uint64_t kbits = 0;                                   // k exactly, not to 6 decimals
                std::memcpy(&kbits, &sc.btrg_k, sizeof kbits);
                key = std::to_string(sc.kind) + "/" + std::to_string(sc.ctx->precision) + "/" +
                      std::to_string(kbits) + "/" + std::to_string(chi[i]) + "/" + std::to_string(maxiter[i]);
                for (int l = 0; l < sc.T.rank; ++l) key += "/" + std::to_string(sc.T.d[l]);
            }
            auto it = groupable ? key_to_task.find(key) : key_to_task.end();
            if (it == key_to_task.end()) {
                tasks.push_back(Task());
                tasks.back().idx.push_back(i);
                if (groupable) key_to_task[key] = (int)tasks.size() - 1;
            } else {
                tasks[it->second].idx.push_back(i);
            }
        }
    }
    int st0 = guarded(nullptr, [&] {
        for (auto& t : tasks)
            if (t.idx.size() > 1)
                t.ctx.reset(new Ctx(nullptr, hs[t.idx[0]]->s.ctx->precision, hs[t.idx[0]]->s.ctx->seed));
    });
    if (st0 != TNR_OK) return st0;
    // largest groups first
    std::stable_sort(tasks.begin(), tasks.end(), [](const Task& a, const Task& b) { return a.idx.size() > b.idx.size(); });
    auto task_stream = [&](const Task& t) { return t.ctx ? t.ctx->stream : hs[t.idx[0]]->s.ctx->stream; };
    cudaStream_t ts = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<cudaEvent_t> done;
    st0 = guarded(nullptr, [&] {
        if (device_ms_out) {
            TNR_CUDA(cudaStreamCreateWithFlags(&ts, cudaStreamNonBlocking));
            TNR_CUDA(cudaEventCreate(&e0));
            TNR_CUDA(cudaEventCreate(&e1));
            TNR_CUDA(cudaEventRecord(e0, ts));
            for (auto& t : tasks) TNR_CUDA(cudaStreamWaitEvent(task_stream(t), e0, 0));
        }
    });
    if (st0 != TNR_OK) return st0;
    // one host worker per concurrent task; a task is a lockstep group or a single handle
    // TNR_BATCH_WORKERS (default 32) bounds the host workers; 1 runs the groups one after
    // another (a profiling pass whose per-launch event times then exclude queueing)
    int max_workers = 32;
    if (const char* w = std::getenv("TNR_BATCH_WORKERS")) max_workers = std::max(1, std::min(32, std::atoi(w)));
    const int workers = std::min((int)tasks.size(), max_workers);
    std::vector<int> status(n, TNR_OK);
    std::atomic<int> next{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const auto t0 = std::chrono::steady_clock::now();
    auto work = [&] {
        cudaSetDevice(dev);
        for (;;) {
            int ti = next.fetch_add(1);
            if (ti >= (int)tasks.size()) break;
            Task& t = tasks[ti];
            if (!t.ctx) {
                int i = t.idx[0];
                status[i] = tnr_run(hs[i], chi[i], maxiter[i], finalize_beginning, norms_out + (size_t)i * stride,
                                    stride, n_out + i);
            } else {
                std::vector<Scheme*> mem;
                for (int i : t.idx) mem.push_back(&hs[i]->s);
                std::vector<std::vector<double>> nv;
                int i0 = t.idx[0];
                int st = guarded(hs[i0], [&] { run_group(*t.ctx, mem, chi[i0], maxiter[i0], finalize_beginning != 0, nv); });
                for (size_t j = 0; j < t.idx.size(); ++j) {
                    int i = t.idx[j];
                    status[i] = st;
                    if (st == TNR_OK) {
                        std::memcpy(norms_out + (size_t)i * stride, nv[j].data(), nv[j].size() * sizeof(double));
                        n_out[i] = nv[j].size();
                    } else {
                        hs[i]->s.err = hs[i0]->s.err;
                    }
                }
            }
            const double lat = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            if (latency_ms_out)
                for (int i : t.idx) latency_ms_out[i] = lat;
        }
    };
    std::vector<std::thread> th;
    for (int w = 0; w < workers; ++w) th.emplace_back(work);
    for (auto& t : th) t.join();
    int st1 = guarded(nullptr, [&] {
        if (device_ms_out) {
            for (auto& t : tasks) {
                cudaEvent_t e;
                TNR_CUDA(cudaEventCreate(&e));
                TNR_CUDA(cudaEventRecord(e, task_stream(t)));
                TNR_CUDA(cudaStreamWaitEvent(ts, e, 0));
                done.push_back(e);
            }
            TNR_CUDA(cudaEventRecord(e1, ts));
            TNR_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            TNR_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            *device_ms_out = ms;
        }
    });
    for (auto e : done) cudaEventDestroy(e);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (ts) cudaStreamDestroy(ts);
    for (int i = 0; i < n; ++i)
        if (status[i] != TNR_OK) {
            g_err = "instance " + std::to_string(i) + ": " + hs[i]->s.err;
            return status[i];
        }
    return st1;
}

int tnr_profile_enable(int on) {
    g_prof_on.store(on != 0);
    return TNR_OK;
}

int tnr_profile_reset(void) {
    return guarded(nullptr, [&] { prof_reset(); });
}

int tnr_profile_read(int cls, uint64_t* launches, double* total_ms, double* work) {
    if (cls < 0 || cls >= PROF_NCLASS) return fail(nullptr, TNR_ERR_INVALID_ARG, "unknown profile class");
    return guarded(nullptr, [&] { prof_read(cls, launches, total_ms, work); });
}

int tnr_debug_chol(int precision, int r, double shift, int batch, const double* G, double* Linv, int* breakdown) {
    if (!G || !Linv || !breakdown || r < 1 || batch < 1) return fail(nullptr, TNR_ERR_INVALID_ARG, "bad chol");
    return guarded(nullptr, [&] {
        require_device();
        Ctx c(nullptr, precision, 0);
        const size_t bytes = (size_t)batch * r * r * sizeof(double);
        Buf dG(c.pool.get(), bytes);
        TNR_CUDA(cudaMemcpyAsync(dG.d(), G, bytes, cudaMemcpyHostToDevice, c.stream));
        if (precision == TNR_PREC_SPLIT) chol_inv_f32(c, dG.d(), r, shift, batch);
        else chol_inv(c, dG.d(), r, shift, batch);
        TNR_CUDA(cudaMemcpyAsync(Linv, dG.d(), bytes, cudaMemcpyDeviceToHost, c.stream));
        const int st = c.read_status_and_clear();
        *breakdown = (st & ST_CHOL_BREAKDOWN) ? 1 : 0;
        TNR_REQUIRE((st & ~ST_CHOL_BREAKDOWN) == 0, TNR_ERR_CUDA, "kernel status word " + std::to_string(st));
    });
}

int tnr_debug_gemm(int precision, int ta, int tb, int64_t m, int64_t n, int64_t k, const double* A, int64_t lda,
                   int64_t sA, const double* B, int64_t ldb, int64_t sB, double* C, int64_t ldc, int64_t sC, int batch) {
    if (!A || !B || !C || m < 1 || n < 1 || k < 1 || batch < 1) return fail(nullptr, TNR_ERR_INVALID_ARG, "bad gemm");
    return guarded(nullptr, [&] {
        require_device();
        Ctx c(nullptr, precision, 0);
        // extents of the host buffers (last element + 1)
        auto extent = [](bool t, int64_t rows, int64_t cols, int64_t ld, int64_t stride, int nb) {
            int64_t r = t ? cols : rows, cc = t ? rows : cols;   // stored shape
            return (nb - 1) * stride + (cc - 1) * ld + r;
        };
        const int64_t eA = extent(ta, m, k, lda, sA, batch), eB = extent(tb, k, n, ldb, sB, batch);
        const int64_t eC = (batch - 1) * sC + (n - 1) * ldc + m;
        Buf dA(c.pool.get(), eA * 8), dB(c.pool.get(), eB * 8), dC(c.pool.get(), eC * 8);
        TNR_CUDA(cudaMemcpyAsync(dA.d(), A, eA * 8, cudaMemcpyHostToDevice, c.stream));
        TNR_CUDA(cudaMemcpyAsync(dB.d(), B, eB * 8, cudaMemcpyHostToDevice, c.stream));
        TNR_CUDA(cudaMemsetAsync(dC.d(), 0, eC * 8, c.stream));
        Batch2 bt;
        bt.n1 = batch; bt.sA1 = sA; bt.sB1 = sB; bt.sC1 = sC;
        if (precision == TNR_PREC_SPLIT) {
            // the contraction path: K accumulated in chunks summed in FP64
            bool ran = gemm_split_tc(c, ta, tb, m, n, k, 1.0, dA.d(), lda, dB.d(), ldb, 0.0, dC.d(), ldc, bt,
                                     split_chunk_kb());
            TNR_REQUIRE(ran, TNR_ERR_UNSUPPORTED, "split kernel declined this shape");
        } else {
            gemm_f64(c, ta, tb, m, n, k, 1.0, dA.d(), lda, dB.d(), ldb, 0.0, dC.d(), ldc, bt);
        }
        TNR_CUDA(cudaMemcpyAsync(C, dC.d(), eC * 8, cudaMemcpyDeviceToHost, c.stream));
        int st = c.read_status_and_clear();
        TNR_REQUIRE(st == 0, TNR_ERR_CUDA, "kernel status word " + std::to_string(st));
    });
}

int tnr_gemm_time(int precision, int ta, int tb, int64_t m, int64_t n, int64_t k, int batch, int reps,
                  int contraction, double* ms_out) {
    if (m < 1 || n < 1 || k < 1 || batch < 1 || reps < 1 || !ms_out)
        return fail(nullptr, TNR_ERR_INVALID_ARG, "bad gemm_time arguments");
    if (precision != TNR_PREC_F64 && precision != TNR_PREC_SPLIT)
        return fail(nullptr, TNR_ERR_INVALID_ARG, "unknown precision");
    return guarded(nullptr, [&] {
        require_device();
        Ctx c(nullptr, precision, 0);
        const int64_t sA = m * k, sB = k * n, sC = m * n;
        Buf dA(c.pool.get(), (size_t)sA * batch * 8), dB(c.pool.get(), (size_t)sB * batch * 8),
            dC(c.pool.get(), (size_t)sC * batch * 8);
        fill_normal(c, dA.d(), sA * batch, 1);
        fill_normal(c, dB.d(), sB * batch, 2);
        Batch2 bt;
        bt.n1 = batch; bt.sA1 = sA; bt.sB1 = sB; bt.sC1 = sC;
        const int64_t lda = ta ? k : m, ldb = tb ? n : k;
        auto once = [&] {
            if (precision == TNR_PREC_SPLIT) {
                bool ran = gemm_split_tc(c, ta, tb, m, n, k, 1.0, dA.d(), lda, dB.d(), ldb, 0.0, dC.d(), m, bt,
                                         contraction ? split_chunk_kb() : 0);
                TNR_REQUIRE(ran, TNR_ERR_UNSUPPORTED, "split kernel declined this shape");
            } else {
                gemm_f64(c, ta, tb, m, n, k, 1.0, dA.d(), lda, dB.d(), ldb, 0.0, dC.d(), m, bt);
            }
        };
        once();   // warm-up (tensor maps, function attributes)
        cudaEvent_t e0, e1;
        TNR_CUDA(cudaEventCreate(&e0));
        TNR_CUDA(cudaEventCreate(&e1));
        TNR_CUDA(cudaEventRecord(e0, c.stream));
        for (int i = 0; i < reps; ++i) once();
        TNR_CUDA(cudaEventRecord(e1, c.stream));
        TNR_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        TNR_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        int st = c.read_status_and_clear();
        TNR_REQUIRE(st == 0, TNR_ERR_CUDA, "kernel status word " + std::to_string(st));
        *ms_out = (double)ms / reps;
    });
}

int tnr_device_info(int* sm, int* major, int* minor, size_t* hbm) {
    return guarded(nullptr, [&] {
        require_device();
        int dev = 0;
        TNR_CUDA(cudaGetDevice(&dev));
        cudaDeviceProp p;
        TNR_CUDA(cudaGetDeviceProperties(&p, dev));
        if (sm) *sm = p.multiProcessorCount;
        if (major) *major = p.major;
        if (minor) *minor = p.minor;
        if (hbm) *hbm = p.totalGlobalMem;
    });
}

const char* tnr_version(void) { return "tnr-gb300 0.1.0 (sm_103a)"; }

uint64_t tnr_kernel_launches(void) { return g_launches.load(); }

}  // extern "C"
