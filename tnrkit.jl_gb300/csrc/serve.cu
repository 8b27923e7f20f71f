// Serving loop: run!() requests admitted by their HBM footprint, kept resident on the
// device while they iterate, with the steps of every admitted request in flight at once
// (one CUDA stream per request, a pool of host workers).  A request that arrives while
// others run is admitted as soon as a slot and enough of the HBM budget free up.
#include "schemes.cuh"

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>

using namespace tnr;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t id = 0;
    int kind = 0, chi = 0, maxiter = 0;
    std::vector<int64_t> dims;
    std::vector<double> data;
    double btrg_k = -0.5;
    int symmetry_n = 1;
    std::vector<int32_t> charges;   // sum(dims) leg charges when symmetry_n > 1
    size_t footprint = 0;
    Clock::time_point t_submit, t_start, t_done;
    int status = TNR_OK;
    std::string err;
    std::vector<double> norms;
    bool done = false;
};

// Device bytes a request needs at bond dimension chi (tensor, intermediates, workspace),
// from the contraction plans: TRG/BTRG/ATRG hold chi^4-sized tensors, HOTRG two chi^5
// intermediates, HOTRG_3D chi^6 tensors plus one sliced chi^8 intermediate of at most
// 2^31 entries.
size_t footprint_bytes(int kind, int chi, const std::vector<int64_t>& dims) {
    double c = chi;
    double d0 = 1;
    for (auto d : dims) d0 = std::max<double>(d0, (double)d);
    c = std::max(c, d0);
    double entries;
    switch (kind) {
        case TNR_TRG:
        case TNR_BTRG: entries = 12.0 * c * c * c * c + 4.0 * 128 * c * c; break;
        case TNR_HOTRG: entries = 2.2 * c * c * c * c * c + 12.0 * c * c * c * c; break;
        case TNR_ATRG: entries = 16.0 * c * c * c * c + 4.0 * 128 * c * c; break;
        case TNR_ATRG_3D: entries = 14.0 * c * c * c * c * c * c; break;
        default: {
            double c6 = c * c * c * c * c * c;
            entries = 10.0 * c6 + 3.0 * std::min(c6 * c * c, 2147483648.0);
        }
    }
    const double bytes = entries * 8.0 + double(size_t(64) << 20);
    return bytes >= 9.0e18 ? size_t(9000000000000000000ull) : (size_t)bytes;   // saturate, never wrap
}

}  // namespace

struct tnr_server_s {
    size_t budget = 0, in_use = 0;
    int max_active = 1, active = 0, precision = TNR_PREC_F64;
    uint64_t next_id = 1;
    bool stopping = false;
    std::mutex mu;
    std::condition_variable cv, cv_done;
    std::deque<Request*> queue;
    std::map<uint64_t, Request*> all;
    std::vector<std::thread> workers;
    int dev = 0;

    // Requests that can step in lockstep: TRG / BTRG on uncharged tensors with equal legs, chi,
    // maxiter and k (the server's precision is shared).  Such requests admitted together run as
    // one lockstep batch (tnr_run_batch: batched GEMMs, one CTA per member in the small solvers).
    static bool batchable(const Request* r) {
        return (r->kind == TNR_TRG || r->kind == TNR_BTRG) && r->symmetry_n <= 1;
    }
    static bool same_group(const Request* a, const Request* b) {
        return batchable(a) && batchable(b) && a->kind == b->kind && a->dims == b->dims && a->chi == b->chi &&
               a->maxiter == b->maxiter && std::memcmp(&a->btrg_k, &b->btrg_k, sizeof(double)) == 0;
    }
    static constexpr int MAX_GROUP = 64;

    // a handle for request r (its status and message on failure)
    tnr_handle create_for(Request* r) {
        tnr_handle h = nullptr;
        tnr_options o;
        tnr_default_options(&o);
        o.precision = precision;
        o.btrg_k = r->btrg_k;
        if (r->symmetry_n > 1) {
            o.symmetry_n = r->symmetry_n;
            o.leg_charges = r->charges.data();
        }
        const int st = tnr_create(&h, r->kind, (int)r->dims.size(), r->dims.data(), r->data.data(), &o);
        if (st != TNR_OK) {
            char buf[512];
            tnr_last_error(nullptr, buf, sizeof buf);
            r->status = st;
            r->err = buf;
            if (h) tnr_destroy(h);
            return nullptr;
        }
        return h;
    }

    void run_one(Request* r) {
        tnr_handle h = create_for(r);
        if (!h) return;
        const size_t cap = (size_t)std::max(r->maxiter, 1) + 1;
        r->norms.resize(cap);
        size_t n = 0;
        int st = tnr_run(h, r->chi, r->maxiter, 1, r->norms.data(), cap, &n);
        r->norms.resize(n);
        if (st != TNR_OK) {
            char buf[512];
            tnr_last_error(h, buf, sizeof buf);
            r->err = buf;
        }
        tnr_destroy(h);
        r->status = st;
    }

    void run_group_of(std::vector<Request*>& grp) {
        std::vector<tnr_handle> hs;
        std::vector<Request*> live;
        for (Request* r : grp) {
            tnr_handle h = create_for(r);
            if (h) {
                hs.push_back(h);
                live.push_back(r);
            }
        }
        if (hs.empty()) return;
        const int n = (int)hs.size();
        const size_t stride = (size_t)std::max(live[0]->maxiter, 1) + 1;
        std::vector<int> chis(n, live[0]->chi), its(n, live[0]->maxiter);
        std::vector<double> norms(stride * n);
        std::vector<size_t> counts(n, 0);
        const int st = tnr_run_batch(hs.data(), n, chis.data(), its.data(), 1, norms.data(), stride, counts.data(),
                                     nullptr, nullptr);
        std::string msg;
        if (st != TNR_OK) {
            char buf[512];
            tnr_last_error(nullptr, buf, sizeof buf);
            msg = buf;
        }
        for (int i = 0; i < n; ++i) {
            Request* r = live[i];
            r->status = st;
            r->err = msg;
            if (st == TNR_OK) r->norms.assign(norms.begin() + (size_t)i * stride, norms.begin() + (size_t)i * stride + counts[i]);
            tnr_destroy(hs[i]);
        }
    }

    void worker() {
        cudaSetDevice(dev);
        for (;;) {
            std::vector<Request*> grp;
            size_t grp_bytes = 0;
            {
                std::unique_lock<std::mutex> lk(mu);
                // admit the oldest queued request that fits the free budget (first fit)
                cv.wait(lk, [&] {
                    if (stopping) return true;
                    if (active >= max_active) return false;
                    for (Request* q : queue)
                        if (q->footprint <= budget - in_use) return true;
                    return false;
                });
                if (stopping && queue.empty()) return;
                if (stopping) {
                    // drain: fail what never got admitted
                    for (Request* q : queue) {
                        q->status = TNR_ERR_ADMISSION;
                        q->err = "server stopped";
                        q->done = true;
                    }
                    queue.clear();
                    cv_done.notify_all();
                    return;
                }
                for (auto it = queue.begin(); it != queue.end(); ++it)
                    if ((*it)->footprint <= budget - in_use) {
                        grp.push_back(*it);
                        grp_bytes = (*it)->footprint;
                        queue.erase(it);
                        break;
                    }
                // continuous batching: queued requests that can step in lockstep with it join it,
                // as far as the free budget allows
                for (auto it = queue.begin(); it != queue.end() && (int)grp.size() < MAX_GROUP;) {
                    if (same_group(grp[0], *it) && grp_bytes + (*it)->footprint <= budget - in_use) {
                        grp_bytes += (*it)->footprint;
                        grp.push_back(*it);
                        it = queue.erase(it);
                    } else {
                        ++it;
                    }
                }
                in_use += grp_bytes;
                ++active;
            }
            const auto t0 = Clock::now();
            for (Request* r : grp) r->t_start = t0;
            if (grp.size() == 1) run_one(grp[0]);
            else run_group_of(grp);
            const auto t1 = Clock::now();
            {
                std::lock_guard<std::mutex> lk(mu);
                for (Request* r : grp) {
                    r->t_done = t1;
                    r->done = true;
                }
                in_use -= grp_bytes;
                --active;
            }
            cv.notify_all();
            cv_done.notify_all();
        }
    }
};

extern "C" {

int tnr_server_create(tnr_server* out, size_t hbm_budget_bytes, int max_active, int precision) {
    if (!out || max_active < 1 || hbm_budget_bytes == 0) return TNR_ERR_INVALID_ARG;
    if (precision != TNR_PREC_F64 && precision != TNR_PREC_SPLIT) return TNR_ERR_INVALID_ARG;
    tnr_server s = new (std::nothrow) tnr_server_s();
    if (!s) return TNR_ERR_OOM;
    s->budget = hbm_budget_bytes;
    s->max_active = max_active;
    s->precision = precision;
    cudaGetDevice(&s->dev);
    for (int i = 0; i < max_active; ++i) s->workers.emplace_back([s] { s->worker(); });
    *out = s;
    return TNR_OK;
}

int tnr_server_submit(tnr_server s, int kind, int nlegs, const int64_t* dims, const double* data, int chi,
                      int maxiter, double btrg_k, uint64_t* id_out) {
    return tnr_server_submit_sym(s, kind, nlegs, dims, data, 1, nullptr, chi, maxiter, btrg_k, id_out);
}

int tnr_server_submit_sym(tnr_server s, int kind, int nlegs, const int64_t* dims, const double* data,
                          int symmetry_n, const int32_t* leg_charges, int chi, int maxiter, double btrg_k,
                          uint64_t* id_out) {
    if (symmetry_n > 1 && !leg_charges) return TNR_ERR_INVALID_ARG;
    if (!s || !dims || !data || !id_out || chi < 1) return TNR_ERR_INVALID_ARG;
    if ((kind < TNR_TRG || kind > TNR_HOTRG_3D) && kind != TNR_ATRG && kind != TNR_ATRG_3D) return TNR_ERR_INVALID_ARG;
    if (nlegs != (kind == TNR_HOTRG_3D || kind == TNR_ATRG_3D ? 6 : 4)) return TNR_ERR_INVALID_ARG;
    Request* r = new (std::nothrow) Request();
    if (!r) return TNR_ERR_OOM;
    r->kind = kind;
    r->chi = chi;
    r->maxiter = maxiter;
    r->btrg_k = btrg_k;
    r->dims.assign(dims, dims + nlegs);
    int64_t total = 1;
    for (int l = 0; l < nlegs; ++l) {
        if (dims[l] < 1) {
            delete r;
            return TNR_ERR_INVALID_ARG;
        }
        total *= dims[l];
    }
    r->data.assign(data, data + total);
    if (symmetry_n > 1) {
        int64_t nq = 0;
        for (int l = 0; l < nlegs; ++l) nq += dims[l];
        r->symmetry_n = symmetry_n;
        r->charges.assign(leg_charges, leg_charges + nq);
    }
    r->footprint = footprint_bytes(kind, chi, r->dims);
    r->t_submit = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    if (r->footprint > s->budget) {
        // can never fit: refused at submission (admission control)
        delete r;
        return TNR_ERR_ADMISSION;
    }
    r->id = s->next_id++;
    s->all[r->id] = r;
    s->queue.push_back(r);
    *id_out = r->id;
    s->cv.notify_all();
    return TNR_OK;
}

int tnr_server_poll(tnr_server s, uint64_t id, int wait, int* done, double* norms, size_t cap, size_t* n_out,
                    double* latency_ms, double* queue_ms) {
    if (!s || !done) return TNR_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return TNR_ERR_INVALID_ARG;
    Request* r = it->second;
    if (wait) s->cv_done.wait(lk, [&] { return r->done; });
    *done = r->done ? 1 : 0;
    if (!r->done) return TNR_OK;
    if (n_out) *n_out = r->norms.size();
    if (norms) {
        if (cap < r->norms.size()) return TNR_ERR_INVALID_ARG;
        std::memcpy(norms, r->norms.data(), r->norms.size() * sizeof(double));
    }
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    if (queue_ms) *queue_ms = std::chrono::duration<double, std::milli>(r->t_start - r->t_submit).count();
    return r->status;
}

int tnr_server_stats(tnr_server s, int* active, int* queued, size_t* bytes_in_use) {
    if (!s) return TNR_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (active) *active = s->active;
    if (queued) *queued = (int)s->queue.size();
    if (bytes_in_use) *bytes_in_use = s->in_use;
    return TNR_OK;
}

int tnr_server_destroy(tnr_server s) {
    if (!s) return TNR_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv.notify_all();
    for (auto& t : s->workers) t.join();
    for (auto& kv : s->all) delete kv.second;
    delete s;
    return TNR_OK;
}

size_t tnr_footprint_bytes(int kind, int chi, int nlegs, const int64_t* dims) {
    std::vector<int64_t> d(dims, dims + nlegs);
    return footprint_bytes(kind, chi, d);
}

}  // extern "C"
