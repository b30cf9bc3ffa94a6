// tdda_server.cu -- continuous-batching request loop over the C ABI.
//
// Requests (one structure + its incidences each) queue in arrival order.
// Workers run concurrently, each on its own cores and therefore its own CUDA
// stream.  A free worker takes the first queued request whose device memory
// fits what the HBM budget leaves free (first fit, so a large request does
// not hold back small ones behind it; a request alone larger than the budget
// fails), adds queued requests with the same operator (lattice, spacing,
// wavelength, material, background index) up to max_group right-hand sides,
// and solves them in one batched solve (tdda_solve_batch).  Memory is
// released as each solve finishes and waiting requests are admitted at once.
// Every result is computed exactly as the same request alone would be: the
// batched kernels treat every right-hand side independently.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/tdda.h"

namespace {

struct Request {
    unsigned long long id = 0;
    tdda_request_desc d{};
    std::vector<int> R;
    std::vector<double> material, diel_old, nK, nE0, E0;
    std::vector<double> P;  // 3N x nrhs complex
    tdda_request_info info{};
    double bytes = 0;
};

bool same_operator(const Request& a, const Request& b) {
    const tdda_request_desc &x = a.d, &y = b.d;
    return x.Nx == y.Nx && x.Ny == y.Ny && x.Nz == y.Nz && x.N == y.N && x.d == y.d && x.lam == y.lam &&
           x.nback == y.nback && a.material == b.material && a.R == b.R;
}

}  // namespace

struct tdda_server_s {
    tdda_server_desc desc{};
    std::chrono::steady_clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request*> queue;
    std::unordered_map<unsigned long long, std::unique_ptr<Request>> all;
    unsigned long long next_id = 1;
    int running = 0;
    double bytes = 0, peak = 0;
    bool stop = false;
    std::vector<std::thread> workers;

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }

    // first queued request that fits; with nothing in flight the head is
    // admitted (or failed, if it alone exceeds the budget)
    std::vector<Request*> take_group() {
        for (size_t i = 0; i < queue.size(); i++) {
            Request* r = queue[i];
            const bool fits = bytes + r->bytes <= desc.hbm_budget_bytes;
            if (!fits && !(i == 0 && running == 0)) continue;
            std::vector<Request*> g{r};
            queue.erase(queue.begin() + (long)i);
            int rhs = r->d.nrhs;
            double extra = 0;
            for (size_t j = i; j < queue.size();) {
                Request* o = queue[j];
                const double add = tdda_request_bytes(o->d.Nx, o->d.Ny, o->d.Nz, o->d.N, rhs + o->d.nrhs,
                                                      desc.precision) -
                                   tdda_request_bytes(r->d.Nx, r->d.Ny, r->d.Nz, r->d.N, rhs, desc.precision);
                if (same_operator(*o, *r) && rhs + o->d.nrhs <= desc.max_group &&
                    bytes + r->bytes + extra + add <= desc.hbm_budget_bytes) {
                    g.push_back(o);
                    rhs += o->d.nrhs;
                    extra += add;
                    queue.erase(queue.begin() + (long)j);
                } else {
                    j++;
                }
            }
            return g;
        }
        return {};
    }

    void run_group(std::vector<Request*>& g, double gbytes);
    void worker();
};

void tdda_server_s::worker() {
    for (;;) {
        std::vector<Request*> g;
        double gbytes = 0;
        {
            std::unique_lock<std::mutex> lk(mu);
            for (;;) {
                if (!queue.empty()) {
                    g = take_group();
                    if (!g.empty()) break;
                }
                if (stop && queue.empty()) return;
                cv.wait(lk);
            }
            int rhs = 0;
            for (Request* r : g) rhs += r->d.nrhs;
            gbytes = tdda_request_bytes(g[0]->d.Nx, g[0]->d.Ny, g[0]->d.Nz, g[0]->d.N, rhs, desc.precision);
            const double t = now();
            for (Request* r : g) {
                r->info.state = TDDA_REQ_RUNNING;
                r->info.t_start = t;
                r->info.group = rhs;
            }
            running += (int)g.size();
            bytes += gbytes;
            if (bytes > peak) peak = bytes;
        }
        run_group(g, gbytes);
        {
            std::lock_guard<std::mutex> lk(mu);
            running -= (int)g.size();
            bytes -= gbytes;
            const double t = now();
            for (Request* r : g) {
                r->info.t_done = t;
                if (r->info.state == TDDA_REQ_RUNNING) r->info.state = TDDA_REQ_DONE;
            }
        }
        cv.notify_all();
    }
}

void tdda_server_s::run_group(std::vector<Request*>& g, double gbytes) {
    auto fail_all = [&](tdda_status st) {
        for (Request* r : g) {
            r->info.state = TDDA_REQ_FAILED;
            r->info.status = st;
        }
    };
    if (gbytes > desc.hbm_budget_bytes) {
        fail_all(TDDA_ERR_OUT_OF_MEMORY);
        return;
    }
    if (desc.dry_run) {
        std::this_thread::sleep_for(std::chrono::duration<double, std::milli>(desc.dry_run_ms));
        for (Request* r : g) r->info.status = TDDA_OK;
        return;
    }
    const Request& h = *g[0];
    int rhs = 0;
    for (Request* r : g) rhs += r->d.nrhs;
    tdda_core_desc cd;
    cd.Nx = h.d.Nx;
    cd.Ny = h.d.Ny;
    cd.Nz = h.d.Nz;
    cd.N = h.d.N;
    cd.R = h.R.data();
    cd.d = h.d.d;
    cd.lam = h.d.lam;
    cd.nback = h.d.nback;
    cd.material = h.material.data();
    cd.nmat = h.d.nmat;
    cd.method = TDDA_METHOD_LDR;
    cd.max_rhs = rhs;
    cd.device = desc.device;
    tdda_core* core = nullptr;
    tdda_status st = tdda_core_create(&cd, &core);
    if (st != TDDA_OK) {
        fail_all(st);
        return;
    }
    std::vector<tdda_model*> models;
    std::vector<std::pair<Request*, int>> owner;
    for (Request* r : g) {
        for (int k = 0; k < r->d.nrhs && st == TDDA_OK; k++) {
            tdda_model* m = nullptr;
            st = tdda_model_create(core, &r->nK[3 * k], r->E0[k], &r->nE0[3 * k], r->diel_old.data(), &m);
            if (st == TDDA_OK) {
                models.push_back(m);
                owner.emplace_back(r, k);
            }
        }
    }
    std::vector<tdda_solve_info> infos(models.size());
    if (st == TDDA_OK) {
        st = tdda_solve_batch(models.data(), (int)models.size(), desc.precision, desc.max_it, desc.tol, infos.data());
        if (st == TDDA_NOT_CONVERGED || st == TDDA_BREAKDOWN || st == TDDA_ERR_NAN) st = TDDA_OK;  // per RHS below
    }
    if (st != TDDA_OK) {
        fail_all(st);
    } else {
        for (Request* r : g) {
            r->info.status = TDDA_OK;
            r->info.iterations = 0;
            r->info.error = 0;
        }
        for (size_t i = 0; i < models.size(); i++) {
            Request* r = owner[i].first;
            const int k = owner[i].second;
            const size_t n6 = 6 * (size_t)r->d.N;
            tdda_status gs = tdda_model_get(models[i], TDDA_FIELD_P, r->P.data() + k * n6, TDDA_MEM_HOST);
            const tdda_status ss = gs != TDDA_OK ? gs : (tdda_status)infos[i].status;
            if (ss != TDDA_OK && r->info.status == TDDA_OK) r->info.status = ss;
            if (infos[i].iterations > r->info.iterations) r->info.iterations = infos[i].iterations;
            if (infos[i].error > r->info.error) r->info.error = infos[i].error;
        }
        for (Request* r : g)
            if (r->info.status != TDDA_OK) r->info.state = TDDA_REQ_FAILED;
    }
    for (tdda_model* m : models) tdda_model_destroy(m);
    tdda_core_destroy(core);
}

extern "C" {

tdda_status tdda_server_create(const tdda_server_desc* desc, tdda_server** out) {
    if (!desc || !out || desc->workers < 1 || desc->workers > 64 || !(desc->hbm_budget_bytes > 0) ||
        desc->max_group < 1 || desc->max_group > 64 ||
        (desc->precision != TDDA_FP64 && desc->precision != TDDA_FP32_REFINE))
        return TDDA_ERR_INVALID_ARGUMENT;
    if (!desc->dry_run && tdda_device_count() < 1) return TDDA_ERR_NO_DEVICE;
    tdda_server* s = new tdda_server_s();
    s->desc = *desc;
    s->t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < desc->workers; i++) s->workers.emplace_back([s] { s->worker(); });
    *out = s;
    return TDDA_OK;
}

tdda_status tdda_server_submit(tdda_server* s, const tdda_request_desc* d, unsigned long long* id) {
    if (!s || !d || !id || d->N < 1 || d->nrhs < 1 || d->nrhs > s->desc.max_group || !d->R || !d->material ||
        d->nmat < 1 || !d->diel_old || !d->nK || !d->nE0 || !d->E0)
        return TDDA_ERR_INVALID_ARGUMENT;
    auto r = std::make_unique<Request>();
    r->d = *d;
    r->R.assign(d->R, d->R + 3 * (size_t)d->N);
    r->material.assign(d->material, d->material + 2 * (size_t)d->nmat);
    r->diel_old.assign(d->diel_old, d->diel_old + 3 * (size_t)d->N);
    r->nK.assign(d->nK, d->nK + 3 * (size_t)d->nrhs);
    r->nE0.assign(d->nE0, d->nE0 + 3 * (size_t)d->nrhs);
    r->E0.assign(d->E0, d->E0 + d->nrhs);
    r->P.assign(6 * (size_t)d->N * d->nrhs, 0.0);
    r->bytes = tdda_request_bytes(d->Nx, d->Ny, d->Nz, d->N, d->nrhs, s->desc.precision);
    r->info.state = TDDA_REQ_QUEUED;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        r->info.t_submit = s->now();
        r->info.bytes = r->bytes;
        *id = r->id;
        s->queue.push_back(r.get());
        s->all.emplace(r->id, std::move(r));
    }
    s->cv.notify_all();
    return TDDA_OK;
}

tdda_status tdda_server_result(tdda_server* s, unsigned long long id, int wait, tdda_request_info* info, double* P) {
    if (!s) return TDDA_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return TDDA_ERR_INVALID_ARGUMENT;
    Request* r = it->second.get();
    if (wait)
        s->cv.wait(lk, [r] { return r->info.state == TDDA_REQ_DONE || r->info.state == TDDA_REQ_FAILED; });
    if (info) *info = r->info;
    if (P && (r->info.state == TDDA_REQ_DONE || r->info.state == TDDA_REQ_FAILED))
        std::memcpy(P, r->P.data(), sizeof(double) * r->P.size());
    return TDDA_OK;
}

tdda_status tdda_server_stats(tdda_server* s, int* queued, int* running, double* bytes, double* peak) {
    if (!s) return TDDA_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    if (queued) *queued = (int)s->queue.size();
    if (running) *running = s->running;
    if (bytes) *bytes = s->bytes;
    if (peak) *peak = s->peak;
    return TDDA_OK;
}

double tdda_server_clock(const tdda_server* s) { return s ? s->now() : 0.0; }

tdda_status tdda_server_destroy(tdda_server* s) {
    if (!s) return TDDA_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    for (auto& t : s->workers) t.join();
    delete s;
    return TDDA_OK;
}

}  // extern "C"
