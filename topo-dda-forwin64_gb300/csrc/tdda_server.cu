// tdda_server.cu -- continuous-batching request loop with resident operators.
//
// Requests (one structure + its incidences each) queue in arrival order.
// Workers run concurrently, each on its own CUDA streams.
//
// Operators stay resident.  The operator of a request -- its core: lattice,
// spacing, wavelength, material and background index, hence its Green
// spectrum -- is kept after its requests finish, together with a pool of its
// models (Krylov vectors, densities), and is reused by later requests of the
// same operator (the reference keeps one AProductCore for all of its
// DDAModels, EvoDDAModel.h:14).  Idle operators are evicted least recently
// used first when admission needs their memory.
//
// FP32+refine: continuous batching by FFT grid shape.  A worker runs one shape
// session (tdda_session.h): slots for max_group right-hand sides of lattices
// that share one FFT grid shape, whose FP32 inner solves run in one launch per
// pass.  Between rounds (a round is at most 32 inner steps) the worker frees the
// slots of finished right-hand sides and admits queued requests of the same
// grid shape into free slots, so requests join running work as it finishes.
//
// FP64: a worker takes the first request that fits and the queued requests of
// the same operator (up to max_group right-hand sides) and solves them in one
// batched solve on the operator's core; no refill inside a running FP64 solve.
//
// Admission is first fit under the HBM budget: a request whose memory (a new
// core, models beyond the operator's pool, a new shape) does not fit what the
// budget leaves free waits while requests behind it that fit run; a request
// larger than the whole budget fails.  Every result is computed exactly as the
// same request alone: the batched kernels treat every right-hand side
// independently.
#include <algorithm>
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
#include "tdda_session.h"

namespace {

struct Operator;

struct Request {
    unsigned long long id = 0;
    tdda_request_desc d{};
    std::vector<int> R;
    std::vector<double> material, diel_old, nK, nE0, E0;
    std::vector<double> P;  // 3N x nrhs complex
    tdda_request_info info{};
    double bytes = 0;
    Operator* op = nullptr;  // while admitted
    std::vector<tdda_model*> pooled;  // models taken from the operator's pool at admission
    int remaining = 0;       // right-hand sides not finished
};

bool same_operator(const Request& a, const Request& b) {
    const tdda_request_desc &x = a.d, &y = b.d;
    return x.Nx == y.Nx && x.Ny == y.Ny && x.Nz == y.Nz && x.N == y.N && x.d == y.d && x.lam == y.lam &&
           x.nback == y.nback && a.material == b.material && a.R == b.R;
}

// A resident operator: the core of one (lattice, spacing, wavelength, material,
// background) and a pool of its models.
struct Operator {
    Request key;                     // the operator's fields (a copy of the first request's)
    tdda_core* core = nullptr;       // built by the worker that first admits it
    std::vector<tdda_model*> pool;   // models not in use
    int nmodels = 0;                 // models created (pooled or in use)
    int owner = -1;                  // the worker running its requests, or -1
    int active = 0;                  // its requests admitted and not finished
    double last_used = 0;
    double core_bytes = 0, model_bytes = 0;
    int grid[3] = {0, 0, 0};
    double bytes() const { return core_bytes + nmodels * model_bytes; }
};

struct IdleShape {
    int grid[3];
    tdda_session::Shape* s;
    double bytes;
    double last_used;
};

// An evicted operator (its core and pooled models) or shape, destroyed outside
// the server's lock
struct Evicted {
    tdda_core* core = nullptr;
    std::vector<tdda_model*> models;
    tdda_session::Shape* shape = nullptr;
};

// Idle operators and shapes kept resident beyond what the budget forces out.
// Hundreds of cores alive at once (their allocations, streams and pinned state)
// slowed every later request of the process by about a third, also after they
// were destroyed, while a stream of requests rarely returns to an operator
// long after its last use.
constexpr int kMaxIdleOperators = 32;
constexpr int kMaxIdleShapes = 48;

}  // namespace

struct tdda_server_s {
    tdda_server_desc desc{};
    std::chrono::steady_clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request*> queue;
    std::unordered_map<unsigned long long, std::unique_ptr<Request>> all;
    std::vector<std::unique_ptr<Operator>> ops;  // resident operators
    std::vector<IdleShape> idle_shapes;
    unsigned long long next_id = 1;
    int running = 0;
    double bytes = 0, peak = 0;  // resident operators and models, shapes, dry-run requests
    bool stop = false;
    std::vector<std::thread> workers;
    tdda_server_counters counters{};
    // evicted operators and shapes not yet destroyed: a core's teardown waits for
    // graph operations of other streams, so workers destroy them after leaving mu
    std::vector<Evicted> graveyard;

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    void add_bytes(double b) {
        bytes += b;
        if (bytes > peak) peak = bytes;
    }

    int core_rhs() const { return desc.precision == TDDA_FP64 ? desc.max_group : 1; }

    Operator* find_op(const Request* r) {
        for (auto& o : ops)
            if (same_operator(o->key, *r)) return o.get();
        return nullptr;
    }

    // bytes a request adds: its operator's core if not resident, its models beyond
    // the operator's free pool
    double need_of(const Request* r, const Operator* op) const {
        const double mb = tdda_session::model_bytes(r->d.N, desc.precision);
        const double core = op ? 0.0 : tdda_session::core_bytes(r->d.Nx, r->d.Ny, r->d.Nz, r->d.N, core_rhs());
        const int extra = std::max(0, r->d.nrhs - (op ? (int)op->pool.size() : 0));
        return core + extra * mb;
    }

    // evict idle resident operators and idle shapes, least recently used first,
    // until `need` more bytes fit the budget (never `keep`); called with mu held
    bool make_room(double need, const Operator* keep) {
        while (bytes + need > desc.hbm_budget_bytes) {
            int best = -1, kind = 0;
            double t = 1e300;
            for (size_t i = 0; i < ops.size(); i++) {
                const Operator* o = ops[i].get();
                if (o == keep || o->owner >= 0 || o->active > 0 || !o->core) continue;
                if (o->last_used < t) t = o->last_used, best = (int)i, kind = 0;
            }
            for (size_t i = 0; i < idle_shapes.size(); i++)
                if (idle_shapes[i].last_used < t) t = idle_shapes[i].last_used, best = (int)i, kind = 1;
            if (best < 0) return false;
            if (kind == 0) evict_operator(best);
            else evict_shape(best);
        }
        return true;
    }

    // move an idle operator or shape to the graveyard (mu held); its bytes are
    // counted free now, and the worker that evicted it destroys it (drain) before
    // it allocates anything
    void evict_operator(int i) {
        Operator* o = ops[i].get();
        Evicted e;
        e.core = o->core;
        e.models = std::move(o->pool);
        graveyard.push_back(std::move(e));
        bytes -= o->bytes();
        counters.operators_evicted++;
        ops.erase(ops.begin() + i);
    }
    void evict_shape(int i) {
        Evicted e;
        e.shape = idle_shapes[i].s;
        graveyard.push_back(std::move(e));
        bytes -= idle_shapes[i].bytes;
        idle_shapes.erase(idle_shapes.begin() + i);
    }

    // keep at most kMaxIdleOperators idle operators and kMaxIdleShapes idle
    // shapes, least recently used out first (mu held)
    void trim_idle() {
        for (;;) {
            int idle = 0, best = -1;
            double t = 1e300;
            for (size_t i = 0; i < ops.size(); i++) {
                const Operator* o = ops[i].get();
                if (o->owner >= 0 || o->active > 0 || !o->core) continue;
                idle++;
                if (o->last_used < t) t = o->last_used, best = (int)i;
            }
            if (idle <= kMaxIdleOperators) break;
            evict_operator(best);
        }
        while ((int)idle_shapes.size() > kMaxIdleShapes) {
            int best = 0;
            for (size_t i = 1; i < idle_shapes.size(); i++)
                if (idle_shapes[i].last_used < idle_shapes[best].last_used) best = (int)i;
            evict_shape(best);
        }
    }

    // destroy what was evicted (outside mu)
    void drain() {
        std::vector<Evicted> g;
        {
            std::lock_guard<std::mutex> lk(mu);
            g.swap(graveyard);
        }
        for (Evicted& e : g) {
            for (tdda_model* m : e.models) tdda_model_destroy(m);
            if (e.core) tdda_core_destroy(e.core);
            if (e.shape) tdda_session::shape_destroy(e.shape);
        }
    }

    // reserve the operator entry and the memory of request r for worker `me`
    // (mu held); false when it does not fit now
    bool reserve(Request* r, int me) {
        Operator* op = find_op(r);
        if (op && op->owner >= 0 && op->owner != me) return false;  // another worker runs it
        const double need = need_of(r, op);
        if (!make_room(need, op)) return false;
        if (!op) {
            auto o = std::make_unique<Operator>();
            o->key = *r;
            o->key.P.clear();
            o->core_bytes = tdda_session::core_bytes(r->d.Nx, r->d.Ny, r->d.Nz, r->d.N, core_rhs());
            o->model_bytes = tdda_session::model_bytes(r->d.N, desc.precision);
            tdda_session::grid_of_box(r->d.Nx, r->d.Ny, r->d.Nz, o->grid);
            op = o.get();
            ops.push_back(std::move(o));
        } else {
            counters.operator_hits++;
        }
        add_bytes(need);
        op->nmodels += std::max(0, r->d.nrhs - (int)op->pool.size());
        // the pooled models this request will use leave the pool now, so a request
        // reserved after it cannot count them again
        while ((int)r->pooled.size() < r->d.nrhs && !op->pool.empty()) {
            r->pooled.push_back(op->pool.back());
            op->pool.pop_back();
        }
        op->owner = me;
        op->active++;
        op->last_used = now();
        r->op = op;
        r->remaining = r->d.nrhs;
        r->info.state = TDDA_REQ_RUNNING;
        r->info.t_start = now();
        running++;
        return true;
    }

    // the first queued request that can start (first fit); with nothing in flight
    // a request that cannot fit even alone fails
    Request* take_first(int me, const int* grid) {
        for (size_t i = 0; i < queue.size(); i++) {
            Request* r = queue[i];
            if (grid) {
                int g[3];
                tdda_session::grid_of_box(r->d.Nx, r->d.Ny, r->d.Nz, g);
                if (g[0] != grid[0] || g[1] != grid[1] || g[2] != grid[2]) continue;
            }
            if (reserve(r, me)) {
                queue.erase(queue.begin() + (long)i);
                return r;
            }
            if (!grid && running == 0 && i == 0) {
                // alone beyond the budget: nothing resident can be evicted to make room
                queue.erase(queue.begin());
                r->info.state = TDDA_REQ_FAILED;
                r->info.status = TDDA_ERR_OUT_OF_MEMORY;
                r->info.t_done = now();
                cv.notify_all();
                i--;
            }
        }
        return nullptr;
    }

    void finish_request(Request* r, double t) {
        r->info.t_done = t;
        if (r->info.state == TDDA_REQ_RUNNING) r->info.state = r->info.status == TDDA_OK ? TDDA_REQ_DONE
                                                                                      : TDDA_REQ_FAILED;
        running--;
        if (r->op) {
            r->op->active--;
            r->op->last_used = t;
            r->op = nullptr;
        }
    }

    void worker(int me);
    void run_dry(int me);
    void run_fp64(int me);
    void run_fp32(int me);
    // the models of a request on its operator's core (pool or new), set to its
    // incidences and densities; outside mu
    tdda_status models_for(Request* r, std::vector<tdda_model*>& out);
};

tdda_status tdda_server_s::models_for(Request* r, std::vector<tdda_model*>& out) {
    Operator* op = r->op;
    if (!op->core) {
        tdda_core_desc cd;
        cd.Nx = r->d.Nx;
        cd.Ny = r->d.Ny;
        cd.Nz = r->d.Nz;
        cd.N = r->d.N;
        cd.R = r->R.data();
        cd.d = r->d.d;
        cd.lam = r->d.lam;
        cd.nback = r->d.nback;
        cd.material = r->material.data();
        cd.nmat = r->d.nmat;
        cd.method = TDDA_METHOD_LDR;
        cd.max_rhs = core_rhs();
        cd.device = desc.device;
        tdda_status st = tdda_core_create(&cd, &op->core);
        if (st != TDDA_OK) return st;
        std::lock_guard<std::mutex> lk(mu);
        counters.operators_built++;
    }
    for (int k = 0; k < r->d.nrhs; k++) {
        tdda_model* m = nullptr;
        if (!r->pooled.empty()) {
            m = r->pooled.back();
            r->pooled.pop_back();
        }
        tdda_status st;
        if (m) {
            st = tdda_session::model_reinit(m, &r->nK[3 * k], r->E0[k], &r->nE0[3 * k], r->diel_old.data());
        } else {
            st = tdda_model_create(op->core, &r->nK[3 * k], r->E0[k], &r->nE0[3 * k], r->diel_old.data(), &m);
        }
        if (st != TDDA_OK) {
            std::lock_guard<std::mutex> lk(mu);
            if (m) op->pool.push_back(m);
            for (tdda_model* q : r->pooled) op->pool.push_back(q);
            r->pooled.clear();
            return st;
        }
        out.push_back(m);
    }
    return TDDA_OK;
}

void tdda_server_s::worker(int me) {
    if (desc.dry_run) return run_dry(me);
    if (desc.precision == TDDA_FP64) return run_fp64(me);
    return run_fp32(me);
}

// Scheduler only: a request takes dry_run_ms; the admission and the grouping of
// requests that share an operator are the FP64 path's, without device work
// (the resident operators hold no memory here, so each group reserves its
// request bytes while it runs).
void tdda_server_s::run_dry(int me) {
    (void)me;
    for (;;) {
        std::vector<Request*> g;
        double gbytes = 0;
        {
            std::unique_lock<std::mutex> lk(mu);
            for (;;) {
                for (size_t i = 0; i < queue.size() && g.empty(); i++) {
                    Request* r = queue[i];
                    const bool fits = bytes + r->bytes <= desc.hbm_budget_bytes;
                    if (!fits && !(i == 0 && running == 0)) continue;
                    queue.erase(queue.begin() + (long)i);
                    g.push_back(r);
                    int rhs = r->d.nrhs;
                    double extra = 0;
                    for (size_t j = i; j < queue.size();) {
                        Request* o = queue[j];
                        const double add =
                            tdda_request_bytes(o->d.Nx, o->d.Ny, o->d.Nz, o->d.N, rhs + o->d.nrhs, desc.precision) -
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
                }
                if (!g.empty()) break;
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
            add_bytes(gbytes);
        }
        const bool too_big = gbytes > desc.hbm_budget_bytes;
        if (!too_big) std::this_thread::sleep_for(std::chrono::duration<double, std::milli>(desc.dry_run_ms));
        {
            std::lock_guard<std::mutex> lk(mu);
            bytes -= gbytes;
            const double t = now();
            for (Request* r : g) {
                r->info.status = too_big ? TDDA_ERR_OUT_OF_MEMORY : TDDA_OK;
                if (too_big) r->info.state = TDDA_REQ_FAILED;
                finish_request(r, t);
            }
        }
        cv.notify_all();
    }
}

void tdda_server_s::run_fp64(int me) {
    for (;;) {
        std::vector<Request*> g;
        {
            std::unique_lock<std::mutex> lk(mu);
            for (;;) {
                Request* r = take_first(me, nullptr);
                if (r) {
                    g.push_back(r);
                    int rhs = r->d.nrhs;
                    for (size_t j = 0; j < queue.size();) {  // queued requests of the same operator
                        Request* o = queue[j];
                        if (same_operator(*o, *r) && rhs + o->d.nrhs <= desc.max_group && reserve(o, me)) {
                            g.push_back(o);
                            rhs += o->d.nrhs;
                            queue.erase(queue.begin() + (long)j);
                        } else {
                            j++;
                        }
                    }
                    for (Request* q : g) q->info.group = rhs;
                    break;
                }
                if (stop && queue.empty()) return;
                cv.wait(lk);
            }
        }
        drain();
        std::vector<tdda_model*> models;
        std::vector<std::pair<Request*, int>> owner;
        tdda_status st = TDDA_OK;
        for (Request* r : g) {
            std::vector<tdda_model*> ms;
            if (st == TDDA_OK) st = models_for(r, ms);
            for (size_t k = 0; k < ms.size(); k++) {
                models.push_back(ms[k]);
                owner.emplace_back(r, (int)k);
            }
        }
        std::vector<tdda_solve_info> infos(models.size());
        if (st == TDDA_OK) {
            st = tdda_solve_batch(models.data(), (int)models.size(), TDDA_FP64, desc.max_it, desc.tol, infos.data());
            if (st == TDDA_NOT_CONVERGED || st == TDDA_BREAKDOWN || st == TDDA_ERR_NAN) st = TDDA_OK;  // per RHS
        }
        for (Request* r : g) {
            r->info.status = st;
            r->info.iterations = 0;
            r->info.error = 0;
        }
        if (st == TDDA_OK) {
            for (size_t i = 0; i < models.size(); i++) {
                Request* r = owner[i].first;
                const int k = owner[i].second;
                const size_t n6 = 6 * (size_t)r->d.N;
                tdda_status gs = tdda_model_get(models[i], TDDA_FIELD_P, r->P.data() + k * n6, TDDA_MEM_HOST);
                const tdda_status ss = gs != TDDA_OK ? gs : (tdda_status)infos[i].status;
                if (ss != TDDA_OK && r->info.status == TDDA_OK) r->info.status = ss;
                r->info.iterations = std::max(r->info.iterations, infos[i].iterations);
                r->info.error = std::max(r->info.error, infos[i].error);
            }
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            const double t = now();
            for (tdda_model* m : models) g[0]->op->pool.push_back(m);
            Operator* op = g[0]->op;
            for (Request* r : g) finish_request(r, t);
            if (op && op->active == 0) op->owner = -1;
            trim_idle();
        }
        drain();
        cv.notify_all();
    }
}

void tdda_server_s::run_fp32(int me) {
    for (;;) {
        // the first request that fits opens (or reuses) a shape session of its grid
        Request* first = nullptr;
        tdda_session::Shape* sh = nullptr;
        double sh_bytes = 0;
        int grid[3];
        {
            std::unique_lock<std::mutex> lk(mu);
            for (;;) {
                first = take_first(me, nullptr);
                if (first) break;
                if (stop && queue.empty()) return;
                cv.wait(lk);
            }
            tdda_session::grid_of_box(first->d.Nx, first->d.Ny, first->d.Nz, grid);
            for (size_t i = 0; i < idle_shapes.size(); i++)
                if (std::memcmp(idle_shapes[i].grid, grid, sizeof(grid)) == 0) {
                    sh = idle_shapes[i].s;
                    sh_bytes = idle_shapes[i].bytes;
                    idle_shapes.erase(idle_shapes.begin() + (long)i);
                    break;
                }
            if (!sh) {
                sh_bytes = tdda_session::shape_bytes(grid, desc.max_group);
                make_room(sh_bytes, first->op);
                add_bytes(sh_bytes);  // over budget only if nothing idle was left to evict
                counters.shapes_built++;
            }
        }
        drain();
        tdda_status st = TDDA_OK;
        if (!sh) st = tdda_session::shape_create(desc.device, grid, desc.max_group, &sh);
        // request of each slot's model, and its right-hand side index
        std::vector<std::pair<Request*, int>> slot_of(desc.max_group, {nullptr, 0});
        std::vector<tdda_model*> slot_model(desc.max_group, nullptr);
        auto fail_request = [&](Request* r, tdda_status s2) {
            std::lock_guard<std::mutex> lk(mu);
            r->info.status = s2;
            r->info.state = TDDA_REQ_FAILED;
            finish_request(r, now());
        };
        // admit a reserved request: its models into free slots
        auto admit = [&](Request* r) -> bool {
            std::vector<tdda_model*> ms;
            tdda_status s2 = models_for(r, ms);
            int used = 0;
            for (size_t k = 0; k < ms.size() && s2 == TDDA_OK; k++) {
                int slot = -1;
                s2 = tdda_session::shape_admit(sh, ms[k], desc.max_it, desc.tol, &slot,
                                               desc.precision == TDDA_FP32_JACOBI ? 1
                                               : desc.precision == TDDA_FP32_AUTO ? 2
                                                                                  : 0);
                if (s2 == TDDA_OK) slot_of[slot] = {r, (int)k}, slot_model[slot] = ms[k], used++;
            }
            if (s2 != TDDA_OK) {
                {
                    std::lock_guard<std::mutex> lk(mu);
                    for (size_t k = used; k < ms.size(); k++) r->op->pool.push_back(ms[k]);
                }
                r->remaining -= used;  // admitted slots finish on their own
                if (used == 0) fail_request(r, s2);
                else r->info.status = s2;
                return false;
            }
            return true;
        };
        if (st != TDDA_OK) {
            fail_request(first, st);
            std::lock_guard<std::mutex> lk(mu);
            bytes -= sh_bytes;
            if (first->op && first->op->active == 0) first->op->owner = -1;
            cv.notify_all();
            continue;
        }
        first->info.group = first->d.nrhs;
        admit(first);
        for (;;) {
            // refill: queued requests of this grid shape, into the free slots
            std::vector<Request*> joined;
            {
                std::lock_guard<std::mutex> lk(mu);
                int free_slots = desc.max_group - tdda_session::shape_active(sh);
                for (size_t i = 0; i < queue.size() && free_slots > 0;) {
                    Request* r = queue[i];
                    int g[3];
                    tdda_session::grid_of_box(r->d.Nx, r->d.Ny, r->d.Nz, g);
                    if (std::memcmp(g, grid, sizeof(g)) == 0 && r->d.nrhs <= free_slots && reserve(r, me)) {
                        queue.erase(queue.begin() + (long)i);
                        free_slots -= r->d.nrhs;
                        joined.push_back(r);
                    } else {
                        i++;
                    }
                }
            }
            drain();
            const int before = tdda_session::shape_active(sh);
            for (Request* r : joined) {
                r->info.group = before + r->d.nrhs;
                if (admit(r) && before > 0) {
                    std::lock_guard<std::mutex> lk(mu);
                    counters.joined_running++;
                }
            }
            const int active = tdda_session::shape_active(sh);
            if (active == 0) break;
            {
                std::lock_guard<std::mutex> lk(mu);
                counters.max_slots_in_use = std::max(counters.max_slots_in_use, active);
                std::vector<const Operator*> lat;
                for (auto& so : slot_of)
                    if (so.first && std::find(lat.begin(), lat.end(), so.first->op) == lat.end())
                        lat.push_back(so.first->op);
                counters.max_lattices_in_use = std::max(counters.max_lattices_in_use, (int)lat.size());
                counters.rounds++;
            }
            std::vector<tdda_session::Done> done;
            st = tdda_session::shape_step(sh, &done);
            if (st != TDDA_OK) {
                // a device error: fail every request holding a slot, free the slots'
                // models (their state is unknown) and drop the shape
                std::lock_guard<std::mutex> lk(mu);
                const double t = now();
                for (size_t k = 0; k < slot_of.size(); k++) {  // the models first: finishing clears r->op
                    Request* r = slot_of[k].first;
                    if (!r || !slot_model[k]) continue;
                    tdda_model_destroy(slot_model[k]);
                    slot_model[k] = nullptr;
                    if (r->op) {
                        r->op->nmodels--;
                        bytes -= r->op->model_bytes;
                    }
                }
                for (auto& so : slot_of) {
                    Request* r = so.first;
                    if (!r || r->info.state != TDDA_REQ_RUNNING) continue;
                    r->info.status = st;
                    r->info.state = TDDA_REQ_FAILED;
                    finish_request(r, t);
                }
                break;
            }
            for (const auto& dn : done) {
                Request* r = slot_of[dn.slot].first;
                const int k = slot_of[dn.slot].second;
                slot_of[dn.slot] = {nullptr, 0};
                slot_model[dn.slot] = nullptr;
                const size_t n6 = 6 * (size_t)r->d.N;
                tdda_status gs = tdda_model_get(dn.model, TDDA_FIELD_P, r->P.data() + k * n6, TDDA_MEM_HOST);
                const tdda_status ss = gs != TDDA_OK ? gs : (tdda_status)dn.info.status;
                std::lock_guard<std::mutex> lk(mu);
                if (ss != TDDA_OK && r->info.status == TDDA_OK) r->info.status = ss;
                r->info.iterations = std::max(r->info.iterations, dn.info.iterations);
                r->info.error = std::max(r->info.error, dn.info.error);
                r->op->pool.push_back(dn.model);
                if (--r->remaining == 0) finish_request(r, now());
            }
            cv.notify_all();
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            if (st == TDDA_OK) {
                idle_shapes.push_back(IdleShape{{grid[0], grid[1], grid[2]}, sh, sh_bytes, now()});
            } else {
                Evicted e;
                e.shape = sh;
                graveyard.push_back(std::move(e));
                bytes -= sh_bytes;
            }
            for (auto& o : ops)
                if (o->owner == me && o->active == 0) o->owner = -1;
            trim_idle();
        }
        drain();
        cv.notify_all();
    }
}

extern "C" {

tdda_status tdda_server_create(const tdda_server_desc* desc, tdda_server** out) {
    if (!desc || !out || desc->workers < 1 || desc->workers > 64 || !(desc->hbm_budget_bytes > 0) ||
        desc->max_group < 1 || desc->max_group > 64 ||
        (desc->precision != TDDA_FP64 && desc->precision != TDDA_FP32_REFINE && desc->precision != TDDA_FP32_JACOBI &&
         desc->precision != TDDA_FP32_AUTO))
        return TDDA_ERR_INVALID_ARGUMENT;
    if (!desc->dry_run && tdda_device_count() < 1) return TDDA_ERR_NO_DEVICE;
    tdda_server* s = new tdda_server_s();
    s->desc = *desc;
    s->t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < desc->workers; i++) s->workers.emplace_back([s, i] { s->worker(i); });
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

tdda_status tdda_server_counters_get(tdda_server* s, tdda_server_counters* out) {
    if (!s || !out) return TDDA_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->counters;
    out->resident_operators = (int)s->ops.size();
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
    s->drain();
    for (auto& is : s->idle_shapes) tdda_session::shape_destroy(is.s);
    for (auto& o : s->ops) {
        for (tdda_model* m : o->pool) tdda_model_destroy(m);
        if (o->core) tdda_core_destroy(o->core);
    }
    delete s;
    return TDDA_OK;
}

}  // extern "C"
