// server.cpp -- served form: a request loop of generate() calls of different sizes.
//
// fastlem answers one TerrainGenerator::generate() call at a time
// (lem/generator.rs:90-213).  The server takes such calls as they arrive, for models
// registered once, and runs several at once on one GPU:
//   * every registered model keeps a host copy; a request needs a device instance of
//     its model (an fl_graph: graph plus workspace), created on admission and kept
//     resident afterwards for the next request on the same model;
//   * `slots` worker threads each run one request at a time on the instance's own CUDA
//     stream, so the kernels of concurrent requests overlap on the device;
//   * admission is first-come first-served: the oldest waiting request starts when a
//     worker is free and its instance is idle or fits the HBM budget, after evicting
//     idle instances (least recently used first); requests behind it wait, so a large
//     request is never starved by smaller ones;
//   * continuous batching: a request on a small model without a resident instance is
//     solved together with the other such requests waiting at that moment, as one
//     packed model (the batched form, every terrain keeping its own semantics), so the
//     many small solves of a burst of arrivals cost about one;
//   * each request records its queueing time, solve time and latency.
// A request's result is exactly fl_generate's on its own: instances share nothing.

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "fastlem_gb300.h"
#include "kernels.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Model {
    uint32_t n = 0;
    std::vector<uint32_t> row, col, outlets;
    std::vector<double> len, area, xs, ys;
    bool coords = false;
    uint64_t bytes = 0;                 // device bytes of one instance (measured)
    std::vector<fl_graph*> idle;        // resident instances, most recently used last
    uint32_t busy = 0;
};

struct Request {
    uint64_t id = 0;
    uint32_t model = 0;
    std::vector<double> base, k, u, slope;
    std::vector<uint8_t> outlet;
    bool has_slope = false;
    int64_t max_iter = -1;
    double* out = nullptr;
    Clock::time_point arrived, started, finished;
    uint32_t iterations = 0;
    int status = FL_OK;
    std::string error;
    bool done = false;
};

}  // namespace

struct fl_server {
    uint64_t budget = 0;
    uint64_t used = 0;                  // device bytes of all live instances
    uint32_t slots = 0;
    int device = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::vector<std::unique_ptr<Model>> models;
    std::deque<Request*> queue;
    std::map<uint64_t, std::unique_ptr<Request>> requests;
    std::list<std::pair<uint32_t, fl_graph*>> lru;   // idle instances, oldest first
    std::vector<std::thread> workers;
    uint64_t next_id = 1;
    bool stop = false;
    // statistics
    uint32_t active = 0, peak_active = 0;
    uint64_t peak_used = 0, created = 0, evicted = 0, completed = 0, packs = 0,
             packed_requests = 0;
    bool pack = true;                   // continuous batching into packed solves
    uint32_t active_packs = 0;
};

namespace {

// An instance's device footprint before it exists: the measured size of an earlier
// instance of the same model, else fl_model_device_bytes's bound.
uint64_t footprint(const Model& m) {
    if (m.bytes) return m.bytes;
    return fl_model_device_bytes(m.n, m.col.size());
}

void drop_idle(fl_server* s, uint32_t model, fl_graph* g) {
    s->lru.remove(std::make_pair(model, g));
    auto& v = s->models[model]->idle;
    v.erase(std::remove(v.begin(), v.end(), g), v.end());
}

enum Admission { kWait = 0, kAdmit, kNever };

// Continuous batching: requests on models of up to kPackMaxSites sites that find no
// resident instance share packed solves of up to kPackMaxTotal sites.
constexpr uint32_t kPackMaxSites = 1u << 21;
constexpr uint64_t kPackMaxTotal = 24ull << 20;
constexpr size_t kPackMaxRequests = 256;
constexpr uint32_t kMaxPacks = 2;               // packed solves running at a time

// With the lock held: can the head request start now?  Takes an idle instance
// (*inst) or reserves budget for a new one (*reserve), evicting idle instances of
// other models as needed (collected in *evict, destroyed outside the lock).  kNever:
// no instance of the model is idle and a new one is larger than the whole budget (the
// measured size of an earlier instance can exceed the bound checked at submission).
Admission admit(fl_server* s, Request* r, fl_graph** inst, uint64_t* reserve,
                std::vector<fl_graph*>* evict) {
    Model& m = *s->models[r->model];
    if (!m.idle.empty()) {
        *inst = m.idle.back();
        drop_idle(s, r->model, *inst);
        return kAdmit;
    }
    const uint64_t need = footprint(m);
    if (need > s->budget) return kNever;
    uint64_t freeable = 0;
    for (auto& e : s->lru) freeable += s->models[e.first]->bytes;
    if (s->used + need > s->budget + freeable) return kWait;
    while (s->used + need > s->budget && !s->lru.empty()) {
        auto e = s->lru.front();
        s->lru.pop_front();
        auto& v = s->models[e.first]->idle;
        v.erase(std::remove(v.begin(), v.end(), e.second), v.end());
        s->used -= s->models[e.first]->bytes;
        evict->push_back(e.second);
        s->evicted++;
    }
    s->used += need;
    *reserve = need;
    *inst = nullptr;
    return kAdmit;
}

// A request solved in a pack: packing on, a small model, no resident instance to reuse.
bool packable(const fl_server* s, const Request* q) {
    const Model& m = *s->models[q->model];
    return s->pack && m.idle.empty() && m.n <= kPackMaxSites;
}

// With the lock held, the first packable request r: the waiting requests that can share
// one packed solve with it (continuous batching into the batched form): packable, the
// same iteration limit, in arrival order while the pack's site limit and the HBM budget
// (idle instances counted as freeable) allow.  Reserves the packed model's device bytes,
// evicting idle instances least recently used first.  kNever: r alone can never fit.
Admission admit_pack(fl_server* s, Request* r, std::vector<Request*>* pack, uint64_t* reserve,
                     std::vector<fl_graph*>* evict) {
    pack->clear();
    uint64_t freeable = 0;
    for (auto& e : s->lru) freeable += s->models[e.first]->bytes;
    const uint64_t room = s->budget + freeable > s->used ? s->budget + freeable - s->used : 0;
    uint64_t sites = 0, slots = 0, need = 0;
    for (Request* q : s->queue) {
        if (pack->size() >= kPackMaxRequests) break;
        const Model& m = *s->models[q->model];
        if (!packable(s, q) || q->max_iter != r->max_iter || sites + m.n > kPackMaxTotal)
            continue;
        const uint64_t nd = fl_model_device_bytes((uint32_t)(sites + m.n), slots + m.col.size());
        if (nd > room) {
            if (q == r) {
                const uint64_t alone = fl_model_device_bytes(m.n, m.col.size());
                return alone > s->budget ? kNever : kWait;
            }
            continue;
        }
        pack->push_back(q);
        sites += m.n;
        slots += m.col.size();
        need = nd;
    }
    if (pack->empty()) return kWait;
    while (s->used + need > s->budget && !s->lru.empty()) {
        auto e = s->lru.front();
        s->lru.pop_front();
        auto& v = s->models[e.first]->idle;
        v.erase(std::remove(v.begin(), v.end(), e.second), v.end());
        s->used -= s->models[e.first]->bytes;
        evict->push_back(e.second);
        s->evicted++;
    }
    s->used += need;
    *reserve = need;
    return kAdmit;
}

// Solves a pack as one packed model (fl_batch_create_parts / fl_batch_generate_parts):
// every terrain keeps its own semantics, so each result equals its solo generate().
int solve_pack(fl_server* s, const std::vector<Request*>& pack, std::string* err) {
    const size_t k = pack.size();
    std::vector<uint32_t> sites(k), ndef(k);
    std::vector<const uint32_t*> rows(k), cols(k), defs(k);
    std::vector<const double*> lens(k), areas(k), xs(k), ys(k), base(k), kk(k), uu(k), slope(k);
    std::vector<const uint8_t*> outl(k);
    std::vector<double*> outs(k);
    bool coords = true, any_slope = false;
    for (size_t t = 0; t < k; ++t) {
        const Model& m = *s->models[pack[t]->model];
        const Request& q = *pack[t];
        sites[t] = m.n;
        ndef[t] = (uint32_t)m.outlets.size();
        rows[t] = m.row.data();
        cols[t] = m.col.data();
        lens[t] = m.len.data();
        areas[t] = m.area.data();
        defs[t] = m.outlets.data();
        coords = coords && m.coords;
        xs[t] = m.coords ? m.xs.data() : nullptr;
        ys[t] = m.coords ? m.ys.data() : nullptr;
        base[t] = q.base.data();
        kk[t] = q.k.data();
        uu[t] = q.u.data();
        outl[t] = q.outlet.data();
        slope[t] = q.has_slope ? q.slope.data() : nullptr;
        any_slope = any_slope || q.has_slope;
        outs[t] = q.out;
    }
    fl_graph* g = nullptr;
    int rc = fl_batch_create_parts((uint32_t)k, sites.data(), rows.data(), cols.data(), lens.data(),
                                   areas.data(), ndef.data(), defs.data(),
                                   coords ? xs.data() : nullptr, coords ? ys.data() : nullptr, &g);
    if (rc == FL_OK) {
        fl_graph_set_sized_grids(g, 1);
        std::vector<uint32_t> titer(k, 0);
        uint32_t iters = 0;
        rc = fl_batch_generate_parts(g, base.data(), kk.data(), uu.data(), outl.data(),
                                     any_slope ? slope.data() : nullptr, pack[0]->max_iter,
                                     outs.data(), titer.data(), &iters, nullptr, nullptr);
        for (size_t t = 0; t < k; ++t) pack[t]->iterations = titer[t];
    }
    if (rc != FL_OK) *err = fl_last_error();
    fl_graph_destroy(g);
    return rc;
}

void worker(fl_server* s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        Request* r = nullptr;
        fl_graph* inst = nullptr;
        uint64_t reserve = 0;
        std::vector<fl_graph*> evict;
        std::vector<Request*> pack;
        bool never = false;
        s->cv_work.wait(lk, [&] {
            if (s->stop) return true;
            if (s->queue.empty()) return false;
            // small requests without a resident instance: packed solves, at most
            // kMaxPacks at a time, each taking every such request waiting when it starts
            // (the others keep arriving meanwhile and make the next pack larger)
            Request* first_small = nullptr;
            for (Request* q : s->queue)
                if (packable(s, q)) {
                    first_small = q;
                    break;
                }
            if (first_small && s->active_packs < kMaxPacks) {
                const Admission a = admit_pack(s, first_small, &pack, &reserve, &evict);
                if (a == kAdmit) return true;
                if (a == kNever) {              // fails alone below
                    pack.clear();
                    never = true;
                    r = first_small;
                    return true;
                }
            }
            // everything else solo, in arrival order
            for (Request* q : s->queue) {
                if (packable(s, q)) continue;
                const Admission a = admit(s, q, &inst, &reserve, &evict);
                if (a == kWait) return false;
                never = a == kNever;
                r = q;
                return true;
            }
            return false;
        });
        if (s->stop) return;
        if (!pack.empty()) {                    // a packed solve of several requests
            for (Request* q : pack) {
                s->queue.erase(std::find(s->queue.begin(), s->queue.end(), q));
                s->models[q->model]->busy++;
                q->started = Clock::now();
            }
            s->active++;
            s->active_packs++;
            s->peak_active = std::max(s->peak_active, s->active);
            s->peak_used = std::max(s->peak_used, s->used);
            s->packs++;
            s->packed_requests += pack.size();
            lk.unlock();
            s->cv_work.notify_all();
            for (fl_graph* g : evict) fl_graph_destroy(g);
            std::string err;
            const int rc = solve_pack(s, pack, &err);
            lk.lock();
            s->used -= reserve;
            s->active--;
            s->active_packs--;
            for (Request* q : pack) {
                s->models[q->model]->busy--;
                q->status = rc;
                q->error = err;
                q->finished = Clock::now();
                q->done = true;
                s->completed++;
            }
            s->cv_done.notify_all();
            s->cv_work.notify_all();
            continue;
        }
        s->queue.erase(std::find(s->queue.begin(), s->queue.end(), r));
        if (never) {                          // fails alone; the requests behind it go on
            r->status = FL_ERR_OUT_OF_MEMORY;
            r->error = "fl_server: the model's instance is larger than the HBM budget";
            r->started = r->finished = Clock::now();
            r->done = true;
            s->completed++;
            s->cv_done.notify_all();
            s->cv_work.notify_all();
            continue;
        }
        Model& m = *s->models[r->model];
        m.busy++;
        s->active++;
        s->peak_active = std::max(s->peak_active, s->active);
        r->started = Clock::now();
        lk.unlock();
        s->cv_work.notify_all();           // the next request may fit as well
        for (fl_graph* g : evict) fl_graph_destroy(g);
        int rc = FL_OK;
        std::string err;
        if (!inst) {
            rc = fl_graph_create(m.n, m.row.data(), m.col.data(), m.len.data(), m.area.data(),
                                 m.outlets.data(), (uint32_t)m.outlets.size(),
                                 m.coords ? m.xs.data() : nullptr,
                                 m.coords ? m.ys.data() : nullptr, &inst);
            if (rc != FL_OK) err = fl_last_error();
            // concurrent solves: small models take only part of the GPU
            if (rc == FL_OK) fl_graph_set_sized_grids(inst, 1);
        }
        uint64_t real = inst ? fl_graph_device_bytes(inst) : 0;
        if (rc == FL_OK) {
            rc = fl_generate(inst, m.n, r->base.data(), r->k.data(), r->u.data(),
                             r->outlet.data(), r->has_slope ? r->slope.data() : nullptr,
                             r->max_iter, r->out, &r->iterations);
            if (rc != FL_OK) err = fl_last_error();
        }
        lk.lock();
        if (reserve) {                      // the reservation becomes the measured size
            s->used -= reserve;
            if (inst) {
                s->used += real;
                m.bytes = real;
                s->created++;
            }
        }
        s->peak_used = std::max(s->peak_used, s->used);
        if (inst) {
            if (rc == FL_OK) {
                m.idle.push_back(inst);
                s->lru.emplace_back(r->model, inst);
            } else {                        // a failed instance is not reused
                s->used -= m.bytes;
                lk.unlock();
                fl_graph_destroy(inst);
                lk.lock();
            }
        }
        m.busy--;
        s->active--;
        r->status = rc;
        r->error = err;
        r->finished = Clock::now();
        r->done = true;
        s->completed++;
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

}  // namespace

extern "C" {

int fl_server_create(uint64_t hbm_budget_bytes, uint32_t slots, fl_server** out) {
    if (!out || slots == 0 || hbm_budget_bytes == 0) {
        fl::set_last_error("fl_server_create: invalid arguments");
        return FL_ERR_INVALID_ARGUMENT;
    }
    fl_server* s = new fl_server();
    s->budget = hbm_budget_bytes;
    s->slots = slots;
    if (cudaGetDevice(&s->device) != cudaSuccess) s->device = 0;
    try {
        for (uint32_t i = 0; i < slots; ++i) s->workers.emplace_back(worker, s);
    } catch (const std::system_error&) {
        fl_server_destroy(s);                  // stops and joins the workers started
        fl::set_last_error("fl_server_create: cannot start the worker threads");
        return FL_ERR_OUT_OF_MEMORY;
    }
    *out = s;
    return FL_OK;
}

int fl_server_add_model(fl_server* s, uint32_t n, const uint32_t* row_ptr, const uint32_t* col,
                        const double* len, const double* area, const uint32_t* default_outlets,
                        uint32_t n_default, const double* xs, const double* ys,
                        uint32_t* model_id) {
    if (!s || !row_ptr || !area || !model_id || n == 0 || (n_default && !default_outlets) ||
        (row_ptr[n] && (!col || !len))) {
        fl::set_last_error("fl_server_add_model: invalid arguments");
        return FL_ERR_INVALID_ARGUMENT;
    }
    auto m = std::make_unique<Model>();
    m->n = n;
    m->row.assign(row_ptr, row_ptr + n + 1);
    const uint64_t nnz = row_ptr[n];
    m->col.assign(col, col + nnz);
    m->len.assign(len, len + nnz);
    m->area.assign(area, area + n);
    m->outlets.assign(default_outlets, default_outlets + n_default);
    if (xs && ys) {
        m->coords = true;
        m->xs.assign(xs, xs + n);
        m->ys.assign(ys, ys + n);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    *model_id = (uint32_t)s->models.size();
    s->models.push_back(std::move(m));
    return FL_OK;
}

int fl_server_submit(fl_server* s, uint32_t model_id, const double* base,
                     const double* erodibility, const double* uplift, const uint8_t* is_outlet,
                     const double* max_slope, int64_t max_iteration, double* out_elev,
                     uint64_t* ticket) {
    if (!s || !ticket) return FL_ERR_INVALID_ARGUMENT;
    if (!base || !erodibility || !uplift || !is_outlet) return FL_ERR_PARAMETERS_NOT_SET;
    if (!out_elev) return FL_ERR_INVALID_ARGUMENT;
    std::unique_ptr<Request> r(new Request());
    uint32_t n = 0;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (model_id >= s->models.size()) return FL_ERR_MODEL_NOT_SET;
        n = s->models[model_id]->n;
        if (s->budget < footprint(*s->models[model_id]) && s->models[model_id]->idle.empty()) {
            fl::set_last_error("fl_server_submit: the model does not fit the HBM budget");
            return FL_ERR_OUT_OF_MEMORY;
        }
    }
    r->model = model_id;
    r->base.assign(base, base + n);
    r->k.assign(erodibility, erodibility + n);
    r->u.assign(uplift, uplift + n);
    r->outlet.assign(is_outlet, is_outlet + n);
    if (max_slope) {
        r->has_slope = true;
        r->slope.assign(max_slope, max_slope + n);
    }
    r->max_iter = max_iteration;
    r->out = out_elev;
    r->arrived = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        *ticket = r->id;
        s->queue.push_back(r.get());
        s->requests[r->id] = std::move(r);
    }
    s->cv_work.notify_all();
    return FL_OK;
}

int fl_server_wait(fl_server* s, uint64_t ticket, uint32_t* out_iterations, double* latency_ms,
                   double* queue_ms, double* solve_ms) {
    if (!s) return FL_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(ticket);
    if (it == s->requests.end()) {
        fl::set_last_error("fl_server_wait: unknown ticket");
        return FL_ERR_INVALID_ARGUMENT;
    }
    Request* r = it->second.get();
    s->cv_done.wait(lk, [&] { return r->done; });
    if (out_iterations) *out_iterations = r->iterations;
    if (latency_ms) *latency_ms = ms_between(r->arrived, r->finished);
    if (queue_ms) *queue_ms = ms_between(r->arrived, r->started);
    if (solve_ms) *solve_ms = ms_between(r->started, r->finished);
    const int rc = r->status;
    if (rc != FL_OK) fl::set_last_error(r->error.c_str());
    s->requests.erase(it);
    return rc;
}

int fl_server_stats(fl_server* s, uint64_t* out, uint32_t cap) {
    if (!s || !out) return FL_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    const uint64_t v[] = {s->completed, s->peak_active, s->peak_used, s->used, s->created,
                          s->evicted, (uint64_t)s->queue.size(), s->packs, s->packed_requests};
    for (uint32_t i = 0; i < cap && i < sizeof v / sizeof v[0]; ++i) out[i] = v[i];
    return FL_OK;
}

int fl_server_set_packing(fl_server* s, int enable) {
    if (!s) return FL_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    s->pack = enable != 0;
    return FL_OK;
}

void fl_server_destroy(fl_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->workers) t.join();
    for (auto& m : s->models)
        for (fl_graph* g : m->idle) fl_graph_destroy(g);
    delete s;
}

}  // extern "C"
