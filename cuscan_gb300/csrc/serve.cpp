// Fit-request server: continuous batching of HDBSCAN fits on one GPU.
//
// Requests are queued in arrival order and admitted onto execution slots as slots and device
// memory free up. Every slot owns a context (its own CUDA stream and workspace) and a worker
// thread, so the fits of different slots overlap on the device: while one slot's host thread
// waits for a Borůvka round or runs the host extraction, the kernels of the others run.
//
// Admission is by device-memory budget. A slot's commitment is the larger of the workspace
// it already holds and, while it runs a request, the upper bound cuscan_fit_workspace_bytes
// gives for that request. The head of the queue is admitted only while the sum of all
// commitments stays within the budget; an idle slot whose retained workspace is in the way is
// told to release it first. A request whose own bound exceeds the budget fails with
// CUSCAN_MEMORY at once. The queue is first in, first out: a request that does not fit is
// never overtaken, so no request starves.
//
// Small fits are packed: a slot that admits a fit of at most CUSCAN_PACK_MAX_ROWS rows at the
// head of the queue also takes the small fits queued right behind it (in order, up to the pack
// limit, while the budget allows) and runs them as one pack (cuscan_fit_core_packed: each step
// of every fit in one launch). A pack commits the sum of its requests' bounds on top of the
// workspace the slot holds, since its fits use buffers of their own.
//
// A request runs the estimator flow of crates/hdbscan/src/estimator.rs:1034-1392 for one
// point set: non-finite rows are set aside (crates/hdbscan-core/src/finite.rs:65-131), the
// fit core runs on the finite rows (cuscan_fit_core), and the host extraction
// (cuscan_clusters_from_spanning_tree) gives labels and membership strengths; rows set aside
// get label -1 and strength 0. Results stay on the server until cuscan_server_release.
//
// The reference has no serving layer; this is the request loop around its fit entry point.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "cuscan_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

void set_err(char *err, size_t len, const char *msg) {
    if (err && len) std::snprintf(err, len, "%s", msg);
}

enum class Kind { Fit = 0, Predict = 1 };

struct Request {
    int64_t id = 0;
    Kind kind = Kind::Fit;
    const cuscan_predictor *predictor = nullptr;  // predict requests
    const float *x = nullptr;
    int64_t n = 0;
    int32_t d = 0;
    int32_t min_samples = 0;
    int32_t precision = 0;
    cuscan_extract_config cfg{};
    int64_t bytes = 0;  // admission bound
    Clock::time_point t_submit, t_admit, t_done;
    double prep_ms = 0, fit_ms = 0, extract_ms = 0;  // host wall time of the three phases
    int slot = -1;
    int32_t pack_size = 1;
    bool done = false;
    int status = CUSCAN_OK;
    std::string error;
    // results
    int64_t finite_rows = 0;
    int32_t clusters = 0;
    std::vector<int32_t> labels;
    std::vector<float> probabilities;
    std::vector<float> core;
    std::vector<double> sorted_mst;
    cuscan_fit_stats stats{};
    std::vector<double> strengths;      // predict requests
    std::vector<int32_t> connectors;
};

enum class Task { None, Fit, Release, Stop };

struct Slot {
    int index = 0;
    cuscan_ctx *ctx = nullptr;
    int64_t reserved = 0;   // workspace held (bytes)
    int64_t running = 0;    // admission bound of the request it runs (sum over a pack)
    Task task = Task::None;
    Request *req = nullptr;
    std::vector<Request *> pack;  // two or more small fits run as one pack
    std::condition_variable cv;
};

// Runs one request on a slot. The device executor drives the fit core; the simulated one
// (a scheduling test double) only waits and reports reservations.
struct Executor {
    virtual ~Executor() = default;
    virtual void run(Slot &slot, Request &r) = 0;
    virtual void run_pack(Slot &slot, std::vector<Request *> &pack) {
        for (Request *r : pack) run(slot, *r);
    }
    virtual void release(Slot &slot) = 0;
    virtual int64_t reserved(Slot &slot) = 0;
};

struct DeviceExecutor : Executor {
    void run(Slot &slot, Request &r) override;
    void run_pack(Slot &slot, std::vector<Request *> &pack) override;
    void predict(Slot &slot, Request &r);
    void release(Slot &slot) override { cuscan_ctx_release_workspace(slot.ctx); }
    int64_t reserved(Slot &slot) override { return cuscan_ctx_reserved_bytes(slot.ctx); }
};

struct SimulatedExecutor : Executor {
    double us_per_kpoint;
    std::vector<int64_t> held;
    SimulatedExecutor(int slots, double us) : us_per_kpoint(us), held(slots, 0) {}
    static int index(Slot &slot) { return slot.index; }
    void run(Slot &slot, Request &r) override {
        std::this_thread::sleep_for(std::chrono::microseconds(
            (int64_t)(us_per_kpoint * (double)r.n / 1000.0) + 1));
        held[index(slot)] = std::max(held[index(slot)], r.bytes);
        r.status = CUSCAN_OK;
        r.finite_rows = r.n;
    }
    void release(Slot &slot) override { held[index(slot)] = 0; }
    int64_t reserved(Slot &slot) override { return held[index(slot)]; }
};

// approximate_predict of one query batch against a resident predictor.
void DeviceExecutor::predict(Slot &slot, Request &r) {
    const Clock::time_point t0 = Clock::now();
    r.labels.resize((size_t)r.n);
    r.strengths.resize((size_t)r.n);
    r.connectors.resize((size_t)r.n);
    r.finite_rows = r.n;
    const int rc = cuscan_predictor_predict(slot.ctx, r.predictor, r.x, r.n, r.labels.data(),
                                            r.strengths.data(), r.connectors.data());
    r.fit_ms = ms_between(t0, Clock::now());
    r.status = rc;
    if (rc) r.error = cuscan_last_error(slot.ctx);
}

// The finite rows of a fit request (finite.rs:65-131): their original indices and, when some
// rows are set aside, a compact copy. Prepares the request's outputs (-1 / 0 for every row).
struct FiniteRows {
    std::vector<int64_t> index;
    std::vector<float> compact;
    const float *x = nullptr;
    int64_t n = 0;
};

void split_finite(Request &r, FiniteRows &f) {
    const int64_t n = r.n;
    const int32_t d = r.d;
    f.index.clear();
    f.index.reserve((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        const float *row = r.x + i * d;
        bool ok = true;
        for (int32_t c = 0; c < d; ++c)
            if (!std::isfinite(row[c])) {
                ok = false;
                break;
            }
        if (ok) f.index.push_back(i);
    }
    f.n = (int64_t)f.index.size();
    r.finite_rows = f.n;
    f.x = r.x;
    if (f.n != n) {
        f.compact.resize((size_t)f.n * d);
        for (int64_t i = 0; i < f.n; ++i)
            std::memcpy(f.compact.data() + i * d, r.x + f.index[(size_t)i] * d,
                        sizeof(float) * d);
        f.x = f.compact.data();
    }
    r.labels.assign((size_t)n, -1);
    r.probabilities.assign((size_t)n, 0.0f);
    r.core.assign((size_t)f.n, INFINITY);
    r.sorted_mst.clear();
}

// Fit-core outputs of one request, and the host extraction that turns them into labels.
struct CoreOutputs {
    std::vector<float> core_sq, wsq;
    std::vector<uint32_t> src, dst;
    void size_for(int64_t nf) {
        core_sq.resize((size_t)nf);
        wsq.resize((size_t)(nf - 1));
        src.resize((size_t)(nf - 1));
        dst.resize((size_t)(nf - 1));
    }
};

void finish(Request &r, const FiniteRows &f, const CoreOutputs &o) {
    const Clock::time_point t0 = Clock::now();
    const int64_t nf = f.n, m = nf - 1;
    for (int64_t i = 0; i < nf; ++i) r.core[(size_t)i] = std::sqrt(o.core_sq[(size_t)i]);
    std::vector<double> w((size_t)m);
    for (int64_t e = 0; e < m; ++e) w[(size_t)e] = std::sqrt((double)o.wsq[(size_t)e]);
    cuscan_clustering *c = nullptr;
    char err[512] = {0};
    int rc = cuscan_clusters_from_spanning_tree(o.src.data(), o.dst.data(), w.data(), m, &r.cfg,
                                                &c, err, sizeof(err));
    if (rc) {
        r.status = rc;
        r.error = err;
        return;
    }
    std::vector<int32_t> lab((size_t)nf);
    std::vector<float> prob((size_t)nf);
    r.sorted_mst.resize((size_t)m * 3);
    cuscan_clustering_read(c, lab.data(), prob.data(), nullptr, r.sorted_mst.data(), nullptr,
                           nullptr, nullptr, nullptr);
    cuscan_clustering_free(c);
    int32_t top = -1;
    for (int64_t i = 0; i < nf; ++i) {
        r.labels[(size_t)f.index[(size_t)i]] = lab[(size_t)i];
        r.probabilities[(size_t)f.index[(size_t)i]] = prob[(size_t)i];
        top = std::max(top, lab[(size_t)i]);
    }
    r.clusters = top + 1;
    r.status = CUSCAN_OK;
    r.extract_ms = ms_between(t0, Clock::now());
}

void DeviceExecutor::run(Slot &slot, Request &r) {
    if (r.kind == Kind::Predict) {
        predict(slot, r);
        return;
    }
    const Clock::time_point t0 = Clock::now();
    FiniteRows f;
    split_finite(r, f);
    if (f.n < 2) {  // one finite row or none: all noise, empty trees (hdbscan-core lib.rs:40-50)
        r.status = CUSCAN_OK;
        return;
    }
    CoreOutputs o;
    o.size_for(f.n);
    int64_t edges = 0;
    const Clock::time_point t1 = Clock::now();
    r.prep_ms = ms_between(t0, t1);
    int rc = cuscan_fit_core(slot.ctx, f.x, f.n, r.d, r.min_samples, r.precision, nullptr,
                             nullptr, o.core_sq.data(), o.src.data(), o.dst.data(), o.wsq.data(),
                             &edges, &r.stats);
    r.fit_ms = ms_between(t1, Clock::now());
    if (rc) {
        r.status = rc;
        r.error = cuscan_last_error(slot.ctx);
        return;
    }
    finish(r, f, o);
}

// Small fits of one pack: finite split of each, one packed call for all fit cores, then the
// extraction of each.
void DeviceExecutor::run_pack(Slot &slot, std::vector<Request *> &pack) {
    const size_t count = pack.size();
    std::vector<FiniteRows> f(count);
    std::vector<CoreOutputs> o(count);
    std::vector<cuscan_fit_item> items;
    std::vector<size_t> owner;  // request of each item
    items.reserve(count);
    for (size_t i = 0; i < count; ++i) {
        Request &r = *pack[i];
        const Clock::time_point t0 = Clock::now();
        split_finite(r, f[i]);
        r.prep_ms = ms_between(t0, Clock::now());
        if (f[i].n < 2) {
            r.status = CUSCAN_OK;
            continue;
        }
        o[i].size_for(f[i].n);
        cuscan_fit_item it;
        std::memset(&it, 0, sizeof(it));
        it.data = f[i].x;
        it.n = f[i].n;
        it.d = r.d;
        it.min_samples = r.min_samples;
        it.precision = r.precision;
        it.core_sq = o[i].core_sq.data();
        it.mst_src = o[i].src.data();
        it.mst_dst = o[i].dst.data();
        it.mst_wsq = o[i].wsq.data();
        items.push_back(it);
        owner.push_back(i);
    }
    if (items.empty()) return;
    const Clock::time_point t1 = Clock::now();
    const int rc = cuscan_fit_core_packed(slot.ctx, items.data(), (int32_t)items.size());
    const double fit_ms = ms_between(t1, Clock::now());
    const std::string msg = rc ? cuscan_last_error(slot.ctx) : std::string();
    for (size_t j = 0; j < items.size(); ++j) {
        Request &r = *pack[owner[j]];
        r.fit_ms = fit_ms;
        r.stats = items[j].stats;
        // a call-wide failure (CUDA error, rejected pack) leaves the item statuses at OK
        const int st = items[j].status ? items[j].status : rc;
        if (st) {
            r.status = st;
            r.error = msg;
            continue;
        }
        finish(r, f[owner[j]], o[owner[j]]);
    }
}

}  // namespace

struct cuscan_server {
    int device = 0;
    int64_t budget = 0;
    bool simulated = false;
    std::unique_ptr<Executor> exec;
    std::vector<std::unique_ptr<Slot>> slots;
    std::vector<std::thread> workers;
    std::mutex mu;
    std::condition_variable cv_done;
    std::deque<Request *> queue;
    std::unordered_map<int64_t, std::unique_ptr<Request>> requests;
    std::deque<int64_t> finished;  // completion order, for wait_any
    int64_t next_id = 1;
    int64_t submitted = 0, completed = 0, failed = 0, releases = 0;
    int64_t peak_committed = 0;
    // Packs of up to 8 small fits by default: a pack launches each step once for all of its
    // fits and reads the host once per few rounds, where eight slots running one small fit
    // each launch every step eight times and read the host once per round each.
    int32_t pack_limit = 8;
    int64_t packs = 0, packed_requests = 0;
    Clock::time_point t0 = Clock::now();
    bool stopping = false;

    // A slot commits the larger of what it holds and what its request may grow it to; a pack
    // runs on buffers of its own, so it commits its bounds on top of what the slot holds.
    static int64_t commitment(const Slot &s) {
        return s.pack.empty() ? std::max(s.reserved, s.running) : s.reserved + s.running;
    }

    int64_t committed_locked() const {
        int64_t total = 0;
        for (auto &s : slots) total += commitment(*s);
        return total;
    }

    // a fit the packed path accepts (a request outside its limits runs on its own, so that it
    // fails or succeeds exactly as alone and never takes a pack's other fits with it)
    static bool small_fit(const Request *r) {
        return r->kind == Kind::Fit && r->n <= CUSCAN_PACK_MAX_ROWS &&
               r->d <= CUSCAN_PACK_MAX_FEATURES;
    }

    // Admit queued requests onto idle slots while the budget allows (called with mu held).
    void schedule_locked() {
        while (!queue.empty() && !stopping) {
            Request *r = queue.front();
            Slot *best = nullptr;
            // an idle slot that already holds enough workspace (smallest such), else the idle
            // slot holding the most (least growth)
            for (auto &s : slots) {
                if (s->task != Task::None) continue;
                if (s->reserved >= r->bytes) {
                    if (!best || best->reserved < r->bytes || s->reserved < best->reserved)
                        best = s.get();
                } else if (!best || (best->reserved < r->bytes && s->reserved > best->reserved)) {
                    best = s.get();
                }
            }
            if (!best) return;  // every slot is busy
            const int64_t others = committed_locked() - commitment(*best);
            if (others + std::max(best->reserved, r->bytes) <= budget) {
                queue.pop_front();
                best->task = Task::Fit;
                best->req = r;
                best->running = r->bytes;
                r->slot = index_of(best);
                r->t_admit = Clock::now();
                // small fits queued right behind a small head join it in one pack
                if (small_fit(r) && pack_limit > 1) {
                    int64_t sum = r->bytes;
                    std::vector<Request *> pack{r};
                    while (!queue.empty() && (int)pack.size() < pack_limit &&
                           small_fit(queue.front()) &&
                           others + best->reserved + sum + queue.front()->bytes <= budget) {
                        Request *q = queue.front();
                        queue.pop_front();
                        q->slot = r->slot;
                        q->t_admit = r->t_admit;
                        sum += q->bytes;
                        pack.push_back(q);
                    }
                    if (pack.size() > 1) {
                        for (Request *q : pack) q->pack_size = (int32_t)pack.size();
                        best->pack = std::move(pack);
                        best->running = sum;
                        ++packs;
                        packed_requests += (int64_t)best->pack.size();
                    }
                }
                peak_committed = std::max(peak_committed, committed_locked());
                best->cv.notify_one();
                continue;
            }
            // over budget: have the idle slot holding the most workspace (other than best
            // when best itself is too small) release it, then try again when it reports back
            Slot *victim = nullptr;
            for (auto &s : slots)
                if (s->task == Task::None && s->reserved > 0 &&
                    (!victim || s->reserved > victim->reserved))
                    victim = s.get();
            if (victim) {
                victim->task = Task::Release;
                ++releases;
                victim->cv.notify_one();
            }
            return;  // wait for a completion or a release
        }
    }

    int index_of(const Slot *s) const {
        for (size_t i = 0; i < slots.size(); ++i)
            if (slots[i].get() == s) return (int)i;
        return -1;
    }

    void worker(int i) {
        Slot &slot = *slots[(size_t)i];
        for (;;) {
            Task task;
            Request *r;
            std::vector<Request *> pack;
            {
                std::unique_lock<std::mutex> lk(mu);
                slot.cv.wait(lk, [&] { return slot.task != Task::None; });
                task = slot.task;
                r = slot.req;
                pack = slot.pack;
            }
            if (task == Task::Stop) return;
            if (task == Task::Fit && !pack.empty()) exec->run_pack(slot, pack);
            else if (task == Task::Fit) exec->run(slot, *r);
            else exec->release(slot);
            if (pack.empty() && task == Task::Fit) pack.push_back(r);
            const int64_t held = exec->reserved(slot);
            {
                std::lock_guard<std::mutex> lk(mu);
                slot.reserved = held;
                slot.running = 0;
                slot.req = nullptr;
                slot.pack.clear();
                if (slot.task != Task::Stop) slot.task = Task::None;
                if (task == Task::Fit) {
                    const Clock::time_point now = Clock::now();
                    for (Request *q : pack) {
                        q->t_done = now;
                        q->done = true;
                        ++completed;
                        if (q->status) ++failed;
                        finished.push_back(q->id);
                    }
                }
                schedule_locked();
            }
            cv_done.notify_all();
        }
    }

    // Queue a request (or finish it at once when its bound exceeds the budget).
    int enqueue(std::unique_ptr<Request> r, int64_t *request_id) {
        std::lock_guard<std::mutex> lk(mu);
        if (stopping) return CUSCAN_INVALID_INPUT;
        r->id = next_id++;
        *request_id = r->id;
        ++submitted;
        Request *raw = r.get();
        requests.emplace(r->id, std::move(r));
        if (raw->bytes > budget) {
            raw->status = CUSCAN_MEMORY;
            raw->error = "the request's workspace bound exceeds the server's memory budget";
            raw->done = true;
            raw->t_admit = raw->t_done = raw->t_submit;
            ++completed;
            ++failed;
            finished.push_back(raw->id);
            cv_done.notify_all();
            return CUSCAN_OK;
        }
        queue.push_back(raw);
        schedule_locked();
        return CUSCAN_OK;
    }

    void fill_info(const Request &r, cuscan_server_info *info) const {
        std::memset(info, 0, sizeof(*info));
        info->request_id = r.id;
        info->kind = (int32_t)r.kind;
        info->pack_size = r.pack_size;
        info->status = r.done ? r.status : CUSCAN_PENDING;
        info->slot = r.slot;
        info->n = r.n;
        info->d = r.d;
        info->finite_rows = r.finite_rows;
        info->n_clusters = r.clusters;
        info->workspace_bound_bytes = r.bytes;
        info->prep_ms = r.prep_ms;
        info->fit_ms = r.fit_ms;
        info->extract_ms = r.extract_ms;
        info->submit_ms = ms_between(t0, r.t_submit);
        if (r.slot >= 0) info->queued_ms = ms_between(r.t_submit, r.t_admit);
        if (r.done) {
            info->run_ms = ms_between(r.t_admit, r.t_done);
            info->latency_ms = ms_between(r.t_submit, r.t_done);
            info->done_ms = ms_between(t0, r.t_done);
        }
        info->stats = r.stats;
    }
};

namespace {

int start_server(cuscan_server *s, int32_t slots, char *err, size_t err_len) {
    for (int32_t i = 0; i < slots; ++i) {
        auto slot = std::make_unique<Slot>();
        slot->index = i;
        if (!s->simulated) {
            int rc = cuscan_ctx_create(s->device, &slot->ctx);
            if (rc) {
                set_err(err, err_len, "could not create a CUDA context for a server slot");
                for (auto &t : s->slots) cuscan_ctx_destroy(t->ctx);
                s->slots.clear();
                return rc;
            }
        }
        s->slots.push_back(std::move(slot));
    }
    for (int32_t i = 0; i < slots; ++i) s->workers.emplace_back([s, i] { s->worker(i); });
    return CUSCAN_OK;
}

}  // namespace

extern "C" {

int cuscan_server_create(int device, int32_t slots, int64_t budget_bytes, cuscan_server **out,
                         char *err, size_t err_len) {
    if (!out) return CUSCAN_INVALID_INPUT;
    *out = nullptr;
    if (slots <= 0 || slots > 64 || budget_bytes <= 0) {
        set_err(err, err_len, "a server needs 1..64 slots and a positive memory budget");
        return CUSCAN_INVALID_CONFIG;
    }
    auto s = std::make_unique<cuscan_server>();
    s->device = device;
    s->budget = budget_bytes;
    s->exec = std::make_unique<DeviceExecutor>();
    int rc = start_server(s.get(), slots, err, err_len);
    if (rc) return rc;
    *out = s.release();
    return CUSCAN_OK;
}

int cuscan_server_create_simulated(int32_t slots, int64_t budget_bytes, double us_per_kpoint,
                                   cuscan_server **out, char *err, size_t err_len) {
    if (!out) return CUSCAN_INVALID_INPUT;
    *out = nullptr;
    if (slots <= 0 || slots > 64 || budget_bytes <= 0 || !(us_per_kpoint >= 0.0)) {
        set_err(err, err_len, "a server needs 1..64 slots and a positive memory budget");
        return CUSCAN_INVALID_CONFIG;
    }
    auto s = std::make_unique<cuscan_server>();
    s->budget = budget_bytes;
    s->simulated = true;
    s->exec = std::make_unique<SimulatedExecutor>(slots, us_per_kpoint);
    start_server(s.get(), slots, err, err_len);
    *out = s.release();
    return CUSCAN_OK;
}

void cuscan_server_destroy(cuscan_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
        for (Request *r : s->queue) {
            r->status = CUSCAN_INVALID_INPUT;
            r->error = "server stopped before the request was admitted";
            r->done = true;
        }
        s->queue.clear();
    }
    // let running requests finish, then stop every worker
    for (auto &slot : s->slots) {
        std::unique_lock<std::mutex> lk(s->mu);
        s->cv_done.wait(lk, [&] { return slot->task == Task::None; });
        slot->task = Task::Stop;
        slot->cv.notify_one();
    }
    for (auto &t : s->workers) t.join();
    if (!s->simulated)
        for (auto &slot : s->slots) cuscan_ctx_destroy(slot->ctx);
    delete s;
}

int cuscan_server_submit_fit(cuscan_server *s, const float *data, int64_t n, int32_t d,
                             int32_t min_samples, int32_t precision,
                             const cuscan_extract_config *config, int64_t *request_id) {
    if (!s || !request_id || !config) return CUSCAN_INVALID_INPUT;
    *request_id = 0;
    if (n <= 0 || d <= 0 || (!data && !s->simulated)) return CUSCAN_INVALID_INPUT;
    if (n > INT32_MAX - 1) return CUSCAN_OVERFLOW;
    if (min_samples <= 0 || config->min_cluster_size <= 0) return CUSCAN_INVALID_CONFIG;
    if (precision != CUSCAN_PRECISION_PLAIN && precision != CUSCAN_PRECISION_BF16_REFINED &&
        precision != CUSCAN_PRECISION_FP16_REFINED)
        return CUSCAN_INVALID_CONFIG;
    auto r = std::make_unique<Request>();
    r->x = data;
    r->n = n;
    r->d = d;
    r->min_samples = min_samples;
    r->precision = precision;
    r->cfg = *config;
    r->bytes = cuscan_fit_workspace_bytes(n < 2 ? 2 : n, d, min_samples, precision);
    r->t_submit = Clock::now();
    return s->enqueue(std::move(r), request_id);
}

int cuscan_server_submit_predict(cuscan_server *s, const cuscan_predictor *predictor,
                                 const float *queries, int64_t m, int64_t *request_id) {
    if (!s || !request_id || !predictor) return CUSCAN_INVALID_INPUT;
    *request_id = 0;
    if (m <= 0 || (!queries && !s->simulated)) return CUSCAN_INVALID_INPUT;
    if (m > INT32_MAX) return CUSCAN_OVERFLOW;
    auto r = std::make_unique<Request>();
    r->kind = Kind::Predict;
    r->predictor = predictor;
    r->x = queries;
    r->n = m;
    int64_t nf = 0;
    int32_t d = 0, ms = 0;
    cuscan_predictor_shape(predictor, &nf, &d, &ms);
    r->d = d;
    r->min_samples = ms;
    r->bytes = cuscan_predict_workspace_bytes(predictor, m);
    r->t_submit = Clock::now();
    return s->enqueue(std::move(r), request_id);
}

int cuscan_server_read_predict(cuscan_server *s, int64_t request_id, int32_t *labels,
                               double *strengths, int32_t *connecting_points) {
    if (!s) return CUSCAN_INVALID_INPUT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end()) return CUSCAN_INVALID_INPUT;
    const Request &r = *it->second;
    if (r.kind != Kind::Predict) return CUSCAN_INVALID_INPUT;
    if (!r.done) return CUSCAN_PENDING;
    if (r.status) return r.status;
    if (s->simulated) return CUSCAN_INVALID_INPUT;  // the test double computes no result
    if (labels) std::memcpy(labels, r.labels.data(), r.labels.size() * sizeof(int32_t));
    if (strengths) std::memcpy(strengths, r.strengths.data(), r.strengths.size() * sizeof(double));
    if (connecting_points)
        std::memcpy(connecting_points, r.connectors.data(), r.connectors.size() * sizeof(int32_t));
    return CUSCAN_OK;
}

int cuscan_server_wait(cuscan_server *s, int64_t request_id, double timeout_ms,
                       cuscan_server_info *info) {
    if (!s) return CUSCAN_INVALID_INPUT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end()) return CUSCAN_INVALID_INPUT;
    Request *r = it->second.get();
    auto ready = [&] { return r->done; };
    if (timeout_ms < 0) s->cv_done.wait(lk, ready);
    else s->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready);
    if (info) s->fill_info(*r, info);
    return r->done ? CUSCAN_OK : CUSCAN_PENDING;
}

int cuscan_server_wait_any(cuscan_server *s, double timeout_ms, int64_t *request_id) {
    if (!s || !request_id) return CUSCAN_INVALID_INPUT;
    *request_id = 0;
    std::unique_lock<std::mutex> lk(s->mu);
    auto ready = [&] { return !s->finished.empty(); };
    if (timeout_ms < 0) s->cv_done.wait(lk, ready);
    else s->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready);
    if (s->finished.empty()) return CUSCAN_PENDING;
    *request_id = s->finished.front();
    s->finished.pop_front();
    return CUSCAN_OK;
}

int cuscan_server_read_fit(cuscan_server *s, int64_t request_id, int32_t *labels,
                           float *probabilities, float *core_distances, double *sorted_mst) {
    if (!s) return CUSCAN_INVALID_INPUT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end()) return CUSCAN_INVALID_INPUT;
    const Request &r = *it->second;
    if (r.kind != Kind::Fit) return CUSCAN_INVALID_INPUT;
    if (!r.done) return CUSCAN_PENDING;
    if (r.status) return r.status;
    if (s->simulated) return CUSCAN_INVALID_INPUT;  // the test double computes no result
    if (labels) std::memcpy(labels, r.labels.data(), r.labels.size() * sizeof(int32_t));
    if (probabilities)
        std::memcpy(probabilities, r.probabilities.data(), r.probabilities.size() * sizeof(float));
    if (core_distances) std::memcpy(core_distances, r.core.data(), r.core.size() * sizeof(float));
    if (sorted_mst)
        std::memcpy(sorted_mst, r.sorted_mst.data(), r.sorted_mst.size() * sizeof(double));
    return CUSCAN_OK;
}

int cuscan_server_request_error(cuscan_server *s, int64_t request_id, char *buf, size_t len) {
    if (!s || !buf || !len) return CUSCAN_INVALID_INPUT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end()) return CUSCAN_INVALID_INPUT;
    std::snprintf(buf, len, "%s", it->second->error.c_str());
    return CUSCAN_OK;
}

int cuscan_server_release(cuscan_server *s, int64_t request_id) {
    if (!s) return CUSCAN_INVALID_INPUT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end()) return CUSCAN_INVALID_INPUT;
    if (!it->second->done) return CUSCAN_PENDING;
    s->requests.erase(it);
    // a released request is no longer reported by wait_any
    auto f = std::find(s->finished.begin(), s->finished.end(), request_id);
    if (f != s->finished.end()) s->finished.erase(f);
    return CUSCAN_OK;
}

int cuscan_server_get_stats(cuscan_server *s, cuscan_server_stats *out) {
    if (!s || !out) return CUSCAN_INVALID_INPUT;
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->slots = (int32_t)s->slots.size();
    out->budget_bytes = s->budget;
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->failed = s->failed;
    out->queued = (int64_t)s->queue.size();
    for (auto &slot : s->slots)
        if (slot->task == Task::Fit) ++out->running;
    out->committed_bytes = s->committed_locked();
    out->peak_committed_bytes = s->peak_committed;
    out->workspace_releases = s->releases;
    out->packs = s->packs;
    out->packed_requests = s->packed_requests;
    return CUSCAN_OK;
}

int cuscan_server_set_pack_limit(cuscan_server *s, int32_t max_fits) {
    if (!s) return CUSCAN_INVALID_INPUT;
    if (max_fits < 1 || max_fits > CUSCAN_PACK_MAX_FITS) return CUSCAN_INVALID_CONFIG;
    std::lock_guard<std::mutex> lk(s->mu);
    s->pack_limit = max_fits;
    return CUSCAN_OK;
}

}  // extern "C"
