// server.cpp -- the request loop over batches (include/armon_gb300.h, armon_server_*).
//
// Requests wait in submission order.  A round admits the head of the queue while its state fits
// in the memory budget (head-of-line: a large request is not overtaken, so it cannot starve),
// enqueues cycles_per_step cycles in every batch that has running solves, then polls the batches
// (each batch has its own stream, so all batches' work is on the device before the first wait),
// and retires the solves whose loop ended.  Solves of one (precision, scheme, projection,
// splitting) share a batch, whose fused launch advances all of them with their own dt and time.
// A finished solve keeps its device state, and its share of the budget, until it is released.
#include <array>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "armon_gb300.h"
#include "host_common.h"

using armon::set_error;

namespace {

using Clock = std::chrono::steady_clock;
using BatchKey = std::array<int32_t, 4>;   // precision, scheme, projection, splitting

struct Request {
    armon_params p{};
    armon_sod_interface sod{};
    bool has_sod = false;
    armon_server_request info{};
    armon_batch* batch = nullptr;
    int32_t dom = -1;
    bool released = false;
};

}  // namespace

struct armon_server {
    armon_server_opts o{};
    Clock::time_point t0;
    std::map<BatchKey, armon_batch*> batches;
    std::map<armon_batch*, bool> busy;  // cycles enqueued and not yet collected
    std::map<BatchKey, int64_t> inflight_cells;   // real cells of the running solves per batch
    std::vector<Request> reqs;
    std::deque<int64_t> queue;        // waiting, in submission order
    std::vector<int64_t> running;     // on the device, loop not ended
    std::deque<int64_t> finished;     // ended, not yet reported by next_done
    int64_t bytes = 0;                // state of admitted, unreleased requests
};

namespace {

double now(const armon_server* s)
{
    return std::chrono::duration<double>(Clock::now() - s->t0).count();
}

BatchKey key_of(const armon_params& p, int32_t precision)
{
    return BatchKey{precision, p.scheme, p.projection, p.axis_splitting};
}

int batch_for(armon_server* s, const armon_params& p, int32_t precision, armon_batch** out)
{
    BatchKey key = key_of(p, precision);
    auto it = s->batches.find(key);
    if (it != s->batches.end()) {
        *out = it->second;
        return ARMON_OK;
    }
    armon_batch_opts bo;
    armon_batch_opts_default(&bo);
    bo.precision = precision;
    bo.cycles_per_graph = s->o.cycles_per_step;
    bo.block_lines = s->o.block_lines;
    bo.waves = s->o.waves;
    armon_batch* b = nullptr;
    int rc = armon_batch_create(&bo, nullptr, &b);   // its own stream
    if (rc != ARMON_OK) return rc;
    s->batches[key] = b;
    *out = b;
    return ARMON_OK;
}

int lookup(armon_server* s, int64_t req, Request** r)
{
    if (req < 0 || req >= (int64_t)s->reqs.size()) { set_error("unknown request"); return ARMON_ERR_PARAMS; }
    *r = &s->reqs[(size_t)req];
    return ARMON_OK;
}

// Admits waiting requests in order while the memory budget allows.  A request whose batch is at
// its cell limit stays (and so do the later requests for that batch); requests for other batches
// may pass it.  The memory budget stops admission at the first request that does not fit.
int admit(armon_server* s)
{
    std::set<BatchKey> full;
    for (auto it = s->queue.begin(); it != s->queue.end();) {
        const int64_t id = *it;
        Request& r = s->reqs[(size_t)id];
        const BatchKey key = key_of(r.p, r.info.precision);
        if (full.count(key)) { ++it; continue; }
        const int64_t cells = (int64_t)r.p.nx * r.p.ny;
        int64_t& inflight = s->inflight_cells[key];
        if (s->o.max_inflight_cells > 0 && inflight > 0 && inflight + cells > s->o.max_inflight_cells) {
            full.insert(key);
            ++it;
            continue;
        }
        const int64_t need = armon_batch_domain_bytes(&r.p, r.info.precision);
        if (s->o.memory_budget > 0 && s->bytes + need > s->o.memory_budget) break;
        armon_batch* b = nullptr;
        int rc = batch_for(s, r.p, r.info.precision, &b);
        if (rc != ARMON_OK) return rc;
        int32_t dom = -1;
        rc = r.has_sod ? armon_batch_add_sod(b, &r.p, &r.sod, &dom) : armon_batch_add(b, &r.p, nullptr, &dom);
        if (rc == ARMON_ERR_NOMEM) break;          // the device is full after all: retry next round
        it = s->queue.erase(it);
        if (rc != ARMON_OK) {                      // this request cannot run: report it as failed
            r.info.status = ARMON_REQ_FAILED;
            r.info.t_done = now(s);
            s->finished.push_back(id);
            continue;
        }
        r.batch = b;
        r.dom = dom;
        r.info.status = ARMON_REQ_RUNNING;
        r.info.bytes = need;
        r.info.t_admit = now(s);
        s->bytes += need;
        inflight += cells;
        s->running.push_back(id);
    }
    return ARMON_OK;
}

}  // namespace

extern "C" {

void armon_server_opts_default(armon_server_opts* o)
{
    std::memset(o, 0, sizeof(*o));
    o->memory_budget = 150000000000ll;
    o->cycles_per_step = 8;
    o->block_lines = 128;
}

int armon_server_create(const armon_server_opts* opts, armon_server** out)
{
    armon_server* s = new armon_server();
    if (opts) s->o = *opts; else armon_server_opts_default(&s->o);
    if (s->o.cycles_per_step <= 0) s->o.cycles_per_step = 8;
    if (s->o.block_lines <= 0) s->o.block_lines = 128;
    s->t0 = Clock::now();
    *out = s;
    return ARMON_OK;
}

void armon_server_destroy(armon_server* s)
{
    if (!s) return;
    for (auto& kv : s->batches) armon_batch_destroy(kv.second);
    delete s;
}

int armon_server_submit(armon_server* s, const armon_params* p, int32_t precision, const armon_sod_interface* sod,
                        int64_t* req)
{
    *req = -1;
    if (precision != 32 && precision != 64) { set_error("precision must be 32 or 64"); return ARMON_ERR_PARAMS; }
    if (!armon_params_check(p)) { set_error("invalid parameters (Params::check)"); return ARMON_ERR_PARAMS; }
    if (sod && sod->shape != 0 && sod->shape != 1) { set_error("interface shape must be 0 or 1"); return ARMON_ERR_PARAMS; }
    Request r;
    r.p = *p;
    if (sod) { r.sod = *sod; r.has_sod = true; }
    r.info.status = ARMON_REQ_QUEUED;
    r.info.precision = precision;
    r.info.nx = p->nx;
    r.info.ny = p->ny;
    r.info.t_submit = now(s);
    r.info.t_admit = -1;
    r.info.t_done = -1;
    r.info.bytes = armon_batch_domain_bytes(p, precision);
    s->reqs.push_back(r);
    *req = (int64_t)s->reqs.size() - 1;
    s->queue.push_back(*req);
    return ARMON_OK;
}

int armon_server_step(armon_server* s, int32_t* in_flight, int32_t* queued)
{
    int rc = admit(s);
    if (rc != ARMON_OK) return rc;
    // idle batches with running solves get their next cycles
    for (auto& kv : s->batches) {
        armon_batch* b = kv.second;
        if (s->busy[b]) continue;
        bool any = false;
        for (int64_t id : s->running)
            if (s->reqs[(size_t)id].batch == b) { any = true; break; }
        if (!any) continue;
        rc = armon_batch_enqueue_cycles(b, s->o.cycles_per_step);
        if (rc != ARMON_OK) return rc;
        s->busy[b] = true;
    }
    // wait for the first batch to finish its cycles, then collect every finished one
    std::vector<armon_batch*> ready;
    for (;;) {
        bool any_busy = false;
        for (auto& kv : s->busy) {
            if (!kv.second) continue;
            any_busy = true;
            if (armon_batch_ready(kv.first)) ready.push_back(kv.first);
        }
        if (!ready.empty() || !any_busy) break;
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    for (armon_batch* b : ready) {
        rc = armon_batch_poll(b, nullptr);
        if (rc != ARMON_OK) return rc;
        s->busy[b] = false;
    }
    const double t = now(s);
    std::vector<int64_t> still;
    still.reserve(s->running.size());
    for (int64_t id : s->running) {
        Request& r = s->reqs[(size_t)id];
        if (s->busy[r.batch] || armon_batch_domain_done(r.batch, r.dom) != 1) {
            still.push_back(id);
            continue;
        }
        armon_params fp;
        int32_t status = 0;
        armon_batch_domain_state(r.batch, r.dom, &fp, &status);
        r.info.status = status == 0 ? ARMON_REQ_DONE : ARMON_REQ_FAILED;
        s->inflight_cells[key_of(r.p, r.info.precision)] -= (int64_t)r.p.nx * r.p.ny;
        r.info.cycle = fp.cycle;
        r.info.time = fp.time;
        r.info.t_done = t;
        s->finished.push_back(id);
    }
    s->running.swap(still);
    if (in_flight) *in_flight = (int32_t)s->running.size();
    if (queued) *queued = (int32_t)s->queue.size();
    return ARMON_OK;
}

int armon_server_next_done(armon_server* s, int64_t* req)
{
    if (s->finished.empty()) return 0;
    *req = s->finished.front();
    s->finished.pop_front();
    return 1;
}

int armon_server_request_info(armon_server* s, int64_t req, armon_server_request* info)
{
    Request* r = nullptr;
    int rc = lookup(s, req, &r);
    if (rc != ARMON_OK) return rc;
    *info = r->info;
    return ARMON_OK;
}

int armon_server_download(armon_server* s, int64_t req, int which, double* host)
{
    Request* r = nullptr;
    int rc = lookup(s, req, &r);
    if (rc != ARMON_OK) return rc;
    if (r->info.status < ARMON_REQ_DONE || r->released || !r->batch) {
        set_error("the request has no finished state on the device");
        return ARMON_ERR_STATE;
    }
    return armon_batch_download(r->batch, r->dom, which, host);
}

int armon_server_release(armon_server* s, int64_t req)
{
    Request* r = nullptr;
    int rc = lookup(s, req, &r);
    if (rc != ARMON_OK) return rc;
    if (r->info.status < ARMON_REQ_DONE) { set_error("the request has not finished"); return ARMON_ERR_STATE; }
    if (r->released || !r->batch) return ARMON_OK;
    rc = armon_batch_remove(r->batch, r->dom);
    if (rc != ARMON_OK) return rc;
    s->bytes -= r->info.bytes;
    r->released = true;
    return ARMON_OK;
}

int64_t armon_server_bytes_in_use(armon_server* s) { return s->bytes; }

int64_t armon_server_kernel_launches(armon_server* s)
{
    int64_t n = 0;
    for (auto& kv : s->batches) n += armon_batch_kernel_launches(kv.second);
    return n;
}

}  // extern "C"
