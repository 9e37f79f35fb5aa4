// server.cu -- a continuous-batching request loop over resident columns.
//
// Requests (a predicate and the aggregates wanted, over 1..8 columns) are
// queued by any thread.  A dispatcher thread owns `slots` workspaces, each
// with its own stream: whenever a slot is free it admits queued requests in
// arrival order while the slot's accumulator and work-item capacity last (the
// memory footprint of a request is one accumulator per chunk of its columns),
// builds one mixed-codec batch from them (batch.cu) and launches it.  Requests
// that arrive while batches run on the device go into the next free slot, so
// batches overlap on the GPU.  A finished slot's per-column results are
// combined per request in column order (sum in order, min, max), stamped and
// handed back; every result equals the request run alone.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "column.h"

namespace {

uint64_t now_ns() {
    return static_cast<uint64_t>(
        std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch()).count());
}

int sfail(int code, const std::string& msg) {
    set_last_error(msg);
    return code;
}

struct Pending {
    ebi_request req;
    uint64_t ticket;
    uint64_t submit_ns;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    QueryParams* d_qp = nullptr;
    BatchItem* d_items = nullptr;
    ChunkAcc* d_acc = nullptr;
    QueryResult* d_res = nullptr;
    unsigned int* d_counter = nullptr;
    QueryParams* h_qp = nullptr;
    BatchItem* h_items = nullptr;
    QueryResult* h_res = nullptr;
    std::vector<Pending> reqs;   // requests of the batch in flight
    std::vector<uint32_t> qindex;  // (request, column) in request order -> its query in the batch
    bool busy = false;
    uint64_t launch_ns = 0;
};

}  // namespace

struct ebi_server {
    std::vector<ebi_column*> cols;
    ebi_server_config cfg{};
    int sms = 1;
    std::vector<Slot> slots;
    // queues
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Pending> pending;
    std::deque<ebi_response> done;
    uint64_t next_ticket = 1;
    bool stop = false;
    int error = 0;
    std::thread worker;
    BatchTiling tiling{};
    // statistics
    uint64_t batches = 0, batched_requests = 0, max_in_flight = 0;
    std::atomic<uint64_t> items{0}, build_ns{0};  // written by the dispatcher outside the lock
};

namespace {

// Items and accumulators a request needs (its memory footprint).
void footprint(const ebi_server* s, const ebi_request& r, uint64_t* chunks, uint64_t* items) {
    uint64_t c = 0, it = 0;
    for (uint32_t k = 0; k < r.n_columns; ++k) {
        const ebi_column* col = s->cols[r.columns[k]];
        c += col->n_chunks;
        it += column_item_count(col->scheme, col->n_chunks, static_cast<uint32_t>(col->tiles.tiles.size()),
                                col->n_records, s->tiling);
    }
    *chunks = c;
    *items = it;
}

// Builds and launches slot sl's batch from its admitted requests.
cudaError_t launch_slot(ebi_server* s, Slot& sl) {
    const uint64_t t_build = now_ns();
    // The batch's queries in column order, so that the queries on one column
    // are consecutive: a Chimp-family chunk is then decoded once for all of
    // them (items naming up to 32 consecutive queries), a group of Gorilla
    // chunks once for up to kGorillaShareWide.
    struct Ent { uint32_t col, req, k; };
    std::vector<Ent> ents;
    std::vector<uint32_t> base(sl.reqs.size() + 1, 0);
    for (uint32_t ri = 0; ri < sl.reqs.size(); ++ri) {
        const Pending& p = sl.reqs[ri];
        base[ri + 1] = base[ri] + p.req.n_columns;
        for (uint32_t k = 0; k < p.req.n_columns; ++k) ents.push_back({p.req.columns[k], ri, k});
    }
    std::stable_sort(ents.begin(), ents.end(), [](const Ent& a, const Ent& b) { return a.col < b.col; });
    sl.qindex.assign(ents.size(), 0);
    const uint32_t nq = static_cast<uint32_t>(ents.size());
    uint64_t acc_used = 0;
    for (uint32_t qi = 0; qi < nq; ++qi) {
        const Ent& en = ents[qi];
        const Pending& p = sl.reqs[en.req];
        const ebi_column* c = s->cols[en.col];
        QueryParams q = column_params(c);
        q.op = OP_FILTER_AGG;
        q.pred = p.req.pred;
        q.pred_on = 1;
        q.agg = p.req.aggregates & AGG_ALL;
        q.out_mask = nullptr;
        q.out_atomic = 1;
        q.stage_bytes = 0;
        q.acc = sl.d_acc + acc_used;
        acc_used += c->n_chunks;
        sl.h_qp[qi] = q;
        sl.qindex[base[en.req] + en.k] = qi;
    }
    std::vector<BatchItem> items;
    for (uint32_t g = 0; g < nq;) {
        uint32_t h = g;
        while (h < nq && ents[h].col == ents[g].col) ++h;  // queries g .. h - 1: one column
        const ebi_column* c = s->cols[ents[g].col];
        shared_column_items(c->scheme, c->n_chunks, static_cast<uint32_t>(c->tiles.tiles.size()), c->n_records,
                            s->tiling, g, h - g, items);
        g = h;
    }
    order_by_cost(items);
    std::memcpy(sl.h_items, items.data(), items.size() * sizeof(BatchItem));
    s->items.fetch_add(items.size(), std::memory_order_relaxed);
    s->build_ns.fetch_add(now_ns() - t_build, std::memory_order_relaxed);
    cudaError_t e = cudaMemcpyAsync(sl.d_qp, sl.h_qp, nq * sizeof(QueryParams), cudaMemcpyHostToDevice, sl.stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.d_items, sl.h_items, items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice, sl.stream);
    const uint32_t grid = static_cast<uint32_t>(s->sms) * 2;
    if (e == cudaSuccess) e = launch_batch(sl.d_qp, sl.d_items, static_cast<uint32_t>(items.size()), sl.d_counter, grid, sl.stream);
    if (e == cudaSuccess) e = launch_batch_finalize(sl.d_qp, sl.d_res, nq, sl.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sl.h_res, sl.d_res, nq * sizeof(QueryResult), cudaMemcpyDeviceToHost, sl.stream);
    if (e == cudaSuccess) e = cudaEventRecord(sl.done, sl.stream);
    sl.launch_ns = now_ns();
    return e;
}

// Combines a finished slot's per-column results into one response per request.
void finish_slot(ebi_server* s, Slot& sl, std::vector<ebi_response>& out) {
    const uint64_t t = now_ns();
    uint32_t pos = 0;
    const double inf = __builtin_inf();
    for (const Pending& p : sl.reqs) {
        ebi_response r{};
        r.ticket = p.ticket;
        r.submit_ns = p.submit_ns;
        r.launch_ns = sl.launch_ns;
        r.done_ns = t;
        r.sum = 0.0;
        r.min = inf;
        r.max = -inf;
        for (uint32_t k = 0; k < p.req.n_columns; ++k, ++pos) {
            const QueryResult& q = sl.h_res[sl.qindex[pos]];
            if (q.status && !r.status) r.status = static_cast<int32_t>(q.status);
            r.sum += q.sum;
            r.min = std::fmin(r.min, q.min);
            r.max = std::fmax(r.max, q.max);
            r.count += q.count;
        }
        const double nan = __builtin_nan("");
        if (!(p.req.aggregates & AGG_SUM)) r.sum = nan;  // aggregates not asked for come back as NaN
        if (!(p.req.aggregates & AGG_MIN)) r.min = nan;
        if (!(p.req.aggregates & AGG_MAX)) r.max = nan;
        out.push_back(r);
    }
    s->batches += 1;
    s->batched_requests += sl.reqs.size();
    sl.reqs.clear();
    sl.busy = false;
}

void run(ebi_server* s) {
    if (cudaSetDevice(s->cfg.device) != cudaSuccess) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->error = EBI_E_CUDA;
        return;
    }
    std::vector<ebi_response> finished;
    for (;;) {
        bool progressed = false;
        // 1. retire finished slots
        for (Slot& sl : s->slots) {
            if (!sl.busy) continue;
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaErrorNotReady) continue;
            if (q != cudaSuccess) {
                std::lock_guard<std::mutex> lk(s->mu);
                s->error = EBI_E_CUDA;
            }
            finish_slot(s, sl, finished);
            progressed = true;
        }
        // 2. admit queued requests into free slots
        std::unique_lock<std::mutex> lk(s->mu);
        for (ebi_response& r : finished) s->done.push_back(r);
        finished.clear();
        if (s->stop && s->pending.empty()) {
            bool idle = true;
            for (Slot& sl : s->slots) idle = idle && !sl.busy;
            if (idle) return;
        }
        uint64_t in_flight = 0;
        for (Slot& sl : s->slots) {
            if (sl.busy) { ++in_flight; continue; }
            if (s->pending.empty()) continue;
            uint64_t chunks = 0, items = 0, queries = 0;
            while (!s->pending.empty()) {
                uint64_t c, it;
                footprint(s, s->pending.front().req, &c, &it);
                const uint64_t qn = s->pending.front().req.n_columns;
                if (!sl.reqs.empty() && (chunks + c > s->cfg.max_chunks_per_batch || items + it > s->cfg.max_items_per_batch ||
                                         queries + qn > s->cfg.max_queries_per_batch))
                    break;
                chunks += c;
                items += it;
                queries += qn;
                sl.reqs.push_back(s->pending.front());
                s->pending.pop_front();
            }
            sl.busy = true;
            ++in_flight;
            lk.unlock();
            if (launch_slot(s, sl) != cudaSuccess) {
                lk.lock();
                s->error = EBI_E_CUDA;
                lk.unlock();
            }
            lk.lock();
            progressed = true;
        }
        if (in_flight > s->max_in_flight) s->max_in_flight = in_flight;
        if (!progressed) {
            // nothing to admit and nothing finished: wait briefly for a request or a slot
            s->cv.wait_for(lk, std::chrono::microseconds(in_flight ? 20 : 200));
        }
    }
}

template <typename T>
cudaError_t salloc(T** p, size_t n) { return cudaMalloc(reinterpret_cast<void**>(p), (n ? n : 1) * sizeof(T)); }

}  // namespace

extern "C" {

int ebi_server_create(ebi_column* const* columns, uint32_t n_columns, const ebi_server_config* config,
                      ebi_server** out) {
    if (!out || !columns || !n_columns || !config) return sfail(EBI_E_INVALID, "columns, config or out is null");
    *out = nullptr;
    const ebi_server_config& cf = *config;
    if (cf.slots == 0 || cf.slots > 64 || cf.max_queries_per_batch == 0 || cf.max_chunks_per_batch == 0 ||
        cf.max_items_per_batch == 0)
        return sfail(EBI_E_INVALID, "server config: slots 1..64 and non-zero batch capacities");
    ebi_server* s = new (std::nothrow) ebi_server();
    if (!s) return sfail(EBI_E_OOM, "host allocation failed");
    s->cols.assign(columns, columns + n_columns);
    s->cfg = cf;
    s->tiling = default_tiling();
    for (int b = 0; b < kSizeBuckets; ++b) {
        if (cf.buff_tiles_per_item) s->tiling.buff_tiles[b] = std::min(cf.buff_tiles_per_item, kMaxItemTiles);
        if (cf.value_chunks_per_item) s->tiling.value_chunks[b] = std::min(cf.value_chunks_per_item, kMaxItemTiles);
        if (cf.gorilla_chunks_per_item)
            s->tiling.gorilla_chunks[b] = std::min(cf.gorilla_chunks_per_item, kMaxGorillaChunks);
    }
    for (ebi_column* c : s->cols) {
        if (!c) { delete s; return sfail(EBI_E_INVALID, "null column"); }
        const uint64_t its = column_item_count(c->scheme, c->n_chunks, static_cast<uint32_t>(c->tiles.tiles.size()),
                                               c->n_records, s->tiling);
        if (c->n_chunks > cf.max_chunks_per_batch || its > cf.max_items_per_batch) {
            delete s;
            return sfail(EBI_E_INVALID, "a column is larger than one batch's capacity");
        }
    }
    cudaSetDevice(cf.device);
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, cf.device);
    cudaError_t e = prepare_batch_kernel();
    s->slots.resize(cf.slots);
    for (Slot& sl : s->slots) {
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = salloc(&sl.d_qp, cf.max_queries_per_batch);
        if (e == cudaSuccess) e = salloc(&sl.d_items, cf.max_items_per_batch);
        if (e == cudaSuccess) e = salloc(&sl.d_acc, cf.max_chunks_per_batch);
        if (e == cudaSuccess) e = salloc(&sl.d_res, cf.max_queries_per_batch);
        if (e == cudaSuccess) e = salloc(&sl.d_counter, 1);
        if (e == cudaSuccess) e = cudaMallocHost(&sl.h_qp, cf.max_queries_per_batch * sizeof(QueryParams));
        if (e == cudaSuccess) e = cudaMallocHost(&sl.h_items, cf.max_items_per_batch * sizeof(BatchItem));
        if (e == cudaSuccess) e = cudaMallocHost(&sl.h_res, cf.max_queries_per_batch * sizeof(QueryResult));
        if (e == cudaSuccess) e = launch_acc_init(sl.d_acc, static_cast<uint32_t>(cf.max_chunks_per_batch), sl.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(sl.stream);
    }
    if (e != cudaSuccess) {
        ebi_server_destroy(s);
        return sfail(e == cudaErrorMemoryAllocation ? EBI_E_OOM : EBI_E_CUDA,
                     std::string("server workspace: ") + cudaGetErrorString(e));
    }
    s->worker = std::thread(run, s);
    *out = s;
    return EBI_OK;
}

int ebi_server_submit(ebi_server* s, const ebi_request* req, uint64_t* ticket) {
    if (!s || !req) return sfail(EBI_E_INVALID, "server or request is null");
    if (req->n_columns == 0 || req->n_columns > 8) return sfail(EBI_E_INVALID, "a request reads 1..8 columns");
    for (uint32_t k = 0; k < req->n_columns; ++k)
        if (req->columns[k] >= s->cols.size()) return sfail(EBI_E_INVALID, "column id out of range");
    const ebi_predicate& p = req->pred;
    if (p.kind < EBI_PRED_EQ || p.kind > EBI_PRED_RANGE) return sfail(EBI_E_INVALID, "bad predicate kind");
    uint64_t c, it;
    footprint(s, *req, &c, &it);
    if (c > s->cfg.max_chunks_per_batch || it > s->cfg.max_items_per_batch ||
        req->n_columns > s->cfg.max_queries_per_batch)
        return sfail(EBI_E_INVALID, "request larger than one batch's capacity");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->error) return sfail(s->error, "server failed");
        const uint64_t t = s->next_ticket++;
        s->pending.push_back(Pending{*req, t, now_ns()});
        if (ticket) *ticket = t;
    }
    s->cv.notify_one();
    return EBI_OK;
}

int ebi_server_poll(ebi_server* s, ebi_response* out, uint32_t max, uint32_t* n_out) {
    if (!s || !n_out || (!out && max)) return sfail(EBI_E_INVALID, "server or output is null");
    std::lock_guard<std::mutex> lk(s->mu);
    uint32_t n = 0;
    while (n < max && !s->done.empty()) {
        out[n++] = s->done.front();
        s->done.pop_front();
    }
    *n_out = n;
    return s->error ? sfail(s->error, "server failed") : EBI_OK;
}

int ebi_server_get_stats(ebi_server* s, ebi_server_stats* out) {
    if (!s || !out) return sfail(EBI_E_INVALID, "server or output is null");
    std::lock_guard<std::mutex> lk(s->mu);
    out->batches = s->batches;
    out->requests = s->batched_requests;
    out->max_in_flight = s->max_in_flight;
    out->pending = s->pending.size();
    out->items = s->items.load(std::memory_order_relaxed);
    out->build_ns = s->build_ns.load(std::memory_order_relaxed);
    return EBI_OK;
}

int ebi_server_replay(ebi_server* s, const ebi_request* reqs, const uint64_t* arrival_ns, uint64_t n,
                      ebi_response* out) {
    if (!s || (!reqs && n) || (!out && n)) return sfail(EBI_E_INVALID, "server, requests or output is null");
    std::vector<uint64_t> first(1, 0);
    const uint64_t t0 = now_ns();
    uint64_t base_ticket = 0, got = 0;
    std::vector<ebi_response> buf(256);
    auto drain = [&]() -> int {
        uint32_t k = 0;
        const int st = ebi_server_poll(s, buf.data(), static_cast<uint32_t>(buf.size()), &k);
        for (uint32_t j = 0; j < k; ++j) {
            const uint64_t idx = buf[j].ticket - base_ticket;
            if (idx < n) out[idx] = buf[j];
        }
        got += k;
        return st;
    };
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t due = t0 + (arrival_ns ? arrival_ns[i] : 0);
        while (now_ns() < due) {
            if (int st = drain()) return st;
        }
        uint64_t t = 0;
        if (int st = ebi_server_submit(s, &reqs[i], &t)) return st;
        if (i == 0) base_ticket = t;
    }
    while (got < n) {
        if (int st = drain()) return st;
        std::this_thread::yield();
    }
    return EBI_OK;
}

int ebi_run_plain(ebi_column* const* columns, uint32_t n_columns, const ebi_request* reqs, uint64_t n,
                  ebi_response* out, void* stream) {
    if (!columns || (!reqs && n) || (!out && n)) return sfail(EBI_E_INVALID, "columns, requests or output is null");
    const double inf = __builtin_inf();
    for (uint64_t i = 0; i < n; ++i) {
        const ebi_request& r = reqs[i];
        ebi_response o{};
        o.submit_ns = o.launch_ns = now_ns();
        o.sum = 0.0;
        o.min = inf;
        o.max = -inf;
        for (uint32_t k = 0; k < r.n_columns; ++k) {
            if (r.columns[k] >= n_columns) return sfail(EBI_E_INVALID, "column id out of range");
            double sm = 0, mn = inf, mx = -inf;
            uint64_t cnt = 0;
            const int st = ebi_filter_agg(columns[r.columns[k]], &r.pred, nullptr, -1, nullptr,
                                          (r.aggregates & AGG_SUM) ? &sm : nullptr, (r.aggregates & AGG_MIN) ? &mn : nullptr,
                                          (r.aggregates & AGG_MAX) ? &mx : nullptr, &cnt, stream);
            if (st && !o.status) o.status = st;
            o.sum += sm;
            o.min = std::fmin(o.min, mn);
            o.max = std::fmax(o.max, mx);
            o.count += cnt;
        }
        const double nan = __builtin_nan("");
        if (!(r.aggregates & AGG_SUM)) o.sum = nan;
        if (!(r.aggregates & AGG_MIN)) o.min = nan;
        if (!(r.aggregates & AGG_MAX)) o.max = nan;
        o.done_ns = now_ns();
        o.ticket = i;
        out[i] = o;
    }
    return EBI_OK;
}

int ebi_server_destroy(ebi_server* s) {
    if (!s) return EBI_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        void* d[] = {sl.d_qp, sl.d_items, sl.d_acc, sl.d_res, sl.d_counter};
        for (void* p : d) if (p) cudaFree(p);
        if (sl.h_qp) cudaFreeHost(sl.h_qp);
        if (sl.h_items) cudaFreeHost(sl.h_items);
        if (sl.h_res) cudaFreeHost(sl.h_res);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    delete s;
    return EBI_OK;
}

}  // extern "C"
