// batch_host.cu -- ebi_batch: a fixed set of filter+aggregate queries over
// many resident columns, run as one persistent mixed-codec launch plus one
// fold launch, captured once into a CUDA graph and replayed.
//
// Every query owns its per-chunk accumulators (the same column may appear in
// several queries).  On the first run the batch times a few launch shapes
// (persistent CTAs per SM, order of the work items) by replaying each shape's
// graph, keeps the fastest and reuses it for every later run.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "column.h"

namespace {

int bfail(int code, const std::string& msg) {
    set_last_error(msg);
    return code;
}
#define BCK(expr)                                                                               \
    do {                                                                                        \
        cudaError_t _e = (expr);                                                                \
        if (_e != cudaSuccess) return bfail(EBI_E_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
    } while (0)

struct Shape {
    uint32_t ctas_per_sm;
    uint32_t order;  // 0: cost-descending, 1: query order
};
constexpr Shape kShapes[] = {{2, 0}, {1, 0}, {2, 1}, {1, 1}};
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);

}  // namespace

struct ebi_batch {
    std::vector<ebi_batch_query> queries;
    std::vector<BatchItem> items_cost, items_query;
    uint64_t n_chunks = 0;
    int sms = 1;
    // device
    QueryParams* d_qp = nullptr;
    BatchItem* d_items[2] = {nullptr, nullptr};
    ChunkAcc* d_acc = nullptr;
    QueryResult* d_res = nullptr;
    unsigned int* d_counter = nullptr;
    // pinned host
    QueryParams* h_qp = nullptr;
    QueryResult* h_res = nullptr;
    // capture and tuning stream (capture is not allowed on the legacy default stream)
    cudaStream_t cap = nullptr;
    // the chosen graph
    cudaGraphExec_t exec = nullptr;
    int shape = -1;
    double shape_ms[kNumShapes] = {0, 0, 0, 0};
};

namespace {

// Records one run of the batch with launch shape `sh` on stream s (captured).
int record(ebi_batch* b, int sh, cudaStream_t s) {
    const uint32_t n = static_cast<uint32_t>(b->queries.size());
    const size_t n_items = b->items_cost.size();
    BCK(cudaMemcpyAsync(b->d_qp, b->h_qp, n * sizeof(QueryParams), cudaMemcpyHostToDevice, s));
    for (const ebi_batch_query& q : b->queries)
        if (q.d_out_mask) BCK(cudaMemsetAsync(q.d_out_mask, 0, ((ebi_column_num_records(q.col) + 63) / 64) * 8, s));
    const uint32_t grid = static_cast<uint32_t>(b->sms) * kShapes[sh].ctas_per_sm;
    BCK(launch_batch(b->d_qp, b->d_items[kShapes[sh].order], static_cast<uint32_t>(n_items), b->d_counter, grid, s));
    BCK(launch_batch_finalize(b->d_qp, b->d_res, n, s));
    BCK(cudaMemcpyAsync(b->h_res, b->d_res, n * sizeof(QueryResult), cudaMemcpyDeviceToHost, s));
    return EBI_OK;
}

int capture(ebi_batch* b, int sh, cudaStream_t s, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    BCK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int st = record(b, sh, s);
    const cudaError_t e = cudaStreamEndCapture(s, &g);
    if (st) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    BCK(e);
    const cudaError_t ei = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    BCK(ei);
    return EBI_OK;
}

// Times every launch shape (one warm-up and two timed replays each) and keeps the fastest.
int tune(ebi_batch* b, cudaStream_t user) {
    BCK(prepare_batch_kernel());
    BCK(cudaStreamSynchronize(user));  // the batch's inputs were written on the caller's stream
    cudaStream_t s = b->cap;
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    double best = 1e30;
    int st = EBI_OK;
    for (int sh = 0; sh < kNumShapes && !st; ++sh) {
        cudaGraphExec_t ex = nullptr;
        if ((st = capture(b, sh, s, &ex))) break;
        cudaError_t e = cudaGraphLaunch(ex, s);
        if (e == cudaSuccess) e = cudaEventRecord(e0, s);
        for (int r = 0; r < 2 && e == cudaSuccess; ++r) e = cudaGraphLaunch(ex, s);
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e != cudaSuccess) {
            cudaGraphExecDestroy(ex);
            st = bfail(EBI_E_CUDA, std::string("batch tuning: ") + cudaGetErrorString(e));
            break;
        }
        b->shape_ms[sh] = ms / 2.0;
        if (b->shape_ms[sh] < best) {
            best = b->shape_ms[sh];
            if (b->exec) cudaGraphExecDestroy(b->exec);
            b->exec = ex;
            b->shape = sh;
        } else {
            cudaGraphExecDestroy(ex);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return st;
}

template <typename T>
int balloc(T** p, size_t n) {
    void* v = nullptr;
    const cudaError_t e = cudaMalloc(&v, (n ? n : 1) * sizeof(T));
    if (e != cudaSuccess) return bfail(e == cudaErrorMemoryAllocation ? EBI_E_OOM : EBI_E_CUDA, "batch allocation failed");
    *p = static_cast<T*>(v);
    return EBI_OK;
}

}  // namespace

extern "C" {

int ebi_batch_create(const ebi_batch_query* queries, uint64_t n, void* stream, ebi_batch** out) {
    if (!out || (!queries && n)) return bfail(EBI_E_INVALID, "queries or out is null");
    *out = nullptr;
    if (n == 0 || n > 0xffffffffull) return bfail(EBI_E_INVALID, "a batch holds 1 .. 2^32 - 1 queries");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ebi_batch* b = new (std::nothrow) ebi_batch();
    if (!b) return bfail(EBI_E_OOM, "host allocation failed");
    b->queries.assign(queries, queries + n);
    std::vector<QueryParams> qp(n);
    std::vector<uint64_t> acc_off(n);
    for (uint64_t i = 0; i < n; ++i) {
        const ebi_batch_query& bq = queries[i];
        if (!bq.col) { delete b; return bfail(EBI_E_INVALID, "query without a column"); }
        const ebi_predicate& p = bq.pred;
        if (p.kind < EBI_PRED_EQ || p.kind > EBI_PRED_RANGE ||
            (p.kind == EBI_PRED_RANGE && (p.start_kind < 0 || p.start_kind > 2 || p.end_kind < 0 || p.end_kind > 2))) {
            delete b;
            return bfail(EBI_E_INVALID, "bad predicate in batch query");
        }
        acc_off[i] = b->n_chunks;
        b->n_chunks += bq.col->n_chunks;
        QueryParams q = column_params(bq.col);
        q.op = OP_FILTER_AGG;
        q.pred = p;
        q.pred_on = 1;
        q.agg = bq.aggregates & AGG_ALL;
        q.out_mask = reinterpret_cast<uint32_t*>(bq.d_out_mask);
        q.out_atomic = 1;
        q.stage_bytes = 0;
        qp[i] = q;
        // work items of this query's column
        const ebi_column* c = bq.col;
        column_items(c->scheme, c->n_chunks, static_cast<uint32_t>(c->tiles.tiles.size()), static_cast<uint32_t>(i),
                     b->items_query);
    }
    b->items_cost = b->items_query;
    std::stable_sort(b->items_cost.begin(), b->items_cost.end(), [](const BatchItem& x, const BatchItem& y) {
        return item_cost(x.kind, x.count) > item_cost(y.kind, y.count);
    });
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    int st = balloc(&b->d_qp, n);
    if (!st) st = balloc(&b->d_items[0], b->items_cost.size());
    if (!st) st = balloc(&b->d_items[1], b->items_query.size());
    if (!st) st = balloc(&b->d_acc, b->n_chunks);
    if (!st) st = balloc(&b->d_res, n);
    if (!st) st = balloc(&b->d_counter, 1);
    if (!st && cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) != cudaSuccess)
        st = bfail(EBI_E_CUDA, "batch stream creation failed");
    if (!st && cudaMallocHost(&b->h_qp, n * sizeof(QueryParams)) != cudaSuccess) st = bfail(EBI_E_OOM, "pinned allocation failed");
    if (!st && cudaMallocHost(&b->h_res, n * sizeof(QueryResult)) != cudaSuccess) st = bfail(EBI_E_OOM, "pinned allocation failed");
    if (!st) {
        for (uint64_t i = 0; i < n; ++i) {
            qp[i].acc = b->d_acc + acc_off[i];
            b->h_qp[i] = qp[i];
        }
        cudaError_t e = cudaMemcpyAsync(b->d_items[0], b->items_cost.data(), b->items_cost.size() * sizeof(BatchItem),
                                        cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(b->d_items[1], b->items_query.data(), b->items_query.size() * sizeof(BatchItem),
                                cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = launch_acc_init(b->d_acc, static_cast<uint32_t>(b->n_chunks), s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = bfail(EBI_E_CUDA, std::string("batch upload: ") + cudaGetErrorString(e));
    }
    if (st) {
        ebi_batch_destroy(b);
        return st;
    }
    *out = b;
    return EBI_OK;
}

int ebi_batch_run(ebi_batch* b, const ebi_predicate* preds, ebi_batch_result* results, void* stream) {
    if (!b) return bfail(EBI_E_INVALID, "batch is null");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t n = b->queries.size();
    if (preds) {
        for (size_t i = 0; i < n; ++i) {
            const ebi_predicate& p = preds[i];
            if (p.kind < EBI_PRED_EQ || p.kind > EBI_PRED_RANGE) return bfail(EBI_E_INVALID, "bad predicate kind");
            b->h_qp[i].pred = p;
            b->queries[i].pred = p;
        }
    }
    if (!b->exec) {
        if (int st = tune(b, s)) return st;
    }
    const uint64_t launches0 = ebi_kernel_launches();
    BCK(cudaGraphLaunch(b->exec, s));
    count_launch(2);  // the batch kernel and the fold replayed by the graph
    (void)launches0;
    BCK(cudaStreamSynchronize(s));
    int first_err = EBI_OK;
    for (size_t i = 0; i < n; ++i) {
        const QueryResult& r = b->h_res[i];
        if (results) {
            results[i].sum = r.sum;
            results[i].min = r.min;
            results[i].max = r.max;
            results[i].count = r.count;
            results[i].status = static_cast<int32_t>(r.status);
            results[i].bad_chunk = r.bad_chunk;
        }
        if (r.status && !first_err) first_err = static_cast<int>(r.status);
    }
    if (first_err) {
        char buf[96];
        std::snprintf(buf, sizeof buf, "a batch query failed with status %d (see its result)", first_err);
        return bfail(first_err, buf);
    }
    return EBI_OK;
}

int ebi_batch_get_info(const ebi_batch* b, ebi_batch_info* out) {
    if (!b || !out) return bfail(EBI_E_INVALID, "batch or out is null");
    std::memset(out, 0, sizeof *out);
    out->queries = b->queries.size();
    out->items = b->items_cost.size();
    out->chunks = b->n_chunks;
    out->shape = b->shape;
    if (b->shape >= 0) {
        out->ctas_per_sm = kShapes[b->shape].ctas_per_sm;
        out->order = kShapes[b->shape].order;
    }
    for (int i = 0; i < kNumShapes && i < 4; ++i) out->shape_ms[i] = b->shape_ms[i];
    return EBI_OK;
}

int ebi_batch_destroy(ebi_batch* b) {
    if (!b) return EBI_OK;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->cap) cudaStreamDestroy(b->cap);
    void* d[] = {b->d_qp, b->d_items[0], b->d_items[1], b->d_acc, b->d_res, b->d_counter};
    for (void* p : d) if (p) cudaFree(p);
    if (b->h_qp) cudaFreeHost(b->h_qp);
    if (b->h_res) cudaFreeHost(b->h_res);
    delete b;
    return EBI_OK;
}

}  // extern "C"
