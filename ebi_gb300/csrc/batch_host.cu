// batch_host.cu -- ebi_batch: a fixed set of filter+aggregate queries over
// many resident columns, run as one persistent mixed-codec launch plus one
// fold launch, captured once into a CUDA graph and replayed.
//
// Every query owns its per-chunk accumulators (the same column may appear in
// several queries).  The first run tunes the launch (graph replays timed with
// events): the persistent CTAs per SM and the order of the work items, then,
// per codec family and column-size bucket present in the batch, how many BUFF
// tiles, RLE / Uncompressed chunks or Gorilla chunks one work item covers
// (coordinate descent; a candidate is kept when it is at least 2 % faster).
// The winner is reused for every later run and, when a tuning cache file is
// set (ebi_batch_set_tuning_cache), stored under the batch's column shape and
// reused by later batches of the same shape without timing.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
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

// One launch configuration: a shape and a tiling.
struct Config {
    int shape;
    BatchTiling tiling;
};

enum Knob : uint32_t { KNOB_SHAPE = 0, KNOB_BUFF = 1, KNOB_VALUE = 2, KNOB_GORILLA = 3 };
constexpr uint32_t kBuffCand[] = {1, 2, 4, 8, 16};
constexpr uint32_t kValueCand[] = {1, 2, 4, 8, 16};
constexpr uint32_t kGorillaCand[] = {8, 16, 32};

// The process-wide tuning cache: column shape -> configuration (and its time).
struct CacheEntry {
    Config cfg;
    double ms;
};
std::mutex g_cache_mu;
std::string g_cache_path;
std::map<std::string, CacheEntry> g_cache;
bool g_cache_loaded = false;

uint32_t* knob_slot(BatchTiling& t, uint32_t knob, int bucket) {
    return knob == KNOB_BUFF ? &t.buff_tiles[bucket] : knob == KNOB_VALUE ? &t.value_chunks[bucket]
                                                                          : &t.gorilla_chunks[bucket];
}

// Reads the cache file written by save_cache (one entry per line); a line
// that does not parse is skipped.
void load_cache_locked() {
    g_cache_loaded = true;
    if (g_cache_path.empty()) return;
    FILE* f = std::fopen(g_cache_path.c_str(), "r");
    if (!f) return;
    char line[4096];
    while (std::fgets(line, sizeof line, f)) {
        const char* q0 = std::strchr(line, '"');
        const char* q1 = q0 ? std::strchr(q0 + 1, '"') : nullptr;
        if (!q0 || !q1) continue;
        const std::string key(q0 + 1, q1);
        const char* p = q1 + 1;
        CacheEntry e{};
        unsigned c = 0, o = 0, b[3], v[3], g[3];
        double ms = 0;
        const char* fmt =
            ": {\"ctas_per_sm\": %u, \"order\": %u, \"buff_tiles\": [%u, %u, %u], \"value_chunks\": [%u, %u, %u], "
            "\"gorilla_chunks\": [%u, %u, %u], \"ms\": %lf";
        if (std::sscanf(p, fmt, &c, &o, &b[0], &b[1], &b[2], &v[0], &v[1], &v[2], &g[0], &g[1], &g[2], &ms) != 12) continue;
        e.cfg.shape = -1;
        for (int i = 0; i < kNumShapes; ++i)
            if (kShapes[i].ctas_per_sm == c && kShapes[i].order == o) e.cfg.shape = i;
        if (e.cfg.shape < 0) continue;
        bool ok = true;
        for (int k = 0; k < kSizeBuckets; ++k) {
            ok = ok && b[k] >= 1 && b[k] <= kMaxItemTiles && v[k] >= 1 && v[k] <= kMaxItemTiles && g[k] >= 1 &&
                 g[k] <= kMaxGorillaChunks;
            e.cfg.tiling.buff_tiles[k] = b[k];
            e.cfg.tiling.value_chunks[k] = v[k];
            e.cfg.tiling.gorilla_chunks[k] = g[k];
        }
        if (!ok) continue;
        e.ms = ms;
        g_cache[key] = e;
    }
    std::fclose(f);
}

void save_cache_locked() {
    if (g_cache_path.empty()) return;
    const std::string tmp = g_cache_path + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "w");
    if (!f) return;
    std::fprintf(f, "{\n");
    size_t i = 0;
    for (const auto& kv : g_cache) {
        const Config& c = kv.second.cfg;
        const BatchTiling& t = c.tiling;
        std::fprintf(f,
                     "\"%s\": {\"ctas_per_sm\": %u, \"order\": %u, \"buff_tiles\": [%u, %u, %u], \"value_chunks\": "
                     "[%u, %u, %u], \"gorilla_chunks\": [%u, %u, %u], \"ms\": %.4f}%s\n",
                     kv.first.c_str(), kShapes[c.shape].ctas_per_sm, kShapes[c.shape].order, t.buff_tiles[0],
                     t.buff_tiles[1], t.buff_tiles[2], t.value_chunks[0], t.value_chunks[1], t.value_chunks[2],
                     t.gorilla_chunks[0], t.gorilla_chunks[1], t.gorilla_chunks[2], kv.second.ms,
                     ++i < g_cache.size() ? "," : "");
    }
    std::fprintf(f, "}\n");
    const bool ok = std::fclose(f) == 0;
    if (ok) std::rename(tmp.c_str(), g_cache_path.c_str());
    else std::remove(tmp.c_str());
}

}  // namespace

struct ebi_batch {
    std::vector<ebi_batch_query> queries;  // in the caller's order
    // device order: queries on one column consecutive (first appearance order),
    // so that a Chimp-family chunk or a Gorilla chunk group is decoded once for
    // several of them; order[pos] = caller index, slot[caller index] = pos
    std::vector<uint32_t> order, slot;
    uint64_t n_chunks = 0;
    uint64_t max_items = 0;  // the most items any candidate tiling makes
    int sms = 1;
    std::string shape_key;   // column shape (codec family x size bucket counts) + SM count
    bool present[4][kSizeBuckets] = {};  // knob family x bucket: the batch has such columns
    // device
    QueryParams* d_qp = nullptr;
    BatchItem* d_items = nullptr;
    ChunkAcc* d_acc = nullptr;
    QueryResult* d_res = nullptr;
    unsigned int* d_counter = nullptr;
    // pinned host
    QueryParams* h_qp = nullptr;
    QueryResult* h_res = nullptr;
    // capture and tuning stream (capture is not allowed on the legacy default stream)
    cudaStream_t cap = nullptr;
    // the chosen configuration and its graph
    cudaGraphExec_t exec = nullptr;
    Config cfg{-1, {}};
    uint64_t n_items = 0;
    double best_ms = 0;
    bool from_cache = false;
    double shape_ms[kNumShapes] = {0, 0, 0, 0};
    std::vector<ebi_batch_trial> trials;
};

namespace {

// The work items of configuration c (device order: the queries on one column
// share their decodes; then cost order if asked).
void build_items(const ebi_batch* b, const Config& c, std::vector<BatchItem>& items) {
    items.clear();
    const uint32_t n = static_cast<uint32_t>(b->order.size());
    for (uint32_t g = 0; g < n;) {
        const ebi_column* col = b->queries[b->order[g]].col;
        uint32_t h = g + 1;
        while (h < n && b->queries[b->order[h]].col == col) ++h;
        shared_column_items(col->scheme, col->n_chunks, static_cast<uint32_t>(col->tiles.tiles.size()), col->n_records,
                            c.tiling, g, h - g, items);
        g = h;
    }
    if (kShapes[c.shape].order == 0) order_by_cost(items);
}

// Records one run of the batch (configuration c, items already in d_items) on stream s (captured).
int record(ebi_batch* b, const Config& c, uint64_t n_items, cudaStream_t s) {
    const uint32_t n = static_cast<uint32_t>(b->queries.size());
    BCK(cudaMemcpyAsync(b->d_qp, b->h_qp, n * sizeof(QueryParams), cudaMemcpyHostToDevice, s));
    for (const ebi_batch_query& q : b->queries)
        if (q.d_out_mask) BCK(cudaMemsetAsync(q.d_out_mask, 0, ((ebi_column_num_records(q.col) + 63) / 64) * 8, s));
    const uint32_t grid = static_cast<uint32_t>(b->sms) * kShapes[c.shape].ctas_per_sm;
    BCK(launch_batch(b->d_qp, b->d_items, static_cast<uint32_t>(n_items), b->d_counter, grid, s));
    BCK(launch_batch_finalize(b->d_qp, b->d_res, n, s));
    BCK(cudaMemcpyAsync(b->h_res, b->d_res, n * sizeof(QueryResult), cudaMemcpyDeviceToHost, s));
    return EBI_OK;
}

// Uploads configuration c's items and captures its graph.
int prepare(ebi_batch* b, const Config& c, cudaStream_t s, cudaGraphExec_t* out, uint64_t* n_items) {
    std::vector<BatchItem> items;
    build_items(b, c, items);
    if (items.size() > b->max_items) return bfail(EBI_E_INVALID, "batch tiling makes more items than allocated");
    BCK(cudaMemcpyAsync(b->d_items, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice, s));
    BCK(cudaStreamSynchronize(s));  // items is pageable host memory about to go out of scope
    *n_items = items.size();
    cudaGraph_t g = nullptr;
    BCK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int st = record(b, c, items.size(), s);
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

// Device time of one run of configuration c (one warm-up replay, then the mean of two).
int time_config(ebi_batch* b, const Config& c, cudaEvent_t e0, cudaEvent_t e1, double* ms_out) {
    cudaStream_t s = b->cap;
    cudaGraphExec_t ex = nullptr;
    uint64_t n_items = 0;
    if (int st = prepare(b, c, s, &ex, &n_items)) return st;
    cudaError_t e = cudaGraphLaunch(ex, s);
    if (e == cudaSuccess) e = cudaEventRecord(e0, s);
    for (int r = 0; r < 2 && e == cudaSuccess; ++r) e = cudaGraphLaunch(ex, s);
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaGraphExecDestroy(ex);
    if (e != cudaSuccess) return bfail(EBI_E_CUDA, std::string("batch tuning: ") + cudaGetErrorString(e));
    *ms_out = ms / 2.0;
    return EBI_OK;
}

// Chooses the configuration (from the cache or by timing) and captures its graph.
int tune(ebi_batch* b, cudaStream_t user) {
    BCK(prepare_batch_kernel());
    BCK(cudaStreamSynchronize(user));  // the batch's inputs were written on the caller's stream
    bool cached = false;
    {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        if (!g_cache_path.empty()) {
            if (!g_cache_loaded) load_cache_locked();
            auto it = g_cache.find(b->shape_key);
            if (it != g_cache.end()) {
                b->cfg = it->second.cfg;
                b->best_ms = it->second.ms;
                cached = true;
            }
        }
    }
    if (!cached) {
        cudaEvent_t e0, e1;
        BCK(cudaEventCreate(&e0));
        BCK(cudaEventCreate(&e1));
        int st = EBI_OK;
        Config cur{0, default_tiling()};
        double best = 0;
        auto trial = [&](const Config& c, uint32_t knob, uint32_t bucket, uint32_t value, double* ms) {
            const int r = time_config(b, c, e0, e1, ms);
            if (!r) b->trials.push_back(ebi_batch_trial{knob, bucket, value, 0, *ms});
            return r;
        };
        // launch shapes on the default tiling
        for (int sh = 0; sh < kNumShapes && !st; ++sh) {
            Config c = cur;
            c.shape = sh;
            double ms = 0;
            st = trial(c, KNOB_SHAPE, 0, kShapes[sh].ctas_per_sm * 2 + kShapes[sh].order, &ms);
            if (st) break;
            b->shape_ms[sh] = ms;
            if (sh == 0 || ms < best) {
                best = ms;
                cur.shape = sh;
            }
        }
        if (!st) {
            for (ebi_batch_trial& t : b->trials)
                t.kept = t.knob == KNOB_SHAPE && t.value == kShapes[cur.shape].ctas_per_sm * 2 + kShapes[cur.shape].order;
        }
        // tiles per item, one (family, bucket) at a time
        for (uint32_t knob = KNOB_BUFF; knob <= KNOB_GORILLA && !st; ++knob) {
            const uint32_t* cand = knob == KNOB_BUFF ? kBuffCand : knob == KNOB_VALUE ? kValueCand : kGorillaCand;
            const int nc = knob == KNOB_GORILLA ? 3 : 5;
            for (int bk = 0; bk < kSizeBuckets && !st; ++bk) {
                if (!b->present[knob][bk]) continue;
                for (int i = 0; i < nc && !st; ++i) {
                    if (cand[i] == *knob_slot(cur.tiling, knob, bk)) continue;
                    Config c = cur;
                    *knob_slot(c.tiling, knob, bk) = cand[i];
                    double ms = 0;
                    st = trial(c, knob, static_cast<uint32_t>(bk), cand[i], &ms);
                    if (!st && ms < 0.98 * best) {
                        best = ms;
                        cur = c;
                        b->trials.back().kept = 1;
                    }
                }
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (st) return st;
        b->cfg = cur;
        b->best_ms = best;
        std::lock_guard<std::mutex> lk(g_cache_mu);
        if (!g_cache_path.empty()) {
            g_cache[b->shape_key] = CacheEntry{cur, best};
            save_cache_locked();
        }
    }
    b->from_cache = cached;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    return prepare(b, b->cfg, b->cap, &b->exec, &b->n_items);
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
    {
        // device order: by column, columns in order of first appearance, queries stable
        std::map<const ebi_column*, uint32_t> first_seen;
        std::vector<uint32_t> key(n);
        for (uint64_t i = 0; i < n; ++i)
            key[i] = first_seen.emplace(queries[i].col, static_cast<uint32_t>(first_seen.size())).first->second;
        b->order.resize(n);
        for (uint64_t i = 0; i < n; ++i) b->order[i] = static_cast<uint32_t>(i);
        std::stable_sort(b->order.begin(), b->order.end(), [&](uint32_t x, uint32_t y) { return key[x] < key[y]; });
        b->slot.resize(n);
        for (uint64_t p = 0; p < n; ++p) b->slot[b->order[p]] = static_cast<uint32_t>(p);
    }
    std::vector<QueryParams> qp(n);  // device order
    std::vector<uint64_t> acc_off(n);
    std::map<int, uint64_t> shape_count;  // scheme * buckets + bucket -> queries
    for (uint64_t i = 0; i < n; ++i) {
        const ebi_batch_query& bq = queries[b->order[i]];  // position i of the device order
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
        // the batch's column shape and the most items any candidate tiling makes
        const ebi_column* c = bq.col;
        const int bk = size_bucket(c->n_records);
        const uint32_t knob = c->scheme == EBI_BUFF ? KNOB_BUFF
                            : c->scheme == EBI_GORILLA ? KNOB_GORILLA
                            : (c->scheme == EBI_RLE || c->scheme == EBI_UNCOMPRESSED) ? KNOB_VALUE : KNOB_SHAPE;
        if (knob != KNOB_SHAPE) b->present[knob][bk] = true;
        BatchTiling finest = default_tiling();
        for (int k = 0; k < kSizeBuckets; ++k) {
            finest.buff_tiles[k] = 1;
            finest.value_chunks[k] = 1;
            finest.gorilla_chunks[k] = kGorillaCand[0];
        }
        b->max_items += column_item_count(c->scheme, c->n_chunks, static_cast<uint32_t>(c->tiles.tiles.size()),
                                          c->n_records, finest);
        shape_count[c->scheme * kSizeBuckets + bk] += 1;
    }
    if (b->max_items > 0xffffffffull) {
        delete b;
        return bfail(EBI_E_INVALID, "a batch holds at most 2^32 - 1 work items");
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    b->shape_key = "sms=" + std::to_string(b->sms);
    for (const auto& kv : shape_count)
        b->shape_key += ";" + std::to_string(kv.first / kSizeBuckets) + "/" + std::to_string(kv.first % kSizeBuckets) +
                        "x" + std::to_string(kv.second);
    int st = balloc(&b->d_qp, n);
    if (!st) st = balloc(&b->d_items, b->max_items);
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
        cudaError_t e = launch_acc_init(b->d_acc, static_cast<uint32_t>(b->n_chunks), s);
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
            b->h_qp[b->slot[i]].pred = p;
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
        const QueryResult& r = b->h_res[b->slot[i]];
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
    out->items = b->exec ? b->n_items : 0;
    out->chunks = b->n_chunks;
    out->shape = b->exec ? b->cfg.shape : -1;
    if (b->exec) {
        out->ctas_per_sm = kShapes[b->cfg.shape].ctas_per_sm;
        out->order = kShapes[b->cfg.shape].order;
        for (int k = 0; k < kSizeBuckets; ++k) {
            out->buff_tiles[k] = b->cfg.tiling.buff_tiles[k];
            out->value_chunks[k] = b->cfg.tiling.value_chunks[k];
            out->gorilla_chunks[k] = b->cfg.tiling.gorilla_chunks[k];
        }
    }
    for (int i = 0; i < kNumShapes && i < 4; ++i) out->shape_ms[i] = b->shape_ms[i];
    out->trials = static_cast<uint32_t>(b->trials.size());
    out->from_cache = b->from_cache ? 1u : 0u;
    out->best_ms = b->best_ms;
    return EBI_OK;
}

int ebi_batch_get_trials(const ebi_batch* b, ebi_batch_trial* out, uint32_t max, uint32_t* n_out) {
    if (!b || (!out && max) || !n_out) return bfail(EBI_E_INVALID, "batch, output or count is null");
    const uint32_t n = static_cast<uint32_t>(std::min<size_t>(max, b->trials.size()));
    for (uint32_t i = 0; i < n; ++i) out[i] = b->trials[i];
    *n_out = n;
    return EBI_OK;
}

int ebi_batch_set_tuning_cache(const char* path) {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    g_cache.clear();
    g_cache_loaded = false;
    g_cache_path = path ? path : "";
    return EBI_OK;
}

int ebi_batch_destroy(ebi_batch* b) {
    if (!b) return EBI_OK;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->cap) cudaStreamDestroy(b->cap);
    void* d[] = {b->d_qp, b->d_items, b->d_acc, b->d_res, b->d_counter};
    for (void* p : d) if (p) cudaFree(p);
    if (b->h_qp) cudaFreeHost(b->h_qp);
    if (b->h_res) cudaFreeHost(b->h_res);
    delete b;
    return EBI_OK;
}

}  // extern "C"
