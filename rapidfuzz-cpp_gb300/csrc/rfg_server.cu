/*
 * rfg_server.cu -- continuous-batching extract service over device-resident corpora.
 *
 * The reference has no service; its README shows the caller-side extract/extractOne
 * loops (README.md:153-214).  This is their serving form: callers submit requests
 * (one query, a metric, an op, a limit) at any time; a loop thread groups queued
 * requests with the same scoring spec into batches and admits a batch when one of the
 * `max_inflight` stream slots is free and its device memory estimate fits the budget
 * (default: 80 % of the device memory free at start).  Admitted batches run
 * concurrently on their own streams; requests that arrive meanwhile wait in the queue
 * and join the next batches, so work of different requests overlaps on the device.
 * Results are copied to the caller's buffers when their batch completes; each request
 * records submit-to-completion latency.  A request's result does not depend on the
 * batch it rides in: every query is scored against the whole corpus on its own.
 */
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "rapidfuzz_gb300.h"
#include "rfg_device.cuh"

namespace rfg {
rfg_status set_last_error(rfg_status s, const char* msg);
struct ExtractJob;
/* implemented in rfg_api.cu */
rfg_status server_extract_enqueue(rfg_corpus c, const unsigned char* qdata, const int64_t* qoff, int64_t nq,
                                  int width, int metric, int op, const rfg_params* p, rfg_cutoff cut, int k,
                                  int tie_last, cudaStream_t st, void** job, int64_t* est_bytes);
rfg_status server_extract_results(void* job, int64_t* idx, double* score, int32_t* count, cudaStream_t st);
void server_extract_free(void* job);
int64_t corpus_chunks(rfg_corpus c);

/* device bytes one batch holds while it runs: its packed queries, offsets, per-query
 * thresholds and results, and the per-(query, chunk) candidate lists of the extract */
inline int64_t batch_bytes(int64_t query_bytes, int64_t nq, int64_t k, int64_t chunks)
{
    return query_bytes + 8 * (nq + 1) + nq * (8 + 4 + 16 * k) + nq * chunks * k * 16 + (1 << 20);
}
} // namespace rfg

using namespace rfg;
using Clock = std::chrono::steady_clock;

namespace {

struct Req {
    uint64_t ticket;
    rfg_request r;
    std::vector<unsigned char> query;
    Clock::time_point t_submit, t_done;
    bool done = false;
    rfg_status status = RFG_OK;
};

bool same_spec(const rfg_request& a, const rfg_request& b)
{
    return a.corpus == b.corpus && a.metric == b.metric && a.op == b.op && a.limit == b.limit &&
           a.tie_last_wins == b.tie_last_wins && a.query_width == b.query_width &&
           memcmp(&a.params, &b.params, sizeof a.params) == 0 && memcmp(&a.cutoff, &b.cutoff, sizeof a.cutoff) == 0;
}

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;
    std::vector<Req*> reqs;
    void* job = nullptr;
    int64_t bytes = 0;
    int64_t* h_idx = nullptr; /* pinned staging */
    double* h_score = nullptr;
    int32_t* h_count = nullptr;
};

} // namespace

struct rfg_server_s {
    std::vector<rfg_corpus> corpora;
    rfg_server_config cfg{};
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req*> queue;
    std::unordered_map<uint64_t, Req*> reqs;
    uint64_t next_ticket = 1;
    bool stop = false;
    std::thread loop;
    int64_t bytes_in_use = 0;
    int64_t completed = 0, batches = 0, batched_requests = 0;
    rfg_status fault = RFG_OK;

    void run();
    bool admit(Slot& s, std::unique_lock<std::mutex>& lk);
    void complete(Slot& s);
};

bool rfg_server_s::admit(Slot& s, std::unique_lock<std::mutex>& lk)
{
    if (queue.empty()) return false;
    Req* head = queue.front();
    std::vector<Req*> batch;
    for (auto it = queue.begin(); it != queue.end() && (int)batch.size() < cfg.max_batch;) {
        if (same_spec((*it)->r, head->r)) {
            batch.push_back(*it);
            it = queue.erase(it);
        }
        else
            ++it;
    }
    /* pack the queries */
    const int w = head->r.query_width;
    std::vector<int64_t> off(batch.size() + 1, 0);
    for (size_t i = 0; i < batch.size(); ++i) off[i + 1] = off[i] + batch[i]->r.query_len;
    std::vector<unsigned char> data((size_t)off.back() * w + 16);
    for (size_t i = 0; i < batch.size(); ++i)
        if (batch[i]->r.query_len) memcpy(data.data() + off[i] * w, batch[i]->query.data(), batch[i]->query.size());
    /* device memory estimate: queries, thresholds, candidates, results */
    const int64_t k = head->r.limit;
    const int64_t nq = (int64_t)batch.size();
    const int64_t est = batch_bytes((int64_t)data.size(), nq, k, corpus_chunks(corpora[head->r.corpus]));
    if (bytes_in_use + est > cfg.max_device_bytes && bytes_in_use > 0) {
        /* not admitted: back to the front of the queue, in order */
        for (auto it = batch.rbegin(); it != batch.rend(); ++it) queue.push_front(*it);
        return false;
    }
    bytes_in_use += est;
    lk.unlock();
    void* job = nullptr;
    int64_t unused = 0;
    rfg_status st = server_extract_enqueue(corpora[head->r.corpus], data.data(), off.data(), nq, w, head->r.metric,
                                           head->r.op, &head->r.params, head->r.cutoff, (int)k,
                                           head->r.tie_last_wins, s.stream, &job, &unused);
    if (st == RFG_OK) st = server_extract_results(job, s.h_idx, s.h_score, s.h_count, s.stream);
    if (st == RFG_OK && cudaEventRecord(s.done, s.stream) != cudaSuccess) st = RFG_ERR_CUDA;
    lk.lock();
    s.reqs = batch;
    s.job = job;
    s.bytes = est;
    s.busy = true;
    ++batches;
    batched_requests += nq;
    if (st != RFG_OK) {
        for (Req* r : batch) r->status = st;
        if (cudaEventRecord(s.done, s.stream) != cudaSuccess) fault = RFG_ERR_CUDA;
    }
    return true;
}

void rfg_server_s::complete(Slot& s)
{
    const int k = s.reqs.empty() ? 0 : s.reqs[0]->r.limit;
    for (size_t i = 0; i < s.reqs.size(); ++i) {
        Req* r = s.reqs[i];
        if (r->status == RFG_OK) {
            memcpy(r->r.out_index, s.h_idx + i * k, k * sizeof(int64_t));
            memcpy(r->r.out_score, s.h_score + i * k, k * sizeof(double));
            *r->r.out_count = s.h_count[i];
        }
        r->t_done = Clock::now();
        r->done = true;
        ++completed;
    }
    if (s.job) server_extract_free(s.job);
    s.job = nullptr;
    s.reqs.clear();
    bytes_in_use -= s.bytes;
    s.bytes = 0;
    s.busy = false;
}

void rfg_server_s::run()
{
    std::unique_lock<std::mutex> lk(mu);
    while (!stop) {
        bool progressed = false;
        for (Slot& s : slots) {
            if (s.busy && cudaEventQuery(s.done) == cudaSuccess) {
                complete(s);
                progressed = true;
            }
        }
        if (progressed) cv_done.notify_all();
        for (Slot& s : slots) {
            if (!s.busy && !queue.empty()) {
                if (admit(s, lk)) progressed = true;
                else break;
            }
        }
        bool any_busy = false;
        for (Slot& s : slots) any_busy |= s.busy;
        if (!progressed) {
            if (any_busy) {
                lk.unlock();
                std::this_thread::sleep_for(std::chrono::microseconds(20));
                lk.lock();
            }
            else if (queue.empty()) {
                cv_work.wait_for(lk, std::chrono::milliseconds(5));
            }
        }
    }
    /* drain: finish what runs, fail what never got admitted */
    for (Slot& s : slots)
        if (s.busy) {
            lk.unlock();
            cudaEventSynchronize(s.done);
            lk.lock();
            complete(s);
        }
    for (Req* r : queue) {
        r->status = RFG_ERR_BUSY;
        r->t_done = Clock::now();
        r->done = true;
    }
    queue.clear();
    cv_done.notify_all();
}

extern "C" {

rfg_status rfg_server_create(const rfg_corpus* corpora, int32_t ncorpora, const rfg_server_config* cfg,
                             rfg_server* out)
{
    if (!out || !corpora || ncorpora < 1) return set_last_error(RFG_ERR_INVALID_ARGUMENT, "invalid arguments");
    *out = nullptr;
    for (int i = 0; i < ncorpora; ++i)
        if (!corpora[i]) return set_last_error(RFG_ERR_INVALID_ARGUMENT, "NULL corpus");
    rfg_server s = new rfg_server_s();
    s->corpora.assign(corpora, corpora + ncorpora);
    s->cfg.max_inflight = cfg && cfg->max_inflight > 0 ? cfg->max_inflight : 4;
    s->cfg.max_batch = cfg && cfg->max_batch > 0 ? cfg->max_batch : 64;
    s->cfg.max_device_bytes = cfg ? cfg->max_device_bytes : 0;
    if (s->cfg.max_device_bytes <= 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        s->cfg.max_device_bytes = (int64_t)(fr * 0.8);
    }
    s->slots.resize(s->cfg.max_inflight);
    const size_t k = RFG_MAX_TOPK, nb = s->cfg.max_batch;
    for (Slot& sl : s->slots) {
        if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess ||
            cudaHostAlloc((void**)&sl.h_idx, nb * k * 8, 0) != cudaSuccess ||
            cudaHostAlloc((void**)&sl.h_score, nb * k * 8, 0) != cudaSuccess ||
            cudaHostAlloc((void**)&sl.h_count, nb * 4, 0) != cudaSuccess) {
            rfg_server_destroy(s);
            return set_last_error(RFG_ERR_OUT_OF_MEMORY, "server set-up failed (streams / pinned staging)");
        }
    }
    s->loop = std::thread([s] { s->run(); });
    *out = s;
    return RFG_OK;
}

rfg_status rfg_server_submit(rfg_server s, const rfg_request* r, uint64_t* ticket)
{
    if (!s || !r || !ticket) return set_last_error(RFG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (r->corpus < 0 || r->corpus >= (int)s->corpora.size())
        return set_last_error(RFG_ERR_INVALID_ARGUMENT, "unknown corpus");
    if (r->limit < 1 || r->limit > RFG_MAX_TOPK) return set_last_error(RFG_ERR_INVALID_ARGUMENT, "limit in [1, 32]");
    if (r->query_width != 1 && r->query_width != 2 && r->query_width != 4 && r->query_width != 8)
        return set_last_error(RFG_ERR_INVALID_ARGUMENT, "query_width must be 1, 2, 4 or 8");
    if (r->query_len < 0 || (!r->query && r->query_len) || !r->out_index || !r->out_score || !r->out_count)
        return set_last_error(RFG_ERR_INVALID_ARGUMENT, "invalid request buffers");
    if (r->metric < RFG_LEVENSHTEIN || r->metric > RFG_RATIO || r->op < RFG_DISTANCE ||
        r->op > RFG_NORMALIZED_SIMILARITY || (r->metric == RFG_RATIO && r->op != RFG_SIMILARITY))
        return set_last_error(RFG_ERR_INVALID_ARGUMENT, "invalid metric/op");
    /* memory-bounded admission: a request that alone needs more device memory than the
     * server's budget can never run -- refused at once instead of queued */
    const int64_t need = batch_bytes(r->query_len * r->query_width + 16, 1, r->limit, corpus_chunks(s->corpora[r->corpus]));
    if (need > s->cfg.max_device_bytes)
        return set_last_error(RFG_ERR_BUSY, "admission refused: the request needs more device memory than the "
                                            "server's max_device_bytes");
    Req* q = new Req();
    q->r = *r;
    q->query.assign((const unsigned char*)r->query, (const unsigned char*)r->query + r->query_len * r->query_width);
    q->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) {
            delete q;
            return set_last_error(RFG_ERR_BUSY, "server is shutting down");
        }
        q->ticket = s->next_ticket++;
        s->reqs[q->ticket] = q;
        s->queue.push_back(q);
        *ticket = q->ticket;
    }
    s->cv_work.notify_one();
    return RFG_OK;
}

rfg_status rfg_server_wait(rfg_server s, uint64_t ticket, double timeout_s, double* latency_ms)
{
    if (!s) return set_last_error(RFG_ERR_INVALID_ARGUMENT, "server is NULL");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return set_last_error(RFG_ERR_INVALID_ARGUMENT, "unknown ticket");
    Req* q = it->second;
    const auto deadline = Clock::now() + std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 1e9);
    while (!q->done) {
        if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !q->done)
            return set_last_error(RFG_ERR_BUSY, "timed out waiting for the request");
    }
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(q->t_done - q->t_submit).count();
    const rfg_status st = q->status;
    s->reqs.erase(it);
    delete q;
    if (st != RFG_OK) return set_last_error(st, "request failed on the device");
    return RFG_OK;
}

rfg_status rfg_server_stats(rfg_server s, int64_t* completed, int64_t* batches, int64_t* batched_requests)
{
    if (!s) return set_last_error(RFG_ERR_INVALID_ARGUMENT, "server is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    if (completed) *completed = s->completed;
    if (batches) *batches = s->batches;
    if (batched_requests) *batched_requests = s->batched_requests;
    return RFG_OK;
}

rfg_status rfg_server_destroy(rfg_server s)
{
    if (!s) return RFG_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->loop.joinable()) s->loop.join();
    for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.h_idx) cudaFreeHost(sl.h_idx);
        if (sl.h_score) cudaFreeHost(sl.h_score);
        if (sl.h_count) cudaFreeHost(sl.h_count);
    }
    for (auto& kv : s->reqs) delete kv.second;
    delete s;
    return RFG_OK;
}

} /* extern "C" */
