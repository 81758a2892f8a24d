// service.cu — continuous batching of column runs on one GPU.
//
// Requests (one column run each: levels, duration, dt, parameters, an optional alkalinity pulse) are
// submitted from any host thread and queued.  A worker thread owns the column engine and loops:
//   1. admit queued requests while a column slot and arena space (the HBM budget) are free: the
//      initial state goes through a pinned mirror of the arena into the column's block;
//   2. launch one chunk of `chunk_steps` steps for every resident, unfinished column;
//   3. queue the device->host copy of every column that this chunk finishes, behind the chunk;
//   4. retire the chunk before last: once its event has completed, hand the finished results
//      to their requests, free their slots and blocks, and record the latency.
// Two chunks stay queued on the stream, so the host work of (1)-(4) overlaps the kernels and the
// GPU never idles between chunks while work is resident.  A request that arrives while others run
// joins at the next chunk boundary; a column's arithmetic does not depend on the columns it shares
// a launch with, so its result is the same alone and in the mix.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <algorithm>
#include "columns_engine.h"

using namespace obgc;
using namespace obgc::cols;

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
    obgc_column_spec spec;
    std::vector<double> init, kappa, result;
    double t_submit = 0, t_admit = 0, t_done = 0;
    int state = 0;               // 0 queued, 1 resident, 2 done
    int64_t slot = -1;
};

struct Chunk {
    cudaEvent_t ev = nullptr;
    std::vector<std::pair<int64_t, int64_t>> finishing;   // (slot, request id) of columns ending in this chunk
};
// The request table is guarded by the service mutex; the worker alone changes slot_req and the
// engine, so it reads those without the mutex.

}  // namespace

struct obgc_service {
    obgc_columns* eng = nullptr;
    int chunk = 32;
    int max_queue = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    void* pinned = nullptr;               // host mirror of the state arena (state element size)
    void* pinned_kappa = nullptr;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<int64_t> queue;
    std::unordered_map<int64_t, Request> reqs;
    std::unordered_map<int64_t, int64_t> slot_req;   // engine slot -> request id
    std::deque<Chunk> inflight;
    std::vector<cudaEvent_t> free_events;
    int64_t next_id = 1, submitted = 0, admitted = 0, completed = 0, launches = 0;
    std::vector<double> latencies_ms;
    double t_first = -1, t_last = 0;
    bool stop = false;
    int error = OBGC_OK;
    std::string error_msg;
};

namespace {

// Everything the worker does with the GPU; returns a status (the worker stops on an error).
int admit_locked(obgc_service* S, std::unique_lock<std::mutex>& lk) {
    obgc_columns* e = S->eng;
    while (!S->queue.empty()) {
        const int64_t id = S->queue.front();
        Request& r = S->reqs[id];
        int64_t slot = -1;
        if (reserve_column(e, &r.spec, &slot) != OBGC_OK) break;     // no slot or no arena space: wait
        S->queue.pop_front();
        const int64_t off = e->slots[slot].cell_off;
        const int Nz = r.spec.Nz;
        const size_t n = (size_t)e->NT * Nz;
        if (e->ts == 4) {
            float* h = static_cast<float*>(S->pinned) + off * e->NT;
            float* k = static_cast<float*>(S->pinned_kappa) + off;
            for (size_t q = 0; q < n; q++) h[q] = (float)r.init[q];
            for (int f = 0; f <= Nz; f++) k[f] = (float)r.kappa[f];
        } else {
            std::memcpy(static_cast<double*>(S->pinned) + off * e->NT, r.init.data(), 8 * n);
            std::memcpy(static_cast<double*>(S->pinned_kappa) + off, r.kappa.data(), 8 * (Nz + 1));
        }
        const size_t es = e->ts;
        OBGC_CUDA(cudaMemcpyAsync(static_cast<char*>(e->state) + es * off * e->NT,
                                  static_cast<char*>(S->pinned) + es * off * e->NT, es * n, cudaMemcpyHostToDevice,
                                  S->stream));
        OBGC_CUDA(cudaMemcpyAsync(static_cast<char*>(e->kappa) + es * off, static_cast<char*>(S->pinned_kappa) + es * off,
                                  es * (Nz + 1), cudaMemcpyHostToDevice, S->stream));
        r.state = 1;
        r.slot = slot;
        r.t_admit = now_s();
        r.init.clear();
        r.init.shrink_to_fit();
        S->slot_req[slot] = id;
        S->admitted++;
    }
    (void)lk;
    return OBGC_OK;
}

int launch_chunk(obgc_service* S) {
    obgc_columns* e = S->eng;
    // which resident columns end in this chunk
    Chunk ch;
    for (auto& kv : S->slot_req) {
        const ColSlot<double>& c = e->slots[kv.first];
        if (c.live && c.steps_left > 0 && c.steps_left <= S->chunk) ch.finishing.emplace_back(kv.first, kv.second);
    }
    const int npacks = stage_tables(e, e->cap, S->stream);
    if (npacks < 0) return -npacks;
    if (npacks == 0) return OBGC_OK;
    int rc = prepare_launch(e, e->cap);
    if (rc != OBGC_OK) return rc;
    rc = launch_any(e, npacks, S->chunk, e->threads, e->cap, S->stream);
    if (rc != OBGC_OK) return rc;
    account_steps(e, S->chunk);
    S->launches++;
    // results of the finished columns, behind the chunk, into the pinned mirror of their blocks
    const size_t es = e->ts;
    for (const auto& f : ch.finishing) {
        const ColSlot<double>& c = e->slots[f.first];
        OBGC_CUDA(cudaMemcpyAsync(static_cast<char*>(S->pinned) + es * c.cell_off * e->NT,
                                  static_cast<char*>(e->state) + es * c.cell_off * e->NT, es * (size_t)e->NT * c.Nz,
                                  cudaMemcpyDeviceToHost, S->stream));
    }
    if (S->free_events.empty()) {
        cudaEvent_t ev;
        OBGC_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        S->free_events.push_back(ev);
    }
    ch.ev = S->free_events.back();
    S->free_events.pop_back();
    OBGC_CUDA(cudaEventRecord(ch.ev, S->stream));
    S->inflight.push_back(std::move(ch));
    return OBGC_OK;
}

// Wait for the oldest chunk and hand its finished columns to their requests.
int retire_oldest(obgc_service* S) {
    Chunk ch = std::move(S->inflight.front());
    S->inflight.pop_front();
    OBGC_CUDA(cudaEventSynchronize(ch.ev));
    S->free_events.push_back(ch.ev);
    obgc_columns* e = S->eng;
    const double t = now_s();
    std::lock_guard<std::mutex> lk(S->mu);
    for (const auto& f : ch.finishing) {
        Request& r = S->reqs[f.second];
        const int64_t off = e->slots[r.slot].cell_off;
        const size_t n = (size_t)e->NT * r.spec.Nz;
        r.result.resize(n);
        if (e->ts == 4) {
            const float* h = static_cast<const float*>(S->pinned) + off * e->NT;
            for (size_t q = 0; q < n; q++) r.result[q] = h[q];
        } else {
            std::memcpy(r.result.data(), static_cast<const double*>(S->pinned) + off * e->NT, 8 * n);
        }
        release_column(e, r.slot);
        S->slot_req.erase(r.slot);
        r.slot = -1;
        r.state = 2;
        r.t_done = t;
        S->completed++;
        S->latencies_ms.push_back(1e3 * (r.t_done - r.t_submit));
        S->t_last = t;
    }
    S->cv_done.notify_all();
    return OBGC_OK;
}

bool has_unfinished(const obgc_service* S) {
    for (auto& kv : S->slot_req)
        if (S->eng->slots[kv.first].steps_left > 0) return true;
    return false;
}

void worker_main(obgc_service* S) {
    cudaSetDevice(S->device);
    int rc = OBGC_OK;
    while (rc == OBGC_OK) {
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] {
                return S->stop || !S->queue.empty() || !S->inflight.empty() || has_unfinished(S);
            });
            if (S->stop && S->inflight.empty()) break;
            rc = admit_locked(S, lk);
            if (rc != OBGC_OK) break;
        }
        if (has_unfinished(S)) rc = launch_chunk(S);
        if (rc != OBGC_OK) break;
        // keep two chunks queued; retire the older one (or the last one when nothing else runs)
        if (S->inflight.size() >= 2 || (!S->inflight.empty() && !has_unfinished(S))) rc = retire_oldest(S);
    }
    while (!S->inflight.empty()) {   // leave nothing queued behind
        Chunk ch = std::move(S->inflight.front());
        S->inflight.pop_front();
        cudaEventSynchronize(ch.ev);
        S->free_events.push_back(ch.ev);
    }
    std::lock_guard<std::mutex> lk(S->mu);
    if (rc != OBGC_OK) {
        S->error = rc;
        S->error_msg = obgc_last_error_message();
    }
    S->stop = true;
    S->cv_done.notify_all();
}

}  // namespace

extern "C" int obgc_service_create(const obgc_service_desc* d, obgc_service** out) {
    if (!d || !out) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_service_create: null argument");
    *out = nullptr;
    obgc_columns* e = nullptr;
    int rc = obgc_columns_create(&d->columns, &e);
    if (rc != OBGC_OK) return rc;
    obgc_service* S = new obgc_service();
    S->eng = e;
    S->chunk = d->chunk_steps > 0 ? d->chunk_steps : 32;
    S->max_queue = d->max_queue;
    cudaGetDevice(&S->device);
    cudaError_t err = cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaMallocHost(&S->pinned, e->ts * e->NT * (size_t)d->columns.arena_cells);
    if (err == cudaSuccess) err = cudaMallocHost(&S->pinned_kappa, e->ts * (size_t)d->columns.arena_cells);
    if (err != cudaSuccess) {
        rc = cuda_fail(err, "obgc_service_create");
        if (S->stream) cudaStreamDestroy(S->stream);
        cudaFreeHost(S->pinned);
        cudaFreeHost(S->pinned_kappa);
        obgc_columns_destroy(e);
        delete S;
        return rc;
    }
    S->worker = std::thread(worker_main, S);
    *out = S;
    return OBGC_OK;
}

extern "C" int obgc_service_destroy(obgc_service* S) {
    if (!S) return OBGC_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    if (S->worker.joinable()) S->worker.join();
    cudaStreamSynchronize(S->stream);
    // the engine's last stream is the service stream: release the engine while the stream exists
    obgc_columns_destroy(S->eng);
    S->eng = nullptr;
    for (cudaEvent_t ev : S->free_events) cudaEventDestroy(ev);
    cudaStreamDestroy(S->stream);
    cudaFreeHost(S->pinned);
    cudaFreeHost(S->pinned_kappa);
    delete S;
    return OBGC_OK;
}

extern "C" int obgc_service_submit(obgc_service* S, const obgc_column_spec* sp, const double* init, const double* kappa,
                                   int64_t* id) {
    if (!S || !sp || !init || !kappa || !id || sp->Nz < 1 || sp->Nz > OBGC_COLUMN_MAX_LEVELS || sp->nsteps < 1 ||
        !(sp->dz > 0) || !(sp->dt > 0))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_service_submit: bad request");
    const int NT = S->eng->NT;
    Request r;
    r.spec = *sp;
    r.init.assign(init, init + (size_t)NT * sp->Nz);
    r.kappa.assign(kappa, kappa + sp->Nz + 1);
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) return fail(S->error ? S->error : OBGC_ERR_INVALID_ARGUMENT, "obgc_service_submit: service stopped: " + S->error_msg);
        if (S->max_queue > 0 && (int)S->queue.size() >= S->max_queue)
            return fail(OBGC_ERR_BUSY, "obgc_service_submit: queue full");
        if ((int64_t)sp->Nz + 1 > S->eng->desc.arena_cells)
            return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_service_submit: column larger than the arena");
        r.t_submit = now_s();
        if (S->t_first < 0) S->t_first = r.t_submit;
        *id = S->next_id++;
        S->reqs.emplace(*id, std::move(r));
        S->queue.push_back(*id);
        S->submitted++;
    }
    S->cv_work.notify_one();
    return OBGC_OK;
}

extern "C" int obgc_service_wait(obgc_service* S, int64_t id, double timeout_s, double* state, double* latency_ms) {
    if (!S) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_service_wait: null service");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_service_wait: unknown request");
    const auto until = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    while (it->second.state != 2) {
        if (S->stop && S->error) return fail(S->error, "obgc_service_wait: service stopped: " + S->error_msg);
        if (S->cv_done.wait_until(lk, until) == std::cv_status::timeout && it->second.state != 2)
            return fail(OBGC_ERR_TIMEOUT, "obgc_service_wait: timed out");
        it = S->reqs.find(id);
    }
    if (state) std::memcpy(state, it->second.result.data(), sizeof(double) * it->second.result.size());
    if (latency_ms) *latency_ms = 1e3 * (it->second.t_done - it->second.t_submit);
    S->reqs.erase(it);
    return OBGC_OK;
}

extern "C" int obgc_service_drain(obgc_service* S, double timeout_s) {
    if (!S) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_service_drain: null service");
    std::unique_lock<std::mutex> lk(S->mu);
    const auto until = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    while (S->completed < S->submitted) {
        if (S->stop && S->error) return fail(S->error, "obgc_service_drain: service stopped: " + S->error_msg);
        if (S->cv_done.wait_until(lk, until) == std::cv_status::timeout && S->completed < S->submitted)
            return fail(OBGC_ERR_TIMEOUT, "obgc_service_drain: timed out");
    }
    return OBGC_OK;
}

extern "C" int obgc_service_get_stats(obgc_service* S, obgc_service_stats* out) {
    if (!S || !out) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_service_get_stats: null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = S->submitted;
    out->admitted = S->admitted;
    out->completed = S->completed;
    out->launches = S->launches;
    std::vector<double> l = S->latencies_ms;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto pct = [&](double p) {
            const double x = p * (l.size() - 1);
            const size_t i = (size_t)x;
            const double f = x - i;
            return i + 1 < l.size() ? l[i] * (1 - f) + l[i + 1] * f : l[i];
        };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        out->max_ms = l.back();
        double s = 0;
        for (double v : l) s += v;
        out->mean_ms = s / l.size();
    }
    out->span_s = S->t_first >= 0 && S->t_last > S->t_first ? S->t_last - S->t_first : 0.0;
    return OBGC_OK;
}

extern "C" int obgc_service_reset_stats(obgc_service* S) {
    if (!S) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_service_reset_stats: null service");
    std::lock_guard<std::mutex> lk(S->mu);
    S->latencies_ms.clear();
    S->submitted -= S->completed;
    S->admitted -= S->completed;
    S->completed = 0;
    S->launches = 0;
    S->t_first = -1;
    S->t_last = 0;
    return OBGC_OK;
}

extern "C" int obgc_service_engine(obgc_service* S, obgc_columns** eng) {
    if (!S || !eng) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_service_engine: null argument");
    *eng = S->eng;
    return OBGC_OK;
}
