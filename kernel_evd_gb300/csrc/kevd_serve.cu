// Serving loop: resident models, admission by HBM footprint, continuous
// batching of Nystrom eigenfunction queries.
//
//   factorization request (host X, N x d): admitted when a factor worker is
//       idle and its footprint fits the budget left by running factorizations
//       and resident models.  The worker (own context, own stream) copies X in,
//       runs block RPCholesky, the bistochastic EVD and the Nystrom
//       preparation, keeps only the model (landmark rows and [Z'|p1'])
//       resident and frees the rest.
//   query request (host Y, n x d, model id): queued per model.  The query
//       worker (own context, own stream) takes whatever is queued for the model
//       with the oldest pending query, up to max_query_batch states, evaluates
//       it in one fused launch and scatters the rows back.  Queries arriving
//       while a batch is on the GPU join the next one; query launches overlap
//       the factorizations on the device.
//
// No counterpart exists in the reference (its stages are batch programs).
// The query kernel evaluates every state independently, so a result does not
// depend on the batch it joined.
#include "kevd_internal.cuh"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>

namespace kevd {
namespace {

using Clock = std::chrono::steady_clock;

constexpr int kQueryMaxD = 1024;
constexpr int kQueryMaxOut = 64;

struct Request {
    int64_t id = 0;
    int type = 0;            // 0 factorization, 1 query
    int status = -1;         // -1 pending, else a kevd_status
    Clock::time_point submitted, started, finished;
    int64_t batch = 0;       // states in the launches that served a query
    // factorization
    std::vector<float> X;
    int64_t N = 0;
    int d = 0;
    double scale = 0.0;
    int64_t k = 0;
    int block = 0;
    int k_out = 0;
    uint64_t seed = 0;
    int precision = KEVD_MIXED;
    size_t footprint = 0;
    int64_t model_id = -1;
    double trace_error = 0.0;
    int64_t rank = 0;
    std::string message;     // failure description
    // query
    const float* Y = nullptr;
    int64_t n = 0;
    float* out = nullptr;
};

struct ResidentModel {
    kevd_model* model = nullptr;
    size_t bytes = 0;
    int d = 0;
    int k_out = 0;
    bool busy = false;       // a query batch is using it
    std::deque<std::shared_ptr<Request>> queries;
};

struct Worker {
    kevd_ctx* ctx = nullptr;
    cudaStream_t stream = nullptr;
    size_t held = 0;         // device bytes its workspace keeps between requests
    size_t running = 0;      // footprint of the request it runs (0: idle)
};

}  // namespace
}  // namespace kevd

struct kevd_server {
    kevd_server_config cfg;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    int64_t next_id = 1;
    int64_t next_model = 1;
    size_t used = 0;         // resident models
    bool trim = false;       // idle workers release their workspaces
    int active = 0;
    int peak_active = 0;
    std::map<int64_t, std::shared_ptr<kevd::Request>> requests;
    std::deque<std::shared_ptr<kevd::Request>> fact_queue;
    std::map<int64_t, kevd::ResidentModel> models;
    std::vector<kevd::Worker> ws;   // factor workers, then the query worker
    std::vector<std::thread> threads;
    std::vector<double> lat[2];
};

namespace kevd {
namespace {

// Device bytes a factorization holds at its peak: X, F and its column-major
// copy, the residual-update column block, N-length FP64 vectors, k x k FP64
// matrices, the EVD output and Ritz buffers (FP64 factors double F).
size_t factorization_footprint(int64_t N, int d, int64_t k, int k_out, int precision) {
    const double f = (precision == KEVD_FP64 ? 8.0 : 4.0) * (double)N * (double)k;
    const double b = 4.0 * N * d + 2.0 * f + 4.0 * N * 64 + 10.0 * 8.0 * N + 8.0 * 8.0 * (double)k * k +
                     4.0 * N * (2.0 * k_out + 2);
    return (size_t)(1.1 * b) + ((size_t)64 << 20);
}

// Bytes charged against the budget: resident models, and per factor worker
// the larger of the workspace it keeps and the footprint of what it runs.
size_t charged_locked(const kevd_server* s, int skip) {
    size_t c = s->used;
    for (int i = 0; i < s->cfg.factor_workers; ++i)
        if (i != skip) c += std::max(s->ws[i].held, s->ws[i].running);
    return c;
}

size_t model_bytes(int64_t r, int d, int k_out) {
    return (size_t)r * (size_t)d * 4 + (size_t)r * (size_t)(k_out + 1) * 8;
}

void finish_locked(kevd_server* s, const std::shared_ptr<Request>& r, int status) {
    r->finished = Clock::now();
    r->status = status;
    s->lat[r->type].push_back(std::chrono::duration<double>(r->finished - r->submitted).count());
}

void factor_worker(kevd_server* s, int wi) {
    Worker& w = s->ws[wi];
    cudaSetDevice(s->cfg.device);
    while (true) {
        std::shared_ptr<Request> r;
        bool do_trim = false;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            auto fits = [&] {
                const size_t fp = s->fact_queue.front()->footprint;
                return charged_locked(s, wi) + std::max(w.held, fp) <= s->cfg.hbm_budget_bytes;
            };
            // Trims happen only while a queued request cannot be admitted.
            s->cv_work.wait(lk, [&] {
                if (s->stop) return true;
                if (s->fact_queue.empty()) return false;
                if (fits()) return true;
                // the head request does not fit: release this worker's own
                // workspace if that is what is in the way, else ask the idle
                // workers to release theirs
                if (w.held > s->fact_queue.front()->footprint) return true;
                if (s->trim && w.held > 0) return true;
                bool idle_held = false;
                for (int i = 0; i < s->cfg.factor_workers; ++i)
                    if (i != wi && s->ws[i].running == 0 && s->ws[i].held > 0) idle_held = true;
                if (idle_held && !s->trim) {
                    s->trim = true;
                    s->cv_work.notify_all();
                }
                return false;
            });
            if (s->stop) break;
            if (!fits()) {
                do_trim = true;   // w.held > 0 here
            } else {
                r = s->fact_queue.front();
                s->fact_queue.pop_front();
                if (s->fact_queue.empty()) s->trim = false;
                w.running = r->footprint;
                ++s->active;
                s->peak_active = std::max(s->peak_active, s->active);
                r->started = Clock::now();
            }
        }
        if (do_trim) {
            w.ctx->arena.release();
            std::lock_guard<std::mutex> lk(s->mu);
            w.held = 0;
            bool any = false;
            for (int i = 0; i < s->cfg.factor_workers; ++i)
                if (s->ws[i].running == 0 && s->ws[i].held > 0) any = true;
            if (!any) s->trim = false;
            s->cv_work.notify_all();
            continue;
        }
        int rc = KEVD_OK;
        kevd_model* model = nullptr;
        const size_t fbytes = (size_t)r->N * (size_t)r->k * (r->precision == KEVD_FP64 ? 8 : 4);
        // the dataset and the factor live in the worker's workspace, which it
        // keeps for the next request (no allocation or free per request)
        float* X = arena_get<float>(w.ctx, "srv.X", (size_t)r->N * r->d, &rc);
        void* F = arena_get<uint8_t>(w.ctx, "srv.F", fbytes, &rc);
        std::vector<int64_t> piv((size_t)r->k);
        kevd_rpchol_result res = {0, 0, 0.0};
        if (rc == KEVD_OK && cudaMemcpyAsync(X, r->X.data(), (size_t)r->N * r->d * 4, cudaMemcpyHostToDevice,
                                             w.stream) != cudaSuccess)
            rc = KEVD_ERR_CUDA;
        if (rc == KEVD_OK) {
            kevd_rpchol_params p;
            std::memset(&p, 0, sizeof(p));
            p.k_max = r->k;
            p.block = r->block;
            p.max_rounds = (int32_t)(4 * ((r->k + r->block - 1) / r->block) + 8);
            p.tol = 1e-10;
            p.seed = r->seed;
            p.precision = r->precision;
            rc = kevd_rpchol(w.ctx, X, r->N, r->d, r->scale, &p, F, r->k, piv.data(), nullptr, nullptr, &res,
                             w.stream);
        }
        if (rc == KEVD_OK && res.rank < r->k_out) rc = KEVD_ERR_ARG;   // rank-deficient dataset
        if (rc == KEVD_OK)
            rc = kevd_nystrom_prepare(w.ctx, X, r->N, r->d, r->scale, F, r->precision, r->k, piv.data(), res.rank,
                                      r->k_out, &model, w.stream);
        cudaStreamSynchronize(w.stream);
        const size_t held = w.ctx->arena.total();
        std::string msg;
        if (rc != KEVD_OK) {
            const char* e = kevd_last_error(w.ctx);
            msg = (rc == KEVD_ERR_ARG && res.rank > 0 && res.rank < r->k_out) ? "rank below k_out"
                                                                            : std::string(e ? e : "");
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            w.running = 0;
            w.held = held;
            --s->active;
            if (rc == KEVD_OK) {
                const int64_t mid = s->next_model++;
                ResidentModel& rm = s->models[mid];
                rm.model = model;
                rm.bytes = model_bytes(res.rank, r->d, r->k_out);
                rm.d = r->d;
                rm.k_out = r->k_out;
                s->used += rm.bytes;
                r->model_id = mid;
                r->trace_error = res.trace_error;
                r->rank = res.rank;
            } else if (model) {
                kevd_model_destroy(model);
            }
            std::vector<float>().swap(r->X);
            r->message = msg;
            finish_locked(s, r, rc);
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

void query_worker(kevd_server* s, int wi) {
    Worker& w = s->ws[wi];
    cudaSetDevice(s->cfg.device);
    const int64_t cap = s->cfg.max_query_batch;
    float *hY = nullptr, *hU = nullptr, *dY = nullptr, *dU = nullptr;
    int init_rc = KEVD_OK;
    if (cudaMallocHost(&hY, (size_t)cap * kQueryMaxD * 4) != cudaSuccess ||
        cudaMallocHost(&hU, (size_t)cap * kQueryMaxOut * 4) != cudaSuccess ||
        cudaMalloc(&dY, (size_t)cap * kQueryMaxD * 4) != cudaSuccess ||
        cudaMalloc(&dU, (size_t)cap * kQueryMaxOut * 4) != cudaSuccess) {
        cudaGetLastError();
        init_rc = KEVD_ERR_NOMEM;
    }
    while (true) {
        std::vector<std::shared_ptr<Request>> batch;
        int64_t mid = -1;
        kevd_model* model = nullptr;
        int d = 0, kout = 0;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            auto ready = [&] {
                if (s->stop) return true;
                for (auto& kv : s->models)
                    if (!kv.second.queries.empty()) return true;
                return false;
            };
            s->cv_work.wait(lk, ready);
            if (s->stop) break;
            if (s->cfg.batch_window_us > 0) {
                lk.unlock();
                std::this_thread::sleep_for(std::chrono::duration<double, std::micro>(s->cfg.batch_window_us));
                lk.lock();
            }
            Clock::time_point oldest = Clock::time_point::max();
            for (auto& kv : s->models)
                if (!kv.second.queries.empty() && kv.second.queries.front()->submitted < oldest) {
                    oldest = kv.second.queries.front()->submitted;
                    mid = kv.first;
                }
            if (mid < 0) continue;
            ResidentModel& rm = s->models[mid];
            model = rm.model;
            d = rm.d;
            kout = rm.k_out;
            // whole requests while they fit; a request larger than the cap runs
            // alone, in cap-sized launches
            int64_t rows = 0;
            while (!rm.queries.empty() && (rows == 0 || rows + rm.queries.front()->n <= cap)) {
                auto q = rm.queries.front();
                rm.queries.pop_front();
                q->started = Clock::now();
                rows += q->n;
                batch.push_back(q);
                if (rows >= cap) break;
            }
            rm.busy = true;
        }
        int rc = init_rc;
        int64_t rows = 0;
        for (auto& q : batch) rows += q->n;
        if (rc == KEVD_OK && (d > kQueryMaxD || kout > kQueryMaxOut)) rc = KEVD_ERR_ARG;
        size_t qi = 0;
        int64_t q_off = 0;
        while (rc == KEVD_OK && qi < batch.size()) {
            // pack up to cap rows, possibly across requests
            int64_t packed = 0;
            std::vector<std::tuple<size_t, int64_t, int64_t>> pieces;   // request, first row, rows
            while (packed < cap && qi < batch.size()) {
                const int64_t take = std::min(cap - packed, batch[qi]->n - q_off);
                std::memcpy(hY + packed * d, batch[qi]->Y + q_off * d, (size_t)take * d * 4);
                pieces.emplace_back(qi, q_off, take);
                packed += take;
                q_off += take;
                if (q_off == batch[qi]->n) {
                    ++qi;
                    q_off = 0;
                }
            }
            if (cudaMemcpyAsync(dY, hY, (size_t)packed * d * 4, cudaMemcpyHostToDevice, w.stream) != cudaSuccess) {
                rc = KEVD_ERR_CUDA;
                break;
            }
            rc = kevd_nystrom_eval(w.ctx, model, dY, packed, dU, w.stream);
            if (rc != KEVD_OK) break;
            if (cudaMemcpyAsync(hU, dU, (size_t)packed * kout * 4, cudaMemcpyDeviceToHost, w.stream) !=
                    cudaSuccess ||
                cudaStreamSynchronize(w.stream) != cudaSuccess) {
                rc = KEVD_ERR_CUDA;
                break;
            }
            int64_t pos = 0;
            for (auto& pc : pieces) {
                const auto& q = batch[std::get<0>(pc)];
                std::memcpy(q->out + std::get<1>(pc) * kout, hU + pos * kout, (size_t)std::get<2>(pc) * kout * 4);
                pos += std::get<2>(pc);
            }
        }
        std::string msg;
        if (rc != KEVD_OK) {
            const char* e = kevd_last_error(w.ctx);
            msg = (rc == KEVD_ERR_NOMEM && init_rc != KEVD_OK) ? "query staging buffers" : std::string(e ? e : "");
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->models[mid].busy = false;
            for (auto& q : batch) {
                q->batch = rows;
                q->message = msg;
                finish_locked(s, q, rc);
            }
        }
        s->cv_done.notify_all();
    }
    if (hY) cudaFreeHost(hY);
    if (hU) cudaFreeHost(hU);
    if (dY) cudaFree(dY);
    if (dU) cudaFree(dU);
}

double percentile(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = p * (double)(v.size() - 1);
    const size_t i = (size_t)pos;
    const double f = pos - (double)i;
    return (i + 1 < v.size()) ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

void destroy_workers(std::vector<Worker>& ws) {
    for (auto& w : ws) {
        if (w.stream) cudaStreamDestroy(w.stream);
        if (w.ctx) kevd_ctx_destroy(w.ctx);
    }
    ws.clear();
}

}  // namespace
}  // namespace kevd

using namespace kevd;

extern "C" {

int64_t kevd_factorization_footprint(int64_t N, int32_t d, int64_t k, int32_t k_out, int32_t precision) {
    if (N < 1 || d < 1 || k < 1 || k_out < 0 || (precision != KEVD_FP64 && precision != KEVD_MIXED)) return -1;
    return (int64_t)factorization_footprint(N, d, k, k_out, precision);
}

int kevd_server_create(const kevd_server_config* cfg, kevd_server** out) {
    if (!cfg || !out || cfg->factor_workers < 1 || cfg->factor_workers > 16 || cfg->max_query_batch < 1 ||
        cfg->max_query_batch > (1 << 20) || !(cfg->batch_window_us >= 0))
        return KEVD_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || cfg->device < 0 || cfg->device >= ndev) {
        cudaGetLastError();
        return KEVD_ERR_CUDA;
    }
    std::vector<Worker> ws;
    for (int i = 0; i < cfg->factor_workers + 1; ++i) {
        Worker w;
        int rc = kevd_ctx_create(cfg->device, &w.ctx);
        if (rc == KEVD_OK && cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking) != cudaSuccess)
            rc = KEVD_ERR_CUDA;
        ws.push_back(w);
        if (rc != KEVD_OK) {
            destroy_workers(ws);
            return rc;
        }
    }
    kevd_server* s = new kevd_server();
    s->cfg = *cfg;
    s->ws = ws;
    for (int i = 0; i < cfg->factor_workers; ++i) s->threads.emplace_back(factor_worker, s, i);
    s->threads.emplace_back(query_worker, s, cfg->factor_workers);
    *out = s;
    return KEVD_OK;
}

void kevd_server_destroy(kevd_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->threads) t.join();
    for (auto& kv : s->models) kevd_model_destroy(kv.second.model);
    destroy_workers(s->ws);
    delete s;
}

int kevd_server_submit_factorization(kevd_server* s, const float* X, int64_t N, int32_t d, double scale,
                                     int64_t k, int32_t block, int32_t k_out, uint64_t seed, int32_t precision,
                                     int64_t* request_id) {
    if (!s || !X || !request_id || N < 2 || d < 1 || d > kMaxFeatures || !(scale > 0.0) || k < 1 || k > N || block < 1 ||
        block > 512 || k_out < 1 || k_out > kQueryMaxOut || k_out > k ||
        (precision != KEVD_FP64 && precision != KEVD_MIXED))
        return KEVD_ERR_ARG;
    const size_t footprint = factorization_footprint(N, d, k, k_out, precision);
    if (footprint > s->cfg.hbm_budget_bytes) return KEVD_ERR_NOMEM;   // could never be admitted
    auto r = std::make_shared<Request>();
    r->type = 0;
    r->X.assign(X, X + (size_t)N * d);
    r->N = N;
    r->d = d;
    r->scale = scale;
    r->k = k;
    r->block = block;
    r->k_out = k_out;
    r->seed = seed;
    r->precision = precision;
    r->footprint = footprint;
    r->submitted = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        s->requests[r->id] = r;
        s->fact_queue.push_back(r);
        *request_id = r->id;
    }
    s->cv_work.notify_all();
    return KEVD_OK;
}

int kevd_server_submit_query(kevd_server* s, int64_t model_id, const float* Y, int64_t n, float* out,
                             int64_t* request_id) {
    if (!s || !Y || !out || !request_id || n < 1) return KEVD_ERR_ARG;
    auto r = std::make_shared<Request>();
    r->type = 1;
    r->Y = Y;
    r->n = n;
    r->out = out;
    r->model_id = model_id;
    r->submitted = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->models.find(model_id);
        if (it == s->models.end()) return KEVD_ERR_ARG;
        r->id = s->next_id++;
        s->requests[r->id] = r;
        it->second.queries.push_back(r);
        *request_id = r->id;
    }
    s->cv_work.notify_all();
    return KEVD_OK;
}

int kevd_server_wait(kevd_server* s, int64_t request_id, double timeout_s, kevd_request_info* info) {
    if (!s || !(timeout_s >= 0)) return KEVD_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end()) return KEVD_ERR_ARG;
    auto r = it->second;
    if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return r->status >= 0; }))
        return KEVD_ERR_TIMEOUT;
    if (info) {
        info->status = r->status;
        info->model_id = r->model_id;
        info->latency_s = std::chrono::duration<double>(r->finished - r->submitted).count();
        info->queue_s = std::chrono::duration<double>(r->started - r->submitted).count();
        info->batch_rows = r->batch;
        info->trace_error = r->trace_error;
        info->rank = r->rank;
        std::memset(info->message, 0, sizeof(info->message));
        std::strncpy(info->message, r->message.c_str(), sizeof(info->message) - 1);
    }
    s->requests.erase(request_id);
    return KEVD_OK;
}

int kevd_server_release_model(kevd_server* s, int64_t model_id) {
    if (!s) return KEVD_ERR_ARG;
    kevd_model* m = nullptr;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->models.find(model_id);
        if (it == s->models.end() || it->second.busy || !it->second.queries.empty()) return KEVD_ERR_ARG;
        m = it->second.model;
        s->used -= it->second.bytes;
        s->models.erase(it);
    }
    kevd_model_destroy(m);
    s->cv_work.notify_all();   // the freed bytes may admit a queued factorization
    return KEVD_OK;
}

int kevd_server_stats(kevd_server* s, int32_t type, double* p50, double* p99, int64_t* count) {
    if (!s || type < 0 || type > 1) return KEVD_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (p50) *p50 = percentile(s->lat[type], 0.50);
    if (p99) *p99 = percentile(s->lat[type], 0.99);
    if (count) *count = (int64_t)s->lat[type].size();
    return KEVD_OK;
}

int kevd_server_memory(kevd_server* s, int64_t* used_bytes, int32_t* active_factorizations, int32_t* models,
                       int32_t* peak_active) {
    if (!s) return KEVD_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (used_bytes) *used_bytes = (int64_t)charged_locked(s, -1);
    if (active_factorizations) *active_factorizations = s->active;
    if (models) *models = (int32_t)s->models.size();
    if (peak_active) *peak_active = s->peak_active;
    return KEVD_OK;
}

}  // extern "C"
