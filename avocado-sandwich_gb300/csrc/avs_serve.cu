// Serving loop: an SVD request server with continuous batching and device
// memory admission, on top of the C ABI of this library.
//
// Execution slots ("workers") each own an avs_handle (stream + workspace) and
// a host thread.  A free slot takes the oldest queued request and every other
// queued request of the same order and type along (up to max_batch) into one
// batched call (FP32: FP32 tiles, double-float stages; FP64: FP64
// throughout), so requests that arrive while others run join the next group
// of their order.  Slots run concurrently, so groups of different orders and
// types overlap on the GPU.  Admission: a slot
// starts a group only while the device bytes held by all slots (workspaces +
// input/output buffers) stay within the budget; otherwise it shrinks the
// group, releases its own cached memory, or waits for others to finish (idle
// slots release theirs when memory is short).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "avs_common.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    int64_t id = 0;
    int64_t n = 0, lda = 0;
    int32_t dtype = AVS_DTYPE_F32;
    int32_t tile = 0;
    const void *A = nullptr;
    void *sigma = nullptr;
    Clock::time_point t_submit, t_done;
    int32_t status = 0;
    bool done = false;
};

struct Slot {
    avs_handle *h = nullptr;
    cudaStream_t s = nullptr;
    void *io = nullptr;  // inputs + outputs of a group
    size_t io_bytes = 0;
    size_t held = 0;  // bytes of workspace + io this slot holds (accounted under the server lock)
    bool busy = false;
    std::thread th;
};

}  // namespace

struct avs_server {
    avs_serve_config cfg{};
    std::mutex mu;
    std::condition_variable cv_work;  // queue changed / memory freed / stop
    std::condition_variable cv_done;  // a request completed
    std::deque<Request *> queue;
    std::unordered_map<int64_t, Request *> reqs;
    std::vector<Slot> slots;
    int64_t next_id = 1;
    bool stop = false;
    bool pressure = false;
    size_t budget = 0, held_total = 0, peak = 0;
    int64_t submitted = 0, completed = 0, failed = 0, batches = 0, batched_reqs = 0;
    std::vector<double> lat_ms;
    bool any_submit = false;
    Clock::time_point t_first, t_last;
};

namespace {

// Tile rule of the serving loop (FP32 measured on GB300: tile 32 is fastest up
// to n = 256 in batched groups, 64 up to 1024, 128 beyond; FP64 likewise).
int32_t rule_tile(int64_t n) {
    int32_t t = n <= 256 ? 32 : (n <= 1024 ? 64 : 128);
    while (t > 16 && (n % t != 0 || t > n)) t >>= 1;
    return t;
}

// The server's plan for a request: tile, precision mode, and whether
// requests of its order and type share batched calls.  FP32 requests of order
// >= 2048 with tiles >= 128 run alone with the split-BF16 tensor-core update
// (measured on GB300, tile 128: n = 8192 0.45 s against 0.58 s for the FP32
// SIMT update; the tensor-core update takes one matrix per call); smaller FP32
// requests run in batched groups (FP32 SIMT updates).  FP64 requests run in
// batched groups with the double-float trailing updates (AVS_PREC_FP64X2).
void plan_of(int64_t n, int32_t dtype, int32_t tile_req, int32_t *tile, int32_t *prec, int32_t *batched) {
    const int32_t t = tile_req > 0 ? tile_req : rule_tile(n);
    *tile = t;
    if (dtype == AVS_DTYPE_F64) {
        *prec = AVS_PREC_FP64X2;
        *batched = 1;
    } else if (n >= 2048 && t >= 128) {
        *prec = AVS_PREC_BF16X3;
        *batched = 0;
    } else {
        *prec = AVS_PREC_FP32;
        *batched = 1;
    }
}

int32_t pick_tile(avs_server *S, Slot &sl, const Request *r) {
    if (r->tile > 0) return r->tile;
    if (S->cfg.autotune && r->dtype == AVS_DTYPE_F32 && r->n >= 64) {
        int32_t best = 0;
        const int32_t sample = (int32_t)std::max<int64_t>(1, std::min<int64_t>(16, (1LL << 22) / (r->n * r->n)));
        if (avs_autotune_tile(sl.h, r->n, sample, &best) == AVS_SUCCESS && best > 0) return best;
    }
    return rule_tile(r->n);
}

// Bytes a slot holds after running a group of `cnt` requests of order n (a
// batched group of either type): the batched workspace grows to what the
// group needs, the single-call workspace stays.
size_t held_after(const Slot &sl, int64_t ws_single, int64_t ws_batched, int64_t n, int32_t tile, int32_t dtype,
                  int cnt) {
    int64_t need = 0;
    int32_t t = 0, prec = 0, batched = 0;
    plan_of(n, dtype, tile, &t, &prec, &batched);
    const size_t elem = dtype == AVS_DTYPE_F64 ? 8 : 4;
    const size_t io = (size_t)cnt * (size_t)(n * n + n) * elem + 256;
    if (!batched) {  // one single-matrix call: its workspace grows, the batched one stays
        avs_estimate_bytes(n, t, prec, 0, &need);
        return (size_t)std::max(ws_single, need) + (size_t)ws_batched + std::max(sl.io_bytes, io);
    }
    avs_estimate_bytes(n, t, dtype == AVS_DTYPE_F64 ? AVS_PREC_FP64 : AVS_PREC_FP32, cnt, &need);
    return (size_t)ws_single + (size_t)std::max(ws_batched, need) + std::max(sl.io_bytes, io);
}

void release_slot(avs_server *S, Slot &sl, std::unique_lock<std::mutex> &lk) {
    const size_t was = sl.held;
    lk.unlock();
    avs_trim(sl.h);
    if (sl.io) cudaFree(sl.io);
    sl.io = nullptr;
    sl.io_bytes = 0;
    lk.lock();
    S->held_total -= was;
    sl.held = 0;
    S->cv_work.notify_all();
}

// One batched call for a group of same-order requests of type T (FP32 tiles
// with double-float stages, or FP64 throughout).
template <typename T>
int run_group(Slot &sl, std::vector<Request *> &g, int32_t tile, int32_t prec, bool batched) {
    const int cnt = (int)g.size();
    const int64_t n = g[0]->n;
    const size_t need = (size_t)cnt * (size_t)(n * n + n) * sizeof(T) + 256;
    if (sl.io_bytes < need) {
        if (sl.io) cudaFree(sl.io);
        sl.io = nullptr;
        sl.io_bytes = 0;
        if (cudaMalloc(&sl.io, need) != cudaSuccess) {
            cudaGetLastError();
            return AVS_ERR_OOM;
        }
        sl.io_bytes = need;
    }
    T *dA = reinterpret_cast<T *>(sl.io);
    T *dS = dA + (size_t)cnt * n * n;
    std::vector<int64_t> nn(cnt, n), ld(cnt, n);
    std::vector<int32_t> tt(cnt, tile);
    std::vector<const T *> pa(cnt);
    std::vector<T *> ps(cnt);
    for (int i = 0; i < cnt; ++i) {
        pa[i] = dA + (size_t)i * n * n;
        ps[i] = dS + (size_t)i * n;
        AVS_CUDA_TRY(cudaMemcpy2DAsync(const_cast<T *>(pa[i]), sizeof(T) * n, g[i]->A, sizeof(T) * g[i]->lda,
                                       sizeof(T) * n, n, cudaMemcpyHostToDevice, sl.s));
    }
    avs_opts o{};
    o.stream = sl.s;
    o.precision = prec;
    int rc;
    if (!batched) {  // a request that runs alone (cnt == 1)
        if constexpr (sizeof(T) == 8)
            rc = avs_svdvals_dev_d(sl.h, n, n, n, tile, pa[0], ps[0], &o, nullptr);
        else
            rc = avs_svdvals_dev_s(sl.h, n, n, n, tile, pa[0], ps[0], &o, nullptr);
    } else if constexpr (sizeof(T) == 8) {
        rc = avs_svdvals_batched_dev_d(sl.h, cnt, nn.data(), ld.data(), tt.data(), pa.data(), ps.data(), &o, nullptr);
    } else {
        rc = avs_svdvals_batched_dev_s(sl.h, cnt, nn.data(), ld.data(), tt.data(), pa.data(), ps.data(), &o, nullptr);
    }
    if (rc != AVS_SUCCESS) return rc;
    for (int i = 0; i < cnt; ++i)
        AVS_CUDA_TRY(cudaMemcpyAsync(g[i]->sigma, ps[i], sizeof(T) * n, cudaMemcpyDeviceToHost, sl.s));
    AVS_CUDA_TRY(cudaStreamSynchronize(sl.s));
    return AVS_SUCCESS;
}

void slot_loop(avs_server *S, int k) {
    Slot &sl = S->slots[k];
    cudaSetDevice(S->cfg.device);
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        if (S->queue.empty()) {
            if (S->stop) break;
            if (S->pressure && sl.held > 0) {
                release_slot(S, sl, lk);
                continue;
            }
            S->cv_work.wait(lk);
            continue;
        }
        // the oldest request heads the group
        Request *head = S->queue.front();
        const int32_t tile = head->tile > 0 ? head->tile : rule_tile(head->n);
        int32_t plan_tile = 0, plan_prec = 0, plan_batched = 0;
        plan_of(head->n, head->dtype, head->tile, &plan_tile, &plan_prec, &plan_batched);
        std::vector<Request *> g{head};
        for (size_t q = 1; plan_batched && q < S->queue.size() && (int)g.size() < S->cfg.max_batch; ++q) {
            Request *r = S->queue[q];
            if (r->dtype == head->dtype && r->n == head->n && (r->tile == head->tile)) g.push_back(r);
        }
        int64_t ws_single = 0, ws_batched = 0;
        avs_workspace_bytes(sl.h, &ws_single, &ws_batched);
        auto fits = [&](int cnt) {
            const size_t after = held_after(sl, ws_single, ws_batched, head->n, tile, head->dtype, cnt);
            return S->held_total - sl.held + after <= S->budget;
        };
        while (g.size() > 1 && !fits((int)g.size())) g.resize(std::max<size_t>(1, g.size() / 2));
        if (!fits((int)g.size())) {
            if (sl.held > 0) {  // give back what this slot caches, then retry
                release_slot(S, sl, lk);
                continue;
            }
            bool others_busy = false;
            for (auto &o : S->slots) others_busy |= (&o != &sl) && (o.busy || o.held > 0);
            if (!others_busy) {  // cannot fit even on an empty device budget
                S->queue.pop_front();
                head->status = AVS_ERR_OOM;
                head->done = true;
                head->t_done = Clock::now();
                ++S->failed;
                S->cv_done.notify_all();
                continue;
            }
            S->pressure = true;
            S->cv_work.notify_all();
            S->cv_work.wait(lk);
            continue;
        }
        S->pressure = false;
        // take the group out of the queue
        for (Request *r : g) S->queue.erase(std::find(S->queue.begin(), S->queue.end(), r));
        const size_t reserve = held_after(sl, ws_single, ws_batched, head->n, tile, head->dtype, (int)g.size());
        S->held_total += reserve - sl.held;
        sl.held = reserve;
        S->peak = std::max(S->peak, S->held_total);
        sl.busy = true;
        ++S->batches;
        S->batched_reqs += (int64_t)g.size();
        lk.unlock();

        int32_t t = tile;
        if (head->tile <= 0 && S->cfg.autotune) t = pick_tile(S, sl, head);
        const int rc = head->dtype == AVS_DTYPE_F32 ? run_group<float>(sl, g, t, plan_prec, plan_batched != 0)
                                                    : run_group<double>(sl, g, t, plan_prec, plan_batched != 0);
        int64_t ws_s = 0, ws_b = 0;
        avs_workspace_bytes(sl.h, &ws_s, &ws_b);
        const int64_t ws_after = ws_s + ws_b;
        const Clock::time_point now = Clock::now();

        lk.lock();
        sl.busy = false;
        const size_t actual = (size_t)ws_after + sl.io_bytes;
        S->held_total += actual - sl.held;
        sl.held = actual;
        S->peak = std::max(S->peak, S->held_total);
        for (Request *r : g) {
            r->status = rc;
            r->done = true;
            r->t_done = now;
            if (rc == AVS_SUCCESS) {
                ++S->completed;
                S->lat_ms.push_back(std::chrono::duration<double, std::milli>(now - r->t_submit).count());
            } else {
                ++S->failed;
            }
        }
        S->t_last = now;
        S->cv_done.notify_all();
        S->cv_work.notify_all();
    }
    lk.unlock();
    avs_trim(sl.h);
}

}  // namespace

extern "C" int avs_serve_plan(int64_t n, int32_t dtype, int32_t tile, int32_t *tile_out, int32_t *precision,
                   int32_t *batched) {
    if (n <= 0) return -1;
    if (dtype != AVS_DTYPE_F32 && dtype != AVS_DTYPE_F64) return -2;
    int32_t t = 0, p = 0, b = 0;
    plan_of(n, dtype, tile, &t, &p, &b);
    if (tile_out) *tile_out = t;
    if (precision) *precision = p;
    if (batched) *batched = b;
    return AVS_SUCCESS;
}

extern "C" int avs_serve_create(avs_server **out, const avs_serve_config *cfg) {
    if (!out) return -1;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return AVS_ERR_NO_DEVICE;
    }
    avs_server *S = new (std::nothrow) avs_server();
    if (!S) return AVS_ERR_INTERNAL;
    if (cfg) S->cfg = *cfg;
    if (S->cfg.device < 0 || S->cfg.device >= count) {
        delete S;
        return -2;
    }
    if (S->cfg.workers <= 0) S->cfg.workers = 4;
    if (S->cfg.max_batch <= 0) S->cfg.max_batch = 512;
    cudaSetDevice(S->cfg.device);
    if (S->cfg.hbm_budget_bytes <= 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        S->budget = (size_t)(0.8 * (double)fr);
    } else {
        S->budget = (size_t)S->cfg.hbm_budget_bytes;
    }
    S->slots.resize(S->cfg.workers);
    for (auto &sl : S->slots) {
        int rc = avs_create(&sl.h, S->cfg.device);
        if (rc == AVS_SUCCESS && cudaStreamCreateWithFlags(&sl.s, cudaStreamNonBlocking) != cudaSuccess)
            rc = AVS_ERR_CUDA;
        if (rc != AVS_SUCCESS) {
            for (auto &o : S->slots) {
                if (o.s) cudaStreamDestroy(o.s);
                if (o.h) avs_destroy(o.h);
            }
            delete S;
            return rc;
        }
    }
    for (int k = 0; k < S->cfg.workers; ++k) S->slots[k].th = std::thread(slot_loop, S, k);
    *out = S;
    return AVS_SUCCESS;
}

extern "C" int avs_serve_submit(avs_server *S, int64_t n, int64_t lda, int32_t dtype, int32_t tile, const void *A,
                                void *sigma, int64_t *id) {
    if (!S) return -1;
    if (n <= 0) return -2;
    if (lda < n) return -3;
    if (dtype != AVS_DTYPE_F32 && dtype != AVS_DTYPE_F64) return -4;
    if (tile != 0) {
        if (tile < 16 || (tile & (tile - 1)) || n % tile != 0 || tile > n) return AVS_ERR_NOT_IMPLEMENTED;
        if (tile > 256) return AVS_ERR_UNSUPPORTED;
    } else if (n % 16 != 0) {
        return AVS_ERR_NOT_IMPLEMENTED;  // no power-of-two tile >= 16 divides n
    }
    if (!A) return -6;
    if (!sigma) return -7;
    Request *r = new (std::nothrow) Request();
    if (!r) return AVS_ERR_INTERNAL;
    r->n = n;
    r->lda = lda;
    r->dtype = dtype;
    r->tile = tile;
    r->A = A;
    r->sigma = sigma;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) {
            delete r;
            return AVS_ERR_INTERNAL;
        }
        r->id = S->next_id++;
        if (!S->any_submit) {
            S->any_submit = true;
            S->t_first = r->t_submit;
        }
        S->reqs[r->id] = r;
        S->queue.push_back(r);
        ++S->submitted;
    }
    S->cv_work.notify_one();
    if (id) *id = r->id;
    return AVS_SUCCESS;
}

extern "C" int avs_serve_wait(avs_server *S, int64_t id, double timeout_ms, int32_t *status, double *latency_ms) {
    if (!S) return -1;
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return -2;
    Request *r = it->second;
    auto pred = [&] { return r->done; };
    if (timeout_ms < 0) {
        S->cv_done.wait(lk, pred);
    } else if (!S->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), pred)) {
        return AVS_ERR_TIMEOUT;
    }
    if (status) *status = r->status;
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    const int rc = r->status;
    S->reqs.erase(it);
    delete r;
    return rc;
}

extern "C" int avs_serve_stats_get(avs_server *S, avs_serve_stats *out) {
    if (!S) return -1;
    if (!out) return -2;
    std::lock_guard<std::mutex> lk(S->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = S->submitted;
    out->completed = S->completed;
    out->failed = S->failed;
    out->queued = (int64_t)S->queue.size();
    out->batches = S->batches;
    out->mean_batch = S->batches ? (double)S->batched_reqs / (double)S->batches : 0.0;
    out->peak_bytes = (int64_t)S->peak;
    out->budget_bytes = (int64_t)S->budget;
    if (!S->lat_ms.empty()) {
        std::vector<double> v = S->lat_ms;
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) {
            const size_t i = (size_t)std::min<double>((double)v.size() - 1, std::ceil(p * (double)v.size()) - 1);
            return v[i];
        };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        double sum = 0;
        for (double x : v) sum += x;
        out->mean_ms = sum / (double)v.size();
        out->max_ms = v.back();
        const double span = std::chrono::duration<double>(S->t_last - S->t_first).count();
        out->throughput_rps = span > 0 ? (double)S->completed / span : 0.0;
    }
    return AVS_SUCCESS;
}

extern "C" int avs_serve_destroy(avs_server *S) {
    if (!S) return AVS_SUCCESS;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    for (auto &sl : S->slots)
        if (sl.th.joinable()) sl.th.join();
    for (auto &sl : S->slots) {
        if (sl.io) {
            cudaSetDevice(S->cfg.device);
            cudaFree(sl.io);
        }
        if (sl.s) cudaStreamDestroy(sl.s);
        avs_destroy(sl.h);
    }
    for (auto &kv : S->reqs) delete kv.second;
    delete S;
    return AVS_SUCCESS;
}
