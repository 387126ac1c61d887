// server.cu -- request server: resident matrices under an HBM budget and
// continuous batching of SpMV / SpMM requests into persistent launches.
//
// Threads.  Callers submit requests into a FIFO queue.  One worker thread
// forms batches: it takes queued requests in order while the batch still has
// room (requests, nonzero chunks, staging bytes), loading matrices that are not
// resident (and evicting idle ones, least recently used first), then issues
// the batch on the stream of a free workspace -- one H2D copy of the packed
// descriptors and small vectors, the batched CSR launches (persistent stream
// kernels of every (value type, k) group, one CUDA graph per workspace),
// per-request launches for the other formats, one D2H copy of the packed
// small results -- and hands it to the completion thread.  With `num_inflight` workspaces, the next batch is formed
// and issued while earlier ones run, so requests that arrive while the GPU is
// busy join the next batch as soon as a workspace is free.  The completion
// thread waits for each batch in issue order, copies packed results into the
// callers' buffers and stamps the requests done.
//
// Staging.  Each workspace holds a device input arena (descriptors, then
// packed X of small requests from the front, X of large requests from the
// back) with a pinned mirror of its front part, and a device output arena
// (packed Y of small requests from the front, large ones from the back) with a
// pinned mirror.  X / Y larger than stage_limit_bytes are copied directly
// between the caller's buffer and the arena.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "plan.cuh"
#include "serve.cuh"

namespace sspmv {

sspmv_status check_dims(int32_t vt, int64_t m, int64_t n, int64_t nnz);

namespace {

int64_t now_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

inline size_t up256(size_t v) { return (v + 255) & ~(size_t)255; }

union DeviceMatrix {
    sspmv_csr csr;
    sspmv_coo coo;
    sspmv_ell ell;
    sspmv_s_ell sell;
    sspmv_sell_c_sigma scs;
    sspmv_sell_c_R scr;
    sspmv_dia dia;
    sspmv_bsr bsr;
    sspmv_csr5 csr5;
};

struct Matrix {
    int32_t id = 0, vt = 0, fmt = 0;
    int32_t params[4] = {0, 0, 0, 0};
    int64_t m = 0, n = 0, nnz = 0;
    const int32_t *h_rp = nullptr, *h_ci = nullptr;
    const void *h_val = nullptr;
    bool resident = false;
    DeviceMatrix dev;
    int64_t bytes = 0;
    int64_t refs = 0;        // requests in batches not yet completed (or being formed)
    uint64_t last_use = 0;   // LRU clock
    const int32_t *row_start = nullptr;  // CSR stream plan: first row of each 256-nonzero chunk
    int64_t chunks = 0;
    bool batchable = false;              // the batched stream kernel takes this matrix
    // The plan of a matrix (carry buffers) is shared by its per-request
    // launches: launches on different streams are ordered through this event.
    cudaEvent_t ev = nullptr;
    cudaStream_t ev_stream = nullptr;
};

struct Request {
    sspmv_request r;
    Matrix *mat = nullptr;
    int64_t ticket = 0;
    sspmv_request_info info{};
    sspmv_request_info *out = nullptr;  // replay: written at completion, then the request is freed
    std::atomic<int64_t> *replay_left = nullptr;
    bool done = false;
    // placement in the workspace
    int group = -1;          // batched CSR group, or -1: own launch
    bool stage_x = false, stage_y = false;
    size_t x_bytes = 0, y_bytes = 0;
    size_t x_off = 0, y_off = 0;  // front offset (staged) or back offset (direct)
    void *d_x = nullptr, *d_y = nullptr;
};

// Requests of a batch that are not in the batched CSR launch (other formats,
// other k) run on up to kAuxStreams streams of their workspace at once,
// forked from and joined back into the workspace stream.
constexpr int kAuxStreams = 4;

struct Workspace {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    cudaStream_t aux[kAuxStreams] = {nullptr};
    cudaEvent_t fork = nullptr, join[kAuxStreams] = {nullptr};
    unsigned char *h_in = nullptr, *d_in = nullptr, *h_out = nullptr, *d_out = nullptr;
    void *carry = nullptr;
    cudaGraphExec_t graph = nullptr;  // all groups' batch kernels (ensure_graph)
    bool busy = false;
};

struct Batch {
    int ws = 0;
    int64_t id = 0;
    std::vector<Request *> reqs;
    size_t staged_y_bytes = 0;
    cudaError_t err = cudaSuccess;
    sspmv_status st = SSPMV_OK;
};

// Device bytes a resident matrix holds (arrays; plans counted as chunk
// starts + carries).
int64_t device_bytes(const Matrix &M) {
    const int64_t V = (int64_t)vsize(M.vt), m = M.m, nnz = M.nnz;
    const int64_t plan = 2 * ((m + nnz) / 1024 + 2) * 152;
    const DeviceMatrix &d = M.dev;
    switch (M.fmt) {
    case SSPMV_FMT_CSR: return (m + 1) * 4 + nnz * (4 + V) + plan;
    case SSPMV_FMT_COO: return nnz * (8 + V) + plan;
    case SSPMV_FMT_ELL: return m * (int64_t)d.ell.max_row_width * (4 + V);
    case SSPMV_FMT_SELL: return d.sell.total_slots * (4 + V) + (int64_t)d.sell.chunk_num * 12 + 8 + plan;
    case SSPMV_FMT_SELL_C_SIGMA:
        return d.scs.total_slots * (4 + V) + (int64_t)d.scs.validchunkNum * 12 + 8 + m * 4 + plan;
    case SSPMV_FMT_SELL_C_R: return d.scr.total_slots * (4 + V) + (int64_t)d.scr.validchunkNum * 12 + 8 + m * 4 + plan;
    case SSPMV_FMT_DIA: return (int64_t)d.dia.stride * d.dia.complete_ndiags * V + (int64_t)d.dia.complete_ndiags * 8;
    case SSPMV_FMT_BSR: return d.bsr.nnzb * (d.bsr.blockNNZ * V + 4) + (d.bsr.mb + 1) * 4;
    case SSPMV_FMT_CSR5:
        return (m + 1) * 4 + nnz * (4 + V) + ((int64_t)d.csr5._p + 1) * 8 +
               (int64_t)d.csr5._p * d.csr5.omega * d.csr5.num_packets * 4 + (int64_t)d.csr5.num_offsets * 4 + plan;
    }
    return 0;
}

sspmv_status convert(const sspmv_csr *csr, Matrix &M, sspmv_stream_t s) {
    const int32_t *p = M.params;
    DeviceMatrix &d = M.dev;
    switch (M.fmt) {
    case SSPMV_FMT_COO: return sspmv_csr_to_coo(csr, &d.coo, s);
    case SSPMV_FMT_ELL: return sspmv_csr_to_ell(csr, p[0], &d.ell, s);
    case SSPMV_FMT_SELL: return sspmv_csr_to_sell(csr, p[0], p[1], &d.sell, s);
    case SSPMV_FMT_SELL_C_SIGMA: return sspmv_csr_to_sell_c_sigma(csr, p[0], p[1], p[2], &d.scs, s);
    case SSPMV_FMT_SELL_C_R: return sspmv_csr_to_sell_c_R(csr, p[0], p[1], &d.scr, s);
    case SSPMV_FMT_DIA: return sspmv_csr_to_dia(csr, p[0], p[1], &d.dia, s);
    case SSPMV_FMT_BSR: return sspmv_csr_to_bsr(csr, p[0] > 0 ? p[0] : 4, p[1] > 0 ? p[1] : 4, &d.bsr, s);
    case SSPMV_FMT_CSR5: return sspmv_csr_to_csr5(csr, p[0], p[1], &d.csr5, s);
    }
    return fail(SSPMV_INVALID_ARG, "unknown format %d", M.fmt);
}

sspmv_status spmm(const Matrix &M, double alpha, int32_t k, const void *X, int64_t ldx, double beta, void *Y,
                  int64_t ldy, sspmv_stream_t s) {
    const DeviceMatrix &d = M.dev;
    switch (M.fmt) {
    case SSPMV_FMT_CSR: return sspmv_spmm_csr(alpha, &d.csr, k, X, ldx, beta, Y, ldy, s);
    case SSPMV_FMT_COO: return sspmv_spmm_coo(alpha, &d.coo, k, X, ldx, beta, Y, ldy, s);
    case SSPMV_FMT_ELL: return sspmv_spmm_ell(alpha, &d.ell, k, X, ldx, beta, Y, ldy, s);
    case SSPMV_FMT_SELL: return sspmv_spmm_sell(alpha, &d.sell, k, X, ldx, beta, Y, ldy, s);
    case SSPMV_FMT_SELL_C_SIGMA: return sspmv_spmm_sell_c_sigma(alpha, &d.scs, k, X, ldx, beta, Y, ldy, s);
    case SSPMV_FMT_SELL_C_R: return sspmv_spmm_sell_c_R(alpha, &d.scr, k, X, ldx, beta, Y, ldy, s);
    case SSPMV_FMT_DIA: return sspmv_spmm_dia(alpha, &d.dia, k, X, ldx, beta, Y, ldy, s);
    case SSPMV_FMT_BSR: return sspmv_spmm_bsr(alpha, &d.bsr, k, X, ldx, beta, Y, ldy, s);
    case SSPMV_FMT_CSR5: return sspmv_spmm_csr5(alpha, &d.csr5, k, X, ldx, beta, Y, ldy, s);
    }
    return fail(SSPMV_INVALID_ARG, "unknown format %d", M.fmt);
}

void release(Matrix &M) {
    DeleteWithoutDeviceSync nosync;
    DeviceMatrix &d = M.dev;
    switch (M.fmt) {
    case SSPMV_FMT_CSR: sspmv_delete_csr(&d.csr); break;
    case SSPMV_FMT_COO: sspmv_delete_coo(&d.coo); break;
    case SSPMV_FMT_ELL: sspmv_delete_ell(&d.ell); break;
    case SSPMV_FMT_SELL: sspmv_delete_sell(&d.sell); break;
    case SSPMV_FMT_SELL_C_SIGMA: sspmv_delete_sell_c_sigma(&d.scs); break;
    case SSPMV_FMT_SELL_C_R: sspmv_delete_sell_c_R(&d.scr); break;
    case SSPMV_FMT_DIA: sspmv_delete_dia(&d.dia); break;
    case SSPMV_FMT_BSR: sspmv_delete_bsr(&d.bsr); break;
    case SSPMV_FMT_CSR5: sspmv_delete_csr5(&d.csr5); break;
    }
    if (M.ev) cudaEventDestroy(M.ev);
    M.ev = nullptr;
    M.ev_stream = nullptr;
    M.row_start = nullptr;
    M.batchable = false;
    M.resident = false;
}

}  // namespace

struct Server {
    sspmv_server_config cfg{};
    int device = 0;
    size_t desc_bytes = 0, in_bytes = 0, out_bytes = 0;
    std::vector<Workspace> ws;
    cudaStream_t load_stream = nullptr;
    cudaStream_t capture_stream = nullptr;  // idle stream the batch graphs are captured on

    std::mutex mu;
    std::condition_variable cv_queue, cv_ws, cv_inflight, cv_done;
    std::deque<Request *> queue;
    std::deque<Batch> inflight;
    std::unordered_map<int32_t, std::unique_ptr<Matrix>> matrices;
    std::unordered_map<int64_t, std::unique_ptr<Request>> tickets;
    int64_t next_ticket = 1;
    int64_t next_batch = 0;
    uint64_t lru_clock = 0;
    int64_t resident_bytes = 0, resident_count = 0;
    bool stopping = false, worker_done = false;
    sspmv_server_stats stats{};
    std::thread worker, completer;

    sspmv_status init();
    void shutdown();
    void worker_loop();
    void completion_loop();
    sspmv_status load(Matrix &M);
    sspmv_status make_room(int64_t need);
    sspmv_status ensure_resident(Matrix &M, bool *wait);
    void issue(Batch &b);
    sspmv_status ensure_graph(Workspace &w);
    sspmv_status launch_groups(Workspace &w, uint32_t mask);
    void finish(Request *r, int32_t status, int64_t t);
};

// ------------------------------------------------------------- lifecycle --
sspmv_status Server::init() {
    SSPMV_CUDA_TRY(cudaGetDevice(&device));
    const int nin = cfg.num_inflight;
    desc_bytes = up256(sizeof(BatchHeader) + (size_t)cfg.max_batch_requests * sizeof(BatchItem));
    in_bytes = desc_bytes + (size_t)cfg.arena_bytes;
    out_bytes = (size_t)cfg.arena_bytes;
    ws.resize(nin);
    for (auto &w : ws) {
        SSPMV_CUDA_TRY(cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking));
        SSPMV_CUDA_TRY(cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming));
        SSPMV_CUDA_TRY(cudaEventCreateWithFlags(&w.fork, cudaEventDisableTiming));
        for (int a = 0; a < kAuxStreams; a++) {
            SSPMV_CUDA_TRY(cudaStreamCreateWithFlags(&w.aux[a], cudaStreamNonBlocking));
            SSPMV_CUDA_TRY(cudaEventCreateWithFlags(&w.join[a], cudaEventDisableTiming));
        }
        SSPMV_CUDA_TRY(cudaMalloc(&w.d_in, in_bytes));
        SSPMV_CUDA_TRY(cudaMalloc(&w.d_out, out_bytes));
        SSPMV_CUDA_TRY(cudaMallocHost(&w.h_in, in_bytes));
        SSPMV_CUDA_TRY(cudaMallocHost(&w.h_out, out_bytes));
        SSPMV_CUDA_TRY(cudaMalloc(&w.carry, (size_t)cfg.max_batch_tiles * kBatchSlotBytes));
    }
    SSPMV_CUDA_TRY(cudaStreamCreateWithFlags(&load_stream, cudaStreamNonBlocking));
    SSPMV_CUDA_TRY(cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking));
    for (int g = 0; g < kBatchGroups; g++) csr_batch_grid(g);  // kernel attributes, before any capture
    if (cfg.use_graphs && cfg.mode == SSPMV_SERVE_BATCHED)
        for (auto &w : ws) SSPMV_TRY(ensure_graph(w));
    worker = std::thread([this] { worker_loop(); });
    completer = std::thread([this] { completion_loop(); });
    return SSPMV_OK;
}

void Server::shutdown() {
    {
        std::lock_guard<std::mutex> g(mu);
        stopping = true;
    }
    cv_queue.notify_all();
    cv_ws.notify_all();
    if (worker.joinable()) worker.join();
    {
        std::lock_guard<std::mutex> g(mu);
        worker_done = true;
    }
    cv_inflight.notify_all();
    if (completer.joinable()) completer.join();
    cudaSetDevice(device);
    for (auto &kv : matrices)
        if (kv.second->resident) release(*kv.second);
    for (auto &w : ws) {
        if (w.stream) cudaStreamSynchronize(w.stream);
        if (w.graph) cudaGraphExecDestroy(w.graph);
        cudaFree(w.d_in);
        cudaFree(w.d_out);
        cudaFreeHost(w.h_in);
        cudaFreeHost(w.h_out);
        cudaFree(w.carry);
        if (w.done) cudaEventDestroy(w.done);
        for (int a = 0; a < kAuxStreams; a++) {
            if (w.aux[a]) {
                cudaStreamSynchronize(w.aux[a]);
                cudaStreamDestroy(w.aux[a]);
            }
            if (w.join[a]) cudaEventDestroy(w.join[a]);
        }
        if (w.fork) cudaEventDestroy(w.fork);
        if (w.stream) cudaStreamDestroy(w.stream);
    }
    if (load_stream) {
        cudaStreamSynchronize(load_stream);
        cudaStreamDestroy(load_stream);
    }
    if (capture_stream) cudaStreamDestroy(capture_stream);
}

// -------------------------------------------------------------- residency --
// Frees idle resident matrices, least recently used first, until `need`
// more bytes fit in the budget.  Called by the worker thread with mu held.
sspmv_status Server::make_room(int64_t need) {
    while (resident_bytes + need > cfg.hbm_budget_bytes) {
        Matrix *victim = nullptr;
        for (auto &kv : matrices) {
            Matrix *M = kv.second.get();
            if (M->resident && M->refs == 0 && (!victim || M->last_use < victim->last_use)) victim = M;
        }
        if (!victim) return SSPMV_BUDGET_EXCEEDED;
        resident_bytes -= victim->bytes;
        resident_count--;
        stats.evictions++;
        release(*victim);
    }
    return SSPMV_OK;
}

sspmv_status Server::load(Matrix &M) {
    sspmv_stream_t s = reinterpret_cast<sspmv_stream_t>(load_stream);
    sspmv_csr csr;
    SSPMV_TRY(sspmv_csr_create(&csr, M.vt, M.m, M.n, M.nnz, M.h_rp, M.h_ci, M.h_val, 1, s));
    sspmv_status st = SSPMV_OK;
    if (M.fmt == SSPMV_FMT_CSR) {
        M.dev.csr = csr;
        int32_t gap = 0;
        st = csr_stream_plan(&M.dev.csr, &M.row_start, &M.chunks, &gap, s);
        M.batchable = st == SSPMV_OK && csr_stream_takes(M.nnz, gap);
    } else {
        st = convert(&csr, M, s);
        cudaStreamSynchronize(load_stream);
        DeleteWithoutDeviceSync nosync;
        sspmv_delete_csr(&csr);
        if (st != SSPMV_OK) return st;
    }
    if (st == SSPMV_OK) {
        cudaError_t e = cudaEventCreateWithFlags(&M.ev, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaStreamSynchronize(load_stream);
        if (e != cudaSuccess) st = fail(SSPMV_CUDA_ERROR, "server load: %s", cudaGetErrorString(e));
    }
    if (st != SSPMV_OK) {
        M.resident = true;
        release(M);
        return st;
    }
    M.ev_stream = nullptr;
    M.resident = true;
    M.bytes = device_bytes(M);
    return SSPMV_OK;
}

// Makes M resident.  *wait is set when the budget is held by matrices of
// batches still in flight (the caller retries after they complete).
sspmv_status Server::ensure_resident(Matrix &M, bool *wait) {
    *wait = false;
    if (M.resident) return SSPMV_OK;
    const int64_t V = (int64_t)vsize(M.vt);
    const int64_t csr_bytes = (M.m + 1) * 4 + M.nnz * (4 + V);
    // transient peak of a load: the CSR plus a converted copy (padding allowed for)
    const int64_t need = M.fmt == SSPMV_FMT_CSR ? csr_bytes + 2 * ((M.m + M.nnz) / 1024 + 2) * 152 : 3 * csr_bytes;
    if (need > cfg.hbm_budget_bytes) return fail(SSPMV_BUDGET_EXCEEDED, "matrix %d alone exceeds the HBM budget", M.id);
    {
        std::lock_guard<std::mutex> g(mu);
        if (make_room(need) != SSPMV_OK) {
            *wait = true;
            return SSPMV_BUDGET_EXCEEDED;
        }
    }
    SSPMV_TRY(load(M));
    std::lock_guard<std::mutex> g(mu);
    resident_bytes += M.bytes;
    resident_count++;
    stats.loads++;
    return SSPMV_OK;
}

// ----------------------------------------------------------------- worker --
void Server::finish(Request *r, int32_t status, int64_t t) {
    // mu held
    r->info.status = status;
    r->info.done_ns = t;
    r->done = true;
    if (status == SSPMV_OK) stats.requests_done++;
    else stats.requests_failed++;
    if (r->out) {
        *r->out = r->info;
        std::atomic<int64_t> *left = r->replay_left;
        tickets.erase(r->ticket);
        left->fetch_sub(1);
    }
}

void Server::worker_loop() {
    cudaSetDevice(device);
    int next_ws = 0;
    std::vector<Request *> held;  // requests taken from the queue for the batch being formed
    for (;;) {
        Workspace &w = ws[next_ws];
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_ws.wait(lk, [&] { return !w.busy; });
            cv_queue.wait(lk, [&] { return !queue.empty() || stopping; });
            if (queue.empty() && stopping) break;
        }
        Batch b;
        b.ws = next_ws;
        const size_t in_cap = in_bytes - desc_bytes;
        size_t x_front = 0, x_back = 0, y_front = 0, y_back = 0;
        int64_t tiles = 0;
        const bool per_request = cfg.mode == SSPMV_SERVE_PER_REQUEST;
        const size_t max_reqs = per_request ? 1 : (size_t)cfg.max_batch_requests;
        for (;;) {
            Request *r = nullptr;
            {
                std::lock_guard<std::mutex> g(mu);
                if (queue.empty() || b.reqs.size() >= max_reqs) break;
                r = queue.front();
                queue.pop_front();
            }
            Matrix &M = *r->mat;
            bool wait = false;
            sspmv_status st = ensure_resident(M, &wait);
            if (wait) {
                std::unique_lock<std::mutex> lk(mu);
                if (!b.reqs.empty() || !inflight.empty() || std::any_of(ws.begin(), ws.end(), [](const Workspace &q) { return q.busy; })) {
                    queue.push_front(r);  // retry once running batches release their matrices
                    if (b.reqs.empty()) cv_ws.wait_for(lk, std::chrono::milliseconds(1));
                    break;
                }
                finish(r, SSPMV_BUDGET_EXCEEDED, now_ns());
                cv_done.notify_all();
                continue;
            }
            if (st != SSPMV_OK) {
                std::lock_guard<std::mutex> g(mu);
                finish(r, st, now_ns());
                cv_done.notify_all();
                continue;
            }
            const size_t V = vsize(M.vt);
            const int32_t k = r->r.k;
            const bool on_device = (r->r.flags & SSPMV_REQ_DEVICE_BUFFERS) != 0;
            r->x_bytes = M.n > 0 && !on_device ? (size_t)((M.n - 1) * r->r.ldx + k) * V : 0;
            r->y_bytes = M.m > 0 && !on_device ? (size_t)((M.m - 1) * r->r.ldy + k) * V : 0;
            r->stage_x = !on_device && (int64_t)r->x_bytes <= cfg.stage_limit_bytes;
            r->stage_y = !on_device && (int64_t)r->y_bytes <= cfg.stage_limit_bytes;
            const bool batched = !per_request && M.fmt == SSPMV_FMT_CSR && M.batchable &&
                                 (k == 1 || k == 2 || k == 4 || k == 8);
            const int64_t t = batched ? M.chunks : 0;
            const size_t xa = up256(r->x_bytes), ya = up256(r->y_bytes);
            const bool fits = x_front + x_back + xa <= in_cap && y_front + y_back + ya <= out_bytes &&
                              tiles + t <= cfg.max_batch_tiles;
            if (!fits) {
                std::lock_guard<std::mutex> g(mu);
                if (b.reqs.empty()) {
                    set_error("request on matrix %d needs more staging or nonzero chunks than one batch holds", M.id);
                    finish(r, SSPMV_INVALID_ARG, now_ns());
                    cv_done.notify_all();
                    continue;
                }
                queue.push_front(r);
                break;
            }
            if (r->stage_x) { r->x_off = x_front; x_front += xa; }
            else { x_back += xa; r->x_off = x_back; }
            if (r->stage_y) { r->y_off = y_front; y_front += ya; }
            else { y_back += ya; r->y_off = y_back; }
            r->group = batched ? batch_group(M.vt, k) : -1;
            tiles += t;
            {
                std::lock_guard<std::mutex> g(mu);
                M.refs++;
                M.last_use = ++lru_clock;
            }
            b.reqs.push_back(r);
        }
        if (b.reqs.empty()) continue;
        b.staged_y_bytes = y_front;
        {
            std::lock_guard<std::mutex> g(mu);
            b.id = next_batch++;
            w.busy = true;
        }
        issue(b);
        {
            std::lock_guard<std::mutex> g(mu);
            inflight.push_back(std::move(b));
        }
        cv_inflight.notify_all();
        next_ws = (next_ws + 1) % (int)ws.size();
    }
}

// The workspace's batch graph: every group's stream kernel and fix-up as
// parallel branches (a group without requests in a batch exits at once), so
// one graph serves every batch and is captured before the first one.
// Captured on an idle stream (kernel arguments name only this workspace's
// buffers); streams and events are made beforehand.
sspmv_status Server::ensure_graph(Workspace &w) {
    if (w.graph) return SSPMV_OK;
    BatchHeader *d_hdr = reinterpret_cast<BatchHeader *>(w.d_in);
    BatchItem *d_items = reinterpret_cast<BatchItem *>(w.d_in + sizeof(BatchHeader));
    std::vector<cudaStream_t> side(kBatchGroups - 1, nullptr);
    std::vector<cudaEvent_t> evs(kBatchGroups, nullptr);  // [0]: fork, [1..]: joins
    cudaError_t e = cudaSuccess;
    for (auto &bs : side)
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking);
    for (auto &ev : evs)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    sspmv_status st = SSPMV_OK;
    cudaStream_t cs = capture_stream;
    if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaEventRecord(evs[0], cs);
        for (int g = 0; g < kBatchGroups; g++) {
            cudaStream_t bs = g == 0 ? cs : side[g - 1];
            if (g > 0) cudaStreamWaitEvent(bs, evs[0], 0);
            if (st == SSPMV_OK)
                st = launch_csr_batch_group(g, d_hdr, d_items, w.carry, cfg.max_batch_tiles,
                                            reinterpret_cast<sspmv_stream_t>(bs));
            if (g > 0) {
                cudaEventRecord(evs[g], bs);
                cudaStreamWaitEvent(cs, evs[g], 0);
            }
        }
        e = cudaStreamEndCapture(cs, &graph);
        if (e == cudaSuccess && st == SSPMV_OK) e = cudaGraphInstantiate(&exec, graph, 0);
    }
    if (graph) cudaGraphDestroy(graph);
    for (auto ev : evs)
        if (ev) cudaEventDestroy(ev);
    for (auto bs : side)
        if (bs) cudaStreamDestroy(bs);
    SSPMV_TRY(st);
    if (e != cudaSuccess) return fail(SSPMV_CUDA_ERROR, "batch graph capture: %s", cudaGetErrorString(e));
    w.graph = exec;
    return SSPMV_OK;
}

sspmv_status Server::launch_groups(Workspace &w, uint32_t mask) {
    if (!cfg.use_graphs) {
        BatchHeader *d_hdr = reinterpret_cast<BatchHeader *>(w.d_in);
        BatchItem *d_items = reinterpret_cast<BatchItem *>(w.d_in + sizeof(BatchHeader));
        sspmv_stream_t s = reinterpret_cast<sspmv_stream_t>(w.stream);
        for (int g = 0; g < kBatchGroups; g++)
            if (mask & (1u << g)) SSPMV_TRY(launch_csr_batch_group(g, d_hdr, d_items, w.carry, cfg.max_batch_tiles, s));
        return SSPMV_OK;
    }
    SSPMV_TRY(ensure_graph(w));
    SSPMV_CUDA_TRY(cudaGraphLaunch(w.graph, w.stream));
    return SSPMV_OK;
}

// Issues batch b on its workspace (worker thread).
void Server::issue(Batch &b) {
    Workspace &w = ws[b.ws];
    const int64_t t_launch = now_ns();
    // --- placement: device addresses; descriptors grouped by batch group ---
    BatchHeader hdr;
    std::memset(&hdr, 0, sizeof(hdr));
    int counts[kBatchGroups] = {0};
    for (Request *r : b.reqs)
        if (r->group >= 0) counts[r->group]++;
    int begin = 0;
    for (int g = 0; g < kBatchGroups; g++) {
        hdr.item_begin[g] = begin;
        begin += counts[g];
    }
    const size_t x_base = desc_bytes;
    size_t staged_x_end = x_base;
    for (Request *r : b.reqs) {
        if (r->r.flags & SSPMV_REQ_DEVICE_BUFFERS) {
            r->d_x = const_cast<void *>(r->r.x);
            r->d_y = r->r.y;
            continue;
        }
        r->d_x = r->stage_x ? (void *)(w.d_in + x_base + r->x_off) : (void *)(w.d_in + in_bytes - r->x_off);
        r->d_y = r->stage_y ? (void *)(w.d_out + r->y_off) : (void *)(w.d_out + out_bytes - r->y_off);
        if (r->stage_x) staged_x_end = std::max(staged_x_end, x_base + r->x_off + r->x_bytes);
    }
    BatchItem *items = reinterpret_cast<BatchItem *>(w.h_in + sizeof(BatchHeader));
    int fill[kBatchGroups] = {0};
    int64_t group_tiles[kBatchGroups] = {0};
    uint32_t mask = 0;
    for (Request *r : b.reqs) {
        if (r->group < 0) continue;
        const int g = r->group;
        const Matrix &M = *r->mat;
        BatchItem &it = items[hdr.item_begin[g] + fill[g]++];
        it.row_offset = M.dev.csr.row_offset;
        it.col_index = M.dev.csr.col_index;
        it.values = M.dev.csr.values;
        it.row_start = M.row_start;
        it.x = r->d_x;
        it.y = r->d_y;
        it.ldx = r->r.ldx;
        it.ldy = r->r.ldy;
        it.alpha = r->r.alpha;
        it.beta = r->r.beta;
        it.chunk_begin = group_tiles[g];
        it.nnz = M.nnz;
        it.m = (int32_t)M.m;
        it.num_chunks = (int32_t)M.chunks;
        it.vec = ((reinterpret_cast<uintptr_t>(M.dev.csr.col_index) | reinterpret_cast<uintptr_t>(M.dev.csr.values)) &
                  15) == 0;
        it.xvec = xrow_vec(r->d_x, r->r.ldx, g >= 4 ? 8 : 4, r->r.k);
        group_tiles[g] += M.chunks;
        mask |= 1u << g;
    }
    int64_t carry = 0;
    for (int g = 0; g < kBatchGroups; g++) {
        hdr.n_items[g] = counts[g];
        hdr.total_chunks[g] = group_tiles[g];
        hdr.carry_base[g] = carry;
        carry += group_tiles[g];
    }
    std::memcpy(w.h_in, &hdr, sizeof(hdr));
    // --- host staging of small X (and of Y when beta != 0) ---
    bool y_in_staged = false;
    for (Request *r : b.reqs) {
        if (r->stage_x && r->x_bytes) std::memcpy(w.h_in + x_base + r->x_off, r->r.x, r->x_bytes);
        if (r->r.beta != 0.0 && r->stage_y && r->y_bytes) {
            std::memcpy(w.h_out + r->y_off, r->r.y, r->y_bytes);
            y_in_staged = true;
        }
    }
    cudaError_t e = cudaMemcpyAsync(w.d_in, w.h_in, staged_x_end, cudaMemcpyHostToDevice, w.stream);
    if (e == cudaSuccess && y_in_staged)
        e = cudaMemcpyAsync(w.d_out, w.h_out, b.staged_y_bytes, cudaMemcpyHostToDevice, w.stream);
    for (Request *r : b.reqs) {
        if (e != cudaSuccess) break;
        if (!r->stage_x && r->x_bytes) e = cudaMemcpyAsync(r->d_x, r->r.x, r->x_bytes, cudaMemcpyHostToDevice, w.stream);
        if (e == cudaSuccess && r->r.beta != 0.0 && !r->stage_y && r->y_bytes)
            e = cudaMemcpyAsync(r->d_y, r->r.y, r->y_bytes, cudaMemcpyHostToDevice, w.stream);
    }
    sspmv_status st = SSPMV_OK;
    if (e == cudaSuccess && mask) st = launch_groups(w, mask);
    // Own launches: with more than one, spread over the auxiliary streams
    // (forked after the copies in), so independent requests overlap on the
    // GPU; launches on one matrix stay ordered through its event.
    int own = 0;
    for (Request *r : b.reqs)
        if (r->group < 0 && r->mat->m > 0) own++;
    bool used[kAuxStreams] = {false};
    if (own > 1 && e == cudaSuccess) e = cudaEventRecord(w.fork, w.stream);
    int j = 0;
    for (Request *r : b.reqs) {
        if (e != cudaSuccess || st != SSPMV_OK) break;
        if (r->group >= 0) continue;
        Matrix &M = *r->mat;
        if (M.m == 0) continue;
        cudaStream_t cs = w.stream;
        if (own > 1) {
            const int a = j++ % kAuxStreams;
            cs = w.aux[a];
            if (!used[a]) {
                cudaStreamWaitEvent(cs, w.fork, 0);
                used[a] = true;
            }
        }
        if (M.ev_stream && M.ev_stream != cs) cudaStreamWaitEvent(cs, M.ev, 0);
        st = spmm(M, r->r.alpha, r->r.k, r->d_x, r->r.ldx, r->r.beta, r->d_y, r->r.ldy,
                  reinterpret_cast<sspmv_stream_t>(cs));
        cudaEventRecord(M.ev, cs);
        M.ev_stream = cs;
    }
    for (int a = 0; a < kAuxStreams; a++)
        if (used[a]) {
            cudaEventRecord(w.join[a], w.aux[a]);
            cudaStreamWaitEvent(w.stream, w.join[a], 0);
        }
    if (e == cudaSuccess && st == SSPMV_OK && b.staged_y_bytes)
        e = cudaMemcpyAsync(w.h_out, w.d_out, b.staged_y_bytes, cudaMemcpyDeviceToHost, w.stream);
    for (Request *r : b.reqs) {
        if (e != cudaSuccess || st != SSPMV_OK) break;
        if (!r->stage_y && r->y_bytes) e = cudaMemcpyAsync(r->r.y, r->d_y, r->y_bytes, cudaMemcpyDeviceToHost, w.stream);
    }
    cudaError_t e2 = cudaEventRecord(w.done, w.stream);
    if (e == cudaSuccess) e = e2;
    b.err = e;
    b.st = st;
    if (e != cudaSuccess) set_error("server batch: %s", cudaGetErrorString(e));
    for (Request *r : b.reqs) {
        r->info.launch_ns = t_launch;
        r->info.batch_id = b.id;
        r->info.batch_size = (int32_t)b.reqs.size();
    }
    std::lock_guard<std::mutex> g(mu);
    stats.batches++;
    if (mask) {
        stats.batched_requests += begin;
        stats.graph_launches += cfg.use_graphs ? 1 : 0;
        for (int q = 0; q < kBatchGroups; q++) stats.batched_tiles += group_tiles[q];
    }
}

// ------------------------------------------------------------- completion --
void Server::completion_loop() {
    cudaSetDevice(device);
    for (;;) {
        Batch b;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_inflight.wait(lk, [&] { return !inflight.empty() || worker_done; });
            if (inflight.empty()) break;
            b = std::move(inflight.front());
            inflight.pop_front();
        }
        Workspace &w = ws[b.ws];
        cudaError_t e = b.err;
        if (e == cudaSuccess) {
            while ((e = cudaEventQuery(w.done)) == cudaErrorNotReady) std::this_thread::yield();
        }
        sspmv_status st = b.st;
        if (st == SSPMV_OK && e != cudaSuccess) st = SSPMV_CUDA_ERROR;
        if (st == SSPMV_OK)
            for (Request *r : b.reqs)
                if (r->stage_y && r->y_bytes) std::memcpy(r->r.y, w.h_out + r->y_off, r->y_bytes);
        const int64_t t = now_ns();
        {
            std::lock_guard<std::mutex> g(mu);
            for (Request *r : b.reqs) {
                r->mat->refs--;
                finish(r, st, t);
            }
            w.busy = false;
        }
        cv_ws.notify_all();
        cv_done.notify_all();
    }
}

}  // namespace sspmv

using namespace sspmv;

struct sspmv_server {
    Server s;
};

extern "C" sspmv_status sspmv_server_create(const sspmv_server_config *cfg, sspmv_server **out) {
    if (!out) return fail(SSPMV_INVALID_ARG, "null output");
    *out = nullptr;
    sspmv_server_config c{};
    if (cfg) c = *cfg;
    if (c.mode != SSPMV_SERVE_BATCHED && c.mode != SSPMV_SERVE_PER_REQUEST) return fail(SSPMV_INVALID_ARG, "bad mode");
    if (c.max_batch_requests <= 0) c.max_batch_requests = 1024;
    if (c.max_batch_tiles <= 0) c.max_batch_tiles = 1 << 20;
    if (c.arena_bytes <= 0) c.arena_bytes = 512ll << 20;
    if (c.stage_limit_bytes <= 0) c.stage_limit_bytes = 1 << 20;
    if (c.hbm_budget_bytes <= 0) c.hbm_budget_bytes = 120000000000ll;
    if (c.num_inflight <= 0) c.num_inflight = 2;
    if (c.num_inflight > 16) return fail(SSPMV_INVALID_ARG, "num_inflight must be <= 16");
    c.arena_bytes = (int64_t)up256((size_t)c.arena_bytes);
    auto *srv = new (std::nothrow) sspmv_server();
    if (!srv) return fail(SSPMV_OUT_OF_MEMORY, "server allocation failed");
    srv->s.cfg = c;
    sspmv_status st = srv->s.init();
    if (st != SSPMV_OK) {
        srv->s.shutdown();
        delete srv;
        return st;
    }
    *out = srv;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_server_destroy(sspmv_server *srv) {
    if (!srv) return SSPMV_OK;
    srv->s.shutdown();
    delete srv;
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_server_add_matrix(sspmv_server *srv, int32_t id, int32_t value_type, int64_t num_rows,
                                                int64_t num_cols, int64_t num_nnzs, const int32_t *row_offset,
                                                const int32_t *col_index, const void *values, int32_t format,
                                                const int32_t *params) {
    if (!srv) return fail(SSPMV_INVALID_ARG, "null server");
    SSPMV_TRY(check_dims(value_type, num_rows, num_cols, num_nnzs));
    if (format < SSPMV_FMT_CSR || format > SSPMV_FMT_CSR5) return fail(SSPMV_INVALID_ARG, "unknown format %d", format);
    if (!row_offset || (num_nnzs > 0 && (!col_index || !values))) return fail(SSPMV_INVALID_ARG, "null array");
    auto M = std::make_unique<Matrix>();
    M->id = id;
    M->vt = value_type;
    M->fmt = format;
    if (params)
        for (int i = 0; i < 4; i++) M->params[i] = params[i];
    M->m = num_rows;
    M->n = num_cols;
    M->nnz = num_nnzs;
    M->h_rp = row_offset;
    M->h_ci = col_index;
    M->h_val = values;
    Server &s = srv->s;
    std::lock_guard<std::mutex> g(s.mu);
    if (s.matrices.count(id)) return fail(SSPMV_INVALID_ARG, "matrix id %d already registered", id);
    s.matrices.emplace(id, std::move(M));
    return SSPMV_OK;
}

extern "C" sspmv_status sspmv_server_preload(sspmv_server *srv, int32_t id) {
    if (!srv) return fail(SSPMV_INVALID_ARG, "null server");
    Server &s = srv->s;
    Matrix *M = nullptr;
    {
        std::lock_guard<std::mutex> g(s.mu);
        auto it = s.matrices.find(id);
        if (it == s.matrices.end()) return fail(SSPMV_INVALID_ARG, "matrix id %d not registered", id);
        M = it->second.get();
        if (M->resident) return SSPMV_OK;
        if (!s.queue.empty() || !s.inflight.empty())
            return fail(SSPMV_INVALID_ARG, "preload only while the server is idle");
        M->refs++;  // keeps the worker's eviction away while loading here
    }
    SSPMV_CUDA_TRY(cudaSetDevice(s.device));
    bool wait = false;
    sspmv_status st = s.ensure_resident(*M, &wait);
    std::lock_guard<std::mutex> g(s.mu);
    M->refs--;
    M->last_use = ++s.lru_clock;
    return st;
}

namespace {
sspmv_status enqueue(Server &s, const sspmv_request *req, int64_t arrival, sspmv_request_info *out,
                     std::atomic<int64_t> *left, int64_t *ticket) {
    if (!req) return fail(SSPMV_INVALID_ARG, "null request");
    std::unique_lock<std::mutex> lk(s.mu);
    auto it = s.matrices.find(req->matrix_id);
    if (it == s.matrices.end()) return fail(SSPMV_INVALID_ARG, "matrix id %d not registered", req->matrix_id);
    Matrix *M = it->second.get();
    if (req->k < 1 || req->ldx < req->k || req->ldy < req->k)
        return fail(SSPMV_INVALID_ARG, "k must be >= 1 and ldx, ldy >= k");
    if ((M->n > 0 && !req->x) || (M->m > 0 && !req->y)) return fail(SSPMV_INVALID_ARG, "null x or y");
    if (s.stopping) return fail(SSPMV_INVALID_ARG, "server is shutting down");
    auto r = std::make_unique<Request>();
    r->r = *req;
    r->mat = M;
    r->ticket = s.next_ticket++;
    r->info.arrival_ns = arrival;
    r->info.status = -1;
    r->out = out;
    r->replay_left = left;
    if (ticket) *ticket = r->ticket;
    s.queue.push_back(r.get());
    s.tickets.emplace(r->ticket, std::move(r));
    lk.unlock();
    s.cv_queue.notify_one();
    return SSPMV_OK;
}
}  // namespace

extern "C" sspmv_status sspmv_server_submit(sspmv_server *srv, const sspmv_request *req, int64_t *ticket) {
    if (!srv || !ticket) return fail(SSPMV_INVALID_ARG, "null server or ticket");
    return enqueue(srv->s, req, now_ns(), nullptr, nullptr, ticket);
}

extern "C" sspmv_status sspmv_server_wait(sspmv_server *srv, int64_t ticket, double timeout_s,
                                          sspmv_request_info *info) {
    if (!srv) return fail(SSPMV_INVALID_ARG, "null server");
    Server &s = srv->s;
    std::unique_lock<std::mutex> lk(s.mu);
    auto it = s.tickets.find(ticket);
    if (it == s.tickets.end() || it->second->out) return fail(SSPMV_INVALID_ARG, "unknown ticket %lld", (long long)ticket);
    Request *r = it->second.get();
    auto ready = [&] { return r->done; };
    if (timeout_s < 0) s.cv_done.wait(lk, ready);
    else if (!s.cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready))
        return fail(SSPMV_DEVICE_TIMEOUT, "request %lld not completed within %.3f s", (long long)ticket, timeout_s);
    if (info) *info = r->info;
    const sspmv_status st = (sspmv_status)r->info.status;
    s.tickets.erase(it);
    return st;
}

extern "C" sspmv_status sspmv_server_replay(sspmv_server *srv, int64_t n, const sspmv_request *reqs,
                                            const int64_t *arrival_ns, sspmv_request_info *infos) {
    if (!srv || n < 0 || (n > 0 && (!reqs || !arrival_ns || !infos))) return fail(SSPMV_INVALID_ARG, "bad replay arguments");
    Server &s = srv->s;
    std::atomic<int64_t> left{n};
    const int64_t t0 = now_ns() + 200000;  // start 0.2 ms from now
    sspmv_status first_err = SSPMV_OK;
    for (int64_t i = 0; i < n; i++) {
        const int64_t target = t0 + arrival_ns[i];
        for (;;) {
            const int64_t d = target - now_ns();
            if (d <= 0) break;
            if (d > 200000) std::this_thread::sleep_for(std::chrono::nanoseconds(d - 100000));
        }
        infos[i].status = -1;
        sspmv_status st = enqueue(s, &reqs[i], target, &infos[i], &left, nullptr);
        if (st != SSPMV_OK) {
            infos[i].status = st;
            if (first_err == SSPMV_OK) first_err = st;
            left.fetch_sub(1);
        }
    }
    std::unique_lock<std::mutex> lk(s.mu);
    s.cv_done.wait(lk, [&] { return left.load() == 0; });
    return first_err;
}

extern "C" sspmv_status sspmv_server_get_stats(const sspmv_server *srv, sspmv_server_stats *stats) {
    if (!srv || !stats) return fail(SSPMV_INVALID_ARG, "null argument");
    Server &s = const_cast<Server &>(srv->s);
    std::lock_guard<std::mutex> g(s.mu);
    *stats = s.stats;
    stats->resident_matrices = s.resident_count;
    stats->resident_bytes = s.resident_bytes;
    return SSPMV_OK;
}
