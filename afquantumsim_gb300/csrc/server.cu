// Serving runtime: independent requests (circuit from |0...0>, then seeded
// measure-all shots) admitted by arrival time and HBM onto concurrent lanes.
//
// The reference runs one circuit per QSimulator (QSimulator::simulate,
// src/quantum.cpp:277; peek_measure_all, src/quantum.cpp:343-358).  Here one
// worker thread owns the device side:
//   * a slab of HBM cut into power-of-two register blocks by a buddy
//     allocator (a register of n qubits takes 2^n amplitudes, so blocks fit
//     exactly and the slab never fragments below the largest register);
//   * lanes, each an engine context with its own stream, reserved scratch and
//     pinned staging, so a running request neither allocates nor blocks;
//   * completion by polling one event per lane.
// Submitting callers do the host work (validation, lowering, fusion and tile
// planning) on their own thread, so the worker only copies op tables and
// enqueues kernels.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <set>
#include <thread>

#include "aqsg_internal.h"

namespace aqsg {

// Power-of-two blocks inside `tops` top blocks of 2^top_order bytes each.
class Buddy {
   public:
    void init(int top_order, uint64_t tops, int min_order) {
        top_ = top_order;
        min_ = min_order;
        free_.assign(top_ - min_ + 1, {});
        for (uint64_t t = 0; t < tops; ++t) free_[top_ - min_].insert(t << top_);
    }
    int order_for(uint64_t bytes) const {
        int o = min_;
        while ((1ull << o) < bytes) ++o;
        return o;
    }
    bool alloc(int order, uint64_t* off) {
        int k = order;
        while (k <= top_ && free_[k - min_].empty()) ++k;
        if (k > top_) return false;
        auto it = free_[k - min_].begin();
        const uint64_t o = *it;
        free_[k - min_].erase(it);
        while (k > order) {
            --k;
            free_[k - min_].insert(o + (1ull << k));
        }
        *off = o;
        return true;
    }
    void release(uint64_t off, int order) {
        int k = order;
        while (k < top_) {
            const uint64_t buddy = off ^ (1ull << k);
            auto& fl = free_[k - min_];
            auto it = fl.find(buddy);
            if (it == fl.end()) break;
            fl.erase(it);
            off = std::min(off, buddy);
            ++k;
        }
        free_[k - min_].insert(off);
    }

   private:
    int top_ = 0, min_ = 0;
    std::vector<std::set<uint64_t>> free_;
};

struct Request {
    uint64_t ticket = 0;
    int n = 0;
    uint32_t shots = 0;
    uint64_t seed = 0;
    double arrival = 0;
    uint64_t* outcomes = nullptr;
    TilePlan plan;
    size_t table_bytes = 0;  // plan.table padded + plan.pool
    int fused_ops = 0;
    int passed_over = 0;
    double admit = 0;
    uint64_t off = 0;
    int order = 0;
};

constexpr size_t kLaneTableBytes = 16u << 20;
constexpr int kMaxPassOver = 64;

struct Lane {
    aqsg_ctx ctx = nullptr;
    cudaEvent_t done = nullptr;
    unsigned char* pinned_table = nullptr;
    uint64_t* pinned_out = nullptr;
    int* pinned_err = nullptr;
    double* d_norms = nullptr;
    aqsg_state_s st;
    Request* cur = nullptr;
};

}  // namespace aqsg

using namespace aqsg;
using Clock = std::chrono::steady_clock;

struct aqsg_server_s {
    int device = 0, dtype = AQSG_C64, max_qubits = 0;
    uint32_t max_shots = 0;
    void* slab = nullptr;
    uint64_t slab_bytes = 0;
    Buddy buddy;
    std::vector<Lane> lanes;

    std::mutex mu;
    std::condition_variable cv_work, cv_idle;
    std::map<std::pair<double, uint64_t>, Request*> pending;  // by arrival, then ticket
    std::deque<aqsg_server_done> done;
    uint64_t next_ticket = 1, submitted = 0, completed = 0, failed = 0, unfinished = 0;
    uint64_t hbm_bytes = 0;  // algorithmic HBM bytes of the completed requests
    bool stop = false, started = false;
    Clock::time_point t0;
    std::thread worker;

    // worker-only
    uint64_t used = 0, peak = 0;
    int running = 0, peak_running = 0;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

void finish(aqsg_server_s* s, Lane& L, int status) {
    Request* r = L.cur;
    aqsg_server_done d{};
    d.ticket = r->ticket;
    d.n = r->n;
    d.lane = (int)(&L - s->lanes.data());
    d.fused_ops = r->fused_ops;
    d.arrival_s = r->arrival;
    d.admit_s = r->admit;
    if (status == AQSG_OK && *L.pinned_err) {
        status = AQSG_ERR_TIMEOUT;
        *L.pinned_err = 0;
        cudaMemsetAsync(L.ctx->d_err, 0, sizeof(int), L.ctx->stream);
    }
    if (status == AQSG_OK && r->shots) std::memcpy(r->outcomes, L.pinned_out, sizeof(uint64_t) * r->shots);
    d.status = status;
    // clear to |0...0>, the plan (with its renormalisation), and sampling:
    // one read for the chunk sums, 2^min(n, 12) amplitudes per shot
    const uint64_t ab = amp_bytes(r->plan.dtype), reg = ab << r->n;
    const uint64_t traffic = reg + plan_hbm_bytes(r->plan, true) +
                             (r->shots ? reg + (uint64_t)r->shots * (ab << (r->n < 12 ? r->n : 12)) : 0);
    s->buddy.release(r->off, r->order);
    s->used -= 1ull << r->order;
    --s->running;
    L.cur = nullptr;
    delete r;
    d.done_s = s->now();
    std::lock_guard<std::mutex> g(s->mu);
    s->done.push_back(d);
    ++s->completed;
    if (status == AQSG_OK) s->hbm_bytes += traffic;
    if (status != AQSG_OK) ++s->failed;
    if (--s->unfinished == 0) s->cv_idle.notify_all();
}

int launch(aqsg_server_s* s, Lane& L, Request* r) {
    L.st.ctx = L.ctx;
    L.st.n = r->n;
    L.st.dtype = s->dtype;
    L.st.amps = 1ull << r->n;
    L.st.d = (char*)s->slab + r->off;
    cudaStream_t stream = L.ctx->stream;
    if (int rc = launch_set_basis(&L.st, 0)) return rc;
    if (!r->plan.passes.empty()) {
        const size_t poff = r->plan.pool_offset();
        std::memcpy(L.pinned_table, r->plan.table.data(), r->plan.table.size());
        if (!r->plan.pool.empty()) std::memcpy(L.pinned_table + poff, r->plan.pool.data(), r->plan.pool.size());
        AQSG_CUDA_TRY(cudaMemcpyAsync(L.ctx->ops.ptr, L.pinned_table, r->table_bytes, cudaMemcpyHostToDevice, stream));
        if (int rc = run_plan_async(&L.st, r->plan, L.ctx->ops.ptr, L.d_norms)) return rc;
    }
    if (r->shots)
        if (int rc = sample_seeded_async(&L.st, r->seed, r->shots, AQSG_SAMPLE_REFERENCE, L.pinned_out)) return rc;
    AQSG_CUDA_TRY(cudaMemcpyAsync(L.pinned_err, L.ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    AQSG_CUDA_TRY(cudaEventRecord(L.done, stream));
    return AQSG_OK;
}

void worker_main(aqsg_server_s* s) {
    cudaSetDevice(s->device);
    std::vector<Request*> admit;
    std::vector<Lane*> idle;
    for (;;) {
        bool progress = false;
        for (Lane& L : s->lanes) {
            if (!L.cur) continue;
            const cudaError_t q = cudaEventQuery(L.done);
            if (q == cudaErrorNotReady) continue;
            finish(s, L, q == cudaSuccess ? AQSG_OK : cuda_error(q, "request"));
            progress = true;
        }
        idle.clear();
        for (Lane& L : s->lanes)
            if (!L.cur) idle.push_back(&L);
        admit.clear();
        double next_arrival = -1;
        bool quit = false;
        {
            std::unique_lock<std::mutex> g(s->mu);
            const double t = s->started ? s->now() : 0.0;
            Request* blocked = nullptr;
            if (s->stop) quit = s->running == 0;
            for (auto it = s->pending.begin();
                 s->started && !s->stop && it != s->pending.end() && admit.size() < idle.size();) {
                Request* r = it->second;
                if (r->arrival > t) {
                    next_arrival = r->arrival;
                    break;
                }
                if (blocked && blocked->passed_over >= kMaxPassOver) break;
                if (s->buddy.alloc(r->order, &r->off)) {
                    if (blocked) ++blocked->passed_over;
                    r->admit = t;
                    admit.push_back(r);
                    it = s->pending.erase(it);
                } else {
                    if (!blocked) blocked = r;
                    ++it;
                }
            }
            if (!quit && admit.empty() && s->running == 0 && !progress) {
                if (!s->stop && s->started && next_arrival >= 0)
                    s->cv_work.wait_for(g, std::chrono::duration<double>(std::max(0.0, next_arrival - t)));
                else if (!s->stop && (!s->started || s->pending.empty()))
                    s->cv_work.wait(g, [&] { return s->stop || (s->started && !s->pending.empty()); });
            }
        }
        if (quit) break;
        for (size_t i = 0; i < admit.size(); ++i) {
            Request* r = admit[i];
            Lane& L = *idle[i];
            L.cur = r;
            s->used += 1ull << r->order;
            s->peak = std::max(s->peak, s->used);
            ++s->running;
            s->peak_running = std::max(s->peak_running, s->running);
            if (int rc = launch(s, L, r)) {
                cudaStreamSynchronize(L.ctx->stream);  // nothing of it may still run on the block
                finish(s, L, rc);
            }
        }
        if (!progress && admit.empty() && s->running > 0) std::this_thread::yield();
    }
}

void destroy_lanes(aqsg_server_s* s) {
    for (Lane& L : s->lanes) {
        if (L.done) cudaEventDestroy(L.done);
        if (L.pinned_table) cudaFreeHost(L.pinned_table);
        if (L.pinned_out) cudaFreeHost(L.pinned_out);
        if (L.d_norms) cudaFree(L.d_norms);
        if (L.ctx) aqsg_shutdown(L.ctx);
    }
    s->lanes.clear();
}

}  // namespace

extern "C" {

int aqsg_server_create(int device, int dtype, uint64_t hbm_budget_bytes, int lanes, int max_qubits,
                       uint32_t max_shots, aqsg_server* out) {
    if (!out) return set_error(AQSG_ERR_NULL, "NULL output handle");
    *out = nullptr;
    if (dtype != AQSG_C64 && dtype != AQSG_C128) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown dtype");
    if (max_qubits < 1 || max_qubits > AQSG_MAX_QUBITS)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Invalid qubit count");
    if (lanes < 1 || lanes > 64) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Lanes must be 1 to 64");
    if (max_shots > (1u << 24)) return set_error(AQSG_ERR_INVALID_ARGUMENT, "At most 2^24 shots per request");
    const int amp_order = dtype == AQSG_C128 ? 4 : 3;
    const int top_order = max_qubits + amp_order;
    const uint64_t tops = hbm_budget_bytes >> top_order;
    if (tops < 1) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Budget holds no register of max_qubits qubits");
    AQSG_ON_DEVICE(device);
    auto* s = new aqsg_server_s();
    s->device = device;
    s->dtype = dtype;
    s->max_qubits = max_qubits;
    s->max_shots = max_shots;
    s->slab_bytes = tops << top_order;
    s->buddy.init(top_order, tops, std::min(top_order, 8));
    s->lanes.resize(lanes);
    int rc = AQSG_OK;
    for (Lane& L : s->lanes) {
        if ((rc = aqsg_init(device, &L.ctx))) break;
        if ((rc = reserve_scratch(L.ctx, max_qubits, max_shots ? max_shots : 1))) break;
        if ((rc = ensure_scratch(L.ctx->ops, kLaneTableBytes))) break;
        cudaError_t e = cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMallocHost((void**)&L.pinned_table, kLaneTableBytes);
        if (e == cudaSuccess) e = cudaMallocHost((void**)&L.pinned_out, sizeof(uint64_t) * (max_shots + 8));
        if (e == cudaSuccess) e = cudaMalloc((void**)&L.d_norms, sizeof(double) * tc_norm_doubles(L.ctx));
        if (e != cudaSuccess) {
            rc = cuda_error(e, "aqsg_server_create");
            break;
        }
        L.pinned_err = (int*)(L.pinned_out + max_shots + 4);
        *L.pinned_err = 0;
    }
    if (rc == AQSG_OK) {
        cudaError_t e = cudaMalloc(&s->slab, s->slab_bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            rc = e == cudaErrorMemoryAllocation ? set_error(AQSG_ERR_OUT_OF_MEMORY, "Cannot allocate the register slab")
                                                : cuda_error(e, "aqsg_server_create");
        }
    }
    if (rc != AQSG_OK) {
        destroy_lanes(s);
        delete s;
        return rc;
    }
    s->worker = std::thread(worker_main, s);
    *out = s;
    return AQSG_OK;
}

int aqsg_server_submit(aqsg_server s, int n, const aqsg_op* ops, int count, int fuse_qubits, uint32_t shots,
                       uint64_t seed, double arrival_s, uint64_t* outcomes, uint64_t* ticket) {
    if (!s) return set_error(AQSG_ERR_NULL, "NULL server");
    if (n < 1 || n > s->max_qubits)
        return set_error(AQSG_ERR_OUT_OF_RANGE, "Register larger than the server's max_qubits");
    if (shots > s->max_shots) return set_error(AQSG_ERR_OUT_OF_RANGE, "More shots than the server's max_shots");
    if (shots && !outcomes) return set_error(AQSG_ERR_NULL, "NULL outcome buffer");
    if (fuse_qubits < 0 || fuse_qubits > AQSG_MAX_UNITARY_QUBITS)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Fusion width must be 0 to 5 qubits");
    if (int rc = aqsg_check_ops(n, ops, count)) return rc;
    auto* r = new Request();
    r->n = n;
    r->shots = shots;
    r->seed = seed;
    r->outcomes = outcomes;
    int rc = AQSG_OK;
    int fused_ops = 0;
    if (fuse_qubits > 0) {
        // encoded straight from the program's ops (no copy of the fused
        // matrices)
        aqsg_program p = nullptr;
        rc = aqsg_compile(n, s->dtype, ops, count, fuse_qubits, &p);
        if (rc == AQSG_OK) {
            fused_ops = (int)program_ops(p).size();
            rc = encode_tiled(n, s->dtype, program_ops(p), true, &r->plan);
            aqsg_program_free(p);
        }
    } else {
        std::vector<LOp> low;
        low.reserve(count);
        for (int i = 0; i < count && rc == AQSG_OK; ++i) {
            LOp o;
            rc = lower_op(n, s->dtype, ops[i], &o);
            if (rc == AQSG_OK && o.cls != L_NOP) low.push_back(std::move(o));
        }
        fused_ops = (int)low.size();
        if (rc == AQSG_OK) rc = encode_tiled(n, s->dtype, low, true, &r->plan);
    }
    if (rc == AQSG_OK && !r->plan.passes.empty()) {
        r->table_bytes = r->plan.pool_offset() + r->plan.pool.size();
        if (r->table_bytes + 16 > kLaneTableBytes)
            rc = set_error(AQSG_ERR_INVALID_ARGUMENT, "Circuit's op table exceeds the 16 MiB a lane holds");
    }
    if (rc != AQSG_OK) {
        delete r;
        return rc;
    }
    r->fused_ops = fused_ops;
    r->order = s->buddy.order_for((uint64_t)amp_bytes(s->dtype) << n);
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (s->stop) {
            delete r;
            return set_error(AQSG_ERR_RUNTIME, "Server is shutting down");
        }
        r->ticket = s->next_ticket++;
        r->arrival = arrival_s < 0 ? (s->started ? s->now() : 0.0) : arrival_s;
        s->pending.emplace(std::make_pair(r->arrival, r->ticket), r);
        ++s->submitted;
        ++s->unfinished;
        if (ticket) *ticket = r->ticket;
    }
    s->cv_work.notify_one();
    return AQSG_OK;
}

int aqsg_server_start(aqsg_server s) {
    if (!s) return set_error(AQSG_ERR_NULL, "NULL server");
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (s->started) return set_error(AQSG_ERR_RUNTIME, "Server already started");
        s->t0 = Clock::now();
        s->started = true;
    }
    s->cv_work.notify_one();
    return AQSG_OK;
}

int aqsg_server_poll(aqsg_server s, aqsg_server_done* out, int capacity, int* count) {
    if (!s) return set_error(AQSG_ERR_NULL, "NULL server");
    if (!count || (capacity > 0 && !out)) return set_error(AQSG_ERR_NULL, "NULL output");
    std::lock_guard<std::mutex> g(s->mu);
    int k = 0;
    while (k < capacity && !s->done.empty()) {
        out[k++] = s->done.front();
        s->done.pop_front();
    }
    *count = k;
    return AQSG_OK;
}

int aqsg_server_wait_idle(aqsg_server s, double timeout_s) {
    if (!s) return set_error(AQSG_ERR_NULL, "NULL server");
    std::unique_lock<std::mutex> g(s->mu);
    if (!s->started && s->unfinished) return set_error(AQSG_ERR_RUNTIME, "Server not started");
    const bool ok = s->cv_idle.wait_for(g, std::chrono::duration<double>(timeout_s),
                                        [&] { return s->unfinished == 0; });
    return ok ? AQSG_OK : set_error(AQSG_ERR_TIMEOUT, "Requests still unfinished");
}

int aqsg_server_get_stats(aqsg_server s, aqsg_server_stats* out) {
    if (!s || !out) return set_error(AQSG_ERR_NULL, "NULL argument");
    std::lock_guard<std::mutex> g(s->mu);
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->failed = s->failed;
    out->slab_bytes = s->slab_bytes;
    out->peak_bytes = s->peak;
    out->peak_running = s->peak_running;
    out->lanes = (int)s->lanes.size();
    uint64_t l = 0;
    for (const Lane& L : s->lanes) l += L.ctx->launches;
    out->launches = l;
    out->hbm_bytes = s->hbm_bytes;
    return AQSG_OK;
}

int aqsg_server_destroy(aqsg_server s) {
    if (!s) return set_error(AQSG_ERR_NULL, "NULL server");
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_one();
    if (s->worker.joinable()) s->worker.join();
    DeviceScope scope(s->device);
    for (auto& kv : s->pending) delete kv.second;
    destroy_lanes(s);
    if (s->slab) cudaFree(s->slab);
    delete s;
    return AQSG_OK;
}

}  // extern "C"
