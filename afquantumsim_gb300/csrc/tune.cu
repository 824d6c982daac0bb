// Autotuner: picks how a circuit runs — one kernel pass per gate, tile passes,
// or tile passes over a program fused into unitaries of 2..5 qubits (with or
// without the tensor cores) — by timing each choice on a scratch register of
// the circuit's size.  Results are cached per context by the circuit's
// structure (gate kinds and operands, not angles or matrix entries), so a
// parameter sweep tunes once.
#include <cstring>
#include <map>
#include <mutex>

#include "aqsg_internal.h"

namespace aqsg {

// FNV-1a over the structural fields of the ops
static uint64_t structure_hash(int n, int dtype, const aqsg_op* ops, int count) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) {
        for (int i = 0; i < 8; ++i) {
            h ^= (v >> (8 * i)) & 0xFFu;
            h *= 1099511628211ull;
        }
    };
    mix((uint64_t)n);
    mix((uint64_t)dtype);
    mix((uint64_t)count);
    for (int i = 0; i < count; ++i) {
        const aqsg_op& o = ops[i];
        mix((uint64_t)o.kind | ((uint64_t)o.num_qubits << 16) | ((uint64_t)o.num_controls << 32));
        mix(o.control_values);
        for (int j = 0; j < o.num_qubits && j < AQSG_OP_MAX_QUBITS; ++j) mix((uint64_t)o.qubits[j]);
        for (int j = 0; j < o.num_controls && j < AQSG_OP_MAX_CONTROLS; ++j) mix((uint64_t)o.controls[j]);
    }
    return h;
}

struct TuneCache {
    std::mutex mu;
    std::map<std::pair<const void*, uint64_t>, aqsg_tune_entry> best;
};

static TuneCache& tune_cache() {
    static TuneCache c;
    return c;
}

int autotune_impl(aqsg_ctx ctx, int n, int dtype, const aqsg_op* ops, int count, int reps, bool tiled_only,
                  aqsg_tune_entry* best, aqsg_tune_entry* all, int capacity, int* count_out);

}  // namespace aqsg

using namespace aqsg;

extern "C" int aqsg_autotune(aqsg_ctx ctx, int n, int dtype, const aqsg_op* ops, int count, int reps,
                             aqsg_tune_entry* best, aqsg_tune_entry* all, int capacity, int* count_out) {
    return autotune_impl(ctx, n, dtype, ops, count, reps, false, best, all, capacity, count_out);
}

namespace aqsg {

void autotune_forget(aqsg_ctx ctx) {
    TuneCache& cache = tune_cache();
    std::lock_guard<std::mutex> g(cache.mu);
    for (auto it = cache.best.begin(); it != cache.best.end();)
        it = it->first.first == (const void*)ctx ? cache.best.erase(it) : std::next(it);
}

// tiled_only: leave out the one-gate-per-pass candidate (callers that only
// run tile passes, such as the batched engine).
int autotune_impl(aqsg_ctx ctx, int n, int dtype, const aqsg_op* ops, int count, int reps, bool tiled_only,
                  aqsg_tune_entry* best, aqsg_tune_entry* all, int capacity, int* count_out) {
    if (!ctx || !best) return set_error(AQSG_ERR_NULL, "NULL argument");
    if (count_out) *count_out = 0;
    if (reps < 1) reps = 1;
    if (int rc = aqsg_check_ops(n, ops, count)) return rc;
    if (dtype != AQSG_C64 && dtype != AQSG_C128) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown dtype");
    const uint64_t key = structure_hash(n, dtype, ops, count) ^ (tiled_only ? 0x9E3779B97F4A7C15ull : 0ull);
    TuneCache& cache = tune_cache();
    if (!all) {
        std::lock_guard<std::mutex> g(cache.mu);
        auto it = cache.best.find({(const void*)ctx, key});
        if (it != cache.best.end()) {
            *best = it->second;
            return AQSG_OK;
        }
    }

    struct Cand {
        int mode, fuse, tc;
    };
    std::vector<Cand> cands;
    if (!tiled_only) cands.push_back({AQSG_EXEC_PER_GATE, 0, 0});
    cands.push_back({AQSG_EXEC_TILED, 0, 0});
    for (int k = 2; k <= AQSG_MAX_UNITARY_QUBITS; ++k) {
        cands.push_back({AQSG_EXEC_TILED, k, 0});
        if (dtype == AQSG_C64) cands.push_back({AQSG_EXEC_TILED, k, 1});
    }

    aqsg_state st = nullptr;
    if (int rc = aqsg_state_alloc(ctx, n, dtype, &st)) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = AQSG_OK;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        rc = set_error(AQSG_ERR_CUDA, "cudaEventCreate failed");
    if (rc == AQSG_OK) rc = aqsg_state_set_basis_index(st, 0);
    const int saved_tc = ctx->tensor_cores;
    std::vector<aqsg_tune_entry> results;
    for (const Cand& c : cands) {
        if (rc != AQSG_OK) break;
        aqsg_program prog = nullptr;
        int fused = count;
        if (c.fuse > 0) {
            if ((rc = aqsg_compile(n, dtype, ops, count, c.fuse, &prog))) break;
            aqsg_program_info(prog, &fused, nullptr);
        }
        ctx->tensor_cores = c.tc;
        auto run = [&]() {
            return prog ? aqsg_run_program(st, prog, c.mode) : aqsg_apply_ops(st, ops, count, c.mode);
        };
        rc = run();  // warm-up (and first-launch setup)
        if (rc == AQSG_OK) {
            cudaEventRecord(e0, ctx->stream);
            for (int r = 0; r < reps && rc == AQSG_OK; ++r) rc = run();
            cudaEventRecord(e1, ctx->stream);
            if (cudaEventSynchronize(e1) != cudaSuccess) rc = set_error(AQSG_ERR_CUDA, "autotune timing failed");
        }
        if (rc == AQSG_OK) {
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            aqsg_tune_entry en;
            std::memset(&en, 0, sizeof(en));
            en.exec_mode = c.mode;
            en.fuse_qubits = c.fuse;
            en.tensor_cores = c.tc;
            en.ops = fused;
            en.ms = (double)ms / reps;
            results.push_back(en);
        }
        if (prog) aqsg_program_free(prog);
    }
    ctx->tensor_cores = saved_tc;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    aqsg_state_free(st);
    if (rc != AQSG_OK) return rc;
    size_t bi = 0;
    for (size_t i = 1; i < results.size(); ++i)
        if (results[i].ms < results[bi].ms) bi = i;
    *best = results[bi];
    {
        std::lock_guard<std::mutex> g(cache.mu);
        cache.best[{(const void*)ctx, key}] = results[bi];
    }
    if (all) {
        const int k = (int)results.size() < capacity ? (int)results.size() : capacity;
        for (int i = 0; i < k; ++i) all[i] = results[i];
        if (count_out) *count_out = (int)results.size();
    }
    return AQSG_OK;
}

}  // namespace aqsg
