// Autotuner: picks how a circuit runs — one kernel pass per gate, tile passes,
// or tile passes over a program fused into unitaries of 2..5 qubits (with or
// without the tensor cores), and for registers of 13-14 qubits (c64) / 12-13
// (c128) the tile shape: the whole register in one CTA's tile, or streaming
// tiles of 2^12 / 2^11 amplitudes over several CTAs — by timing each choice
// on a scratch register of the circuit's size.  Results are cached per
// context by the circuit's structure (gate kinds and operands, not angles or
// matrix entries), so a parameter sweep tunes once.
#include <algorithm>
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
    AQSG_ON_DEVICE(ctx->device);
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

    // tile: the largest register run as one tile (aqsg_set_whole_tile_max);
    // a register of more qubits than a streaming tile that still fits one
    // whole-register tile is timed in both shapes
    struct Cand {
        int mode, fuse, tc, tile;
    };
    const int whole = tile_max_bits(dtype), stream = stream_tile_bits(dtype);
    std::vector<int> shapes = {whole};
    if (n > stream && n <= whole) shapes.push_back(stream);
    std::vector<Cand> cands;
    if (!tiled_only) cands.push_back({AQSG_EXEC_PER_GATE, 0, 0, 0});
    for (int shape : shapes) {
        cands.push_back({AQSG_EXEC_TILED, 0, 0, shape});
        cands.push_back({AQSG_EXEC_TILED, 1, 0, shape});  // consecutive 1-qubit gates merged
        for (int k = 2; k <= AQSG_MAX_UNITARY_QUBITS; ++k) {
            cands.push_back({AQSG_EXEC_TILED, k, 0, shape});
            if (dtype == AQSG_C64) cands.push_back({AQSG_EXEC_TILED, k, 1, shape});
        }
    }

    aqsg_state st = nullptr;
    if (int rc = aqsg_state_alloc(ctx, n, dtype, &st)) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = AQSG_OK;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        rc = set_error(AQSG_ERR_CUDA, "cudaEventCreate failed");
    if (rc == AQSG_OK) rc = aqsg_state_set_basis_index(st, 0);
    const int saved_tc = ctx->tensor_cores, saved_tile = ctx->whole_tile_max;
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
        ctx->whole_tile_max = c.tile;
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
            en.tile_bits = c.mode == AQSG_EXEC_PER_GATE ? 0 : (n <= c.tile ? n : stream);
            results.push_back(en);
        }
        if (prog) aqsg_program_free(prog);
    }
    ctx->tensor_cores = saved_tc;
    ctx->whole_tile_max = saved_tile;
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

namespace aqsg {

// Fusion width and tensor-core use for a large register of the batched
// engine, timed the way the batch runs it: the tile plan over a group of
// replicas whose size depends only on n (so the choice does not depend on
// the rest of the batch), one launch per pass.  Cached per context and
// structure.  A run that trips the device error flag (a bounded wait gave
// up) fails the tuning with AQSG_ERR_TIMEOUT.
int autotune_grouped(aqsg_ctx ctx, int n, const aqsg_op* ops, int count, int* fuse_out, int* tc_out) {
    if (int rc = aqsg_check_ops(n, ops, count)) return rc;
    const uint64_t key = structure_hash(n, AQSG_C64, ops, count) ^ 0xC2B2AE3D27D4EB4Full;
    TuneCache& cache = tune_cache();
    {
        std::lock_guard<std::mutex> g(cache.mu);
        auto it = cache.best.find({(const void*)ctx, key});
        if (it != cache.best.end()) {
            *fuse_out = it->second.fuse_qubits;
            *tc_out = it->second.tensor_cores;
            return AQSG_OK;
        }
    }
    if (n < 13 || n > 30) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Grouped tuning takes 13 to 30 qubits");
    const int replicas = n >= 22 ? 1 : (1 << (22 - n));
    const uint64_t amps = 1ull << n;
    void* regs = nullptr;
    void* tables = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    AQSG_ON_DEVICE(ctx->device);
    int rc = AQSG_OK;
    cudaError_t e = cudaMalloc(&regs, (size_t)replicas * amps * 8);
    if (e == cudaSuccess) e = cudaMemsetAsync(regs, 0, (size_t)replicas * amps * 8, ctx->stream);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) rc = cuda_error(e, "autotune_grouped");
    double best_ms = 1e300;
    int best_fuse = 0, best_tc = 0;
    size_t table_cap = 0;
    const int cand[][2] = {{0, 0}, {1, 0}, {2, 0}, {3, 0}, {4, 0}, {5, 0}, {3, 1}, {4, 1}, {5, 1}};
    for (const auto& fc : cand) {
        const int fuse = fc[0], tc = fc[1];
        if (rc != AQSG_OK) break;
        std::vector<LOp> low;
        if (fuse > 0) {
            aqsg_program p = nullptr;
            if ((rc = aqsg_compile(n, AQSG_C64, ops, count, fuse, &p))) break;
            low = program_ops(p);
            aqsg_program_free(p);
        } else {
            for (int i = 0; i < count && rc == AQSG_OK; ++i) {
                LOp o;
                rc = lower_op(n, AQSG_C64, ops[i], &o);
                if (rc == AQSG_OK && o.cls != L_NOP) low.push_back(std::move(o));
            }
            if (rc) break;
        }
        TilePlan plan;
        if ((rc = encode_tiled(n, AQSG_C64, low, tc != 0, &plan, false))) break;
        if (tc && !plan.any_tc) continue;  // nothing for the tensor cores: same as the plain plan
        const size_t stride = (plan.pool_offset() + plan.pool.size() + 255) & ~size_t(255);
        if (stride * replicas > table_cap) {
            if (tables) cudaFree(tables);
            table_cap = stride * replicas;
            if ((e = cudaMalloc(&tables, table_cap)) != cudaSuccess) {
                tables = nullptr;
                rc = cuda_error(e, "autotune_grouped");
                break;
            }
        }
        for (int r = 0; r < replicas && e == cudaSuccess; ++r) {
            char* dst = (char*)tables + (size_t)r * stride;
            e = cudaMemcpyAsync(dst, plan.table.data(), plan.table.size(), cudaMemcpyHostToDevice, ctx->stream);
            if (e == cudaSuccess && !plan.pool.empty())
                e = cudaMemcpyAsync(dst + plan.pool_offset(), plan.pool.data(), plan.pool.size(),
                                    cudaMemcpyHostToDevice, ctx->stream);
        }
        if (e != cudaSuccess) {
            rc = cuda_error(e, "autotune_grouped");
            break;
        }
        uint64_t launches = 0;
        if ((rc = launch_tile_plan_multi(regs, amps, replicas, plan, tables, stride, ctx->stream, ctx->d_err,
                                         &launches)))
            break;
        // the best of two timed runs (candidates can lie within a few per
        // cent of each other)
        float ms = 1e30f;
        for (int rep = 0; rep < 2 && rc == AQSG_OK; ++rep) {
            cudaEventRecord(e0, ctx->stream);
            if ((rc = launch_tile_plan_multi(regs, amps, replicas, plan, tables, stride, ctx->stream, ctx->d_err,
                                             &launches)))
                break;
            cudaEventRecord(e1, ctx->stream);
            if ((e = cudaEventSynchronize(e1)) != cudaSuccess) {
                rc = cuda_error(e, "autotune_grouped");
                break;
            }
            float t = 0;
            cudaEventElapsedTime(&t, e0, e1);
            ms = std::min(ms, t);
        }
        if (rc != AQSG_OK) break;
        if (plan.any_tc) {
            int flag = 0;
            if ((e = cudaMemcpy(&flag, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess) {
                rc = cuda_error(e, "autotune_grouped");
                break;
            }
            if (flag) {
                cudaMemset(ctx->d_err, 0, sizeof(int));
                rc = set_error(AQSG_ERR_TIMEOUT, "A bounded device wait gave up while tuning");
                break;
            }
        }
        if (ms < best_ms) {
            best_ms = ms;
            best_fuse = fuse;
            best_tc = tc;
        }
    }
    cudaStreamSynchronize(ctx->stream);
    if (tables) cudaFree(tables);
    if (regs) cudaFree(regs);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (rc != AQSG_OK) return rc;
    aqsg_tune_entry en;
    std::memset(&en, 0, sizeof(en));
    en.exec_mode = AQSG_EXEC_TILED;
    en.fuse_qubits = best_fuse;
    en.tensor_cores = best_tc;
    en.ms = best_ms / replicas;
    en.tile_bits = n <= tile_max_bits(AQSG_C64) ? n : stream_tile_bits(AQSG_C64);
    {
        std::lock_guard<std::mutex> g(cache.mu);
        cache.best[{(const void*)ctx, key}] = en;
    }
    *fuse_out = best_fuse;
    *tc_out = best_tc;
    return AQSG_OK;
}

}  // namespace aqsg
