// Batched engine: many independent c64 registers of uneven size, each run
// from |0...0> and reduced to <Z_q> and <Z_q Z_q+1> (FP64), in one CUDA
// graph.  It generalises the reference's VQE cost loop
// (src/quantum_algo.cpp:412-456: simulate, then read expectation values)
// from one circuit at a time to a whole parameter sweep.
//
// Registers of up to 14 qubits never touch HBM: a persistent kernel per size
// class takes circuits from an atomic work counter, one CTA per circuit,
// prepares |0...0> in shared memory, runs the circuit's ops with the tile
// interpreter, and sums the expectation values on chip.  Larger registers
// run as preplanned tile passes over one reused device register.  The whole
// sequence is captured once; aqsg_batch_update swaps in new angles without
// re-planning, and aqsg_batch_run replays the graph.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "../../include/aqsg_debug.h"
#include "tile_device.cuh"

namespace aqsg {

struct SmallItem {
    int32_t n, nops;
    uint32_t op_first;  // first TileOp of this circuit in the class table
    uint32_t out;       // offset (doubles) of its 2n raw results
};

constexpr int kZMaxBits = 14;

__device__ __forceinline__ double warp_sum_b(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block sum; valid in thread 0.  blockDim.x is a multiple of 32.
__device__ __forceinline__ double block_sum_b(double v, double* sh) {
    v = warp_sum_b(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0;
    if (w == 0) {
        r = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
        r = warp_sum_b(r);
    }
    __syncthreads();
    return r;
}

// Raw results per circuit, 2n doubles: S[b] = sum p over indices with bit b
// set (b < n), X[b] = sum p over indices whose bits b and b+1 differ
// (b < n-1), then the total T.  <Z_q> = T - 2 S[n-1-q].
template <int EPT, int MAXT, bool MATK>
__global__ void __launch_bounds__(MAXT, 1)
k_batch_small(const SmallItem* __restrict__ items, int count, int* counter, const TileOp* __restrict__ ops,
              const unsigned char* __restrict__ pool, double* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* s = reinterpret_cast<float2*>(smem_raw);
    __shared__ int cur;
    __shared__ double red[32];
    for (;;) {
        if (threadIdx.x == 0) cur = atomicAdd(counter, 1);
        __syncthreads();
        const int i = cur;
        __syncthreads();
        if (i >= count) break;
        const SmallItem it = items[i];
        const int n = it.n;
        const uint32_t size = 1u << n;
        for (uint32_t j = threadIdx.x; j < size; j += blockDim.x) s[j] = make_float2(j == 0 ? 1.f : 0.f, 0.f);
        __syncthreads();
        tile_run_ops<float, EPT, false, FlatLay, CtaSync, MATK>(s, size, blockDim.x, 0, ops + it.op_first, it.nops,
                                                                pool, nullptr, nullptr);
        // exact |a|^2 and compensated sums on the FP32 pipe, FP64 across threads
        FAcc fT, fS[kZMaxBits], fX[kZMaxBits];
        for (uint32_t j = threadIdx.x; j < size; j += blockDim.x) {
            const float2 a = s[j];
            float h, l;
            norm2_ff(a.x, a.y, h, l);
            fT.add(h, l);
#pragma unroll
            for (int b = 0; b < kZMaxBits; ++b) {
                if (b < n && ((j >> b) & 1u)) fS[b].add(h, l);
                if (b + 1 < n && (((j >> b) ^ (j >> (b + 1))) & 1u)) fX[b].add(h, l);
            }
        }
        double T = fT.value(), S[kZMaxBits], X[kZMaxBits];
#pragma unroll
        for (int b = 0; b < kZMaxBits; ++b) {
            S[b] = fS[b].value();
            X[b] = fX[b].value();
        }
        double* o = out + it.out;
#pragma unroll
        for (int b = 0; b < kZMaxBits; ++b) {
            if (b < n) {
                const double v = block_sum_b(S[b], red);
                if (threadIdx.x == 0) o[b] = v;
            }
            if (b + 1 < n) {
                const double v = block_sum_b(X[b], red);
                if (threadIdx.x == 0) o[n + b] = v;
            }
        }
        const double t = block_sum_b(T, red);
        if (threadIdx.x == 0) o[2 * n - 1] = t;
        __syncthreads();
    }
}

__global__ void k_basis0(float2* sv) { sv[0] = make_float2(1.f, 0.f); }
// |0...0> in each of gridDim.x registers `stride` amplitudes apart (already zeroed)
__global__ void k_basis0_multi(float2* sv, uint64_t stride) {
    sv[(uint64_t)blockIdx.x * stride] = make_float2(1.f, 0.f);
}

// Large registers whose tile plans have the same geometry (qubits, passes,
// tile bits, tensor-core use, table, pool and operand-blob sizes) run as a
// group:
// one launch per pass for all of them, their registers side by side and
// their op tables at a fixed stride in the device plan area.
struct LargeGroup {
    int n = 0;
    std::vector<size_t> members;      // indices into aqsg_batch_s::large / plans
    uint64_t dev_off = 0, stride = 0;  // first member's table in d_large, distance between members
    void* regs = nullptr;              // members x 2^n amplitudes
    double* partials = nullptr;        // members x expz_partial_doubles(n)
    uint64_t* d_out_off = nullptr;     // members result offsets into d_out
};
constexpr uint64_t kGroupBytes = 1ull << 30;  // registers of one group at most

// classes of small registers: (max qubits, threads, elements per thread)
struct SmallClass {
    int max_n, threads;
};
static const SmallClass kClasses[3] = {{10, 128}, {12, 256}, {14, 512}};

// The kernel of a size class, with or without the dense k-qubit op path (a
// class whose circuits have none runs the lighter variant).
struct SmallKernel {
    void (*fn)(const SmallItem*, int, int*, const TileOp*, const unsigned char*, double*);
    int threads;
    void launch(int grid, size_t shm, cudaStream_t st, const SmallItem* items, int cnt, int* counter,
                const TileOp* ops, const unsigned char* pool, double* out) const {
        void* args[] = {(void*)&items, (void*)&cnt, (void*)&counter, (void*)&ops, (void*)&pool, (void*)&out};
        cudaLaunchKernel((const void*)fn, dim3(grid), dim3(threads), args, shm, st);
    }
};

static SmallKernel small_kernel(int c, bool matk) {
    switch (c) {
        case 0: return {matk ? k_batch_small<2, 128, true> : k_batch_small<2, 128, false>, 128};
        case 1: return {matk ? k_batch_small<2, 256, true> : k_batch_small<2, 256, false>, 256};
        default: return {matk ? k_batch_small<2, 512, true> : k_batch_small<2, 512, false>, 512};
    }
}

static int class_of(int n) {
    for (int c = 0; c < 3; ++c)
        if (n <= kClasses[c].max_n) return c;
    return -1;
}

// Where one circuit's encoded ops sit in the batch's plan image: its op
// table, its operand pool, and (small registers) the shift applied to its
// pool offsets, which are relative to the class pool there.
struct PlanSlot {
    uint64_t table_at = 0, pool_at = 0;
    uint64_t table_bytes = 0, pool_bytes = 0;
    int32_t reloc = 0;
    int cls = -1;    // size class, or -1 for a large register
    int large = -1;  // index into the large plans
};

}  // namespace aqsg

using namespace aqsg;

struct aqsg_batch_s {
    aqsg_ctx ctx = nullptr;
    int count = 0;
    std::vector<int> n;
    std::vector<size_t> out_off;  // raw-result offset per circuit
    size_t out_doubles = 0;
    // small classes
    std::vector<SmallItem> items[3];
    std::vector<int> class_circuits[3];
    std::vector<unsigned char> small_table[3], small_pool[3];
    void* d_small_items[3] = {nullptr, nullptr, nullptr};
    void* d_small_ops[3] = {nullptr, nullptr, nullptr};
    int grid[3] = {0, 0, 0};
    bool class_matk[3] = {false, false, false};  // a class has dense k-qubit ops
    // large registers
    std::vector<int> large;  // circuit indices
    std::vector<int> fuse;   // per large circuit: tuned fusion width (0 = none)
    std::vector<int> tc;     // per large circuit: fused unitaries on the tensor cores
    std::vector<TilePlan> plans;
    std::vector<size_t> plan_off;  // offset of each plan's table+pool in d_large
    std::vector<LargeGroup> groups;
    std::vector<char> grouped;     // per large circuit: runs in a group
    void* d_large = nullptr;
    // every plan area in one host image (pinned) and its device copy,
    // uploaded with one copy: the three class tables (pool after each),
    // then the large plans.  d_small_ops and d_large point into d_plans.
    std::vector<PlanSlot> slots;  // per circuit
    size_t small_base[3] = {0, 0, 0};
    size_t large_base = 0;
    size_t plans_bytes = 0;
    unsigned char* h_plans = nullptr;
    void* d_plans = nullptr;
    // host-only batches (the plan-image check): no device, the fusion width
    // and tensor-core choice of each large register given, not tuned
    bool host_only = false;
    const int* preset_fuse = nullptr;
    const int* preset_tc = nullptr;
    // parallel branches of the graph: large circuits go round-robin to
    // branch streams, each with its own register and reduction scratch
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> joins;
    cudaEvent_t fork = nullptr;
    std::vector<void*> regs, partials;
    // results and counters
    double* d_out = nullptr;
    double* h_out = nullptr;  // pinned
    int* d_counters = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t kernels = 0;  // kernel launches in one replay
};

namespace aqsg {

int launch_expz_raw(const void* sv, int n, int dtype, double* partial, double* out_raw, cudaStream_t stream);
int launch_expz_raw_multi(const void* sv0, uint64_t reg_stride, int members, int n, double* partial,
                          const uint64_t* out_off, double* out_base, cudaStream_t stream);
size_t expz_partial_doubles(int n);

// Lower one circuit (fused at the given width, or gate by gate) and encode
// it as tile passes.  Host-only and independent of every other circuit.
static int encode_circuit(const aqsg_circuit& ci, int fuse, bool tc, TilePlan* plan) {
    std::vector<LOp> low;
    if (fuse > 0) {
        // encode straight from the program's ops (fused matrices are 16 KiB
        // each: no copy)
        aqsg_program p = nullptr;
        if (int rc = aqsg_compile(ci.n, AQSG_C64, ci.ops, ci.count, fuse, &p)) return rc;
        const int rc = encode_tiled(ci.n, AQSG_C64, program_ops(p), tc, plan, false);
        aqsg_program_free(p);
        return rc;
    } else {
        low.reserve(ci.count);
        for (int k = 0; k < ci.count; ++k) {
            LOp o;
            if (int rc = lower_op(ci.n, AQSG_C64, ci.ops[k], &o)) return rc;
            if (o.cls != L_NOP) low.push_back(std::move(o));
        }
    }
    // the tensor-core choice may not depend on parameter values, so that an
    // update keeps the captured graph's shape
    return encode_tiled(ci.n, AQSG_C64, low, tc, plan, false);
}

// Run body(i) for i in [0, count) on up to hardware_concurrency threads,
// in chunks claimed from an atomic counter.
template <class F>
static void parallel_for(int count, F body) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int threads = (int)std::min<unsigned>(hw, (unsigned)std::max(1, count / 16));
    std::atomic<int> next{0};
    auto work = [&]() {
        for (;;) {
            const int at = next.fetch_add(16);
            if (at >= count) return;
            const int end = std::min(count, at + 16);
            for (int i = at; i < end; ++i) body(i);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
}

// Lower and encode every circuit at creation; fills the host-side tables
// of b.  Each large register first gets its fusion width: the width the
// grouped tuner finds fastest for its structure (timed as the batch runs
// it, over a replica count that depends on n only, and cached per
// structure, so a circuit runs the same way alone and in any batch).  The
// per-circuit lowering and encoding then run on all host threads, and the
// tables are assembled in circuit order, so the result does not depend on
// the thread count.
static int encode_batch(aqsg_batch_s* b, const aqsg_circuit* cs) {
    std::vector<int> large_index(b->count, -1);
    int nlarge = 0;
    for (int i = 0; i < b->count; ++i) {
        const aqsg_circuit& ci = cs[i];
        if (int rc = aqsg_check_ops(ci.n, ci.ops, ci.count)) return rc;
        if (class_of(ci.n) >= 0) continue;
        large_index[i] = nlarge++;
        int best_fuse = 0, best_tc = 0;
        if (b->preset_fuse) {
            best_fuse = b->preset_fuse[nlarge - 1];
            best_tc = b->preset_tc ? b->preset_tc[nlarge - 1] : 0;
            if (best_fuse < 0) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Negative fusion width");
        } else if (int rc = autotune_grouped(b->ctx, ci.n, ci.ops, ci.count, &best_fuse, &best_tc)) {
            return rc;
        }
        b->fuse.push_back(best_fuse);
        b->tc.push_back(best_tc);
    }
    std::vector<TilePlan> plans(b->count);
    std::vector<int> rcs(b->count, AQSG_OK);
    std::vector<std::string> msgs(b->count);
    parallel_for(b->count, [&](int i) {
        const int li = large_index[i];
        const int fuse = li >= 0 ? b->fuse[li] : 0;
        const bool tc = li >= 0 && b->tc[li] != 0;
        rcs[i] = encode_circuit(cs[i], fuse, tc, &plans[i]);
        if (rcs[i]) msgs[i] = last_error_message();
    });
    for (int i = 0; i < b->count; ++i)
        if (rcs[i]) return set_error(rcs[i], msgs[i]);
    // assemble the class tables in circuit order
    b->slots.assign(b->count, PlanSlot());
    for (int i = 0; i < b->count; ++i) {
        const int cls = class_of(cs[i].n);
        TilePlan& plan = plans[i];
        PlanSlot& sl = b->slots[i];
        sl.cls = cls;
        sl.table_bytes = plan.table.size();
        sl.pool_bytes = plan.pool.size();
        if (cls >= 0) {
            // one whole-register pass; its ops go to the class table with
            // their pool offsets shifted to the class pool
            const size_t tsz = sizeof(TileOp);
            const uint32_t first = (uint32_t)(b->small_table[cls].size() / tsz);
            const size_t pbase = (b->small_pool[cls].size() + 255) & ~size_t(255);
            b->small_pool[cls].resize(pbase);
            b->small_pool[cls].insert(b->small_pool[cls].end(), plan.pool.begin(), plan.pool.end());
            const size_t w = b->small_table[cls].size();
            b->small_table[cls].insert(b->small_table[cls].end(), plan.table.begin(), plan.table.end());
            if (relocate_tile_matrices(b->small_table[cls].data() + w, plan.table.size() / tsz, (int32_t)pbase))
                b->class_matk[cls] = true;
            sl.table_at = w;     // within the class table, until laid out
            sl.pool_at = pbase;  // within the class pool
            sl.reloc = (int32_t)pbase;
            SmallItem it;
            it.n = cs[i].n;
            it.nops = (int)(plan.table.size() / tsz);
            it.op_first = first;
            it.out = (uint32_t)b->out_off[i];
            b->items[cls].push_back(it);
            b->class_circuits[cls].push_back(i);
        } else {
            sl.large = (int)b->large.size();
            b->large.push_back(i);
            b->plans.push_back(std::move(plan));
        }
    }
    return AQSG_OK;
}

// Group the large registers with equal plan geometry, and lay out the plan
// image: each size class's table then pool, then the large plans (each
// group's members at a fixed stride, then the rest).  Host only.
static void layout_batch(aqsg_batch_s* b) {
    b->grouped.assign(b->large.size(), 0);
    {
        std::map<std::vector<uint64_t>, std::vector<size_t>> by_key;
        for (size_t k = 0; k < b->large.size(); ++k) {
            const TilePlan& p = b->plans[k];
            std::vector<uint64_t> key = {(uint64_t)p.n, p.table.size(), p.pool.size(), p.passes.size()};
            for (const TilePass& ps : p.passes) {
                key.push_back(((uint64_t)ps.m << 48) | ((uint64_t)ps.L << 40) | ((uint64_t)ps.tc << 36) |
                              ((uint64_t)ps.matk << 32) | ps.first);
                key.push_back(ps.count);
                key.push_back(((uint64_t)ps.tc_blob << 32) | ps.tc_bytes);
                uint64_t bits = 0;
                for (int i = 0; i < ps.m; ++i) bits |= 1ull << ps.tbits[i];
                key.push_back(bits);
            }
            by_key[key].push_back(k);
        }
        for (auto& kv : by_key) {
            const int n = b->plans[kv.second[0]].n;
            const size_t per_chunk = std::max<size_t>(1, std::min<size_t>(kGroupBytes >> (n + 3), 65535));
            for (size_t at = 0; at < kv.second.size(); at += per_chunk) {
                LargeGroup gr;
                gr.n = n;
                gr.members.assign(kv.second.begin() + (long)at,
                                  kv.second.begin() + (long)std::min(kv.second.size(), at + per_chunk));
                for (size_t k : gr.members) b->grouped[k] = 1;
                b->groups.push_back(std::move(gr));
            }
        }
    }
    size_t at = 0;
    for (int c = 0; c < 3; ++c) {
        b->small_base[c] = at;
        if (b->items[c].empty()) continue;
        const size_t poff = (b->small_table[c].size() + 255) & ~size_t(255);
        at += (poff + b->small_pool[c].size() + 16 + 255) & ~size_t(255);
    }
    b->large_base = at;
    b->plan_off.assign(b->plans.size(), 0);
    size_t large_bytes = 0;
    for (LargeGroup& gr : b->groups) {
        const TilePlan& p = b->plans[gr.members[0]];
        gr.stride = (p.pool_offset() + p.pool.size() + 255) & ~size_t(255);
        gr.dev_off = large_bytes;
        for (size_t j = 0; j < gr.members.size(); ++j) b->plan_off[gr.members[j]] = large_bytes + j * gr.stride;
        large_bytes += gr.members.size() * gr.stride;
    }
    for (size_t k = 0; k < b->plans.size(); ++k) {
        if (b->grouped[k]) continue;
        const TilePlan& p = b->plans[k];
        b->plan_off[k] = large_bytes;
        large_bytes += (p.pool_offset() + p.pool.size() + 255) & ~size_t(255);
    }
    b->plans_bytes = at + large_bytes;
    // slots as image offsets
    for (PlanSlot& sl : b->slots) {
        if (sl.cls >= 0) {
            const size_t poff = (b->small_table[sl.cls].size() + 255) & ~size_t(255);
            sl.table_at += b->small_base[sl.cls];
            sl.pool_at += b->small_base[sl.cls] + poff;
        } else {
            sl.table_at = b->large_base + b->plan_off[sl.large];
            sl.pool_at = sl.table_at + b->plans[sl.large].pool_offset();
        }
    }
}

// Write the tables assembled at creation into the (zeroed) plan image.
static void fill_image(aqsg_batch_s* b) {
    std::memset(b->h_plans, 0, b->plans_bytes);
    for (int c = 0; c < 3; ++c) {
        if (b->items[c].empty()) continue;
        unsigned char* dst = b->h_plans + b->small_base[c];
        const size_t poff = (b->small_table[c].size() + 255) & ~size_t(255);
        if (!b->small_table[c].empty()) std::memcpy(dst, b->small_table[c].data(), b->small_table[c].size());
        if (!b->small_pool[c].empty()) std::memcpy(dst + poff, b->small_pool[c].data(), b->small_pool[c].size());
    }
    for (size_t k = 0; k < b->plans.size(); ++k) {
        const TilePlan& p = b->plans[k];
        unsigned char* dst = b->h_plans + b->large_base + b->plan_off[k];
        if (!p.table.empty()) std::memcpy(dst, p.table.data(), p.table.size());
        if (!p.pool.empty()) std::memcpy(dst + p.pool_offset(), p.pool.data(), p.pool.size());
    }
}

// New parameter values: re-lower and re-encode every circuit on all host
// threads, each straight into its slot of the plan image.  The structure
// (qubit counts, op classes, table, pool and pass geometry) must be the
// one the batch was created with, since the captured graph's launches
// depend on it.  On an error the image may be partly rewritten; it is not
// uploaded.
static int update_image(aqsg_batch_s* b, const aqsg_circuit* cs) {
    for (int i = 0; i < b->count; ++i) {
        if (cs[i].n != b->n[i]) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Batch structure changed (qubit count)");
        if (cs[i].count > 0 && !cs[i].ops) return set_error(AQSG_ERR_NULL, "NULL op list");
        if (int rc = aqsg_check_ops(cs[i].n, cs[i].ops, cs[i].count)) return rc;
    }
    std::vector<int> rcs(b->count, AQSG_OK);
    std::vector<std::string> msgs(b->count);
    parallel_for(b->count, [&](int i) {
        // one plan per host thread, reused: its buffers keep their capacity
        thread_local TilePlan plan;
        const PlanSlot& sl = b->slots[i];
        const int fuse = sl.large >= 0 ? b->fuse[sl.large] : 0;
        const bool tc = sl.large >= 0 && b->tc[sl.large] != 0;
        int rc = encode_circuit(cs[i], fuse, tc, &plan);
        if (!rc && (plan.table.size() != sl.table_bytes || plan.pool.size() != sl.pool_bytes))
            rc = set_error(AQSG_ERR_INVALID_ARGUMENT, "Batch structure changed (ops)");
        if (!rc && sl.large >= 0) {
            const std::vector<TilePass>& was = b->plans[sl.large].passes;
            if (plan.passes.size() != was.size() ||
                (!was.empty() && std::memcmp(plan.passes.data(), was.data(), was.size() * sizeof(TilePass))))
                rc = set_error(AQSG_ERR_INVALID_ARGUMENT, "Batch structure changed (passes)");
        }
        if (!rc) {
            unsigned char* t = b->h_plans + sl.table_at;
            if (sl.table_bytes) std::memcpy(t, plan.table.data(), sl.table_bytes);
            if (sl.pool_bytes) std::memcpy(b->h_plans + sl.pool_at, plan.pool.data(), sl.pool_bytes);
            if (sl.cls >= 0 && relocate_tile_matrices(t, sl.table_bytes / sizeof(TileOp), sl.reloc) &&
                !b->class_matk[sl.cls])
                rc = set_error(AQSG_ERR_INVALID_ARGUMENT, "Batch structure changed (dense ops)");
        }
        if (rc) {
            rcs[i] = rc;
            msgs[i] = last_error_message();
        }
    });
    for (int i = 0; i < b->count; ++i)
        if (rcs[i]) return set_error(rcs[i], msgs[i]);
    return AQSG_OK;
}

static int upload_batch(aqsg_batch_s* b, cudaStream_t s) {
    if (b->plans_bytes)
        AQSG_CUDA_TRY(cudaMemcpyAsync(b->d_plans, b->h_plans, b->plans_bytes, cudaMemcpyHostToDevice, s));
    AQSG_CUDA_TRY(cudaStreamSynchronize(s));
    return AQSG_OK;
}

// Qubit counts and result offsets of a new batch.
static int init_shape(aqsg_batch_s* b, const aqsg_circuit* cs, int count) {
    b->count = count;
    b->n.resize(count);
    b->out_off.resize(count);
    for (int i = 0; i < count; ++i) {
        const int n = cs[i].n;
        if (n < 1 || n > 30) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Batch registers take 1 to 30 qubits");
        if (cs[i].count > 0 && !cs[i].ops) return set_error(AQSG_ERR_NULL, "NULL op list");
        b->n[i] = n;
        b->out_off[i] = b->out_doubles;
        b->out_doubles += 2 * (size_t)n;
    }
    return AQSG_OK;
}

static constexpr int kMaxBranches = 32;

static int branch_of_large(const aqsg_batch_s* b, size_t k) {
    return (int)((k + 3) % b->streams.size());
}

// The device work of one run (captured into the graph): fork to the branch
// streams, small-register classes on branches 0..2, large registers
// round-robin, join back.
static int record_batch(aqsg_batch_s* b, cudaStream_t s) {
    b->kernels = 0;
    AQSG_CUDA_TRY(cudaMemsetAsync(b->d_counters, 0, 3 * sizeof(int), s));
    const int nb = (int)b->streams.size();
    AQSG_CUDA_TRY(cudaEventRecord(b->fork, s));
    for (int k = 0; k < nb; ++k) AQSG_CUDA_TRY(cudaStreamWaitEvent(b->streams[k], b->fork, 0));
    for (int c = 0; c < 3; ++c) {
        if (b->items[c].empty()) continue;
        cudaStream_t bs = b->streams[c % nb];
        const size_t shm = (size_t)8 << kClasses[c].max_n;
        const size_t poff = (b->small_table[c].size() + 255) & ~size_t(255);
        const TileOp* ops = (const TileOp*)b->d_small_ops[c];
        const unsigned char* pool = (const unsigned char*)b->d_small_ops[c] + poff;
        const SmallItem* items = (const SmallItem*)b->d_small_items[c];
        const int cnt = (int)b->items[c].size();
        small_kernel(c, b->class_matk[c]).launch(b->grid[c], shm, bs, items, cnt, b->d_counters + c, ops, pool,
                                                 b->d_out);
        AQSG_CUDA_TRY(cudaGetLastError());
        b->kernels++;
    }
    for (size_t gi = 0; gi < b->groups.size(); ++gi) {
        const LargeGroup& gr = b->groups[gi];
        cudaStream_t bs = b->streams[(gi + 3) % b->streams.size()];
        const uint64_t amps = 1ull << gr.n;
        const int members = (int)gr.members.size();
        AQSG_CUDA_TRY(cudaMemsetAsync(gr.regs, 0, (size_t)members * amps * 8, bs));
        k_basis0_multi<<<members, 1, 0, bs>>>((float2*)gr.regs, amps);
        AQSG_CUDA_TRY(cudaGetLastError());
        const TilePlan& plan = b->plans[gr.members[0]];
        if (int rc = launch_tile_plan_multi(gr.regs, amps, members, plan, (const char*)b->d_large + gr.dev_off,
                                            gr.stride, bs, b->ctx->d_err, &b->kernels))
            return rc;
        if (int rc = launch_expz_raw_multi(gr.regs, amps, members, gr.n, gr.partials, gr.d_out_off, b->d_out, bs))
            return rc;
        b->kernels += 3;
    }
    for (size_t k = 0; k < b->large.size(); ++k) {
        if (b->grouped[k]) continue;
        const int i = b->large[k];
        const int n = b->n[i];
        const int br = branch_of_large(b, k);
        cudaStream_t bs = b->streams[br];
        void* reg = b->regs[br];
        AQSG_CUDA_TRY(cudaMemsetAsync(reg, 0, (size_t)8 << n, bs));
        k_basis0<<<1, 1, 0, bs>>>((float2*)reg);
        AQSG_CUDA_TRY(cudaGetLastError());
        const void* dev = (const char*)b->d_large + b->plan_off[k];
        if (int rc = launch_tile_plan(reg, b->plans[k], dev, bs, b->ctx->d_err, &b->kernels)) return rc;
        if (int rc = launch_expz_raw(reg, n, AQSG_C64, (double*)b->partials[br], b->d_out + b->out_off[i], bs))
            return rc;
        b->kernels += 3;
    }
    for (int k = 0; k < nb; ++k) {
        AQSG_CUDA_TRY(cudaEventRecord(b->joins[k], b->streams[k]));
        AQSG_CUDA_TRY(cudaStreamWaitEvent(s, b->joins[k], 0));
    }
    return AQSG_OK;
}

static void free_batch(aqsg_batch_s* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->host_only) {  // nothing on the device
        delete[] b->h_plans;
        delete b;
        return;
    }
    for (int c = 0; c < 3; ++c)
        if (b->d_small_items[c]) cudaFree(b->d_small_items[c]);
    if (b->d_plans) cudaFree(b->d_plans);
    if (b->h_plans) cudaFreeHost(b->h_plans);
    for (LargeGroup& gr : b->groups) {
        if (gr.regs) cudaFree(gr.regs);
        if (gr.partials) cudaFree(gr.partials);
        if (gr.d_out_off) cudaFree(gr.d_out_off);
    }
    for (void* p : b->regs)
        if (p) cudaFree(p);
    for (void* p : b->partials)
        if (p) cudaFree(p);
    for (cudaStream_t st : b->streams) cudaStreamDestroy(st);
    for (cudaEvent_t ev : b->joins) cudaEventDestroy(ev);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->d_out) cudaFree(b->d_out);
    if (b->h_out) cudaFreeHost(b->h_out);
    if (b->d_counters) cudaFree(b->d_counters);
    delete b;
}

}  // namespace aqsg

extern "C" {

int aqsg_batch_create(aqsg_ctx ctx, const aqsg_circuit* circuits, int count, aqsg_batch* out) {
    if (!ctx || !out) return set_error(AQSG_ERR_NULL, "NULL argument");
    *out = nullptr;
    if (count < 1) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Empty batch");
    if (!circuits) return set_error(AQSG_ERR_NULL, "NULL circuit list");
    AQSG_ON_DEVICE(ctx->device);
    auto* b = new aqsg_batch_s();
    b->ctx = ctx;
    if (int rc = init_shape(b, circuits, count)) {
        delete b;
        return rc;
    }
    int rc = encode_batch(b, circuits);
    auto fail = [&](int code) {
        free_batch(b);
        return code;
    };
    if (rc) return fail(rc);
    layout_batch(b);
    cudaError_t e = cudaMallocHost((void**)&b->h_plans, std::max<size_t>(b->plans_bytes, 256));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_plans, std::max<size_t>(b->plans_bytes, 256));
    if (e == cudaSuccess) {
        fill_image(b);
        for (int c = 0; c < 3; ++c)
            if (!b->items[c].empty()) b->d_small_ops[c] = (char*)b->d_plans + b->small_base[c];
        b->d_large = (char*)b->d_plans + b->large_base;
    }
    for (int c = 0; c < 3 && e == cudaSuccess; ++c) {
        if (b->items[c].empty()) continue;
        e = cudaMalloc(&b->d_small_items[c], sizeof(SmallItem) * b->items[c].size());
        if (e == cudaSuccess)
            e = cudaMemcpy(b->d_small_items[c], b->items[c].data(), sizeof(SmallItem) * b->items[c].size(),
                           cudaMemcpyHostToDevice);
    }
    for (LargeGroup& gr : b->groups) {
        if (e != cudaSuccess) break;
        const size_t members = gr.members.size();
        e = cudaMalloc(&gr.regs, members * ((size_t)8 << gr.n));
        if (e == cudaSuccess) e = cudaMalloc((void**)&gr.partials, sizeof(double) * members * expz_partial_doubles(gr.n));
        if (e == cudaSuccess) e = cudaMalloc((void**)&gr.d_out_off, sizeof(uint64_t) * members);
        if (e == cudaSuccess) {
            std::vector<uint64_t> off(members);
            for (size_t j = 0; j < members; ++j) off[j] = b->out_off[b->large[gr.members[j]]];
            e = cudaMemcpy(gr.d_out_off, off.data(), sizeof(uint64_t) * members, cudaMemcpyHostToDevice);
        }
    }
    // branch streams: three for the small classes, up to kMaxBranches overall
    int nb = 3;
    if ((int)b->large.size() + 3 > nb) nb = (int)b->large.size() + 3;
    if (nb > kMaxBranches) nb = kMaxBranches;
    b->streams.assign(nb, nullptr);
    b->joins.assign(nb, nullptr);
    b->regs.assign(nb, nullptr);
    b->partials.assign(nb, nullptr);
    for (int k = 0; k < nb && e == cudaSuccess; ++k) {
        e = cudaStreamCreateWithFlags(&b->streams[k], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->joins[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    std::vector<int> branch_max(nb, 0);
    for (size_t k = 0; k < b->large.size(); ++k) {
        if (b->grouped[k]) continue;
        const int br = branch_of_large(b, k);
        branch_max[br] = std::max(branch_max[br], b->n[b->large[k]]);
    }
    for (int k = 0; k < nb && e == cudaSuccess; ++k) {
        if (!branch_max[k]) continue;
        e = cudaMalloc(&b->regs[k], (size_t)8 << branch_max[k]);
        if (e == cudaSuccess) e = cudaMalloc(&b->partials[k], sizeof(double) * expz_partial_doubles(branch_max[k]));
    }
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_out, sizeof(double) * b->out_doubles);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&b->h_out, sizeof(double) * b->out_doubles);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_counters, 4 * sizeof(int));
    if (e != cudaSuccess) return fail(cuda_error(e, "aqsg_batch_create"));
    // persistent grids: resident CTAs per SM x SMs, at most one CTA per circuit
    for (int c = 0; c < 3; ++c) {
        if (b->items[c].empty()) continue;
        const size_t shm = (size_t)8 << kClasses[c].max_n;
        int per_sm = 1;
        const SmallKernel kern = small_kernel(c, b->class_matk[c]);
        cudaFuncSetAttribute(kern.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern.fn, kern.threads, shm);
        if (per_sm < 1) per_sm = 1;
        const int want = per_sm * ctx->sm_count;
        b->grid[c] = (int)b->items[c].size() < want ? (int)b->items[c].size() : want;
    }
    if ((rc = upload_batch(b, ctx->stream))) return fail(rc);
    // capture the run once
    e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return fail(cuda_error(e, "cudaStreamBeginCapture"));
    rc = record_batch(b, ctx->stream);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(ctx->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return fail(rc);
    }
    if (e != cudaSuccess) return fail(cuda_error(e, "cudaStreamEndCapture"));
    b->graph = g;
    e = cudaGraphInstantiate(&b->exec, g, 0);
    if (e != cudaSuccess) return fail(cuda_error(e, "cudaGraphInstantiate"));
    *out = b;
    return AQSG_OK;
}

int aqsg_batch_update(aqsg_batch b, const aqsg_circuit* circuits) {
    if (!b || !circuits) return set_error(AQSG_ERR_NULL, "NULL argument");
    AQSG_ON_DEVICE(b->ctx->device);
    // the previous run has finished reading the device image (runs end
    // with a synchronize), so the pinned image can be rewritten
    if (int rc = update_image(b, circuits)) return rc;
    return upload_batch(b, b->ctx->stream);
}

int aqsg_batch_run(aqsg_batch b, double* z, double* zz) {
    if (!b) return set_error(AQSG_ERR_NULL, "NULL batch");
    aqsg_ctx_s* c = b->ctx;
    AQSG_ON_DEVICE(c->device);
    AQSG_CUDA_TRY(cudaGraphLaunch(b->exec, c->stream));
    c->launches += b->kernels;
    AQSG_CUDA_TRY(cudaMemcpyAsync(b->h_out, b->d_out, sizeof(double) * b->out_doubles, cudaMemcpyDeviceToHost,
                                  c->stream));
    AQSG_CUDA_TRY(cudaMemcpyAsync(c->host_result, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    AQSG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (*reinterpret_cast<volatile int*>(c->host_result) != 0) {  // a tensor-core pass's bounded wait gave up
        AQSG_CUDA_TRY(cudaMemset(c->d_err, 0, sizeof(int)));
        return set_error(AQSG_ERR_TIMEOUT, "A bounded device wait gave up during the batch");
    }
    size_t zo = 0, zzo = 0;
    for (int i = 0; i < b->count; ++i) {
        const int n = b->n[i];
        const double* r = b->h_out + b->out_off[i];
        const double tot = r[2 * n - 1];
        const double inv = tot > 0 ? 1.0 / tot : 0.0;  // the register's norm, in FP64
        for (int q = 0; q < n; ++q)
            if (z) z[zo + q] = (tot - 2.0 * r[n - 1 - q]) * inv;
        for (int q = 0; q + 1 < n; ++q)
            if (zz) zz[zzo + q] = (tot - 2.0 * r[n + (n - 2 - q)]) * inv;
        zo += n;
        zzo += n - 1;
    }
    return AQSG_OK;
}

int aqsg_batch_info(aqsg_batch b, int* small_circuits, int* large_circuits, int* kernels) {
    if (!b) return set_error(AQSG_ERR_NULL, "NULL batch");
    if (small_circuits) *small_circuits = (int)(b->items[0].size() + b->items[1].size() + b->items[2].size());
    if (large_circuits) *large_circuits = (int)b->large.size();
    if (kernels) *kernels = (int)b->kernels;
    return AQSG_OK;
}

int aqsg_batch_traffic(aqsg_batch b, uint64_t* hbm_bytes) {
    if (!b || !hbm_bytes) return set_error(AQSG_ERR_NULL, "NULL argument");
    uint64_t t = 0;
    for (size_t k = 0; k < b->large.size(); ++k)
        t += 2 * ((uint64_t)8 << b->n[b->large[k]]) + plan_hbm_bytes(b->plans[k], false);
    *hbm_bytes = t;
    return AQSG_OK;
}

int aqsg_batch_tuning(aqsg_batch b, int* fuse_qubits, int* tensor_cores) {
    if (!b) return set_error(AQSG_ERR_NULL, "NULL batch");
    for (size_t k = 0; k < b->large.size(); ++k) {
        if (fuse_qubits) fuse_qubits[k] = b->fuse[k];
        if (tensor_cores) tensor_cores[k] = b->tc[k];
    }
    return AQSG_OK;
}

int aqsg_debug_batch_image(const aqsg_circuit* circuits, int count, const int* fuse, const int* tc,
                           const aqsg_circuit* update, void* image, size_t capacity, size_t* bytes) {
    if (!circuits || !bytes) return set_error(AQSG_ERR_NULL, "NULL argument");
    if (count < 1) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Empty batch");
    auto* b = new aqsg_batch_s();
    b->host_only = true;
    std::vector<int> zeros(count, 0);  // at most one large register per circuit
    b->preset_fuse = fuse ? fuse : zeros.data();
    b->preset_tc = tc ? tc : zeros.data();
    int rc = init_shape(b, circuits, count);
    if (!rc) rc = encode_batch(b, circuits);
    if (!rc) {
        layout_batch(b);
        b->h_plans = new unsigned char[std::max<size_t>(b->plans_bytes, 1)];
        fill_image(b);
        if (update) rc = update_image(b, update);
    }
    if (!rc) {
        *bytes = b->plans_bytes;
        if (image) {
            if (capacity < b->plans_bytes)
                rc = set_error(AQSG_ERR_OUT_OF_RANGE, "Image buffer too small");
            else
                std::memcpy(image, b->h_plans, b->plans_bytes);
        }
    }
    free_batch(b);
    return rc;
}

int aqsg_batch_free(aqsg_batch b) {
    if (!b) return set_error(AQSG_ERR_NULL, "NULL batch");
    DeviceScope scope(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    free_batch(b);
    return AQSG_OK;
}

}  // extern "C"
