// Shared-memory tile passes: a run of gates costs one HBM read-write pass.
//
// A tile is 2^m amplitudes: the L lowest index bits (contiguous rows of
// 2^L amplitudes, 256 B, so loads and stores stay coalesced) plus m - L
// further "high" bits chosen by the planner.  Every non-diagonal gate of a
// pass acts on tile bits only; its controls and every diagonal gate may sit
// on any bit, because bits outside the tile are constant within a tile (they
// are the tile's base index).  When n is small enough the whole register is
// one tile and the circuit runs in a single launch (the 12-qubit plain
// workload is one CTA).
//
// Consecutive diagonal gates run element-wise from registers: each thread
// keeps the same elements across the run, so the run needs no barrier and
// one shared-memory round trip.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "tile_device.cuh"

namespace aqsg {

int tile_max_bits(int dtype) { return dtype == AQSG_C64 ? 14 : 13; }
static int stream_tile_bits(int dtype) { return dtype == AQSG_C64 ? 12 : 11; }
static int row_bits(int dtype) { return dtype == AQSG_C64 ? 5 : 4; }

// EPT: elements per thread in register runs; MAXT/MINB: launch bounds (the
// whole-register variant runs up to 512 threads in one CTA, the streaming
// variant 256 threads with several CTAs per SM).  TC: fused unitaries with
// k >= 3 go through tc_apply (c64, 4096-amplitude tiles, 128 threads).
template <typename R, int EPT, int MAXT, int MINB, bool TC>
__global__ void __launch_bounds__(MAXT, MINB)
k_tile(typename Cx<R>::T* __restrict__ sv, const TileGeom g, const TileOp* __restrict__ ops,
       int nops, const unsigned char* __restrict__ pool, int* err) {
    using T = typename Cx<R>::T;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const int m = g.m, L = g.L;
    const uint32_t size = 1u << m;
    T* s = reinterpret_cast<T*>(smem_raw);
    uint64_t* rowoff = reinterpret_cast<uint64_t*>(smem_raw + sizeof(T) * size);
    const uint32_t rows = 1u << (m - L), rowlen = 1u << L;
    const int nthr = blockDim.x;

    TcShared tcs;
    uint32_t tc_phase = 0;
    if constexpr (TC) {
        // after the tile (32 KiB) and its row table (<= 1 KiB), 1 KiB aligned
        unsigned char* p = smem_raw + sizeof(T) * size + 1024;
        tcs.a = p;
        tcs.b = p + 2 * kTcABytes;
        tcs.bar = reinterpret_cast<uint64_t*>(tcs.b + 2 * kTcBBytes);
        tcs.tmem = reinterpret_cast<uint32_t*>(tcs.bar + 1);
        tcs.offr = tcs.tmem + 1;
        tcs.err = err;
        if (threadIdx.x < 32) {
            asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                         ::"r"(smem_u32(tcs.tmem)), "r"(kTcTmemCols));
            asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
        }
        if (threadIdx.x == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(tcs.bar)), "r"(1));
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }

    // base index of this tile: the block index spread over the non-tile bits
    uint64_t base = blockIdx.x;
    for (int i = 0; i < m; ++i) {
        const int b = g.tbits[i];
        const uint64_t lo = base & ((1ull << b) - 1ull);
        base = ((base - lo) << 1) | lo;
    }
    for (uint32_t r = threadIdx.x; r < rows; r += nthr) {
        uint64_t off = 0;
        for (int k = 0; k < m - L; ++k)
            if ((r >> k) & 1u) off |= 1ull << g.tbits[L + k];
        rowoff[r] = off;
    }
    __syncthreads();

    // load (128-bit accesses along rows)
    if constexpr (sizeof(R) == 4) {
        const uint32_t half = size >> 1;
        for (uint32_t i = threadIdx.x; i < half; i += nthr) {
            const uint32_t j = i << 1;
            const uint64_t gi = base + rowoff[j >> L] + (j & (rowlen - 1));
            const float4 f = __ldcs(reinterpret_cast<const float4*>(sv) + (gi >> 1));
            reinterpret_cast<float4*>(s)[i] = f;
        }
    } else {
        for (uint32_t j = threadIdx.x; j < size; j += nthr)
            s[j] = __ldcs(sv + base + rowoff[j >> L] + (j & (rowlen - 1)));
    }
    __syncthreads();

    tile_run_ops<R, EPT, TC>(s, size, base, ops, nops, pool, tcs, tc_phase);

    // store
    if constexpr (sizeof(R) == 4) {
        const uint32_t half = size >> 1;
        for (uint32_t i = threadIdx.x; i < half; i += nthr) {
            const uint32_t j = i << 1;
            const uint64_t gi = base + rowoff[j >> L] + (j & (rowlen - 1));
            __stcs(reinterpret_cast<float4*>(sv) + (gi >> 1), reinterpret_cast<const float4*>(s)[i]);
        }
    } else {
        for (uint32_t j = threadIdx.x; j < size; j += nthr)
            __stcs(sv + base + rowoff[j >> L] + (j & (rowlen - 1)), s[j]);
    }
    if constexpr (TC) {
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (threadIdx.x < 32) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                         ::"r"(*tcs.tmem), "r"(kTcTmemCols));
        }
    }
}

// ---- planner ------------------------------------------------------------------

struct Pass {
    std::vector<int> bits;  // global bits of the tile, ascending
    std::vector<const LOp*> ops;
};

static uint64_t targets_of(const LOp& o) {
    switch (o.cls) {
        case L_MAT2: case L_PERM_X: case L_PERM_OR: return 1ull << o.t0;
        case L_PERM_SWAP: return (1ull << o.t0) | (1ull << o.t1);
        case L_MATK: {
            uint64_t t = 0;
            for (int j = 0; j < o.k; ++j) t |= 1ull << o.tb[j];
            return t;
        }
        default: return 0;  // diagonal
    }
}

static std::vector<int> bits_of(uint64_t mask) {
    std::vector<int> v;
    for (int b = 0; b < 64; ++b)
        if ((mask >> b) & 1ull) v.push_back(b);
    return v;
}

// Greedy in-order grouping: a pass takes ops while the union of their target
// bits (plus the L row bits) fits in m tile bits.
static std::vector<Pass> plan(int n, int dtype, const std::vector<LOp>& ops) {
    std::vector<Pass> passes;
    const bool whole = n <= tile_max_bits(dtype);
    const int m = whole ? n : stream_tile_bits(dtype);
    const int L = whole ? n : row_bits(dtype);
    const uint64_t rowmask = (L >= 64) ? ~0ull : ((1ull << L) - 1ull);
    uint64_t S = rowmask;
    Pass cur;
    for (const LOp& o : ops) {
        const uint64_t t = targets_of(o);
        if ((S | t) != S && __builtin_popcountll(S | t) > m) {
            passes.push_back(std::move(cur));
            cur = Pass();
            S = rowmask | t;
        } else {
            S |= t;
        }
        cur.ops.push_back(&o);
        cur.bits = bits_of(S);
    }
    if (!cur.ops.empty()) passes.push_back(std::move(cur));
    // pad each pass's bit set to exactly m bits with the lowest unused bits,
    // so every tile of a pass has the same shape
    for (Pass& p : passes) {
        uint64_t s = 0;
        for (int b : p.bits) s |= 1ull << b;
        for (int b = 0; b < n && __builtin_popcountll(s) < m; ++b) s |= 1ull << b;
        p.bits = bits_of(s);
    }
    return passes;
}

static uint64_t compress(uint64_t x, const std::vector<int>& bits) {
    uint64_t r = 0;
    for (size_t i = 0; i < bits.size(); ++i)
        if ((x >> bits[i]) & 1ull) r |= 1ull << i;
    return r;
}

// Host bf16 (round to nearest even) for the tensor-core operands.
static uint16_t host_bf16(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
static float host_bf16_val(uint16_t h) {
    const uint32_t u = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// B operand of tc_apply for a fused unitary: Urf = [[Ur, -Ui], [Ui, Ur]]
// (N = K = 2D) split into bf16 hi and lo, no-swizzle K-major layout.
static void tc_operand(const std::vector<double>& mk, int k, std::vector<unsigned char>& out) {
    const uint32_t D = 1u << k, K = 2 * D, N = 2 * D;
    const size_t split = 2ull * N * K;
    const size_t at = out.size();
    out.resize(at + 2 * split, 0);
    for (uint32_t n = 0; n < N; ++n)
        for (uint32_t kk = 0; kk < K; ++kk) {
            const uint32_t r = n % D, c = kk % D;
            const double re = mk[2 * (r * D + c)], im = mk[2 * (r * D + c) + 1];
            double v;
            if (n < D) v = kk < D ? re : -im;
            else v = kk < D ? im : re;
            const uint16_t hi = host_bf16((float)v);
            const uint16_t lo = host_bf16((float)(v - (double)host_bf16_val(hi)));
            const uint32_t off = kmajor_off(n, kk, K);
            std::memcpy(&out[at + off], &hi, 2);
            std::memcpy(&out[at + split + off], &lo, 2);
        }
}

// A matrix with one non-zero per row, each 1 (a permutation), is applied on
// CUDA cores, where x * 1 + 0 * y is exact; the split-bf16 tensor-core
// product keeps only 16 significant bits of each amplitude.
static bool is_permutation(const std::vector<double>& mk, int k) {
    const int D = 1 << k;
    for (int r = 0; r < D; ++r) {
        int ones = 0;
        for (int c = 0; c < D; ++c) {
            const double re = mk[2 * (r * D + c)], im = mk[2 * (r * D + c) + 1];
            if (im != 0.0) return false;
            if (re == 1.0) ++ones;
            else if (re != 0.0) return false;
        }
        if (ones != 1) return false;
    }
    return true;
}

static void pad_to(std::vector<unsigned char>& v, size_t align) {
    v.resize((v.size() + align - 1) / align * align, 0);
}

// Encode the passes of `ops` into a table of TileOps and an operand pool.
int encode_tiled(int n, int dtype, const std::vector<LOp>& ops, bool tc_on, TilePlan* plan) {
    plan->table.clear();
    plan->pool.clear();
    plan->passes.clear();
    plan->any_tc = false;
    plan->n = n;
    plan->dtype = dtype;
    std::vector<Pass> passes = aqsg::plan(n, dtype, ops);
    const size_t tsize = sizeof(TileOp);
    for (const Pass& p : passes) {
        TilePass tp;
        std::memset(&tp, 0, sizeof(tp));
        tp.first = (uint32_t)(plan->table.size() / tsize);
        tp.m = (int)p.bits.size();
        tp.L = tp.m == n ? n : row_bits(dtype);
        for (int i = 0; i < tp.m; ++i) tp.tbits[i] = p.bits[i];
        uint64_t S = 0;
        for (int b : p.bits) S |= 1ull << b;
        std::vector<int> local(64, -1);
        for (size_t i = 0; i < p.bits.size(); ++i) local[p.bits[i]] = (int)i;
        const bool tc_pass = tc_on && dtype == AQSG_C64 && tp.m == kTcTileBits;
        for (const LOp* o : p.ops) {
            TileOp t;
            std::memset(&t, 0, sizeof(t));
            t.cls = o->cls;
            t.lt0 = o->t0 >= 0 ? local[o->t0] : -1;
            t.lt1 = o->t1 >= 0 ? local[o->t1] : -1;
            t.ext_t = -1;
            if (o->cls == L_DIAG2 && t.lt0 < 0) t.ext_t = o->t0;
            t.k = o->k;
            for (int j = 0; j < o->k; ++j) t.ltb[j] = local[o->tb[j]];
            t.cm_loc = compress(o->cmask & S, p.bits);
            t.cv_loc = compress(o->cval & S, p.bits);
            t.cm_ext = o->cmask & ~S;
            t.cv_ext = o->cval & ~S;
            t.am_loc = compress(o->amask & S, p.bits);
            t.am_ext = o->amask & ~S;
            for (int e = 0; e < 8; ++e) t.m[e] = o->m[e];
            if (o->cls == L_MATK) {
                pad_to(plan->pool, 256);
                t.mat = (int32_t)plan->pool.size();
                if (tc_pass && o->k >= 3 && t.cm_loc == 0 && !is_permutation(o->mk, o->k)) {
                    t.pad = 1;  // tensor-core op
                    tp.tc = 1;
                    tc_operand(o->mk, o->k, plan->pool);
                } else {
                    const int D = 1 << o->k;
                    const size_t esz = dtype == AQSG_C64 ? 8 : 16;
                    for (int e = 0; e < D * D; ++e) {
                        const size_t at = plan->pool.size();
                        plan->pool.resize(at + esz);
                        if (dtype == AQSG_C64) {
                            const float v[2] = {(float)o->mk[2 * e], (float)o->mk[2 * e + 1]};
                            std::memcpy(&plan->pool[at], v, 8);
                        } else {
                            std::memcpy(&plan->pool[at], &o->mk[2 * e], 16);
                        }
                    }
                }
            }
            const size_t at = plan->table.size();
            plan->table.resize(at + tsize);
            std::memcpy(&plan->table[at], &t, tsize);
        }
        tp.count = (uint32_t)(plan->table.size() / tsize) - tp.first;
        plan->any_tc = plan->any_tc || tp.tc;
        plan->passes.push_back(tp);
    }
    return AQSG_OK;
}

size_t TilePlan::pool_offset() const { return (table.size() + 255) & ~size_t(255); }

template <typename R>
static int launch_plan_t(void* sv, const TilePlan& plan, const void* dev, cudaStream_t stream, int* d_err,
                         uint64_t* launches) {
    using T = typename Cx<R>::T;
    const int n = plan.n;
    const TileOp* dops = (const TileOp*)dev;
    const unsigned char* dpool = (const unsigned char*)dev + plan.pool_offset();
    constexpr int EPT_WHOLE = sizeof(R) == 4 ? 32 : 16;  // 2^14 / 512, 2^13 / 512
    constexpr int EPT_STREAM = sizeof(R) == 4 ? 16 : 8;  // 2^12 / 256, 2^11 / 256
    auto kwhole = k_tile<R, EPT_WHOLE, 512, 1, false>;
    auto kstream = k_tile<R, EPT_STREAM, 256, 3, false>;
    auto ktc = k_tile<float, 32, kTcThreads, 1, true>;
    const int max_shm = (int)(sizeof(T) << tile_max_bits(plan.dtype)) + 512 * 8;
    AQSG_CUDA_TRY(cudaFuncSetAttribute(kwhole, cudaFuncAttributeMaxDynamicSharedMemorySize, max_shm));
    // tile + row table (1 KiB) + A hi/lo + B hi/lo + barrier, tmem slot, row offsets
    const int tc_shm = (int)((8u << kTcTileBits) + 1024 + 2 * kTcABytes + 2 * kTcBBytes + 256);
    if (plan.any_tc)
        AQSG_CUDA_TRY(cudaFuncSetAttribute(ktc, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_shm));
    for (const TilePass& p : plan.passes) {
        TileGeom geo;
        std::memset(&geo, 0, sizeof(geo));
        geo.n = n;
        geo.m = p.m;
        geo.L = p.L;
        for (int i = 0; i < p.m; ++i) geo.tbits[i] = p.tbits[i];
        const uint32_t size = 1u << geo.m;
        const size_t rows = size_t(1) << (geo.m - geo.L);
        const size_t shm = sizeof(T) * size + rows * sizeof(uint64_t);
        const unsigned grid = (unsigned)(1ull << (n - geo.m));
        if (p.tc) {
            ktc<<<grid, kTcThreads, tc_shm, stream>>>((float2*)sv, geo, dops + p.first, (int)p.count, dpool, d_err);
        } else if (geo.m == n) {
            int threads = (int)(size / EPT_WHOLE);
            threads = threads < 32 ? 32 : (threads > 512 ? 512 : threads);
            kwhole<<<grid, threads, shm, stream>>>((T*)sv, geo, dops + p.first, (int)p.count, dpool, nullptr);
        } else {
            kstream<<<grid, 256, shm, stream>>>((T*)sv, geo, dops + p.first, (int)p.count, dpool, nullptr);
        }
        if (launches) ++*launches;
        AQSG_CUDA_TRY(cudaGetLastError());
    }
    return AQSG_OK;
}

int launch_tile_plan(void* sv, const TilePlan& plan, const void* dev, cudaStream_t stream, int* d_err,
                     uint64_t* launches) {
    return plan.dtype == AQSG_C64 ? launch_plan_t<float>(sv, plan, dev, stream, d_err, launches)
                                  : launch_plan_t<double>(sv, plan, dev, stream, d_err, launches);
}

int run_tiled(aqsg_state_s* st, const std::vector<LOp>& ops) {
    aqsg_ctx_s* c = st->ctx;
    TilePlan plan;
    if (int rc = encode_tiled(st->n, st->dtype, ops, c->tensor_cores != 0, &plan)) return rc;
    if (plan.passes.empty()) return AQSG_OK;
    const size_t poff = plan.pool_offset();
    if (int rc = ensure_scratch(c->ops, poff + plan.pool.size() + 16)) return rc;
    AQSG_CUDA_TRY(cudaMemcpyAsync(c->ops.ptr, plan.table.data(), plan.table.size(), cudaMemcpyHostToDevice,
                                  c->stream));
    if (!plan.pool.empty())
        AQSG_CUDA_TRY(cudaMemcpyAsync((char*)c->ops.ptr + poff, plan.pool.data(), plan.pool.size(),
                                      cudaMemcpyHostToDevice, c->stream));
    // The tensor-core products lose a little norm in a biased way (~1e-7 per
    // fused op); a run that uses them restores the input's FP64 norm at the
    // end (one read pass before, one read and one scale pass after).
    double norm_before = 0;
    if (plan.any_tc)
        if (int rc = reduce_prob(st, 0, 0, &norm_before)) return rc;
    if (int rc = launch_tile_plan(st->d, plan, c->ops.ptr, c->stream, c->d_err, &c->launches)) return rc;
    if (plan.any_tc) {  // a tensor-core wait that gave up leaves a flag
        AQSG_CUDA_TRY(cudaMemcpyAsync(c->host_result, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        AQSG_CUDA_TRY(cudaStreamSynchronize(c->stream));
        int flag = 0;
        std::memcpy(&flag, c->host_result, sizeof(int));
        if (flag) {
            AQSG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
            return set_error(AQSG_ERR_TIMEOUT, "Tensor-core tile pass timed out waiting for its MMAs");
        }
        double norm_after = 0;
        if (int rc = reduce_prob(st, 0, 0, &norm_after)) return rc;
        if (norm_after > 0 && norm_before > 0)
            if (int rc = launch_scale(st, std::sqrt(norm_before / norm_after))) return rc;
    }
    return AQSG_OK;
}

int run_plan_async(aqsg_state_s* st, const TilePlan& plan, const void* dev_table, double* d_norms) {
    aqsg_ctx_s* c = st->ctx;
    if (plan.passes.empty()) return AQSG_OK;
    if (plan.any_tc)
        if (int rc = launch_norm_to_device(st, d_norms)) return rc;
    if (int rc = launch_tile_plan(st->d, plan, dev_table, c->stream, c->d_err, &c->launches)) return rc;
    if (plan.any_tc) {
        if (int rc = launch_norm_to_device(st, d_norms + 1)) return rc;
        if (int rc = launch_renorm_device(st, d_norms, d_norms + 1)) return rc;
    }
    return AQSG_OK;
}

}  // namespace aqsg
