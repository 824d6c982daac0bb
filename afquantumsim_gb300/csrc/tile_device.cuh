// Device side of the shared-memory tile engine, shared by the tile passes
// (tile_kernels.cu) and the batched engine (batch.cu): the per-tile op table
// format, the op interpreter and the tensor-core (tcgen05) fused-unitary path.
#pragma once

#include <cuda_bf16.h>

#include <type_traits>

#include "aqsg_internal.h"
#include "common.cuh"

namespace aqsg {

struct TileOp {
    int32_t cls;
    int32_t lt0, lt1;  // local target bits; DIAG2 with an external target: lt0 = -1
    int32_t k;
    int32_t ltb[AQSG_MAX_UNITARY_QUBITS];
    int32_t mat;       // MATK: byte offset of its matrix (or tensor-core operand) in the pool
    int32_t ext_t;     // DIAG2 external target: global bit, else -1
    int32_t pad;       // MATK: 1 = apply on the tensor cores
    uint64_t cm_loc, cv_loc, cm_ext, cv_ext, am_loc, am_ext;
    double m[8];
};

struct TileGeom {
    int n, m, L;
    int tbits[16];      // global bit of each local bit, ascending; tbits[i] = i for i < L
    uint32_t tc_blob;   // tensor-core passes: pool offset and size of the operand blob
    uint32_t tc_bytes;
};

__device__ __forceinline__ uint32_t ins0(uint32_t p, int b) {
    return ((p >> b) << (b + 1)) | (p & ((1u << b) - 1u));
}

template <typename T>
__device__ __forceinline__ T ld_coef(const double* m, int i) {
    T t;
    t.x = m[2 * i];
    t.y = m[2 * i + 1];
    return t;
}

// Position of tile element j in shared memory: the identity, or rows of 2^L
// elements followed by PAD elements of padding.  The streaming passes keep
// 256-byte rows at a 288-byte stride, so elements of different rows that
// share their low index bits fall into different shared-memory banks.
template <int L, int PAD>
struct TileLay {
    static __device__ __forceinline__ uint32_t at(uint32_t j) { return PAD ? j + (j >> L) * (uint32_t)PAD : j; }
};
using FlatLay = TileLay<0, 0>;

// Barrier among the threads that run a tile's ops: the whole CTA, or (in a
// warp-specialised kernel) one compute group (GroupSync below).
struct CtaSync {
    static __device__ __forceinline__ void sync() { __syncthreads(); }
};
// Barrier among the N threads of this thread's compute group (aligned
// blocks of N threads; group q uses named barrier 1 + q), for warp-
// specialised kernels whose groups each run their own tile.
template <int N>
struct GroupSync {
    static __device__ __forceinline__ void sync() {
        asm volatile("bar.sync %0, %1;" ::"r"(1u + threadIdx.x / (uint32_t)N), "n"(N) : "memory");
    }
};

// Index of this thread among the nthr threads (a power of two) that run a
// tile's ops: compute groups are aligned blocks of nthr threads.
__device__ __forceinline__ uint32_t tile_tid(uint32_t nthr) { return threadIdx.x & (nthr - 1u); }

// ---- asynchronous copies and barriers (sm_90+ bulk copies, mbarriers) -----------

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ uint32_t mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok;
}

// Wait for the phase of `bar` with the given parity, at most kWaitNs of
// waiting (for winding down: copies or MMAs already issued must land before
// the shared or tensor memory goes, whatever the error flag says).
__device__ __forceinline__ bool mbar_wait_timeout(uint64_t* bar, uint32_t parity) {
    WaitClock clk;
    for (uint32_t it = 0;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63u) == 63u && clk.expired()) return false;
    }
}

// Wait for the phase of `bar` with the given parity; gives up after kWaitNs
// of waiting, or early once the device error flag is set.  Returns whether
// the phase completed.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, const int* err) {
    WaitClock clk;
    for (uint32_t it = 0;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63u) == 63u && (clk.expired() || *(volatile const int*)err != 0)) return false;
    }
}

// global -> shared bulk copy completing on `bar` (bytes: multiple of 16,
// both addresses 16-byte aligned)
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

// 16-byte global -> shared copy (cp.async, L2 only); completion is tracked
// by cp_async_arrive on an mbarrier
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
// one arrival on `bar` once this thread's earlier cp.async copies have landed
// (the barrier's expected count includes it)
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void cp_async_arrive(uint64_t* bar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// order this thread's shared-memory writes before later async-proxy accesses
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- tensor-core path (tcgen05) for fused 3..5-qubit unitaries -----------------
//
// On a 4096-amplitude c64 tile, a fused unitary U (D x D, D = 2^k) on k tile
// bits is Y = U X with X the tile viewed as D rows (the target bits) by
// C = 4096 / D columns (the other bits).  In real form, with the complex
// components interleaved (index 2r = real part of row r, 2r + 1 = imaginary
// part),
//   Y[2r]   = sum_c Ur[r][c] X[2c] - Ui[r][c] X[2c+1]
//   Y[2r+1] = sum_c Ui[r][c] X[2c] + Ur[r][c] X[2c+1].
// With the data as the M side, D_tmem[col][n] = sum_kk A[col][kk] B[n][kk]
// where A[col][kk] = X[kk] of data column col (M = 128 columns per block,
// K = 2D) and B is the real form above (N = 2D).  Both operands are split
// into BF16 hi + lo parts; D = Ahi Bhi + Ahi Blo + Alo Bhi accumulates in
// FP32 in tensor memory (the dropped Alo Blo term is ~2^-18 relative).
// A sits in tensor memory (one data column per TMEM lane, one amplitude per
// 32-bit column: the interleaved K order lets one bf16x2 conversion turn an
// amplitude into one operand word); B sits in shared memory in the
// no-swizzle K-major canonical layout: 8 x 16-byte core matrices,
// K-direction stride 128 B, N-direction stride (K/8) * 128 B.

constexpr int kTcTileBits = 12;
constexpr int kTcThreads = 768;                    // compute threads: 24 warps in 3 groups of 8
constexpr uint32_t kTcTmemCols = 128;              // per compute group: A hi, A lo, D (32 + 32 + 64)
// A pass's tensor-core operands (per op: B hi and lo splits, then the index
// tables) are loaded into shared memory once per CTA; at most this many bytes
// (three 5-qubit unitaries: 3 x 17 KiB).
constexpr uint32_t kTcBlobMax = 52u * 1024u;

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= 1ull << 46;  // descriptor version of tcgen05; base offset 0, no swizzle
    return d;
}

// kind::f16 instruction descriptor: D f32, A and B bf16, both K-major.
__host__ __device__ constexpr uint32_t tc_idesc(uint32_t M, uint32_t N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(smem_u32(bar)) : "memory");
}

// 32 lanes x 16 columns of 32-bit words; the caller waits (tc_ld_wait)
__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
          "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
          "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tc_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Byte offset of element (row, kk) in a no-swizzle K-major operand with
// K elements per row.
__host__ __device__ __forceinline__ uint32_t kmajor_off(uint32_t row, uint32_t kk, uint32_t K) {
    return ((row >> 3) * (K >> 3) + (kk >> 3)) * 128u + (row & 7u) * 16u + (kk & 7u) * 2u;
}

struct TcSmem {
    const unsigned char* blob;  // the pass's operands; an op's B hi at blob + op.mat
    uint64_t* mma_bar;     // MMAs done
    uint32_t tmem;         // tensor-memory base address (kTcTmemCols columns)
    int* err;              // device error flag
};

struct TcPhase {
    uint32_t mma = 0;
};

// ---- fused unitaries with the data operand in tensor memory ---------------------
//
// Each thread gathers the amplitudes of one data column (its TMEM lane = the
// MMA's M row) from the tile, splits them into BF16 hi and lo and stores
// them to its lane with tcgen05.st; the MMAs read A from tensor memory and B
// from the pass's operand blob, so the operand never makes a round trip
// through shared memory.  A compute
// group of 8 warps owns 128 TMEM columns: A hi at [0, 32), A lo at [32, 64)
// (block b of the data columns at 32-bit column b * D, one column per
// matrix row r = the (re, im) BF16 pair of K indices 2r, 2r + 1), and the
// FP32 accumulators D at [64, 128) (block b at 64 + b * N).
//
// Thread (warp w, lane l) of the group: lane quarter q = w % 4, half
// h = w / 4, M row 32 q + l of block b (b = 0 for 5 qubits, b = h for 4, b
// = h and h + 2 for 3); it gathers rows [r0, r0 + RPT) of that column (r0 =
// 16 h for 5 qubits, else 0) and later writes back the same amplitudes, so
// no two threads touch one amplitude within an op.  The host orders the
// data columns (colbase) so that the 32 lanes of a warp spread over the
// shared-memory banks.

__device__ __forceinline__ void tc_st16(uint32_t taddr, const uint32_t* r) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
        "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
        ::"r"(taddr), "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
          "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
        : "memory");
}
__device__ __forceinline__ void tc_st8(uint32_t taddr, const uint32_t* r) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
                 ::"r"(taddr), "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]),
                   "r"(r[7])
                 : "memory");
}
__device__ __forceinline__ void tc_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// D (+)= A B with A in tensor memory (a_tmem), B in shared memory (desc)
__device__ __forceinline__ void tc_mma_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}"
        ::"r"(d_tmem), "r"(a_tmem), "l"(b), "r"(idesc), "r"(accumulate));
}

template <class LAY, class SYNC, int KQ>
__device__ __forceinline__ void tc_apply_tm(float2* s, const TileOp& op, const TcSmem& t, TcPhase& ph) {
    static_assert(std::is_same<LAY, TileLay<5, 2>>::value, "the index tables are byte offsets in 272-byte rows");
    constexpr uint32_t D = 1u << KQ, K = 2u * D, N = 2u * D;
    constexpr uint32_t blocks = 1u << (kTcTileBits - KQ - 7);  // 1, 2, 4 blocks of 128 data columns
    constexpr uint32_t bsplit = 2u * N * K;
    constexpr uint32_t RPT = KQ == 3 ? 8u : 16u;               // matrix rows per thread and block
    constexpr uint32_t BPT = KQ == 3 ? 2u : 1u;                // blocks per thread
    static_assert(blocks * D == 32u, "A hi and lo take 32 columns each");
    const uint32_t tid = threadIdx.x & 255u, w = tid >> 5, lane = tid & 31u;
    const uint32_t q = w & 3u, h = w >> 2;
    const unsigned char* bsm = t.blob + op.mat;
    // byte offsets in the padded tile (the layout is additive over disjoint
    // index bits, so a data column's offset plus a matrix row's is the
    // amplitude's): colbase[c], offr[r]
    const uint16_t* colbase = reinterpret_cast<const uint16_t*>(bsm + 2u * bsplit);
    const uint16_t* offr = colbase + 512;
    unsigned char* sb = reinterpret_cast<unsigned char*>(s);
    const uint32_t lane_base = t.tmem + ((32u * q) << 16);
    const uint32_t r0 = KQ == 5 ? 16u * h : 0u;

    uint32_t jb[BPT], bk[BPT];
#pragma unroll
    for (uint32_t i = 0; i < BPT; ++i) {
        bk[i] = KQ == 5 ? 0u : (KQ == 4 ? h : h + 2u * i);
        jb[i] = colbase[128u * bk[i] + 32u * q + lane];
    }
#pragma unroll
    for (uint32_t i = 0; i < BPT; ++i) {
        uint32_t hi[RPT], lo[RPT];
#pragma unroll
        for (uint32_t e = 0; e < RPT; ++e) {
            const float2 x = *reinterpret_cast<const float2*>(sb + jb[i] + offr[r0 + e]);
            const __nv_bfloat162 bh = __float22bfloat162_rn(x);
            const float2 hf = __bfloat1622float2(bh);
            const __nv_bfloat162 bl = __float22bfloat162_rn(make_float2(x.x - hf.x, x.y - hf.y));
            hi[e] = *reinterpret_cast<const uint32_t*>(&bh);
            lo[e] = *reinterpret_cast<const uint32_t*>(&bl);
        }
        const uint32_t col = bk[i] * D + r0;
        if constexpr (RPT == 16) {
            tc_st16(lane_base + col, hi);
            tc_st16(lane_base + 32u + col, lo);
        } else {
            tc_st8(lane_base + col, hi);
            tc_st8(lane_base + 32u + col, lo);
        }
    }
    tc_st_wait();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    SYNC::sync();

    if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t idesc = tc_idesc(128, N);
        constexpr uint32_t sbo = (K / 8u) * 128u;
        const uint32_t b_hi = smem_u32(bsm), b_lo = b_hi + bsplit;
#pragma unroll
        for (uint32_t blk = 0; blk < blocks; ++blk) {
            const uint32_t dcol = t.tmem + 64u + blk * N;
            const uint32_t a_hi = t.tmem + blk * D, a_lo = a_hi + 32u;
#pragma unroll
            for (uint32_t st = 0; st < K / 16u; ++st) {
                const uint32_t ko = st * 256u;  // two core matrices of B along K
                tc_mma_ta(dcol, a_hi + 8u * st, tc_desc(b_hi + ko, 128u, sbo), idesc, st > 0 ? 1u : 0u);
                tc_mma_ta(dcol, a_hi + 8u * st, tc_desc(b_lo + ko, 128u, sbo), idesc, 1u);
                tc_mma_ta(dcol, a_lo + 8u * st, tc_desc(b_hi + ko, 128u, sbo), idesc, 1u);
            }
        }
        tc_commit(t.mma_bar);
    }
    if (!mbar_wait_bounded(t.mma_bar, ph.mma, t.err)) atomicExch(t.err, 1);
    ph.mma ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    // D back to the amplitudes this thread gathered: output row r0 + e of
    // block bk is D columns 2 (r0 + e) and 2 (r0 + e) + 1
#pragma unroll
    for (uint32_t i = 0; i < BPT; ++i) {
        const uint32_t dbase = lane_base + 64u + bk[i] * N + 2u * r0;
        // all of a block's accumulator columns in one load and one wait
        uint32_t v[2u * RPT];
        if constexpr (RPT == 16) tc_ld32(dbase, v);
        else tc_ld16(dbase, v);
        tc_ld_wait();
#pragma unroll
        for (uint32_t e = 0; e < RPT; ++e)
            *reinterpret_cast<float2*>(sb + jb[i] + offr[r0 + e]) =
                make_float2(__uint_as_float(v[2 * e]), __uint_as_float(v[2 * e + 1]));
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    SYNC::sync();
}

// One fused unitary of 3..5 qubits on the tile through the tensor cores; all
// 256 threads of the compute group (8 warps) call it.
template <class LAY, class SYNC, int WARPS>
__device__ __forceinline__ void tc_apply(float2* s, const TileOp& op, const TcSmem& t, TcPhase& ph) {
    static_assert(WARPS == 8, "compute groups of 8 warps");
    switch (op.k) {
        case 3: tc_apply_tm<LAY, SYNC, 3>(s, op, t, ph); break;
        case 4: tc_apply_tm<LAY, SYNC, 4>(s, op, t, ph); break;
        default: tc_apply_tm<LAY, SYNC, 5>(s, op, t, ph); break;
    }
}

// k-qubit dense unitary on CUDA cores: each thread updates one group of 2^K
// amplitudes, with the group in registers.  Not inlined, so the registers
// the group needs do not weigh on the passes that never use it.
template <typename T, int K, class LAY>
__device__ __noinline__ void matk_apply(T* s, uint32_t size, uint32_t nthr, const TileOp& op,
                                        const T* __restrict__ mat, uint32_t cm, uint32_t cv) {
    constexpr int D = 1 << K;
    int srt[K];
#pragma unroll
    for (int i = 0; i < K; ++i) srt[i] = op.ltb[i];
#pragma unroll
    for (int i = 1; i < K; ++i)
#pragma unroll
        for (int q = i; q > 0; --q)
            if (srt[q - 1] > srt[q]) {
                const int x = srt[q];
                srt[q] = srt[q - 1];
                srt[q - 1] = x;
            }
    uint32_t tb[K];  // tile bit of matrix-row bit K-1-i
#pragma unroll
    for (int i = 0; i < K; ++i) tb[i] = 1u << op.ltb[i];
    auto off_of = [&](int r) {
        uint32_t off = 0;
#pragma unroll
        for (int i = 0; i < K; ++i)
            if ((r >> (K - 1 - i)) & 1) off |= tb[i];
        return off;
    };
    // G groups per thread and step share each matrix element load (small K)
    constexpr int G = K <= 3 ? 2 : 1;
    const uint32_t groups = size >> K;
    for (uint32_t p0 = tile_tid(nthr); p0 < groups; p0 += G * nthr) {
        uint32_t jg[G];
        bool on[G];
        T v[G][D];
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const uint32_t p = p0 + g * nthr;
            uint32_t j = p;
#pragma unroll
            for (int i = 0; i < K; ++i) j = ins0(j, srt[i]);
            jg[g] = j;
            on[g] = p < groups && (j & cm) == cv;
#pragma unroll
            for (int r = 0; r < D; ++r) v[g][r] = on[g] ? s[LAY::at(j | off_of(r))] : T{};
        }
#pragma unroll 1
        for (int r = 0; r < D; ++r) {
            T acc[G];
#pragma unroll
            for (int g = 0; g < G; ++g) {
                acc[g].x = 0;
                acc[g].y = 0;
            }
#pragma unroll
            for (int c = 0; c < D; ++c) {
                const T mm = mat[r * D + c];
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    cmac(acc[g], mm, v[g][c]);
                }
            }
            uint32_t off = 0;
            for (int i = 0; i < K; ++i)
                if ((r >> (K - 1 - i)) & 1) off |= tb[i];
#pragma unroll
            for (int g = 0; g < G; ++g)
                if (on[g]) s[LAY::at(jg[g] | off)] = acc[g];
        }
    }
}

// ---- register phases -------------------------------------------------------------
//
// A register phase applies a run of ops with one shared-memory round trip:
// the tile is split into slots of 2^RB amplitudes that differ only in the
// phase's RB register bits; a thread loads a slot into registers, applies
// every op of the run to it and stores it back.  Ops whose target bits are
// register bits (2x2 gates, permutations, dense unitaries of 2 or 3 qubits)
// act within the slot; diagonal ops act on any bits.  A control on the
// slot's other bits is one test per thread; a control on register bits is a
// mask of slot elements the host precomputes.
//
// Table layout: a header TileOp (cls T_RPHASE, k = ops in the run, lt0 = RB,
// am_loc = tile position of each register bit, cm_loc = tile position of
// each slot-index bit, 4 bits each), then k ROps in TileOp-sized slots.
enum TileCls : int { T_RPHASE = 8 };

enum RKind : uint32_t {
    RK_MAT2C = 1,  // complex 2x2 on register bit a: coefficients c[0..3]
    RK_MAT2R = 2,  // real 2x2 on register bit a: coefficients r[0..3] (floats of the kernel's type)
    RK_PERM = 3,   // swap the pairs on register bit a (PERM_X / PERM_OR)
    RK_SWAP = 4,   // exchange register bits a < b
    RK_DIAG = 5,   // multiply by c[0], or by c[1] where a target outside the register bits is 1
    RK_DIAGR = 6,  // multiply by c[0] / c[1] where register bit a is 0 / 1
    RK_MATK = 7    // 2^k x 2^k unitary (k = 2, 3) on the register bits of mask a (bits 8-15)
};
constexpr uint32_t RF_EXT = 1u << 16;   // controls outside the tile (cm_ext / cv_ext)
constexpr uint32_t RF_OR = 1u << 17;    // RK_PERM: OR condition (PERM_OR)
constexpr uint32_t RF_TTHR = 1u << 18;  // RK_DIAG: target = slot-index position `extra`
constexpr uint32_t RF_TEXT = 1u << 19;  // RK_DIAG: target = bit ext_t outside the tile

struct ROp {
    uint32_t code;    // kind | a << 8 | b << 12 | flags
    uint32_t ctl;     // control on slot-index bits: tile-position mask (bits 0-15), value (16-31)
    uint32_t em;      // slot elements (the pair's / group's element with target bits 0) whose
                      // register-bit control holds (bits 0-15); RK_PERM: OR mask (16-31)
    uint32_t extra;   // RK_MATK: pool offset of the matrix; RK_DIAG: target position
    uint64_t cm_ext, cv_ext, am_ext;
    int32_t ext_t;    // RK_DIAG with RF_TEXT: global target bit
    uint32_t amt;     // RK_PERM with RF_OR: OR mask on slot-index bits (tile positions)
    unsigned char coef[112];  // 16-byte aligned; complex values of the kernel's type
};
static_assert(sizeof(ROp) == sizeof(TileOp), "register ops overlay the op table");

// Shared-memory position of tile element j with the low S bits XORed with
// the XOR of the higher S-bit groups: the 2^S elements a half warp (c64,
// S = 4) or a quarter warp (c128, S = 3) touches at once fall into distinct
// banks whenever their varying index bits have distinct residues mod S.
// The map is linear over GF(2).
template <int S>
struct SwzLay {
    static __device__ __forceinline__ uint32_t at(uint32_t j) {
        uint32_t f = 0;
#pragma unroll
        for (int sh = S; sh < 16; sh += S) f ^= j >> sh;
        return j ^ (f & ((1u << S) - 1u));
    }
};

template <bool P>
__device__ __forceinline__ bool r_on(uint32_t em, int e) {
    return !P || ((em >> e) & 1u);
}

// In-place updates of register-held amplitudes, written as PTX whose
// outputs are tied to their inputs.  Each op of a register phase rewrites
// the same 2^RB registers; written as plain expressions, the compiler put
// an op's results in fresh registers and copied them back before the next
// op (MOV/IMAD moves were ~40 % of a pass's instructions).  The arithmetic
// is the same: products rounded once, sums fused (mul.rn + fma.rn).
//
// (a, b) <- (m00 a + m01 b, m10 a + m11 b) on one real component
__device__ __forceinline__ void ip_rot(float& a, float& b, float m00, float m01, float m10, float m11) {
    asm("{\n\t.reg .f32 t0, t1;\n\t"
        "mul.rn.f32 t0, %3, %1;\n\t"
        "mul.rn.f32 t1, %4, %0;\n\t"
        "fma.rn.f32 %0, %2, %0, t0;\n\t"
        "fma.rn.f32 %1, %5, %1, t1;\n\t}"
        : "+f"(a), "+f"(b)
        : "f"(m00), "f"(m01), "f"(m10), "f"(m11));
}
__device__ __forceinline__ void ip_rot(double& a, double& b, double m00, double m01, double m10, double m11) {
    asm("{\n\t.reg .f64 t0, t1;\n\t"
        "mul.rn.f64 t0, %3, %1;\n\t"
        "mul.rn.f64 t1, %4, %0;\n\t"
        "fma.rn.f64 %0, %2, %0, t0;\n\t"
        "fma.rn.f64 %1, %5, %1, t1;\n\t}"
        : "+d"(a), "+d"(b)
        : "d"(m00), "d"(m01), "d"(m10), "d"(m11));
}
// (x + iy) <- (px + i py)(x + iy); npy = -py
__device__ __forceinline__ void ip_cmul(float& x, float& y, float px, float py, float npy) {
    asm("{\n\t.reg .f32 t0, t1;\n\t"
        "mul.rn.f32 t0, %4, %1;\n\t"
        "mul.rn.f32 t1, %3, %0;\n\t"
        "fma.rn.f32 %0, %2, %0, t0;\n\t"
        "fma.rn.f32 %1, %2, %1, t1;\n\t}"
        : "+f"(x), "+f"(y)
        : "f"(px), "f"(py), "f"(npy));
}
__device__ __forceinline__ void ip_cmul(double& x, double& y, double px, double py, double npy) {
    asm("{\n\t.reg .f64 t0, t1;\n\t"
        "mul.rn.f64 t0, %4, %1;\n\t"
        "mul.rn.f64 t1, %3, %0;\n\t"
        "fma.rn.f64 %0, %2, %0, t0;\n\t"
        "fma.rn.f64 %1, %2, %1, t1;\n\t}"
        : "+d"(x), "+d"(y)
        : "d"(px), "d"(py), "d"(npy));
}
// exchange a and b; where c only.  Written as XOR exchanges, which keep
// both values in their registers: a permuting op then needs no copies in
// the paths of the other ops of a register phase.
__device__ __forceinline__ void ip_swap(float& a, float& b) {
    asm("{\n\txor.b32 %0, %0, %1;\n\txor.b32 %1, %1, %0;\n\txor.b32 %0, %0, %1;\n\t}" : "+f"(a), "+f"(b));
}
__device__ __forceinline__ void ip_swap(double& a, double& b) {
    asm("{\n\txor.b64 %0, %0, %1;\n\txor.b64 %1, %1, %0;\n\txor.b64 %0, %0, %1;\n\t}" : "+d"(a), "+d"(b));
}
// m: all ones to exchange, zero to keep
__device__ __forceinline__ void ip_cswap(float& a, float& b, bool c) {
    const uint32_t m = 0u - (uint32_t)c;
    asm("{\n\t.reg .b32 d;\n\txor.b32 d, %0, %1;\n\tand.b32 d, d, %2;\n\t"
        "xor.b32 %0, %0, d;\n\txor.b32 %1, %1, d;\n\t}"
        : "+f"(a), "+f"(b)
        : "r"(m));
}
__device__ __forceinline__ void ip_cswap(double& a, double& b, bool c) {
    const uint64_t m = 0ull - (uint64_t)c;
    asm("{\n\t.reg .b64 d;\n\txor.b64 d, %0, %1;\n\tand.b64 d, d, %2;\n\t"
        "xor.b64 %0, %0, d;\n\txor.b64 %1, %1, d;\n\t}"
        : "+d"(a), "+d"(b)
        : "l"(m));
}
template <typename T>
__device__ __forceinline__ void ip_swap2(T& a, T& b) {
    ip_swap(a.x, b.x);
    ip_swap(a.y, b.y);
}
template <typename T>
__device__ __forceinline__ void ip_cswap2(T& a, T& b, bool c) {
    ip_cswap(a.x, b.x, c);
    ip_cswap(a.y, b.y, c);
}

// complex 2x2: (a, b) <- (m00 a + m01 b, m10 a + m11 b).  Every output
// needs every input, so three terms of each output go to a temporary first
// and each output's last term is the one with its own input.
// q = {m00.x, m00.y, m01.x, m01.y, m10.x, m10.y, m11.x, m11.y},
// nq = {-m00.y, -m01.y, -m10.y, -m11.y}.
#define AQSG_IP_CMAT2_BODY(TY)                                               \
    "{\n\t.reg ." TY " ax, ay, bx, by;\n\t"                                  \
    "mul.rn." TY " ax, %6, %2;\n\t"                                          \
    "fma.rn." TY " ax, %13, %3, ax;\n\t"                                     \
    "fma.rn." TY " ax, %12, %1, ax;\n\t"                                     \
    "mul.rn." TY " ay, %6, %3;\n\t"                                          \
    "fma.rn." TY " ay, %7, %2, ay;\n\t"                                      \
    "fma.rn." TY " ay, %5, %0, ay;\n\t"                                      \
    "mul.rn." TY " bx, %8, %0;\n\t"                                          \
    "fma.rn." TY " bx, %14, %1, bx;\n\t"                                     \
    "fma.rn." TY " bx, %15, %3, bx;\n\t"                                     \
    "mul.rn." TY " by, %8, %1;\n\t"                                          \
    "fma.rn." TY " by, %9, %0, by;\n\t"                                      \
    "fma.rn." TY " by, %11, %2, by;\n\t"                                     \
    "fma.rn." TY " %0, %4, %0, ax;\n\t"                                      \
    "fma.rn." TY " %1, %4, %1, ay;\n\t"                                      \
    "fma.rn." TY " %2, %10, %2, bx;\n\t"                                     \
    "fma.rn." TY " %3, %10, %3, by;\n\t}"
__device__ __forceinline__ void ip_cmat2(float2& a, float2& b, const float (&q)[8], const float (&nq)[4]) {
    asm(AQSG_IP_CMAT2_BODY("f32")
        : "+f"(a.x), "+f"(a.y), "+f"(b.x), "+f"(b.y)
        : "f"(q[0]), "f"(q[1]), "f"(q[2]), "f"(q[3]), "f"(q[4]), "f"(q[5]), "f"(q[6]), "f"(q[7]), "f"(nq[0]),
          "f"(nq[1]), "f"(nq[2]), "f"(nq[3]));
}
__device__ __forceinline__ void ip_cmat2(double2& a, double2& b, const double (&q)[8], const double (&nq)[4]) {
    asm(AQSG_IP_CMAT2_BODY("f64")
        : "+d"(a.x), "+d"(a.y), "+d"(b.x), "+d"(b.y)
        : "d"(q[0]), "d"(q[1]), "d"(q[2]), "d"(q[3]), "d"(q[4]), "d"(q[5]), "d"(q[6]), "d"(q[7]), "d"(nq[0]),
          "d"(nq[1]), "d"(nq[2]), "d"(nq[3]));
}
#undef AQSG_IP_CMAT2_BODY

// The leaves below apply one op to the SL slots a thread holds (v[sl]),
// to slot sl only where on[sl] (its control on the slot's other bits
// holds), and within a slot to the elements of mask em where P.
template <typename T, int RB, int I, bool P, int SL, typename R>
__device__ __forceinline__ void r_mat2c(T (&v)[SL][1 << RB], const bool (&on)[SL], const R (&q)[8], uint32_t em) {
    const R nq[4] = {-q[1], -q[3], -q[5], -q[7]};
#pragma unroll
    for (int sl = 0; sl < SL; ++sl) {
        if (!on[sl]) continue;
#pragma unroll
        for (int e = 0; e < (1 << RB); ++e) {
            if (e & (1 << I)) continue;
            if (!r_on<P>(em, e)) continue;
            ip_cmat2(v[sl][e], v[sl][e | (1 << I)], q, nq);
        }
    }
}

// r = {m00, m01, m10, m11}, real
template <typename T, typename R, int RB, int I, bool P, int SL>
__device__ __forceinline__ void r_mat2r(T (&v)[SL][1 << RB], const bool (&on)[SL], const R (&r)[4], uint32_t em) {
#pragma unroll
    for (int sl = 0; sl < SL; ++sl) {
        if (!on[sl]) continue;
#pragma unroll
        for (int e = 0; e < (1 << RB); ++e) {
            if (e & (1 << I)) continue;
            if (!r_on<P>(em, e)) continue;
            ip_rot(v[sl][e].x, v[sl][e | (1 << I)].x, r[0], r[1], r[2], r[3]);
            ip_rot(v[sl][e].y, v[sl][e | (1 << I)].y, r[0], r[1], r[2], r[3]);
        }
    }
}

// pm[sl]: the elements (target bit 0) of slot sl whose pair is exchanged
template <typename T, int RB, int I, bool P, int SL>
__device__ __forceinline__ void r_perm(T (&v)[SL][1 << RB], const bool (&on)[SL], const uint32_t (&pm)[SL]) {
#pragma unroll
    for (int sl = 0; sl < SL; ++sl) {
        if (!on[sl]) continue;
#pragma unroll
        for (int e = 0; e < (1 << RB); ++e) {
            if (e & (1 << I)) continue;
            if (P) ip_cswap2(v[sl][e], v[sl][e | (1 << I)], (pm[sl] >> e) & 1u);
            else ip_swap2(v[sl][e], v[sl][e | (1 << I)]);
        }
    }
}

template <typename T, int RB, int I, int J, bool P, int SL>
__device__ __forceinline__ void r_swap(T (&v)[SL][1 << RB], const bool (&on)[SL], uint32_t em) {
#pragma unroll
    for (int sl = 0; sl < SL; ++sl) {
        if (!on[sl]) continue;
#pragma unroll
        for (int e = 0; e < (1 << RB); ++e) {
            if ((e & (1 << I)) || !(e & (1 << J))) continue;
            const int f = e ^ (1 << I) ^ (1 << J);
            if (P) ip_cswap2(v[sl][e], v[sl][f], (em >> e) & 1u);
            else ip_swap2(v[sl][e], v[sl][f]);
        }
    }
}

// ph[sl]: the phase of slot sl
template <typename T, int RB, bool P, int SL>
__device__ __forceinline__ void r_diag(T (&v)[SL][1 << RB], const bool (&on)[SL], const T (&ph)[SL], uint32_t em) {
#pragma unroll
    for (int sl = 0; sl < SL; ++sl) {
        if (!on[sl]) continue;
        const auto npy = -ph[sl].y;
#pragma unroll
        for (int e = 0; e < (1 << RB); ++e)
            if (r_on<P>(em, e)) ip_cmul(v[sl][e].x, v[sl][e].y, ph[sl].x, ph[sl].y, npy);
    }
}

// c = {c0.x, c0.y, c1.x, c1.y}: c0 where register bit I is 0, c1 where 1
template <typename T, int RB, int I, bool P, int SL, typename R>
__device__ __forceinline__ void r_diagr(T (&v)[SL][1 << RB], const bool (&on)[SL], const R (&c)[4], uint32_t em) {
    const R n0 = -c[1], n1 = -c[3];
#pragma unroll
    for (int sl = 0; sl < SL; ++sl) {
        if (!on[sl]) continue;
#pragma unroll
        for (int e = 0; e < (1 << RB); ++e) {
            if (!r_on<P>(em, e)) continue;
            if ((e >> I) & 1) ip_cmul(v[sl][e].x, v[sl][e].y, c[2], c[3], n1);
            else ip_cmul(v[sl][e].x, v[sl][e].y, c[0], c[1], n0);
        }
    }
}

template <int RM, int K>
__device__ __forceinline__ constexpr int r_dep(int r) {  // matrix index -> slot element bits
    int out = 0, bit = 0;
    for (int b = 0; b < 8; ++b)
        if ((RM >> b) & 1) {
            if ((r >> bit) & 1) out |= 1 << b;
            ++bit;
        }
    return out;
}

template <typename T, int RB, int RM, int SL>
__device__ __forceinline__ void r_matk(T (&vv)[SL][1 << RB], const bool (&on)[SL], const T* __restrict__ mat,
                                       uint32_t em) {
    constexpr int K = __builtin_popcount(RM), D = 1 << K, E = 1 << RB;
#pragma unroll
    for (int sl = 0; sl < SL; ++sl) {
        if (!on[sl]) continue;
        T (&v)[E] = vv[sl];
        T a[E];
#pragma unroll
        for (int e = 0; e < E; ++e) a[e] = v[e];
#pragma unroll
        for (int r = 0; r < D; ++r) {
            T row[D];
#pragma unroll
            for (int c = 0; c < D; ++c) row[c] = mat[r * D + c];
#pragma unroll
            for (int e0 = 0; e0 < E; ++e0) {
                if (e0 & RM) continue;
                if (!((em >> e0) & 1u)) continue;
                T acc;
                acc.x = 0;
                acc.y = 0;
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    const T x = a[e0 | r_dep<RM, K>(c)];
                    cmac(acc, row[c], x);
                }
                v[e0 | r_dep<RM, K>(r)] = acc;
            }
        }
    }
}

// Dispatch of a per-register-bit template over a runtime bit index a < RB
// and the predicated / unpredicated variant.
#define AQSG_R_BIT(RB, a, pred, CALL)                                   \
    do {                                                                \
        if (pred) {                                                     \
            constexpr bool P_ = true;                                   \
            switch (a) {                                                \
                case 0: { constexpr int I_ = 0; CALL; } break;          \
                case 1: { constexpr int I_ = 1; CALL; } break;          \
                case 2: { constexpr int I_ = 2; CALL; } break;          \
                default: if constexpr (RB > 3) { constexpr int I_ = RB > 3 ? 3 : 0; CALL; } break; \
            }                                                           \
        } else {                                                        \
            constexpr bool P_ = false;                                  \
            switch (a) {                                                \
                case 0: { constexpr int I_ = 0; CALL; } break;          \
                case 1: { constexpr int I_ = 1; CALL; } break;          \
                case 2: { constexpr int I_ = 2; CALL; } break;          \
                default: if constexpr (RB > 3) { constexpr int I_ = RB > 3 ? 3 : 0; CALL; } break; \
            }                                                           \
        }                                                               \
    } while (0)

// The op loop's other kinds: permutations (X, CX, Or, Swap and their
// controlled forms) and dense 2- and 3-qubit unitaries on register bits.
template <typename T, int RB, bool MATK, int SL>
__device__ __forceinline__ void rop_other(T (&v)[SL][1 << RB], const bool (&on)[SL], const uint32_t (&jt)[SL],
                                          uint32_t kind, uint32_t code, uint4 hd, uint32_t em, bool pred, int a,
                                          uint64_t base, const ROp* op, const unsigned char* __restrict__ pool) {
    constexpr uint32_t ALL = (1u << (1 << RB)) - 1u;
    switch (kind) {
        case RK_PERM: {
            uint32_t pm[SL];
            bool ppred = false;
#pragma unroll
            for (int sl = 0; sl < SL; ++sl) {
                pm[sl] = em;
                if (code & RF_OR) {
                    const bool or_t = ((jt[sl] & op->amt) != 0u) || ((base & op->am_ext) != 0ull);
                    pm[sl] = em & (or_t ? ALL : (hd.z >> 16));
                }
                ppred |= pm[sl] != ALL;
            }
            AQSG_R_BIT(RB, a, ppred, (r_perm<T, RB, I_, P_, SL>(v, on, pm)));
            break;
        }
        case RK_SWAP: {
            const int b = (code >> 12) & 15;
            if (pred) {
                switch (a * 4 + b) {
                    case 0 * 4 + 1: r_swap<T, RB, 0, 1, true, SL>(v, on, em); break;
                    case 0 * 4 + 2: r_swap<T, RB, 0, 2, true, SL>(v, on, em); break;
                    case 1 * 4 + 2: r_swap<T, RB, 1, 2, true, SL>(v, on, em); break;
                    default:
                        if constexpr (RB > 3) {
                            constexpr int H = RB > 3 ? 3 : 0;
                            switch (a) {
                                case 0: r_swap<T, RB, 0, H, true, SL>(v, on, em); break;
                                case 1: r_swap<T, RB, 1, H, true, SL>(v, on, em); break;
                                default: r_swap<T, RB, 2, H, true, SL>(v, on, em); break;
                            }
                        }
                        break;
                }
            } else {
                switch (a * 4 + b) {
                    case 0 * 4 + 1: r_swap<T, RB, 0, 1, false, SL>(v, on, em); break;
                    case 0 * 4 + 2: r_swap<T, RB, 0, 2, false, SL>(v, on, em); break;
                    case 1 * 4 + 2: r_swap<T, RB, 1, 2, false, SL>(v, on, em); break;
                    default:
                        if constexpr (RB > 3) {
                            constexpr int H = RB > 3 ? 3 : 0;
                            switch (a) {
                                case 0: r_swap<T, RB, 0, H, false, SL>(v, on, em); break;
                                case 1: r_swap<T, RB, 1, H, false, SL>(v, on, em); break;
                                default: r_swap<T, RB, 2, H, false, SL>(v, on, em); break;
                            }
                        }
                        break;
                }
            }
            break;
        }
        default:
            if constexpr (MATK) {
                const T* mat = reinterpret_cast<const T*>(pool + hd.w);
                const int rm = (code >> 8) & 0xFF;
                switch (rm) {
                    case 0x3: r_matk<T, RB, 0x3, SL>(v, on, mat, em); break;
                    case 0x5: r_matk<T, RB, 0x5, SL>(v, on, mat, em); break;
                    case 0x6: r_matk<T, RB, 0x6, SL>(v, on, mat, em); break;
                    case 0x7: r_matk<T, RB, 0x7, SL>(v, on, mat, em); break;
                    default:
                        if constexpr (RB > 3) {
                            switch (rm) {
                                case 0x9: r_matk<T, RB, 0x9, SL>(v, on, mat, em); break;
                                case 0xA: r_matk<T, RB, 0xA, SL>(v, on, mat, em); break;
                                case 0xC: r_matk<T, RB, 0xC, SL>(v, on, mat, em); break;
                                case 0xB: r_matk<T, RB, 0xB, SL>(v, on, mat, em); break;
                                case 0xD: r_matk<T, RB, 0xD, SL>(v, on, mat, em); break;
                                default: r_matk<T, RB, 0xE, SL>(v, on, mat, em); break;
                            }
                        }
                        break;
                }
            }
            break;
    }
}

// One register phase: hp[0] the header, hp[1..k] its ROps.  LAY must be
// linear over GF(2) (the identity or SwzLay): the position of slot element
// e is then at(jt) ^ at(e's register bits), an XOR of per-bit offsets.
// SL: slots a thread holds at once (slot, slot + nthr, ...); the caller
// guarantees that 2^(log2 size - RB) is a multiple of SL x nthr.  Two
// slots per thread halve the per-element cost of decoding each op.
template <typename T, int RB, class LAY, bool MATK, int SL>
__device__ __forceinline__ void rphase_run(T* s, uint32_t size, uint32_t nthr, uint64_t base,
                                           const TileOp* __restrict__ hp, const unsigned char* __restrict__ pool) {
    static_assert(SL == 1 || SL == 2, "one or two slots per thread");
    using R = decltype(T{}.x);
    constexpr int E = 1 << RB;
    constexpr uint32_t ALL = (1u << E) - 1u;
    const int nops = hp[0].k;
    const uint64_t rpos = hp[0].am_loc, tpos = hp[0].cm_loc;
    const int tbits = 31 - __clz(size) - RB;
    const ROp* __restrict__ rops = reinterpret_cast<const ROp*>(hp + 1);
    uint32_t bo[RB];  // byte offset of each register bit under LAY
#pragma unroll
    for (int i = 0; i < RB; ++i) bo[i] = LAY::at(1u << ((rpos >> (4 * i)) & 15u)) * (uint32_t)sizeof(T);
    unsigned char* sb = reinterpret_cast<unsigned char*>(s);
    auto off_of = [&](uint32_t ajt, int e) {
        uint32_t o = ajt;
#pragma unroll
        for (int i = 0; i < RB; ++i)
            if ((e >> i) & 1) o ^= bo[i];
        return o;
    };
    for (uint32_t slot0 = tile_tid(nthr); slot0 < (size >> RB); slot0 += SL * nthr) {
        uint32_t jt[SL], ajt[SL];
        T v[SL][E];
        {
            uint32_t j = 0;
            for (int i = 0; i < tbits; ++i) j |= ((slot0 >> i) & 1u) << ((tpos >> (4 * i)) & 15u);
            jt[0] = j;
        }
        if constexpr (SL == 2) {
            // slot0 + nthr: slot0 has bit log2(nthr) clear (nthr is a power
            // of two and slot0 = tid + k 2 nthr), so one tile bit is added
            jt[1] = jt[0] | (1u << ((tpos >> (4 * (31 - __clz(nthr)))) & 15u));
        }
#pragma unroll
        for (int sl = 0; sl < SL; ++sl) {
            ajt[sl] = LAY::at(jt[sl]) * (uint32_t)sizeof(T);
#pragma unroll
            for (int e = 0; e < E; ++e) v[sl][e] = *reinterpret_cast<const T*>(sb + off_of(ajt[sl], e));
        }
        // the next op's header is loaded while this one runs
        uint4 hd_next = nops > 0 ? *reinterpret_cast<const uint4*>(rops) : make_uint4(0u, 0u, 0u, 0u);
        for (int q = 0; q < nops; ++q) {
            const ROp* op = rops + q;
            const uint4 hd = hd_next;
            if (q + 1 < nops) hd_next = *reinterpret_cast<const uint4*>(rops + q + 1);
            const uint32_t code = hd.x;
            if (code & RF_EXT) {
                if ((base & op->cm_ext) != op->cv_ext) continue;
            }
            bool on[SL];
            bool any = false;
#pragma unroll
            for (int sl = 0; sl < SL; ++sl) {
                on[sl] = (jt[sl] & (hd.y & 0xFFFFu)) == (hd.y >> 16);
                any |= on[sl];
            }
            if (!any) continue;
            const uint32_t em = hd.z & ALL;
            const bool pred = em != ALL;
            const int a = (code >> 8) & 15;
            const uint32_t kind = code & 0xFFu;
            // the leaves read their coefficients from the op table where they
            // use them (loading them into registers ahead measured slower)
            switch (kind) {
                case RK_MAT2C: {
                    const R(&q)[8] = *reinterpret_cast<const R(*)[8]>(op->coef);
                    AQSG_R_BIT(RB, a, pred, (r_mat2c<T, RB, I_, P_, SL>(v, on, q, em)));
                    break;
                }
                case RK_MAT2R: {
                    const R(&r)[4] = *reinterpret_cast<const R(*)[4]>(op->coef);
                    AQSG_R_BIT(RB, a, pred, (r_mat2r<T, R, RB, I_, P_, SL>(v, on, r, em)));
                    break;
                }
                case RK_DIAGR: {
                    const R(&c)[4] = *reinterpret_cast<const R(*)[4]>(op->coef);
                    AQSG_R_BIT(RB, a, pred, (r_diagr<T, RB, I_, P_, SL>(v, on, c, em)));
                    break;
                }
                case RK_DIAG: {
                    const R* cf = reinterpret_cast<const R*>(op->coef);
                    T ph[SL];
#pragma unroll
                    for (int sl = 0; sl < SL; ++sl) {
                        bool one = false;
                        if (code & RF_TTHR) one = (jt[sl] >> hd.w) & 1u;
                        else if (code & RF_TEXT) one = (base >> op->ext_t) & 1ull;
                        ph[sl].x = one ? cf[2] : cf[0];
                        ph[sl].y = one ? cf[3] : cf[1];
                    }
                    if (pred) r_diag<T, RB, true, SL>(v, on, ph, em);
                    else r_diag<T, RB, false, SL>(v, on, ph, em);
                    break;
                }
                default:
                    rop_other<T, RB, MATK, SL>(v, on, jt, kind, code, hd, em, pred, a, base, op, pool);
                    break;
            }
        }
#pragma unroll
        for (int sl = 0; sl < SL; ++sl)
#pragma unroll
            for (int e = 0; e < E; ++e) *reinterpret_cast<T*>(sb + off_of(ajt[sl], e)) = v[sl][e];
    }
}
#undef AQSG_R_BIT

// Apply a pass's ops to the 2^m-amplitude tile s in shared memory (all
// nthr threads that SYNC covers call this; EPT x nthr >= 2^m).  base = the
// tile's global base index (its bits outside the tile).  With TC, ops the
// host marked go through tc_apply (tcs, ph).  Without MATK the kernel has no
// dense k-qubit path (passes the host knows to be free of them).  A run of
// consecutive diagonal
// ops runs from registers: each thread keeps the same EPT elements for the
// whole run, so the run costs one shared-memory round trip and one barrier.
template <typename R, int EPT, bool TC, class LAY, class SYNC = CtaSync, bool MATK = true, bool RPH = !TC,
          int TCW = 16, int SL = 1>
__device__ __forceinline__ void tile_run_ops(typename Cx<R>::T* s, uint32_t size, uint32_t nthr, uint64_t base,
                                             const TileOp* __restrict__ ops, int nops,
                                             const unsigned char* __restrict__ pool, const TcSmem* tcs,
                                             TcPhase* ph) {
    using T = typename Cx<R>::T;
    for (int oi = 0; oi < nops;) {
        const TileOp& op = ops[oi];
        const int cls = op.cls;
        if constexpr (RPH) {
            if (cls == T_RPHASE) {
                rphase_run<T, (sizeof(R) == 4 ? 4 : 3), LAY, MATK, SL>(s, size, nthr, base, ops + oi, pool);
                SYNC::sync();
                oi += 1 + op.k;
                continue;
            }
        }
        if (cls == L_DIAG1 || cls == L_DIAG2) {
            T reg[EPT];
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
                const uint32_t j = tile_tid(nthr) + e * nthr;
                if (j < size) reg[e] = s[LAY::at(j)];
            }
            int q = oi;
            for (; q < nops; ++q) {
                const TileOp& d = ops[q];
                if (d.cls != L_DIAG1 && d.cls != L_DIAG2) break;
                if ((base & d.cm_ext) != d.cv_ext) continue;
                T ph0 = ld_coef<T>(d.m, 0);
                const T ph1 = ld_coef<T>(d.m, 1);
                const int lt = d.lt0;
                if (d.cls == L_DIAG2 && lt < 0)  // target outside the tile: one phase
                    ph0 = ((base >> d.ext_t) & 1ull) ? ph1 : ph0;
                const bool two = d.cls == L_DIAG2 && lt >= 0;
                const uint32_t cm = (uint32_t)d.cm_loc, cv = (uint32_t)d.cv_loc;
#pragma unroll
                for (int e = 0; e < EPT; ++e) {
                    const uint32_t j = tile_tid(nthr) + e * nthr;
                    if (j < size && (j & cm) == cv) reg[e] = cmul((two && ((j >> lt) & 1u)) ? ph1 : ph0, reg[e]);
                }
            }
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
                const uint32_t j = tile_tid(nthr) + e * nthr;
                if (j < size) s[LAY::at(j)] = reg[e];
            }
            SYNC::sync();
            oi = q;
            continue;
        }
        ++oi;
        if ((base & op.cm_ext) != op.cv_ext) continue;
        if constexpr (TC) {
            if (cls == L_MATK && op.pad) {  // tensor-core op (host marks it)
                tc_apply<LAY, SYNC, TCW>(reinterpret_cast<float2*>(s), op, *tcs, *ph);
                continue;
            }
        }
        const uint32_t cm = (uint32_t)op.cm_loc, cv = (uint32_t)op.cv_loc;
        if (cls == L_MAT2 || cls == L_PERM_X || cls == L_PERM_OR) {
            const int lt = op.lt0;
            const uint32_t tb = 1u << lt;
            const T m00 = ld_coef<T>(op.m, 0), m01 = ld_coef<T>(op.m, 1);
            const T m10 = ld_coef<T>(op.m, 2), m11 = ld_coef<T>(op.m, 3);
            const bool or_all = (base & op.am_ext) != 0;
            const uint32_t am = (uint32_t)op.am_loc;
            for (uint32_t p = tile_tid(nthr); p < (size >> 1); p += nthr) {
                const uint32_t j0 = ins0(p, lt);
                if ((j0 & cm) != cv) continue;
                const uint32_t a0 = LAY::at(j0), a1 = LAY::at(j0 | tb);
                const T a = s[a0], b = s[a1];
                if (cls == L_MAT2) {
                    s[a0] = cmul2(m00, a, m01, b);
                    s[a1] = cmul2(m10, a, m11, b);
                } else if (cls == L_PERM_X || or_all || (j0 & am)) {
                    s[a0] = b;
                    s[a1] = a;
                }
            }
        } else if (cls == L_PERM_SWAP) {
            const int lo = min(op.lt0, op.lt1), hi = max(op.lt0, op.lt1);
            const uint32_t ma = 1u << op.lt0, mb = 1u << op.lt1;
            for (uint32_t p = tile_tid(nthr); p < (size >> 2); p += nthr) {
                const uint32_t j = ins0(ins0(p, lo), hi) | mb;  // a = 0, b = 1
                if ((j & cm) != cv) continue;
                const uint32_t a0 = LAY::at(j), a1 = LAY::at(j ^ (ma | mb));
                const T x = s[a0];
                s[a0] = s[a1];
                s[a1] = x;
            }
        } else if (MATK && cls == L_MATK) {
            const T* mat = reinterpret_cast<const T*>(pool + op.mat);
            switch (op.k) {
                case 2: matk_apply<T, 2, LAY>(s, size, nthr, op, mat, cm, cv); break;
                case 3: matk_apply<T, 3, LAY>(s, size, nthr, op, mat, cm, cv); break;
                case 4: matk_apply<T, 4, LAY>(s, size, nthr, op, mat, cm, cv); break;
                default: matk_apply<T, 5, LAY>(s, size, nthr, op, mat, cm, cv); break;
            }
        }
        SYNC::sync();
    }
}

}  // namespace aqsg
