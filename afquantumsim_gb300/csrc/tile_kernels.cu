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
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>

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
    int tbits[16];  // global bit of each local bit, ascending; tbits[i] = i for i < L
};

int tile_max_bits(int dtype) { return dtype == AQSG_C64 ? 14 : 13; }
static int stream_tile_bits(int dtype) { return dtype == AQSG_C64 ? 12 : 11; }
static int row_bits(int dtype) { return dtype == AQSG_C64 ? 5 : 4; }

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

// ---- tensor-core path (tcgen05) for fused 3..5-qubit unitaries -----------------
//
// On a 4096-amplitude c64 tile, a fused unitary U (D x D, D = 2^k) on k tile
// bits is Y = U X with X the tile viewed as D rows (the target bits) by
// C = 4096 / D columns (the other bits).  In real form
//   [Yr; Yi] = [[Ur, -Ui], [Ui, Ur]] [Xr; Xi]
// and with the data as the M side, D_tmem[c][n] = sum_kk A[c][kk] B[n][kk]
// where A[c][kk] = Xrf[kk][c] (M = 128 columns per block, K = 2D) and
// B[n][kk] = Urf[n][kk] (N = 2D).  Both operands are split into BF16 hi + lo
// parts; D = Ahi Bhi + Ahi Blo + Alo Bhi accumulates in FP32 in tensor memory
// (the dropped Alo Blo term is ~2^-18 relative).  Operands sit in shared
// memory in the no-swizzle K-major canonical layout: 8 x 16-byte core
// matrices, K-direction stride 128 B, M/N-direction stride (K/8) * 128 B.

constexpr int kTcTileBits = 12;
constexpr int kTcThreads = 128;
constexpr uint32_t kTcTmemCols = 64;            // 2^(12+1) / 128
constexpr uint32_t kTcABytes = 4u << kTcTileBits;  // one split of A: 2^(m+1) bf16 = 2^(m+2) B
constexpr uint32_t kTcBBytes = 2u * 64 * 64;       // one split of B at k = 5
constexpr uint64_t kTcWaitNs = 200000000ull;  // 0.2 s per wait

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

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

__device__ __forceinline__ uint32_t mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok;
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint16_t bf16_bits(float x) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ float bf16_val(uint16_t h) {
    return __uint_as_float((uint32_t)h << 16);
}

// Byte offset of element (row, kk) in a no-swizzle K-major operand with
// K elements per row.
__host__ __device__ __forceinline__ uint32_t kmajor_off(uint32_t row, uint32_t kk, uint32_t K) {
    return ((row >> 3) * (K >> 3) + (kk >> 3)) * 128u + (row & 7u) * 16u + (kk & 7u) * 2u;
}

struct TcShared {
    unsigned char* a;   // A hi, then A lo (kTcABytes each)
    unsigned char* b;   // B hi, then B lo (kTcBBytes each)
    uint64_t* bar;
    uint32_t* tmem;     // allocated tensor-memory address
    uint32_t* offr;     // per matrix row: local offset of its target-bit pattern
    int* err;           // device error flag
};

// One fused unitary on the tile through the tensor cores.  All kTcThreads
// threads of the CTA call this; returns the next mbarrier phase.
__device__ uint32_t tc_apply(float2* s, const TileOp& op, const unsigned char* __restrict__ pool,
                             const TcShared& t, uint32_t phase) {
    const int k = op.k, D = 1 << k;
    const uint32_t K = 2u * D, N = 2u * D;
    const uint32_t cols = 1u << (kTcTileBits - k);  // columns of X
    const uint32_t blocks = cols / 128u;
    const uint32_t bsplit = 2u * N * K;              // bytes of one B split
    const int tid = threadIdx.x;

    // B operand (host-prepared hi and lo splits) and the row offset table
    const uint4* src = reinterpret_cast<const uint4*>(pool + op.mat);
    uint4* dstb = reinterpret_cast<uint4*>(t.b);
    for (uint32_t i = tid; i < 2u * bsplit / 16u; i += kTcThreads) {
        const uint32_t half = i / (bsplit / 16u), w = i % (bsplit / 16u);
        dstb[half * (kTcBBytes / 16u) + w] = __ldg(src + i);
    }
    if (tid < D) {
        uint32_t off = 0;
        for (int i = 0; i < k; ++i)
            if ((tid >> (k - 1 - i)) & 1) off |= 1u << op.ltb[i];
        t.offr[tid] = off;
    }
    uint32_t tmask = 0;
    for (int i = 0; i < k; ++i) tmask |= 1u << op.ltb[i];
    __syncthreads();

    // A operand: column c of X -> row c % 128 of block c / 128
    for (uint32_t c = tid; c < cols; c += kTcThreads) {
        uint32_t basec = 0, cc = c;  // spread c over the non-target tile bits
        for (int b = 0; b < kTcTileBits; ++b) {
            if ((tmask >> b) & 1u) continue;
            basec |= (cc & 1u) << b;
            cc >>= 1;
        }
        unsigned char* ahi = t.a + (c >> 7) * (128u * K * 2u);
        unsigned char* alo = ahi + kTcABytes;
        const uint32_t row = c & 127u;
        for (uint32_t q = 0; q < K / 8u; ++q) {  // 8 consecutive kk per 16-byte chunk
            uint32_t hw[4], lw[4];
#pragma unroll
            for (int e = 0; e < 8; e += 2) {
                float x2[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const uint32_t kk = q * 8u + e + h;
                    const uint32_t r = kk < (uint32_t)D ? kk : kk - D;
                    const float2 a = s[basec | t.offr[r]];
                    x2[h] = kk < (uint32_t)D ? a.x : a.y;
                }
                const uint16_t h0 = bf16_bits(x2[0]), h1 = bf16_bits(x2[1]);
                const uint16_t l0 = bf16_bits(x2[0] - bf16_val(h0)), l1 = bf16_bits(x2[1] - bf16_val(h1));
                hw[e / 2] = (uint32_t)h0 | ((uint32_t)h1 << 16);
                lw[e / 2] = (uint32_t)l0 | ((uint32_t)l1 << 16);
            }
            const uint32_t off = kmajor_off(row, q * 8u, K);
            *reinterpret_cast<uint4*>(ahi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
            *reinterpret_cast<uint4*>(alo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();

    const uint32_t tmem = *t.tmem;
    if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t idesc = tc_idesc(128, N);
        const uint32_t sbo = (K / 8u) * 128u;
        const uint32_t a_hi = smem_u32(t.a), a_lo = a_hi + kTcABytes;
        const uint32_t b_hi = smem_u32(t.b), b_lo = b_hi + kTcBBytes;
        for (uint32_t blk = 0; blk < blocks; ++blk) {
            const uint32_t dcol = tmem + blk * N;
            const uint32_t aoff = blk * (128u * K * 2u);
            for (uint32_t st = 0; st < K / 16u; ++st) {
                const uint32_t ko = st * 256u;  // two core matrices along K
                tc_mma(dcol, tc_desc(a_hi + aoff + ko, 128u, sbo), tc_desc(b_hi + ko, 128u, sbo), idesc,
                       st > 0 ? 1u : 0u);
                tc_mma(dcol, tc_desc(a_hi + aoff + ko, 128u, sbo), tc_desc(b_lo + ko, 128u, sbo), idesc, 1u);
                tc_mma(dcol, tc_desc(a_lo + aoff + ko, 128u, sbo), tc_desc(b_hi + ko, 128u, sbo), idesc, 1u);
            }
        }
        tc_commit(t.bar);
    }
    // bounded wait for the tensor-core work: at most kTcWaitNs of wall time,
    // and none once another CTA has given up
    uint32_t done = 0;
    const uint64_t t0 = globaltimer_ns();
    for (long it = 0; !done; ++it) {
        done = mbar_try_wait(t.bar, phase);
        if (!done && (it & 63) == 63 &&
            (globaltimer_ns() - t0 > kTcWaitNs || *(volatile int*)t.err != 0))
            break;
    }
    if (!done && tid == 0) atomicExch(t.err, 1);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    // D back to the tile: warp w reads TMEM lanes 32w..32w+31 = columns
    const uint32_t warp = tid >> 5, lane_base = warp * 32u;
    for (uint32_t blk = 0; blk < blocks; ++blk) {
        const uint32_t c = blk * 128u + lane_base + (tid & 31u);
        uint32_t basec = 0, cc = c;
        for (int b = 0; b < kTcTileBits; ++b) {
            if ((tmask >> b) & 1u) continue;
            basec |= (cc & 1u) << b;
            cc >>= 1;
        }
        float v[64];
        for (uint32_t chunk = 0; chunk < N / 16u; ++chunk)
            tc_ld16(tmem + (lane_base << 16) + blk * N + chunk * 16u, v + chunk * 16u);
        for (int r = 0; r < D; ++r) s[basec | t.offr[r]] = make_float2(v[r], v[D + r]);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    return phase ^ 1u;
}

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

    T reg[EPT];
    bool in_regs = false;
    for (int oi = 0; oi < nops; ++oi) {
        const TileOp& op = ops[oi];
        const int cls = op.cls;
        if ((base & op.cm_ext) != op.cv_ext) continue;
        const bool diag = cls == L_DIAG1 || cls == L_DIAG2;
        if (diag) {
            if (!in_regs) {
#pragma unroll
                for (int e = 0; e < EPT; ++e) {
                    const uint32_t j = threadIdx.x + e * nthr;
                    if (j < size) reg[e] = s[j];
                }
                in_regs = true;
            }
            T ph0 = ld_coef<T>(op.m, 0), ph1 = ld_coef<T>(op.m, 1);
            int lt = op.lt0;
            if (cls == L_DIAG2 && lt < 0) {  // target outside the tile: one phase
                ph0 = ((base >> op.ext_t) & 1ull) ? ph1 : ph0;
            }
            const uint32_t cm = (uint32_t)op.cm_loc, cv = (uint32_t)op.cv_loc;
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
                const uint32_t j = threadIdx.x + e * nthr;
                if (j < size && (j & cm) == cv) {
                    T ph = ph0;
                    if (cls == L_DIAG2 && lt >= 0 && ((j >> lt) & 1u)) ph = ph1;
                    reg[e] = cmul(ph, reg[e]);
                }
            }
            continue;
        }
        if (in_regs) {
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
                const uint32_t j = threadIdx.x + e * nthr;
                if (j < size) s[j] = reg[e];
            }
            in_regs = false;
            __syncthreads();
        }
        if constexpr (TC) {
            if (cls == L_MATK && op.pad) {  // tensor-core op (host marks it)
                tc_phase = tc_apply(reinterpret_cast<float2*>(s), op, pool, tcs, tc_phase);
                continue;
            }
        }
        const uint32_t cm = (uint32_t)op.cm_loc, cv = (uint32_t)op.cv_loc;
        if (cls == L_MAT2 || cls == L_PERM_X || cls == L_PERM_OR || cls == L_DIAG2) {
            const int lt = op.lt0;
            const uint32_t tb = 1u << lt;
            const T m00 = ld_coef<T>(op.m, 0), m01 = ld_coef<T>(op.m, 1);
            const T m10 = ld_coef<T>(op.m, 2), m11 = ld_coef<T>(op.m, 3);
            const bool or_all = (base & op.am_ext) != 0;
            const uint32_t am = (uint32_t)op.am_loc;
            for (uint32_t p = threadIdx.x; p < (size >> 1); p += nthr) {
                const uint32_t j0 = ins0(p, lt);
                if ((j0 & cm) != cv) continue;
                const T a = s[j0], b = s[j0 | tb];
                if (cls == L_MAT2) {
                    s[j0] = cmul2(m00, a, m01, b);
                    s[j0 | tb] = cmul2(m10, a, m11, b);
                } else if (cls == L_PERM_X || or_all || (j0 & am)) {
                    s[j0] = b;
                    s[j0 | tb] = a;
                }
            }
        } else if (cls == L_PERM_SWAP) {
            const int lo = min(op.lt0, op.lt1), hi = max(op.lt0, op.lt1);
            const uint32_t ma = 1u << op.lt0, mb = 1u << op.lt1;
            for (uint32_t p = threadIdx.x; p < (size >> 2); p += nthr) {
                const uint32_t j = ins0(ins0(p, lo), hi) | mb;  // a = 0, b = 1
                if ((j & cm) != cv) continue;
                const uint32_t jj = j ^ (ma | mb);
                const T x = s[j];
                s[j] = s[jj];
                s[jj] = x;
            }
        } else if (cls == L_MATK) {
            const int k = op.k, D = 1 << k;
            int srt[AQSG_MAX_UNITARY_QUBITS];
            for (int i = 0; i < k; ++i) srt[i] = op.ltb[i];
            for (int i = 1; i < k; ++i)
                for (int q = i; q > 0 && srt[q - 1] > srt[q]; --q) {
                    const int t = srt[q]; srt[q] = srt[q - 1]; srt[q - 1] = t;
                }
            const T* mat = reinterpret_cast<const T*>(pool + op.mat);
            for (uint32_t p = threadIdx.x; p < (size >> k); p += nthr) {
                uint32_t j = p;
                for (int i = 0; i < k; ++i) j = ins0(j, srt[i]);
                if ((j & cm) != cv) continue;
                T v[32];
                for (int r = 0; r < D; ++r) {
                    uint32_t off = 0;
                    for (int i = 0; i < k; ++i)
                        if ((r >> (k - 1 - i)) & 1) off |= 1u << op.ltb[i];
                    v[r] = s[j | off];
                }
                for (int r = 0; r < D; ++r) {
                    T acc;
                    acc.x = 0;
                    acc.y = 0;
                    for (int c = 0; c < D; ++c) {
                        const T mm = mat[r * D + c];
                        acc.x += mm.x * v[c].x - mm.y * v[c].y;
                        acc.y += mm.x * v[c].y + mm.y * v[c].x;
                    }
                    uint32_t off = 0;
                    for (int i = 0; i < k; ++i)
                        if ((r >> (k - 1 - i)) & 1) off |= 1u << op.ltb[i];
                    s[j | off] = acc;
                }
            }
        }
        __syncthreads();
    }
    if (in_regs) {
#pragma unroll
        for (int e = 0; e < EPT; ++e) {
            const uint32_t j = threadIdx.x + e * nthr;
            if (j < size) s[j] = reg[e];
        }
    }
    __syncthreads();

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

static void pad_to(std::vector<unsigned char>& v, size_t align) {
    v.resize((v.size() + align - 1) / align * align, 0);
}

template <typename R>
static int run_tiled_t(aqsg_state_s* st, const std::vector<LOp>& ops) {
    using T = typename Cx<R>::T;
    aqsg_ctx_s* c = st->ctx;
    const int n = st->n;
    std::vector<Pass> passes = plan(n, st->dtype, ops);
    if (passes.empty()) return AQSG_OK;
    const bool tc_on = sizeof(R) == 4 && c->tensor_cores;

    // op tables and operand pool (bytes) of all passes in one upload
    std::vector<TileOp> table;
    std::vector<unsigned char> pool;
    std::vector<size_t> first;
    std::vector<char> pass_tc;
    for (const Pass& p : passes) {
        first.push_back(table.size());
        uint64_t S = 0;
        for (int b : p.bits) S |= 1ull << b;
        std::vector<int> local(64, -1);
        for (size_t i = 0; i < p.bits.size(); ++i) local[p.bits[i]] = (int)i;
        const bool tc_pass = tc_on && (int)p.bits.size() == kTcTileBits;
        bool any_tc = false;
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
                pad_to(pool, 256);
                t.mat = (int32_t)pool.size();
                if (tc_pass && o->k >= 3 && t.cm_loc == 0) {
                    t.pad = 1;  // tensor-core op
                    any_tc = true;
                    tc_operand(o->mk, o->k, pool);
                } else {
                    const int D = 1 << o->k;
                    for (int e = 0; e < D * D; ++e) {
                        T v;
                        v.x = (R)o->mk[2 * e];
                        v.y = (R)o->mk[2 * e + 1];
                        const size_t at = pool.size();
                        pool.resize(at + sizeof(T));
                        std::memcpy(&pool[at], &v, sizeof(T));
                    }
                }
            }
            table.push_back(t);
        }
        pass_tc.push_back(any_tc ? 1 : 0);
    }
    const size_t tbytes = sizeof(TileOp) * table.size();
    const size_t pbytes = pool.size();
    const size_t poff = (tbytes + 255) & ~size_t(255);
    if (int rc = ensure_scratch(c->ops, poff + pbytes + 16)) return rc;
    AQSG_CUDA_TRY(cudaMemcpyAsync(c->ops.ptr, table.data(), tbytes, cudaMemcpyHostToDevice, c->stream));
    if (pbytes)
        AQSG_CUDA_TRY(cudaMemcpyAsync((char*)c->ops.ptr + poff, pool.data(), pbytes,
                                      cudaMemcpyHostToDevice, c->stream));
    const TileOp* dops = (const TileOp*)c->ops.ptr;
    const unsigned char* dpool = (const unsigned char*)c->ops.ptr + poff;

    constexpr int EPT_WHOLE = sizeof(R) == 4 ? 32 : 16;  // 2^14 / 512, 2^13 / 512
    constexpr int EPT_STREAM = sizeof(R) == 4 ? 16 : 8;  // 2^12 / 256, 2^11 / 256
    auto kwhole = k_tile<R, EPT_WHOLE, 512, 1, false>;
    auto kstream = k_tile<R, EPT_STREAM, 256, 3, false>;
    auto ktc = k_tile<R, 32, kTcThreads, 1, true>;
    // largest tile of this dtype plus its row-offset table
    const int max_shm = (int)(sizeof(T) << tile_max_bits(st->dtype)) + 512 * 8;
    AQSG_CUDA_TRY(cudaFuncSetAttribute(kwhole, cudaFuncAttributeMaxDynamicSharedMemorySize, max_shm));
    // tile + row table (1 KiB) + A hi/lo + B hi/lo + barrier, tmem slot, row offsets
    const int tc_shm = (int)((sizeof(T) << kTcTileBits) + 1024 + 2 * kTcABytes + 2 * kTcBBytes + 256);
    bool launched_tc = false;
    if (tc_on) AQSG_CUDA_TRY(cudaFuncSetAttribute(ktc, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_shm));
    // The tensor-core products lose a little norm in a biased way (~1e-7 per
    // fused op); a run that uses them restores the input's FP64 norm at the
    // end (one read pass before, one read and one scale pass after).
    bool any_tc_pass = false;
    for (char f : pass_tc) any_tc_pass = any_tc_pass || f;
    double norm_before = 0;
    if (any_tc_pass)
        if (int rc = reduce_prob(st, 0, 0, &norm_before)) return rc;
    for (size_t pi = 0; pi < passes.size(); ++pi) {
        const Pass& p = passes[pi];
        TileGeom geo;
        std::memset(&geo, 0, sizeof(geo));
        geo.n = n;
        geo.m = (int)p.bits.size();
        const bool whole = geo.m == n;
        geo.L = whole ? n : row_bits(st->dtype);
        for (int i = 0; i < geo.m; ++i) geo.tbits[i] = p.bits[i];
        const uint32_t size = 1u << geo.m;
        const size_t rows = size_t(1) << (geo.m - geo.L);
        const size_t shm = sizeof(T) * size + rows * sizeof(uint64_t);
        const unsigned grid = (unsigned)(1ull << (n - geo.m));
        const int count = (int)((pi + 1 < passes.size() ? first[pi + 1] : table.size()) - first[pi]);
        if (pass_tc[pi]) {
            ktc<<<grid, kTcThreads, tc_shm, c->stream>>>((T*)st->d, geo, dops + first[pi], count, dpool,
                                                         c->d_err);
            launched_tc = true;
        } else if (whole) {
            int threads = (int)(size / EPT_WHOLE);
            threads = threads < 32 ? 32 : (threads > 512 ? 512 : threads);
            kwhole<<<grid, threads, shm, c->stream>>>((T*)st->d, geo, dops + first[pi], count, dpool, nullptr);
        } else {
            kstream<<<grid, 256, shm, c->stream>>>((T*)st->d, geo, dops + first[pi], count, dpool, nullptr);
        }
        c->launches++;
        AQSG_CUDA_TRY(cudaGetLastError());
    }
    if (launched_tc) {  // a tensor-core wait that gave up leaves a flag
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

int run_tiled(aqsg_state_s* st, const std::vector<LOp>& ops) {
    return st->dtype == AQSG_C64 ? run_tiled_t<float>(st, ops) : run_tiled_t<double>(st, ops);
}

}  // namespace aqsg
