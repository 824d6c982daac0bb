// Device side of the shared-memory tile engine, shared by the tile passes
// (tile_kernels.cu) and the batched engine (batch.cu): the per-tile op table
// format, the op interpreter and the tensor-core (tcgen05) fused-unitary path.
#pragma once

#include <cuda_bf16.h>

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
static __device__ uint32_t tc_apply(float2* s, const TileOp& op, const unsigned char* __restrict__ pool,
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

// Apply a pass's ops to the 2^m-amplitude tile s in shared memory (all
// threads of the CTA call this).  base = the tile's global base index (its
// bits outside the tile); TC ops use tcs and advance tc_phase.
template <typename R, int EPT, bool TC>
__device__ __forceinline__ void tile_run_ops(typename Cx<R>::T* s, uint32_t size, uint64_t base,
                                             const TileOp* __restrict__ ops, int nops,
                                             const unsigned char* __restrict__ pool, const TcShared& tcs,
                                             uint32_t& tc_phase) {
    using T = typename Cx<R>::T;
    const int nthr = blockDim.x;
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

}

}  // namespace aqsg
