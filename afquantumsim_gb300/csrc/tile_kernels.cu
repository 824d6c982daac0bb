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
#include <map>
#include <functional>
#include <mutex>
#include <unordered_map>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "tile_device.cuh"

namespace aqsg {

int tile_max_bits(int dtype) { return dtype == AQSG_C64 ? 14 : 13; }
int stream_tile_bits(int dtype) { return dtype == AQSG_C64 ? 12 : 11; }
int whole_tile_limit(int dtype, int setting) {
    if (setting <= 0) return tile_max_bits(dtype);
    return std::max(stream_tile_bits(dtype), std::min(setting, tile_max_bits(dtype)));
}
static int row_bits(int dtype) { return dtype == AQSG_C64 ? 5 : 4; }

// Shared-memory layout of the CUDA-core tile kernels: XOR-swizzled in groups
// of 4 index bits (complex64: 16 x 8 B = the 32 banks) or 3 (complex128).
template <typename R>
using TileSwz = SwzLay<sizeof(R) == 4 ? 4 : 3>;

// Whole-register passes (n <= 14 c64 / 13 c128): one CTA holds the register.
// EPT: elements per thread in register runs; MATK: the pass has dense
// k-qubit ops on CUDA cores.
// ops_smem: the op table is staged in shared memory after the register (one
// CTA reads each op once, so from global memory every op would be a cold
// load on the critical path).
template <typename R, int EPT, bool MATK>
__global__ void __launch_bounds__(512, 1)
k_tile(typename Cx<R>::T* __restrict__ sv, const TileGeom g, const TileOp* __restrict__ ops, int nops,
       const unsigned char* __restrict__ pool, int ops_smem) {
    using T = typename Cx<R>::T;
    using LAY = TileSwz<R>;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t size = 1u << g.m;
    T* s = reinterpret_cast<T*>(smem_raw);
    if (ops_smem) {
        uint4* dst = reinterpret_cast<uint4*>(smem_raw + sizeof(T) * size);
        const uint4* src = reinterpret_cast<const uint4*>(ops);
        const uint32_t words = (uint32_t)nops * (uint32_t)(sizeof(TileOp) / 16);
        for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = __ldg(src + i);
        ops = reinterpret_cast<const TileOp*>(dst);
    }
    if constexpr (sizeof(R) == 4) {
        for (uint32_t i = threadIdx.x; i < (size >> 1); i += blockDim.x) {
            const float4 x = __ldcs(reinterpret_cast<const float4*>(sv) + i);
            s[LAY::at(2 * i)] = make_float2(x.x, x.y);
            s[LAY::at(2 * i + 1)] = make_float2(x.z, x.w);
        }
    } else {
        for (uint32_t j = threadIdx.x; j < size; j += blockDim.x) s[LAY::at(j)] = __ldcs(sv + j);
    }
    __syncthreads();
    tile_run_ops<R, EPT, false, LAY, CtaSync, MATK>(s, size, blockDim.x, 0, ops, nops, pool, nullptr, nullptr);
    if constexpr (sizeof(R) == 4) {
        for (uint32_t i = threadIdx.x; i < (size >> 1); i += blockDim.x) {
            const float2 a = s[LAY::at(2 * i)], b = s[LAY::at(2 * i + 1)];
            __stcs(reinterpret_cast<float4*>(sv) + i, make_float4(a.x, a.y, b.x, b.y));
        }
    } else {
        for (uint32_t j = threadIdx.x; j < size; j += blockDim.x) __stcs(sv + j, s[LAY::at(j)]);
    }
}

// Plain streaming passes (no tensor-core ops): one CTA per tile of 2^m
// amplitudes (rows of 2^L contiguous amplitudes = 256 B at the row offsets of
// the pass's high tile bits); several CTAs per SM overlap one another's
// loads, compute and stores.  MATK: the pass has dense k-qubit ops on CUDA
// cores.  kStreamThreads threads per tile: each holds two slots of every
// register phase (the tile's 2^(m - RB) slots = 2 x kStreamThreads).
constexpr int kStreamThreads = 128;

// Op tables of up to this many bytes are copied into each CTA's shared
// memory (after the tile and its row offsets): the op loop then reads them
// with shared-memory loads instead of L1 hits (a 16 % shorter brick-work
// pass).  140 entries; four CTAs per SM still fit.
constexpr uint32_t kStreamOpsSmemMax = 140u * (uint32_t)sizeof(TileOp);

// SOPS: the op table is staged in shared memory (a compile-time choice, so
// that the op loop's loads are shared-memory loads, not generic ones).
template <typename R, int EPT, bool MATK, bool SOPS>
__device__ __forceinline__ void tile_stream_body(typename Cx<R>::T* __restrict__ sv, const TileGeom& g,
                                                 const TileOp* __restrict__ ops, int nops,
                                                 const unsigned char* __restrict__ pool, uint64_t tile) {
    using T = typename Cx<R>::T;
    using LAY = TileSwz<R>;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // tile size and thread count are compile-time constants (the launch
    // checks g.m): the interpreter's slot loop then runs exactly once per
    // thread and keeps no loop-carried state
    constexpr uint32_t size = (uint32_t)EPT * kStreamThreads;
    constexpr int m = __builtin_ctz(size);
    constexpr uint32_t nthr = kStreamThreads;
    const int L = g.L;
    T* s = reinterpret_cast<T*>(smem_raw);
    uint64_t* rowoff = reinterpret_cast<uint64_t*>(smem_raw + sizeof(T) * size);
    const uint32_t rows = 1u << (m - L), rowlen = 1u << L;
    uint64_t base = tile;  // the tile index spread over the non-tile bits
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
    if constexpr (SOPS) {
        uint4* dst = reinterpret_cast<uint4*>(rowoff + rows);
        const uint4* src = reinterpret_cast<const uint4*>(ops);
        const uint32_t words = (uint32_t)nops * (uint32_t)(sizeof(TileOp) / 16);
        for (uint32_t i = threadIdx.x; i < words; i += nthr) dst[i] = __ldg(src + i);
        ops = reinterpret_cast<const TileOp*>(dst);
    }
    __syncthreads();
    // the tile arrives by asynchronous copies straight into shared memory:
    // all of a thread's copies are in flight at once and hold no registers
    // (one amplitude per copy: the swizzle can reverse a pair's order)
    if constexpr (sizeof(R) == 4) {
        for (uint32_t i = threadIdx.x; i < (size >> 1); i += nthr) {
            const uint32_t j = i << 1;
            const T* src = sv + base + rowoff[j >> L] + (j & (rowlen - 1));
            cp_async8(s + LAY::at(j), src);
            cp_async8(s + LAY::at(j + 1), src + 1);
        }
    } else {
        for (uint32_t j = threadIdx.x; j < size; j += nthr)
            cp_async16(s + LAY::at(j), sv + base + rowoff[j >> L] + (j & (rowlen - 1)));
    }
    cp_async_wait_all();
    __syncthreads();
    tile_run_ops<R, EPT, false, LAY, CtaSync, MATK, true, 16, 2>(s, size, nthr, base, ops, nops, pool, nullptr,
                                                                nullptr);
    if constexpr (sizeof(R) == 4) {
        for (uint32_t i = threadIdx.x; i < (size >> 1); i += nthr) {
            const uint32_t j = i << 1;
            const uint64_t gi = base + rowoff[j >> L] + (j & (rowlen - 1));
            const float2 a = s[LAY::at(j)], b = s[LAY::at(j + 1)];
            __stcs(reinterpret_cast<float4*>(sv) + (gi >> 1), make_float4(a.x, a.y, b.x, b.y));
        }
    } else {
        for (uint32_t j = threadIdx.x; j < size; j += nthr)
            __stcs(sv + base + rowoff[j >> L] + (j & (rowlen - 1)), s[LAY::at(j)]);
    }
}

template <typename R, int EPT, bool MATK, bool SOPS>
__global__ void __launch_bounds__(kStreamThreads, MATK ? 3 : 4)
k_tile_stream(typename Cx<R>::T* __restrict__ sv, const __grid_constant__ TileGeom g,
              const TileOp* __restrict__ ops, int nops, const unsigned char* __restrict__ pool) {
    tile_stream_body<R, EPT, MATK, SOPS>(sv, g, ops, nops, pool, blockIdx.x);
}

// The same pass over `members` registers of equal shape and plan geometry,
// one launch: block b runs tile b % tiles of register b / tiles, whose
// amplitudes start reg_stride amplitudes after the previous register's and
// whose op table + operand pool start dev_stride bytes after the previous
// one's (the batched engine's groups of equal-structure circuits).
template <typename R, int EPT, bool MATK, bool SOPS>
__global__ void __launch_bounds__(kStreamThreads, MATK ? 3 : 4)
k_tile_stream_multi(typename Cx<R>::T* __restrict__ sv0, uint64_t reg_stride, const __grid_constant__ TileGeom g,
                    const unsigned char* __restrict__ dev0, uint64_t dev_stride, uint32_t op_first, int nops,
                    uint64_t pool_off, uint32_t tiles) {
    const uint32_t member = blockIdx.x / tiles, tile = blockIdx.x % tiles;
    const unsigned char* dev = dev0 + (uint64_t)member * dev_stride;
    tile_stream_body<R, EPT, MATK, SOPS>(sv0 + (uint64_t)member * reg_stride, g,
                                         reinterpret_cast<const TileOp*>(dev) + op_first, nops, dev + pool_off, tile);
}

constexpr uint32_t kRowBytes = 256;
constexpr uint32_t kRows = 128;                     // rows of a 2^12-amplitude c64 tile
constexpr int kTcCta = kTcThreads + 32;             // 24 compute warps + 1 producer warp
                                                    // (25 warps: at most 72 registers per thread)
constexpr int kTcGroups = 3;                        // compute groups (tiles in flight) per CTA
constexpr int kTcMaxOps = 24;                       // op tables up to this size go to shared memory
constexpr uint32_t kTcRowStride = 272u;             // padded tile row in the tensor-core kernel
static_assert(sizeof(TileOp) % 16 == 0, "op tables are bulk-copied: 16-byte multiples");

// ---- tile loads by the tensor memory accelerator -----------------------------
//
// A tensor-core pass loads each tile with one cp.async.bulk.tensor.  The
// register is described to the TMA unit as a tensor of rank 2..5: dimension
// 0 is index bits [0, start[1]) (the 32-amplitude row and the non-tile bits
// above it up to the first run of high tile bits), dimension i >= 1 is bits
// [start[i], start[i] + bits[i]) (one run of high tile bits and the
// non-tile bits above it), so a tile is the box of 34 x 2^run_1 x ... rows:
// each row of 32 amplitudes plus the next 2, which land in the row padding
// of the shared-memory layout (272-byte rows).  Amplitudes past the end of a
// dimension read as zero (they only ever reach padding).  A grouped pass
// (several registers back to back) extends the top dimension over the
// members.  Passes whose high tile bits form more than four runs keep the
// cp.async loader (rank 0).
struct TmaGeom {
    int32_t rank;      // 0: no tensor map
    int32_t start[5];  // first index bit of each dimension
    int32_t bits[5];   // index bits each dimension covers
};
constexpr uint32_t kTmaRowBox = 34;  // amplitudes per row the box reads: 32 + the padding

__device__ __forceinline__ void tma_load_tile(void* dst, const CUtensorMap* map, int rank, const int32_t* c,
                                              uint64_t* bar) {
    const uint64_t m = reinterpret_cast<uint64_t>(map);
    const uint32_t d = smem_u32(dst), b = smem_u32(bar);
    switch (rank) {
        case 2:
            asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                         " [%0], [%1, {%2, %3}], [%4];" ::"r"(d), "l"(m), "r"(c[0]), "r"(c[1]), "r"(b) : "memory");
            break;
        case 3:
            asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                         " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(d), "l"(m), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(b)
                         : "memory");
            break;
        case 4:
            asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                         " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(d), "l"(m), "r"(c[0]), "r"(c[1]), "r"(c[2]),
                         "r"(c[3]), "r"(b) : "memory");
            break;
        default:
            asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                         " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(d), "l"(m), "r"(c[0]), "r"(c[1]),
                         "r"(c[2]), "r"(c[3]), "r"(c[4]), "r"(b) : "memory");
            break;
    }
}

// Shared memory of the tensor-core streaming kernel: five tile buffers (the
// three compute groups' tiles and two loading), the row offsets, barriers, the
// op table and the pass's operand blob (the MMAs' data operand lives in
// tensor memory).  Rows are padded by 16 bytes (a 272-byte stride) so the
// operand gathers of rows that share their low index bits spread over the
// banks.
template <int GROUPS>
struct TcStreamSmemT {
    static constexpr int kBufs = 5;
    static constexpr uint32_t kRowStride = kTcRowStride;
    static constexpr uint32_t kBufBytes = kRows * kRowStride;          // 34 KiB
    static constexpr uint32_t kRowOff = kBufs * kBufBytes;              // kRows x u64
    static constexpr uint32_t kBars = kRowOff + kRows * 8u;             // full[5] done[5] mma[3] blob
    static constexpr uint32_t kTmemSlot = kBars + 16u * 8u;
    static constexpr uint32_t kOps = (kTmemSlot + 16u + 127u) & ~127u;  // kTcMaxOps TileOps
    static constexpr uint32_t kBlob = (kOps + kTcMaxOps * (uint32_t)sizeof(TileOp) + 1023u) & ~1023u;
    static constexpr uint32_t kBytes = kBlob + kTcBlobMax;
    static_assert(kBytes <= 232448u, "more shared memory than a CTA may have");
};
using TcStreamSmem = TcStreamSmemT<kTcGroups>;
// tensor-memory columns a CTA allocates: the groups' columns, rounded up to
// a power of two
constexpr uint32_t kTcTmemAlloc = 512;
static_assert(kTcTmemCols * kTcGroups <= kTcTmemAlloc, "tensor memory of the compute groups");

// any(v) over the N threads of this thread's compute group (named barrier
// 1 + group, as GroupSync)
template <int N>
__device__ __forceinline__ bool group_any(bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r) : "r"((uint32_t)v), "r"(1u + threadIdx.x / (uint32_t)N), "n"(N) : "memory");
    return r != 0;
}

// Tensor-core streaming passes (c64, 4096-amplitude tiles).  A persistent
// CTA per SM walks its tiles; a tile is 128 rows of 256 contiguous bytes
// (the 5 low index bits) at the row offsets of the pass's 7 high tile bits.
// Warp 24 is the producer: it loads each tile into one of five
// shared-memory buffers with one TMA copy (full[b] completes on its byte
// count), or, for a pass whose tile bits the tensor map cannot describe, in
// 16-byte cp.async chunks (full[b] completes when all 32 lanes' chunks have
// landed), and loads the next tile into a buffer as soon as the compute
// group that ran its tile has written it back with 128-bit stores and
// released it (done[b]).  The 24 compute warps form GROUPS = 3 groups of 8;
// group g runs the pass's ops on the CTA's tiles g, g + GROUPS, ... with its
// own named barrier, tensor-memory columns and MMA barrier, so the groups'
// gathers, MMAs, waits and write-backs overlap one another (three groups
// instead of two took the fused 30-qubit brick-work from 164 to 132 ms).  The pass's operand blob and op table are
// bulk-loaded into shared memory.  Every wait is bounded: one that gives up
// sets the error flag and the CTA winds down.
//
// MATK: the pass also has dense k-qubit ops on the CUDA cores (the variant
// without that path keeps its registers: the path is a call).
//
// One register (MULTI false): CTA b takes tiles b, b + grid, ...  A group of
// `members` registers of equal plan geometry (MULTI true; the batched
// engine): register m starts reg_stride amplitudes after register m-1, its
// op table and pool dev_stride bytes after m-1's; CTA b takes a contiguous
// run of the members' tiles, and where the run crosses into the next
// register the producer reloads the blob and op table once the compute warps
// have released the last tile of the previous one.
// The CTA's tiles as the compute groups see them: the i-th is tile
// local(i) of register member(i) (MULTI: a contiguous run from `first`;
// otherwise blockIdx.x + i * gridDim.x of register 0).
struct TcTiles {
    uint32_t count, first, ntiles;
    __device__ __forceinline__ uint32_t tile(uint32_t i, bool multi) const {
        return multi ? first + i : blockIdx.x + i * gridDim.x;
    }
};

// Compute group G = threadIdx.x / NT (named barrier 1 + G) of the
// tensor-core streaming kernel: runs the pass's ops on the CTA's tiles G,
// G + GROUPS, ...
template <int NT, int GROUPS, bool MULTI, bool MATK, class LAY>
__device__ __forceinline__ void tc_compute_group(unsigned char* smem_raw, const TileGeom& g, const TcTiles& tl,
                                                 float2* __restrict__ sv0, uint64_t reg_stride,
                                                 const unsigned char* __restrict__ dev0, uint64_t dev_stride,
                                                 uint32_t op_first, int nops, uint64_t pool_off, const TileOp* sops,
                                                 uint64_t* full, uint64_t* done, uint64_t* blob_bar,
                                                 const TcSmem& tcs_in, int* err, uint32_t norm_flags, double& nin,
                                                 double& nout) {
    constexpr int NB = TcStreamSmem::kBufs, M = kTcTileBits;
    constexpr uint32_t kBufBytes = TcStreamSmem::kBufBytes;
    using SYNC = GroupSync<NT>;
    const uint32_t G = threadIdx.x / NT;
    const uint32_t lane = threadIdx.x & 31u;
    const bool gtid0 = (threadIdx.x & (NT - 1)) == 0;
    TcSmem tcs = tcs_in;
    TcPhase tph;
    uint32_t blob_par = 0;
    uint32_t cur = (MULTI && tl.count) ? tl.tile(0, true) / tl.ntiles : 0u;
    // |a|^2 of the tiles before the ops (norm_flags bit 0) and after them
    // (bit 1), over the 16-byte chunks this thread writes back
    FAcc fin, fout;
    auto add_norm = [&](FAcc& f, const uint4& v) {
        float h, l;
        norm2_ff(__uint_as_float(v.x), __uint_as_float(v.y), h, l);
        f.add(h, l);
        norm2_ff(__uint_as_float(v.z), __uint_as_float(v.w), h, l);
        f.add(h, l);
    };
    bool ok = !group_any<NT>(!mbar_wait_bounded(blob_bar, 0, err));
    for (uint32_t i = G; ok && i < tl.count; i += GROUPS) {
        const uint32_t buf = i % NB;
        const uint32_t t = tl.tile(i, MULTI);
        const uint32_t m = MULTI ? t / tl.ntiles : 0u;
        const uint32_t local = MULTI ? t % tl.ntiles : t;
        if (MULTI && m != cur) {  // the producer reloads the blob after the previous register's tiles
            blob_par ^= 1u;
            if (group_any<NT>(!mbar_wait_bounded(blob_bar, blob_par, err))) break;
            cur = m;
        }
        if (group_any<NT>(!mbar_wait_bounded(full + buf, (i / NB) & 1u, err))) break;
        float2* s = reinterpret_cast<float2*>(smem_raw + buf * kBufBytes);
        uint64_t base = local;  // spread over the non-tile bits
        for (int q = 0; q < M; ++q) {
            const int b = g.tbits[q];
            const uint64_t lo = base & ((1ull << b) - 1ull);
            base = ((base - lo) << 1) | lo;
        }
        const unsigned char* dev = dev0 + (uint64_t)m * dev_stride;
        if (norm_flags & 1u) {
            const unsigned char* src = smem_raw + buf * kBufBytes;
            for (uint32_t q = threadIdx.x & (NT - 1u); q < kRows * 16u; q += NT)
                add_norm(fin, *reinterpret_cast<const uint4*>(src + (q >> 4) * TcStreamSmem::kRowStride +
                                                              (q & 15u) * 16u));
        }
        // the op table is in shared memory (the planner keeps tensor-core
        // passes within kTcMaxOps entries)
        tile_run_ops<float, (1 << M) / NT, true, LAY, SYNC, MATK, false, NT / 32>(s, 1u << M, NT, base, sops, nops,
                                                                                dev + pool_off, &tcs, &tph);
        // the group writes its tile back itself (16-byte chunks of the rows,
        // 2048 / NT per thread), so the buffer is free as soon as the last
        // chunk has been read and the producer only issues loads
        {
            const uint64_t* rowoff = reinterpret_cast<const uint64_t*>(smem_raw + TcStreamSmem::kRowOff);
            float2* dstg = sv0 + (uint64_t)m * reg_stride + base;
            const unsigned char* src = smem_raw + buf * kBufBytes;
#pragma unroll 4
            for (uint32_t q = threadIdx.x & (NT - 1u); q < kRows * 16u; q += NT) {
                const uint32_t r = q >> 4, c = q & 15u;
                const uint4 v = *reinterpret_cast<const uint4*>(src + r * TcStreamSmem::kRowStride + c * 16u);
                __stcs(reinterpret_cast<uint4*>(dstg + rowoff[r]) + c, v);
                if (norm_flags & 2u) add_norm(fout, v);
            }
        }
        fence_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(done + buf);
        if (group_any<NT>(gtid0 && *(volatile int*)err != 0)) break;
    }
    if (!ok || *(volatile int*)err != 0) {
        if (gtid0) {
            atomicExch(err, 1);
            // the MMAs this group issued finish before the shared and tensor
            // memory go (the producer waits for its own copies): the last
            // issued commit is the phase of parity tph.mma ^ 1 (already
            // complete, or never started on a fresh barrier, when nothing is
            // outstanding)
            mbar_wait_timeout(tcs.mma_bar, tph.mma ^ 1u);
        }
    }
    nin = fin.value();
    nout = fout.value();
}

template <bool MULTI, bool MATK>
__global__ void __launch_bounds__(kTcCta, 1)
k_stream_tc(float2* __restrict__ sv0, const __grid_constant__ TileGeom g, const unsigned char* __restrict__ dev0,
            uint32_t op_first, int nops, uint64_t pool_off, int* err, uint32_t ntiles, uint32_t members,
            uint64_t reg_stride, uint64_t dev_stride, double* __restrict__ norm_part, uint32_t norm_flags,
            const __grid_constant__ CUtensorMap tmap, const __grid_constant__ TmaGeom tg) {
    using SM = TcStreamSmem;
    constexpr int NB = SM::kBufs;
    constexpr int GROUPS = kTcGroups;
    constexpr int NT = kTcThreads / GROUPS;  // threads per compute group
    constexpr int L = 5, M = 12;
    constexpr uint32_t kRowStride = SM::kRowStride, kBufBytes = SM::kBufBytes;
    using LAY = TileLay<L, (int)((kRowStride - kRowBytes) / sizeof(float2))>;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    uint64_t* rowoff = reinterpret_cast<uint64_t*>(smem_raw + SM::kRowOff);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + SM::kBars);
    uint64_t* done = full + NB;
    uint64_t* mma_bar = full + 2 * NB;  // one per compute group
    uint64_t* blob_bar = mma_bar + GROUPS;
    TileOp* sops = reinterpret_cast<TileOp*>(smem_raw + SM::kOps);
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    double nin = 0.0, nout = 0.0;  // this thread's norm sums (compute warps)

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(smem_raw + SM::kTmemSlot)), "r"(kTcTmemAlloc));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int b = 0; b < NB; ++b) {
            mbar_init(full + b, tg.rank ? 1 : 32);  // the TMA load, or one cp.async arrival per producer lane
            mbar_init(done + b, NT / 32);
        }
        for (int q = 0; q < GROUPS; ++q) mbar_init(mma_bar + q, 1);
        mbar_init(blob_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (uint32_t r = tid; r < kRows; r += kTcCta) {
        uint64_t off = 0;
        for (int q = 0; q < M - L; ++q)
            if ((r >> q) & 1u) off |= 1ull << g.tbits[L + q];
        rowoff[r] = off;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    auto tile_base = [&](uint32_t t) {  // t spread over the non-tile bits
        uint64_t base = t;
        for (int i = 0; i < M; ++i) {
            const int b = g.tbits[i];
            const uint64_t lo = base & ((1ull << b) - 1ull);
            base = ((base - lo) << 1) | lo;
        }
        return base;
    };
    // this CTA's tiles: the i-th is tile local_of(i) of register member_of(i)
    uint32_t count, first = 0;
    if constexpr (MULTI) {
        const uint64_t total = (uint64_t)ntiles * members;
        const uint64_t chunk = (total + gridDim.x - 1) / gridDim.x;
        const uint64_t start = (uint64_t)blockIdx.x * chunk;
        count = start < total ? (uint32_t)(total - start < chunk ? total - start : chunk) : 0u;
        first = (uint32_t)start;
    } else {
        count = blockIdx.x < ntiles ? (ntiles - 1u - blockIdx.x) / gridDim.x + 1u : 0u;
    }
    auto tile_of = [&](uint32_t i) { return MULTI ? first + i : blockIdx.x + i * gridDim.x; };
    auto member_of = [&](uint32_t i) { return MULTI ? tile_of(i) / ntiles : 0u; };
    auto local_of = [&](uint32_t i) { return MULTI ? tile_of(i) % ntiles : tile_of(i); };
    auto dev_of = [&](uint32_t m) { return dev0 + (uint64_t)m * dev_stride; };
    auto sv_of = [&](uint32_t m) { return sv0 + (uint64_t)m * reg_stride; };

    if (warp == kTcThreads / 32) {
        // ---- producer warp ----
        uint32_t blob_loads = 0;
        auto load_blob = [&](uint32_t m) {  // lane 0
            const unsigned char* pool = dev_of(m) + pool_off;
            const uint32_t opb = (uint32_t)nops * (uint32_t)sizeof(TileOp);
            mbar_expect_tx(blob_bar, g.tc_bytes + opb);
            for (uint32_t o = 0; o < g.tc_bytes; o += 32768u) {
                const uint32_t len = g.tc_bytes - o < 32768u ? g.tc_bytes - o : 32768u;
                bulk_load(smem_raw + SM::kBlob + o, pool + g.tc_blob + o, len, blob_bar);
            }
            if (opb) bulk_load(sops, reinterpret_cast<const TileOp*>(dev_of(m)) + op_first, opb, blob_bar);
            ++blob_loads;
        };
        if (lane == 0) load_blob(count ? member_of(0) : 0u);
        auto issue_load = [&](uint32_t i) {
            const uint32_t buf = i % NB;
            unsigned char* dst = smem_raw + buf * kBufBytes;
            if (tg.rank) {  // one TMA load of the whole tile (lane 0)
                if (lane == 0) {
                    const uint64_t base = tile_base(local_of(i));
                    int32_t c[5];
                    for (int d = 0; d < tg.rank; ++d)
                        c[d] = (int32_t)((base >> tg.start[d]) & ((1ull << tg.bits[d]) - 1ull));
                    if (MULTI) c[tg.rank - 1] += (int32_t)(member_of(i) << tg.bits[tg.rank - 1]);
                    mbar_expect_tx(full + buf, kBufBytes);
                    tma_load_tile(dst, &tmap, tg.rank, c, full + buf);
                }
                return;
            }
            const float2* src = sv_of(member_of(i)) + tile_base(local_of(i));
#pragma unroll 8
            for (uint32_t q = lane; q < kRows * 16u; q += 32u) {
                const uint32_t r = q >> 4, c = q & 15u;
                cp_async16(dst + r * kRowStride + c * 16u, src + rowoff[r] + 2u * c);
            }
            cp_async_arrive(full + buf);
        };
        for (uint32_t q = 0; q < count && q < (uint32_t)NB; ++q) issue_load(q);
        for (uint32_t i = 0; i < count; ++i) {
            const uint32_t buf = i % NB;
            if (!mbar_wait_bounded(done + buf, (i / NB) & 1u, err)) {
                if (lane == 0) atomicExch(err, 1);
                break;
            }
            // tiles are released in order (the compute groups have written
            // them back), so every tile up to i is done: at a change of
            // register its blob and op table may be replaced
            if (MULTI && lane == 0 && i + 1 < count && member_of(i + 1) != member_of(i)) load_blob(member_of(i + 1));
            __syncwarp();
            if (i + NB < count) issue_load(i + NB);
        }
        // the copies this warp started have landed before the shared memory
        // goes (a wound-down CTA may leave some unconsumed)
        asm volatile("cp.async.wait_all;" ::: "memory");
        if (lane == 0 && blob_loads > 0) mbar_wait_timeout(blob_bar, (blob_loads - 1u) & 1u);
    } else {
        // ---- compute groups ----
        const uint32_t grp = warp / (NT / 32);
        TcSmem tcs;
        tcs.blob = smem_raw + SM::kBlob;
        tcs.mma_bar = mma_bar + grp;
        tcs.tmem = *reinterpret_cast<volatile uint32_t*>(smem_raw + SM::kTmemSlot) + grp * kTcTmemCols;
        tcs.err = err;
        TcTiles tl;
        tl.count = count;
        tl.first = first;
        tl.ntiles = ntiles;
        tc_compute_group<NT, GROUPS, MULTI, MATK, LAY>(smem_raw, g, tl, sv0, reg_stride, dev0, dev_stride, op_first,
                                                        nops, pool_off, sops, full, done, blob_bar, tcs, err,
                                                        MULTI ? 0u : norm_flags, nin, nout);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            nin += __shfl_down_sync(0xffffffffu, nin, o);
            nout += __shfl_down_sync(0xffffffffu, nout, o);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (!MULTI && norm_flags) {
        // per-CTA partials in a fixed order (the row offsets are no longer
        // needed): the same input gives the same sums on every run
        double* red = reinterpret_cast<double*>(rowoff);
        constexpr int CW = kTcThreads / 32;
        if (warp < CW && lane == 0) {
            red[warp] = nin;
            red[CW + warp] = nout;
        }
        __syncthreads();
        if (tid == 0) {
            double a = 0.0, b = 0.0;
            for (int w = 0; w < CW; ++w) {
                a += red[w];
                b += red[CW + w];
            }
            if (norm_flags & 1u) norm_part[blockIdx.x] = a;
            if (norm_flags & 2u) norm_part[gridDim.x + blockIdx.x] = b;
        }
    }
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(
                         *reinterpret_cast<volatile uint32_t*>(smem_raw + SM::kTmemSlot)),
                     "r"(kTcTmemAlloc));
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

static uint64_t support_of(const LOp& o) {
    uint64_t s = o.cmask | o.amask;
    if (o.t0 >= 0) s |= 1ull << o.t0;
    if (o.t1 >= 0) s |= 1ull << o.t1;
    for (int j = 0; j < o.k; ++j) s |= 1ull << o.tb[j];
    return s;
}

// Passes with lookahead.  A pass scans the remaining ops in order and takes
// each op whose target bits still fit in m tile bits (with the L row bits)
// and that commutes with every op it has passed over: it shares no qubit
// with them, or it and they are all diagonal.  Taking it moves it before the
// ops passed over, which is then exact.  The scan gives up kWindow ops after
// the first one it passed over.
static size_t tc_op_bytes(int k);

// tc_budget: tensor-core passes (c64): a pass also stops taking fused
// unitaries of 3+ qubits once their operands would exceed the shared-memory
// blob of the kernel.
static std::vector<Pass> plan(int n, int dtype, const std::vector<LOp>& ops, bool tc_budget, int whole_max) {
    std::vector<Pass> passes;
    const bool whole = n <= whole_tile_limit(dtype, whole_max);
    const int m = whole ? n : stream_tile_bits(dtype);
    const int L = whole ? n : row_bits(dtype);
    const uint64_t rowmask = (L >= 64) ? ~0ull : ((1ull << L) - 1ull);
    constexpr size_t kWindow = 1024;
    std::vector<const LOp*> rest;
    rest.reserve(ops.size());
    for (const LOp& o : ops) rest.push_back(&o);
    std::vector<const LOp*> left;
    while (!rest.empty()) {
        Pass cur;
        uint64_t S = rowmask, blk_any = 0, blk_nondiag = 0;
        size_t skipped = 0, blob = 0;
        bool has_tc = false;  // a tensor-core pass holds at most kTcMaxOps ops
        left.clear();
        for (size_t i = 0; i < rest.size(); ++i) {
            const LOp* o = rest[i];
            if (skipped > kWindow) {
                left.insert(left.end(), rest.begin() + (long)i, rest.end());
                break;
            }
            const uint64_t sup = support_of(*o), t = targets_of(*o);
            const bool conflict = (sup & (o->diagonal() ? blk_nondiag : blk_any)) != 0;
            const size_t ob = (tc_budget && !whole && o->cls == L_MATK && o->k >= 3) ? tc_op_bytes(o->k) : 0;
            const bool fits_tc = !(has_tc || ob > 0) || cur.ops.size() < (size_t)kTcMaxOps;
            if (!conflict && __builtin_popcountll(S | t) <= m && blob + ob <= kTcBlobMax && fits_tc) {
                S |= t;
                blob += ob;
                has_tc |= ob > 0;
                cur.ops.push_back(o);
            } else {
                left.push_back(o);
                blk_any |= sup;
                if (!o->diagonal()) blk_nondiag |= sup;
                ++skipped;
            }
        }
        cur.bits = bits_of(S);
        passes.push_back(std::move(cur));
        rest.swap(left);
    }
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

// B operand of tc_apply for a fused unitary, in the interleaved real form
// (n = 2r + output part, kk = 2c + input part; part 0 = real, 1 = imaginary):
//   B[2r][2c] = Ur, B[2r][2c+1] = -Ui, B[2r+1][2c] = Ui, B[2r+1][2c+1] = Ur
// (N = K = 2D), split into bf16 hi and lo, no-swizzle K-major layout, the lo
// split right after the hi split.
static void tc_operand(const std::vector<double>& mk, int k, std::vector<unsigned char>& out) {
    const uint32_t D = 1u << k, K = 2 * D, N = 2 * D;
    const size_t split = 2ull * N * K;
    const size_t at = out.size();
    out.resize(at + 2 * split, 0);
    // each component (Ur, Ui of every entry) is split once, in one loop over
    // the matrix; -Ui is the sign-flipped split of Ui (rounding to nearest
    // even is symmetric).  Tensor-core ops have k >= 3: D is a multiple of 4.
    const uint32_t E = 2u * D * D;
    uint16_t sh[2 * 32 * 32], sl[2 * 32 * 32];
    for (uint32_t e = 0; e < E; ++e) {
        const double v = mk[e];
        const uint16_t h = host_bf16((float)v);
        sh[e] = h;
        sl[e] = host_bf16((float)(v - (double)host_bf16_val(h)));
    }
    unsigned char* hi = &out[at];
    unsigned char* lo = hi + split;
    // the 2x2 real block of entry (r, c) sits in one 8x8 core matrix (2r
    // and 2c are even): (2r, 2c) and (2r, 2c+1) are adjacent halves of a
    // 32-bit word (Ur, -Ui), row 2r+1 holds (Ui, Ur) 16 bytes on, and
    // entries c .. c+3 (c a multiple of 4) fill the core matrix's rows 2r and
    // 2r+1: two 16-byte runs per split
    auto words = [](const uint16_t* sp, uint32_t e, uint32_t* w0, uint32_t* w1) {
        for (uint32_t j = 0; j < 4; ++j) {
            const uint32_t r = sp[e + 2 * j], i = sp[e + 2 * j + 1];
            w0[j] = r | ((i ^ 0x8000u) << 16);  // Ur, -Ui
            w1[j] = i | (r << 16);              // Ui, Ur
        }
    };
    for (uint32_t r = 0; r < D; ++r)
        for (uint32_t c = 0; c < D; c += 4) {
            const uint32_t e = 2 * (r * D + c), off = kmajor_off(2 * r, 2 * c, K);
            uint32_t w0[4], w1[4];
            words(sh, e, w0, w1);
            std::memcpy(hi + off, w0, 16);
            std::memcpy(hi + off + 16, w1, 16);
            words(sl, e, w0, w1);
            std::memcpy(lo + off, w0, 16);
            std::memcpy(lo + off + 16, w1, 16);
        }
}

static void pad_to(std::vector<unsigned char>& v, size_t align) {
    v.resize((v.size() + align - 1) / align * align, 0);
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


// Bytes one tensor-core op takes in its pass's blob: B hi and lo splits
// (2 x 2N x K each), the data-column table (u16 per column, padded to 1 KiB)
// and the matrix-row table (32 x u16).
static size_t tc_op_bytes(int k) {
    const size_t D = size_t(1) << k;
    return 2 * (2 * (2 * D) * (2 * D)) + 1024 + 64;
}

// Index tables of a tensor-core op, appended to the blob after its B splits:
// colbase[c] = byte offset of data column c in the padded tile (c over the
// non-target tile bits), offr[r] = byte offset of matrix row r's index bits
// (qubit ltb[0] is the row's most significant bit).  Data column c is the MMA's M row c % 128 of
// block c / 128 and the TMEM lane of the thread that gathers it, so the 32
// lanes of a warp read columns c .. c + 31 at once: the five lowest bits of
// c go to the five non-target tile bits that spread those reads (and the
// write-back) over the most shared-memory banks in the padded tile layout,
// the remaining bits of c to the other non-target bits in ascending order.
// Both tables depend only on the op's tile bits, so they are computed once
// per host thread and bit set.
constexpr size_t kTcTableBytes = 1024 + 64;
static void tc_tables_compute(const TileOp& t, unsigned char* out);

static void tc_tables(TileOp& t, std::vector<unsigned char>& blob) {
    struct Entry {
        unsigned char bytes[kTcTableBytes];
    };
    thread_local std::unordered_map<uint64_t, Entry> memo;
    uint64_t key = (uint64_t)t.k;
    for (int i = 0; i < t.k; ++i) key |= (uint64_t)t.ltb[i] << (4 + 5 * i);
    auto it = memo.find(key);
    if (it == memo.end()) {
        // fused unitaries list their bits in one order (at most 1507 sets of
        // 3..5 of the 12 tile bits); user unitaries may use any order, so
        // the memo is bounded
        if (memo.size() >= 4096) memo.clear();
        Entry e;
        std::memset(e.bytes, 0, sizeof(e.bytes));
        tc_tables_compute(t, e.bytes);
        it = memo.emplace(key, e).first;
    }
    blob.insert(blob.end(), it->second.bytes, it->second.bytes + kTcTableBytes);
    t.lt1 = 0;
}

// Shared-memory wavefronts of 32 lanes reading one float2 each at tile
// indices j[0..31] in the padded layout (row stride kTcRowStride): the most
// distinct 4-byte words any bank must deliver.
static int tc_wavefronts(const uint32_t* j) {
    const uint32_t pad = (kTcRowStride - 256u) / 8u;  // float2 elements of padding per row
    uint32_t words[32][64];
    int cnt[32] = {0};
    int worst = 0;
    for (int l = 0; l < 32; ++l) {
        const uint32_t w0 = 2u * (j[l] + (j[l] >> 5) * pad);  // first 4-byte word
        for (uint32_t w = w0; w < w0 + 2u; ++w) {
            const uint32_t b = w & 31u;
            bool seen = false;
            for (int i = 0; i < cnt[b]; ++i) seen |= words[b][i] == w;
            if (!seen) words[b][cnt[b]++] = w;
            worst = std::max(worst, cnt[b]);
        }
    }
    return worst;
}

static void tc_tables_compute(const TileOp& t, unsigned char* out) {
    const int k = t.k;
    uint32_t tmask = 0;
    for (int i = 0; i < k; ++i) tmask |= 1u << t.ltb[i];
    const uint32_t nmask = ((1u << kTcTileBits) - 1u) & ~tmask;
    std::vector<int> free_bits;
    for (int b = 0; b < kTcTileBits; ++b)
        if ((nmask >> b) & 1u) free_bits.push_back(b);
    const int nf = (int)free_bits.size();  // 12 - k >= 7
    // the five lane bits: every choice of 5 of the free bits, fewest
    // wavefronts first, then the lowest bits
    uint32_t best_sel = 0;
    int best_cost = 1 << 30;
    for (uint32_t sel = 0; sel < (1u << nf); ++sel) {
        if (__builtin_popcount(sel) != 5) continue;
        uint32_t lanes[32];
        for (uint32_t l = 0; l < 32; ++l) {
            uint32_t j = 0, x = l;
            for (int i = 0; i < nf; ++i)
                if ((sel >> i) & 1u) {
                    j |= (x & 1u) << free_bits[i];
                    x >>= 1;
                }
            lanes[l] = j;
        }
        const int cost = tc_wavefronts(lanes);
        if (cost < best_cost) {
            best_cost = cost;
            best_sel = sel;
        }
    }
    std::vector<int> order;  // bit i of c -> tile bit order[i]
    for (int i = 0; i < nf; ++i)
        if ((best_sel >> i) & 1u) order.push_back(free_bits[i]);
    for (int i = 0; i < nf; ++i)
        if (!((best_sel >> i) & 1u)) order.push_back(free_bits[i]);
    // both tables hold byte offsets in the padded tile layout of the
    // tensor-core kernel (row stride kTcRowStride): it is additive over
    // disjoint index bits, so colbase[c] + offr[r] addresses the amplitude
    const uint32_t pad = (kTcRowStride - 256u) / 8u;
    auto byte_at = [pad](uint32_t j) { return (uint16_t)(8u * (j + (j >> 5) * pad)); };
    const uint32_t cols = 1u << nf;
    for (uint32_t c = 0; c < cols; ++c) {
        uint32_t j = 0;
        for (int i = 0; i < nf; ++i) j |= ((c >> i) & 1u) << order[i];
        const uint16_t v = byte_at(j);
        std::memcpy(out + 2 * c, &v, 2);
    }
    for (uint32_t r = 0; r < (1u << k); ++r) {
        uint32_t off = 0;
        for (int i = 0; i < k; ++i)
            if ((r >> (k - 1 - i)) & 1u) off |= 1u << t.ltb[i];
        const uint16_t v = byte_at(off);
        std::memcpy(out + 1024 + 2 * r, &v, 2);
    }
}

// Encode the passes of `ops` into a table of TileOps and an operand pool.
// ---- register phases (host side) ------------------------------------------------
//
// Runs of consecutive ops of a CUDA-core pass become register phases (see
// tile_device.cuh): a run grows while the union of the register bits its
// ops need stays within RB (2x2 gates and permutations need their targets,
// dense unitaries of k <= 3 qubits their k bits, diagonal ops none).  Dense
// unitaries of more qubits stay single ops on the shared-memory path.
constexpr int kPhaseMinSlotBits = 5;  // at least 32 slots (one warp) per tile

static int phase_reg_bits(int dtype) { return dtype == AQSG_C64 ? 4 : 3; }

static bool reg_needs(const TileOp& t, int rb, uint32_t* need) {
    switch (t.cls) {
        case L_DIAG1:
        case L_DIAG2: *need = 0; return true;
        case L_MAT2:
        case L_PERM_X:
        case L_PERM_OR: *need = 1u << t.lt0; return true;
        case L_PERM_SWAP: *need = (1u << t.lt0) | (1u << t.lt1); return true;
        case L_MATK: {
            if (t.pad || t.k > 3 || t.k > rb) return false;
            uint32_t b = 0;
            for (int j = 0; j < t.k; ++j) b |= 1u << t.ltb[j];
            *need = b;
            return true;
        }
        default: return false;
    }
}

static std::vector<TileOp> register_phases(const std::vector<TileOp>& ops, int m, int dtype,
                                           std::vector<unsigned char>& pool) {
    const int rb = phase_reg_bits(dtype);
    if (m < rb + kPhaseMinSlotBits || m > 15) return ops;
    const uint32_t E = 1u << rb;
    std::vector<TileOp> out;
    out.reserve(ops.size() + 8);
    size_t i = 0;
    while (i < ops.size()) {
        uint32_t R = 0;
        if (!reg_needs(ops[i], rb, &R)) {
            out.push_back(ops[i++]);
            continue;
        }
        size_t j = i + 1;
        for (uint32_t nd; j < ops.size() && reg_needs(ops[j], rb, &nd) && __builtin_popcount(R | nd) <= rb; ++j)
            R |= nd;
        // pad the register bits with the highest free positions
        for (int b = m - 1; b >= 0 && __builtin_popcount(R) < rb; --b) R |= 1u << b;
        int rpos[8], rix[16];
        for (int b = 0, c = 0; b < 16; ++b) {
            rix[b] = -1;
            if ((R >> b) & 1u) {
                rix[b] = c;
                rpos[c++] = b;
            }
        }
        // slot-index bits: first one position of each residue mod rb (the
        // bits a half / quarter warp varies fall into distinct banks under
        // the swizzled layout), then the rest in ascending order
        std::vector<int> tpos;
        uint32_t used = 0, seen_res = 0;
        for (int b = 0; b < m; ++b)
            if (!((R >> b) & 1u) && !((seen_res >> (b % rb)) & 1u)) {
                seen_res |= 1u << (b % rb);
                used |= 1u << b;
                tpos.push_back(b);
            }
        for (int b = 0; b < m; ++b)
            if (!((R >> b) & 1u) && !((used >> b) & 1u)) tpos.push_back(b);
        auto dep = [&](uint32_t e) {
            uint32_t o = 0;
            for (int q = 0; q < rb; ++q)
                if ((e >> q) & 1u) o |= 1u << rpos[q];
            return o;
        };
        TileOp h;
        std::memset(&h, 0, sizeof(h));
        h.cls = T_RPHASE;
        h.k = (int32_t)(j - i);
        h.lt0 = rb;
        h.ext_t = -1;
        for (int q = 0; q < rb; ++q) h.am_loc |= (uint64_t)rpos[q] << (4 * q);
        for (size_t q = 0; q < tpos.size(); ++q) h.cm_loc |= (uint64_t)tpos[q] << (4 * q);
        out.push_back(h);
        for (size_t q = i; q < j; ++q) {
            const TileOp& t = ops[q];
            ROp r;
            std::memset(&r, 0, sizeof(r));
            const uint32_t cm = (uint32_t)t.cm_loc, cv = (uint32_t)t.cv_loc;
            r.ctl = (cm & ~R) | ((cv & ~R) << 16);
            r.cm_ext = t.cm_ext;
            r.cv_ext = t.cv_ext;
            r.ext_t = -1;
            uint32_t flags = t.cm_ext ? RF_EXT : 0u;
            auto ctl = [&](uint32_t idx) { return (idx & cm & R) == (cv & R); };
            uint32_t em = 0;
            for (uint32_t e = 0; e < E; ++e)
                if (ctl(dep(e))) em |= 1u << e;
            auto put_complex = [&](int count) {  // t.m[0 .. 2 count) as the kernel's complex type
                if (dtype == AQSG_C64) {
                    float f[8];
                    for (int c = 0; c < 2 * count; ++c) f[c] = (float)t.m[c];
                    std::memcpy(r.coef, f, sizeof(float) * 2 * count);
                } else {
                    std::memcpy(r.coef, t.m, sizeof(double) * 2 * count);
                }
            };
            uint32_t kind = 0, ra = 0, rbb = 0;
            switch (t.cls) {
                case L_MAT2: {
                    ra = (uint32_t)rix[t.lt0];
                    const bool real = t.m[1] == 0.0 && t.m[3] == 0.0 && t.m[5] == 0.0 && t.m[7] == 0.0;
                    if (real) {
                        kind = RK_MAT2R;
                        if (dtype == AQSG_C64) {
                            const float f[4] = {(float)t.m[0], (float)t.m[2], (float)t.m[4], (float)t.m[6]};
                            std::memcpy(r.coef, f, sizeof(f));
                        } else {
                            const double d[4] = {t.m[0], t.m[2], t.m[4], t.m[6]};
                            std::memcpy(r.coef, d, sizeof(d));
                        }
                    } else {
                        kind = RK_MAT2C;
                        put_complex(4);
                    }
                    break;
                }
                case L_PERM_X:
                case L_PERM_OR: {
                    kind = RK_PERM;
                    ra = (uint32_t)rix[t.lt0];
                    if (t.cls == L_PERM_OR) {
                        flags |= RF_OR;
                        if (t.am_ext) flags |= RF_EXT;
                        const uint32_t am = (uint32_t)t.am_loc;
                        r.amt = am & ~R;
                        r.am_ext = t.am_ext;
                        uint32_t om = 0;
                        for (uint32_t e = 0; e < E; ++e)
                            if (dep(e) & am & R) om |= 1u << e;
                        em |= om << 16;
                    }
                    break;
                }
                case L_PERM_SWAP: {
                    kind = RK_SWAP;
                    const int a2 = rix[t.lt0], b2 = rix[t.lt1];
                    ra = (uint32_t)(a2 < b2 ? a2 : b2);
                    rbb = (uint32_t)(a2 < b2 ? b2 : a2);
                    if (a2 > b2) {  // the control is checked at (a = 0, b = 1)
                        em = 0;
                        for (uint32_t e = 0; e < E; ++e)
                            if (ctl(dep(e ^ (1u << a2) ^ (1u << b2)))) em |= 1u << e;
                    }
                    break;
                }
                case L_DIAG1:
                case L_DIAG2: {
                    kind = RK_DIAG;
                    put_complex(2);
                    if (t.cls == L_DIAG2) {
                        if (t.lt0 >= 0 && ((R >> t.lt0) & 1u)) {
                            kind = RK_DIAGR;
                            ra = (uint32_t)rix[t.lt0];
                        } else if (t.lt0 >= 0) {
                            flags |= RF_TTHR;
                            r.extra = (uint32_t)t.lt0;
                        } else {
                            flags |= RF_TEXT;
                            r.ext_t = t.ext_t;
                        }
                    }
                    break;
                }
                default: {  // L_MATK, k <= 3, all bits register bits
                    kind = RK_MATK;
                    const int k = t.k, D = 1 << k;
                    int rmask = 0;
                    for (int q2 = 0; q2 < k; ++q2) rmask |= 1 << rix[t.ltb[q2]];
                    // old matrix bit (k-1-q2) <-> register index rix[ltb[q2]];
                    // new matrix bit b <-> the b-th lowest register index
                    int oldbit_of_new[8];
                    for (int b = 0, c = 0; b < rb; ++b)
                        if ((rmask >> b) & 1)
                            for (int q2 = 0; q2 < k; ++q2)
                                if (rix[t.ltb[q2]] == b) oldbit_of_new[c++] = k - 1 - q2;
                    auto old_index = [&](int nidx) {
                        int o = 0;
                        for (int b = 0; b < k; ++b)
                            if ((nidx >> b) & 1) o |= 1 << oldbit_of_new[b];
                        return o;
                    };
                    const size_t esz = dtype == AQSG_C64 ? 8 : 16;
                    std::vector<unsigned char> src(pool.begin() + t.mat, pool.begin() + t.mat + esz * D * D);
                    for (int rr = 0; rr < D; ++rr)
                        for (int cc = 0; cc < D; ++cc)
                            std::memcpy(&pool[t.mat + esz * (rr * D + cc)],
                                        &src[esz * (old_index(rr) * D + old_index(cc))], esz);
                    ra = (uint32_t)rmask;
                    r.extra = (uint32_t)t.mat;
                    em = 0;
                    for (uint32_t e = 0; e < E; ++e)
                        if (!(e & (uint32_t)rmask) && ctl(dep(e))) em |= 1u << e;
                    break;
                }
            }
            if (r.ext_t >= 0) flags |= RF_EXT;
            r.code = kind | (ra << 8) | (rbb << 12) | flags;
            r.em = em;
            TileOp slot;
            std::memcpy(&slot, &r, sizeof(slot));
            out.push_back(slot);
        }
        i = j;
    }
    return out;
}

// Shift the pool offsets of a pass table's dense matrices by delta (tables
// moved into a larger pool); returns whether the table has any.
bool relocate_tile_matrices(unsigned char* table, size_t count, int32_t delta) {
    bool any = false;
    for (size_t q = 0; q < count; ++q) {
        TileOp t;
        std::memcpy(&t, table + q * sizeof(TileOp), sizeof(TileOp));
        if (t.cls == T_RPHASE) {
            for (int k = 0; k < t.k; ++k) {
                ROp r;
                unsigned char* at = table + (q + 1 + k) * sizeof(TileOp);
                std::memcpy(&r, at, sizeof(ROp));
                if ((r.code & 0xFFu) == RK_MATK) {
                    r.extra += (uint32_t)delta;
                    any = true;
                    std::memcpy(at, &r, sizeof(ROp));
                }
            }
            q += (size_t)t.k;
        } else if (t.cls == L_MATK && !t.pad) {  // (a tensor-core op's offset is into its pass's blob)
            t.mat += delta;
            any = true;
            std::memcpy(table + q * sizeof(TileOp), &t, sizeof(TileOp));
        }
    }
    return any;
}

int encode_tiled(int n, int dtype, const std::vector<LOp>& ops, bool tc_on, TilePlan* plan, bool exact_perm,
                 int whole_max) {
    plan->table.clear();
    plan->pool.clear();
    plan->passes.clear();
    plan->any_tc = false;
    plan->any_stream = false;
    plan->n = n;
    plan->dtype = dtype;
    std::vector<Pass> passes = aqsg::plan(n, dtype, ops, tc_on && dtype == AQSG_C64, whole_max);
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
        // the tensor-core kernel keeps its op table in shared memory: a pass
        // with more ops (a whole 12-qubit register; the planner keeps
        // streaming tensor-core passes within the limit) runs on CUDA cores
        const bool tc_pass = tc_on && dtype == AQSG_C64 && tp.m == kTcTileBits && p.ops.size() <= (size_t)kTcMaxOps;
        std::vector<unsigned char> blob;  // this pass's tensor-core operands
        if (tc_pass) blob.reserve(kTcBlobMax);
        std::vector<TileOp> pops;         // this pass's table
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
                const size_t need = tc_op_bytes(o->k);
                if (tc_pass && o->k >= 3 && t.cm_loc == 0 && !(exact_perm && is_permutation(o->mk, o->k)) &&
                    blob.size() + need <= kTcBlobMax) {
                    t.pad = 1;  // tensor-core op; mat = offset in the pass's blob
                    tp.tc = 1;
                    t.mat = (int32_t)blob.size();
                    tc_operand(o->mk, o->k, blob);
                    tc_tables(t, blob);
                } else {
                    pad_to(plan->pool, 256);
                    t.mat = (int32_t)plan->pool.size();
                    tp.matk = 1;
                    const size_t DD = (size_t)1 << (2 * o->k);
                    const size_t at = plan->pool.size();
                    if (dtype == AQSG_C64) {
                        plan->pool.resize(at + 8 * DD);
                        for (size_t e = 0; e < 2 * DD; ++e) {
                            const float v = (float)o->mk[e];
                            std::memcpy(&plan->pool[at + 4 * e], &v, 4);
                        }
                    } else {
                        plan->pool.resize(at + 16 * DD);
                        std::memcpy(&plan->pool[at], o->mk.data(), 16 * DD);
                    }
                }
            }
            pops.push_back(t);
        }
        // passes on the CUDA cores: runs of ops as register phases
        if (!tp.tc) {
            pops = register_phases(pops, tp.m, dtype, plan->pool);
            // the kernels size their diagonal runs for tiles without phases
            if (tp.m >= phase_reg_bits(dtype) + kPhaseMinSlotBits)
                for (size_t q = 0; q < pops.size(); ++q) {
                    if (pops[q].cls == T_RPHASE) q += (size_t)pops[q].k;  // skip the phase's ROps
                    else if (pops[q].cls == L_DIAG1 || pops[q].cls == L_DIAG2)
                        return set_error(AQSG_ERR_RUNTIME, "Diagonal op outside a register phase");
                }
        }
        for (const TileOp& t : pops) {
            const size_t at = plan->table.size();
            plan->table.resize(at + tsize);
            std::memcpy(&plan->table[at], &t, tsize);
        }
        tp.count = (uint32_t)(plan->table.size() / tsize) - tp.first;
        if (tp.tc) {
            pad_to(plan->pool, 1024);
            tp.tc_blob = (uint32_t)plan->pool.size();
            tp.tc_bytes = (uint32_t)blob.size();
            plan->pool.insert(plan->pool.end(), blob.begin(), blob.end());
        }
        plan->any_tc = plan->any_tc || tp.tc;
        plan->any_stream = plan->any_stream || tp.tc;
        plan->passes.push_back(tp);
    }
    return AQSG_OK;
}

size_t TilePlan::pool_offset() const { return (table.size() + 255) & ~size_t(255); }

// Resident CTAs per SM of a kernel at a dynamic shared-memory size, and
// the SM count, per device (queried once).
struct StreamShape {
    int sms = 0, per_sm = 0;
};

template <typename K>
static int stream_shape(K kernel, int threads, int shm, StreamShape* out) {
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, StreamShape> cache;
    int dev = 0;
    AQSG_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(mu);
    auto key = std::make_pair(dev, (const void*)kernel);
    auto it = cache.find(key);
    if (it != cache.end()) {
        *out = it->second;
        return AQSG_OK;
    }
    StreamShape sh;
    AQSG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shm));
    AQSG_CUDA_TRY(cudaDeviceGetAttribute(&sh.sms, cudaDevAttrMultiProcessorCount, dev));
    AQSG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sh.per_sm, kernel, threads, shm));
    if (sh.per_sm < 1) return set_error(AQSG_ERR_RUNTIME, "Streaming tile kernel does not fit on an SM");
    cache[key] = sh;
    *out = sh;
    return AQSG_OK;
}

// cuTensorMapEncodeTiled from the driver, looked up once (null if the
// driver has none: tile loads then stay on cp.async).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
        else
            cudaGetLastError();
    });
    return fn;
}

// The tensor map of a tensor-core pass's tiles over `members` registers of
// 2^n amplitudes stored back to back at sv (see TmaGeom); tg->rank = 0 when
// the pass's high tile bits form more than four runs or the encoding fails.
static void tile_tensor_map(void* sv, int n, const TilePass& p, uint32_t members, CUtensorMap* map, TmaGeom* tg) {
    std::memset(tg, 0, sizeof(*tg));
    std::memset(map, 0, sizeof(*map));
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || p.m != kTcTileBits || p.L != 5) return;
    int rank = 1;
    int start[5] = {0, 0, 0, 0, 0}, run[5] = {5, 0, 0, 0, 0};
    for (int i = p.L; i < p.m; ++i) {
        const int b = p.tbits[i];
        if (rank > 1 && b == start[rank - 1] + run[rank - 1]) {
            ++run[rank - 1];
            continue;
        }
        if (rank == 5) return;  // a fifth run of high bits
        start[rank] = b;
        run[rank] = 1;
        ++rank;
    }
    cuuint64_t dim[5], stride[4];
    cuuint32_t box[5], estride[5] = {1, 1, 1, 1, 1};
    for (int d = 0; d < rank; ++d) {
        const int end = d + 1 < rank ? start[d + 1] : n;
        tg->start[d] = start[d];
        tg->bits[d] = end - start[d];
        dim[d] = (cuuint64_t)1 << (end - start[d]);
        box[d] = d == 0 ? kTmaRowBox : (cuuint32_t)1 << run[d];
        if (d > 0) stride[d - 1] = ((cuuint64_t)1 << start[d]) * sizeof(float2);
    }
    dim[rank - 1] *= members;
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_INT64, (cuuint32_t)rank, sv, dim, stride, box, estride,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r == CUDA_SUCCESS) tg->rank = rank;
}

template <typename R>
static int launch_plan_t(void* sv, const TilePlan& plan, const void* dev, cudaStream_t stream, int* d_err,
                         uint64_t* launches, double* norm_part, uint32_t* tc_grid) {
    using T = typename Cx<R>::T;
    const int n = plan.n;
    const TileOp* dops = (const TileOp*)dev;
    const unsigned char* dpool = (const unsigned char*)dev + plan.pool_offset();
    // whole registers: register phases cover every diagonal op once the
    // register has 2^(RB + kPhaseMinSlotBits) amplitudes; below that the
    // diagonal runs need 2 elements per thread (threads >= size / 2)
    constexpr int EPT_WHOLE = 2;
    constexpr int M_STREAM = sizeof(R) == 4 ? 12 : 11;
    auto kwhole = k_tile<R, EPT_WHOLE, false>;
    auto kwhole_k = k_tile<R, EPT_WHOLE, true>;
    constexpr int EPT_S = (1 << M_STREAM) / kStreamThreads;
    // [MATK][op table in shared memory]
    void (*const kstream[2][2])(T*, const TileGeom, const TileOp*, int, const unsigned char*) = {
        {k_tile_stream<R, EPT_S, false, false>, k_tile_stream<R, EPT_S, false, true>},
        {k_tile_stream<R, EPT_S, true, false>, k_tile_stream<R, EPT_S, true, true>}};
    static_assert(((1 << M_STREAM) >> (sizeof(R) == 4 ? 4 : 3)) == 2 * kStreamThreads,
                  "two register-phase slots per thread");
    constexpr int kStreamShmMax = (int)(sizeof(T) << M_STREAM) + 8 * 128 + (int)kStreamOpsSmemMax;
    for (int a = 0; a < 2; ++a)
        AQSG_CUDA_TRY(cudaFuncSetAttribute(kstream[a][1], cudaFuncAttributeMaxDynamicSharedMemorySize, kStreamShmMax));
    constexpr int kWholeShmMax = 232448;  // the register plus, where it fits, its op table
    AQSG_CUDA_TRY(cudaFuncSetAttribute(kwhole, cudaFuncAttributeMaxDynamicSharedMemorySize, kWholeShmMax));
    AQSG_CUDA_TRY(cudaFuncSetAttribute(kwhole_k, cudaFuncAttributeMaxDynamicSharedMemorySize, kWholeShmMax));
    StreamShape tshape;
    bool have_t = false;
    for (size_t pi = 0; pi < plan.passes.size(); ++pi) {
        const TilePass& p = plan.passes[pi];
        TileGeom geo;
        std::memset(&geo, 0, sizeof(geo));
        geo.n = n;
        geo.m = p.m;
        geo.L = p.L;
        for (int i = 0; i < p.m; ++i) geo.tbits[i] = p.tbits[i];
        geo.tc_blob = p.tc_blob;
        geo.tc_bytes = p.tc_bytes;
        const uint32_t size = 1u << geo.m;
        if (p.tc) {  // c64, 12 tile bits (streaming, or the whole 12-qubit register)
            if (geo.m != kTcTileBits || sizeof(R) != 4)
                return set_error(AQSG_ERR_RUNTIME, "Tensor-core pass with an unexpected tile shape");
            auto ktc = p.matk ? k_stream_tc<false, true> : k_stream_tc<false, false>;
            if (!have_t) {  // both variants have the same shape
                if (int rc = stream_shape(k_stream_tc<false, true>, kTcCta, (int)TcStreamSmem::kBytes, &tshape))
                    return rc;
                if (int rc = stream_shape(k_stream_tc<false, false>, kTcCta, (int)TcStreamSmem::kBytes, &tshape))
                    return rc;
                have_t = true;
            }
            if (p.tc_bytes > kTcBlobMax) return set_error(AQSG_ERR_RUNTIME, "Tensor-core operands exceed the blob");
            if (p.count > (uint32_t)kTcMaxOps) return set_error(AQSG_ERR_RUNTIME, "Tensor-core pass with too many ops");
            const uint32_t tiles = 1u << (n - geo.m);
            const uint32_t grid = std::min<uint32_t>(tiles, (uint32_t)(tshape.sms * tshape.per_sm));
            if (tc_grid) *tc_grid = grid;
            uint32_t nf = 0;
            if (norm_part) nf = (pi == 0 ? 1u : 0u) | (pi + 1 == plan.passes.size() ? 2u : 0u);
            CUtensorMap map;
            TmaGeom tg;
            tile_tensor_map(sv, n, p, 1u, &map, &tg);
            ktc<<<grid, kTcCta, TcStreamSmem::kBytes, stream>>>(
                (float2*)sv, geo, (const unsigned char*)dev, p.first, (int)p.count, plan.pool_offset(), d_err, tiles,
                1u, 0ull, 0ull, norm_part, nf, map, tg);
        } else if (geo.m == n) {
            const int rb = phase_reg_bits(plan.dtype);
            int threads = (int)(geo.m >= rb + kPhaseMinSlotBits ? size >> rb : size / EPT_WHOLE);
            threads = threads < 32 ? 32 : (threads > 512 ? 512 : threads);
            const size_t reg_bytes = sizeof(T) * size, ops_bytes = sizeof(TileOp) * p.count;
            const int ops_smem = reg_bytes + ops_bytes <= (size_t)kWholeShmMax ? 1 : 0;
            (p.matk ? kwhole_k : kwhole)<<<1, threads, reg_bytes + (ops_smem ? ops_bytes : 0), stream>>>(
                (T*)sv, geo, dops + p.first, (int)p.count, dpool, ops_smem);
        } else {
            if (geo.m != M_STREAM) return set_error(AQSG_ERR_RUNTIME, "Streaming pass with an unexpected tile size");
            const size_t ops_bytes = sizeof(TileOp) * p.count;
            const int ops_smem = ops_bytes <= kStreamOpsSmemMax ? 1 : 0;
            const size_t shm = sizeof(T) * size + (size_t(1) << (geo.m - geo.L)) * sizeof(uint64_t) +
                               (ops_smem ? ops_bytes : 0);
            kstream[p.matk ? 1 : 0][ops_smem]<<<(unsigned)(1ull << (n - geo.m)), kStreamThreads, shm, stream>>>(
                (T*)sv, geo, dops + p.first, (int)p.count, dpool);
        }
        if (launches) ++*launches;
        AQSG_CUDA_TRY(cudaGetLastError());
    }
    return AQSG_OK;
}

int launch_tile_plan_multi(void* sv0, uint64_t reg_stride, int members, const TilePlan& plan, const void* dev0,
                           uint64_t dev_stride, cudaStream_t stream, int* d_err, uint64_t* launches) {
    if (plan.dtype != AQSG_C64) return set_error(AQSG_ERR_RUNTIME, "Grouped tile passes take complex64 plans");
    const int n = plan.n;
    constexpr int EPT = (1 << 12) / kStreamThreads;
    // [MATK][op table in shared memory]
    void (*const kmulti[2][2])(float2*, uint64_t, const TileGeom, const unsigned char*, uint64_t, uint32_t, int,
                               uint64_t, uint32_t) = {
        {k_tile_stream_multi<float, EPT, false, false>, k_tile_stream_multi<float, EPT, false, true>},
        {k_tile_stream_multi<float, EPT, true, false>, k_tile_stream_multi<float, EPT, true, true>}};
    constexpr int kStreamShmMax = (int)(sizeof(float2) << 12) + 8 * 128 + (int)kStreamOpsSmemMax;
    for (int a = 0; a < 2; ++a)
        AQSG_CUDA_TRY(cudaFuncSetAttribute(kmulti[a][1], cudaFuncAttributeMaxDynamicSharedMemorySize, kStreamShmMax));
    StreamShape tshape;
    bool have_t = false;
    for (const TilePass& p : plan.passes) {
        if (p.m != 12 || p.m == n) return set_error(AQSG_ERR_RUNTIME, "Grouped tile passes take streaming plans");
        TileGeom geo;
        std::memset(&geo, 0, sizeof(geo));
        geo.n = n;
        geo.m = p.m;
        geo.L = p.L;
        for (int i = 0; i < p.m; ++i) geo.tbits[i] = p.tbits[i];
        geo.tc_blob = p.tc_blob;
        geo.tc_bytes = p.tc_bytes;
        const uint32_t size = 1u << geo.m;
        const uint32_t tiles = 1u << (n - geo.m);
        const uint64_t blocks = (uint64_t)tiles * (uint64_t)members;
        if (blocks > 0x7fffffffull) return set_error(AQSG_ERR_RUNTIME, "Too many tiles in one grouped pass");
        if (p.tc) {
            auto ktc = p.matk ? k_stream_tc<true, true> : k_stream_tc<true, false>;
            if (!have_t) {  // both variants have the same shape
                if (int rc = stream_shape(k_stream_tc<true, true>, kTcCta, (int)TcStreamSmem::kBytes, &tshape))
                    return rc;
                if (int rc = stream_shape(k_stream_tc<true, false>, kTcCta, (int)TcStreamSmem::kBytes, &tshape))
                    return rc;
                have_t = true;
            }
            if (p.tc_bytes > kTcBlobMax) return set_error(AQSG_ERR_RUNTIME, "Tensor-core operands exceed the blob");
            if (p.count > (uint32_t)kTcMaxOps) return set_error(AQSG_ERR_RUNTIME, "Tensor-core pass with too many ops");
            const uint32_t grid = (uint32_t)std::min<uint64_t>(blocks, (uint64_t)tshape.sms * tshape.per_sm);
            CUtensorMap map;
            TmaGeom tg;
            std::memset(&map, 0, sizeof(map));
            std::memset(&tg, 0, sizeof(tg));
            // the members' registers must lie back to back for one tensor map
            if (reg_stride == (1ull << n)) tile_tensor_map(sv0, n, p, (uint32_t)members, &map, &tg);
            ktc<<<grid, kTcCta, TcStreamSmem::kBytes, stream>>>(
                (float2*)sv0, geo, (const unsigned char*)dev0, p.first, (int)p.count, plan.pool_offset(), d_err,
                tiles, (uint32_t)members, reg_stride, dev_stride, nullptr, 0u, map, tg);
        } else {
            const size_t ops_bytes = sizeof(TileOp) * p.count;
            const int ops_smem = ops_bytes <= kStreamOpsSmemMax ? 1 : 0;
            const size_t shm = sizeof(float2) * size + (size_t(1) << (geo.m - geo.L)) * sizeof(uint64_t) +
                               (ops_smem ? ops_bytes : 0);
            kmulti[p.matk ? 1 : 0][ops_smem]<<<(unsigned)blocks, kStreamThreads, shm, stream>>>(
                (float2*)sv0, reg_stride, geo, (const unsigned char*)dev0, dev_stride, p.first, (int)p.count,
                plan.pool_offset(), tiles);
        }
        if (launches) ++*launches;
        AQSG_CUDA_TRY(cudaGetLastError());
    }
    return AQSG_OK;
}

int launch_tile_plan(void* sv, const TilePlan& plan, const void* dev, cudaStream_t stream, int* d_err,
                     uint64_t* launches, double* norm_part, uint32_t* tc_grid) {
    return plan.dtype == AQSG_C64 ? launch_plan_t<float>(sv, plan, dev, stream, d_err, launches, norm_part, tc_grid)
                                  : launch_plan_t<double>(sv, plan, dev, stream, d_err, launches, norm_part, tc_grid);
}

// ---- plan cache ----------------------------------------------------------------------
//
// Re-running a circuit (a simulator that simulates the same QCircuit again,
// a parameter-free sweep of shots) would lower, plan and encode it and copy
// its table to the device each time; the cache keeps the last few encoded
// plans with their device tables.  Entries are matched on the exact key
// bytes, so a hit runs exactly what a miss would.
constexpr size_t kPlanCacheEntries = 8;

struct PlanCache {
    struct Entry {
        std::vector<unsigned char> key;
        TilePlan plan;
        void* dev = nullptr;
        size_t dev_bytes = 0;
        uint64_t last = 0;
    };
    std::vector<Entry> e;
    uint64_t tick = 0;
};

void plan_cache_free(aqsg_ctx_s* c) {
    if (!c->plans) return;
    for (auto& en : c->plans->e)
        if (en.dev) cudaFree(en.dev);
    delete c->plans;
    c->plans = nullptr;
}

size_t tc_norm_doubles(const aqsg_ctx_s* c) { return 2 + 4 * (size_t)c->sm_count; }

// The tile passes of a plan and, for a run with tensor-core passes, the
// renormalisation to the input's FP64 norm, all on the context stream.  The
// tensor-core products lose a little norm in a biased way (~1e-7 per fused
// op).  The norms before and after come from the first and the last pass
// when those run on the tensor cores (per-CTA partials summed in a fixed
// order, so a run gives the same sums every time), else from a read pass of
// their own (whose reduction scratch the caller reserved); the scale factor
// never leaves the device.  norms: tc_norm_doubles() doubles,
// [before, after, partials...].
static int launch_plan_renorm(aqsg_state_s* st, const TilePlan& plan, const void* dev_table, double* norms) {
    aqsg_ctx_s* c = st->ctx;
    const bool fold_in = plan.any_tc && plan.passes.front().tc;
    const bool fold_out = plan.any_tc && plan.passes.back().tc;
    double* parts = norms + 2;
    if (plan.any_tc && !fold_in)
        if (int rc = launch_norm_to_device(st, norms)) return rc;
    uint32_t tc_grid = 0;
    if (int rc = launch_tile_plan(st->d, plan, dev_table, c->stream, c->d_err, &c->launches,
                                  (fold_in || fold_out) ? parts : nullptr, &tc_grid))
        return rc;
    if (!plan.any_tc) return AQSG_OK;
    if (tc_grid > 2u * (uint32_t)c->sm_count) return set_error(AQSG_ERR_RUNTIME, "Norm partials exceed their scratch");
    if (fold_in)
        if (int rc = launch_sum_partials(c, parts, (int)tc_grid, norms)) return rc;
    if (fold_out) {
        if (int rc = launch_sum_partials(c, parts + tc_grid, (int)tc_grid, norms + 1)) return rc;
    } else {
        if (int rc = launch_norm_to_device(st, norms + 1)) return rc;
    }
    return launch_renorm_device(st, norms, norms + 1);
}

// Run an encoded plan whose table is on the device (dev_table): the passes
// with their renormalisation, then the error-flag check.
static int run_encoded(aqsg_state_s* st, const TilePlan& plan, const void* dev_table) {
    aqsg_ctx_s* c = st->ctx;
    double* norms = nullptr;
    if (plan.any_tc) {
        if (int rc = ensure_scratch(c->tcnorm, sizeof(double) * tc_norm_doubles(c))) return rc;
        norms = (double*)c->tcnorm.ptr;
        if (!plan.passes.front().tc || !plan.passes.back().tc)  // a read pass's reduction scratch
            if (int rc = reserve_scratch(c, st->n, 1)) return rc;
    }
    if (int rc = launch_plan_renorm(st, plan, dev_table, norms)) return rc;
    if (plan.any_stream) {  // a bounded wait that gave up leaves a flag
        AQSG_CUDA_TRY(cudaMemcpyAsync(c->host_result, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        AQSG_CUDA_TRY(cudaStreamSynchronize(c->stream));
        int flag = 0;
        std::memcpy(&flag, c->host_result, sizeof(int));
        if (flag) {
            AQSG_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
            return set_error(AQSG_ERR_TIMEOUT, "Tile pass timed out waiting for its copies or MMAs");
        }
    }
    return AQSG_OK;
}

uint64_t plan_hbm_bytes(const TilePlan& plan, bool renorm) {
    const uint64_t reg = (uint64_t)amp_bytes(plan.dtype) << plan.n;
    return renorm ? plan_run_bytes(plan) : 2 * reg * (uint64_t)plan.passes.size();
}

uint64_t plan_run_bytes(const TilePlan& plan) {
    const uint64_t reg = (uint64_t)amp_bytes(plan.dtype) << plan.n;
    uint64_t b = 2 * reg * (uint64_t)plan.passes.size();
    if (plan.any_tc)
        b += 2 * reg + (plan.passes.front().tc ? 0 : reg) + (plan.passes.back().tc ? 0 : reg);
    return b;
}

int run_tiled_cached(aqsg_state_s* st, const std::vector<unsigned char>& key_ops,
                     const std::function<int(std::vector<LOp>*)>& lower) {
    aqsg_ctx_s* c = st->ctx;
    if (!c->plans) c->plans = new PlanCache();
    PlanCache& pc = *c->plans;
    // the tile shape is part of the plan
    const int32_t whole_max = whole_tile_limit(st->dtype, c->whole_tile_max);
    std::vector<unsigned char> key = key_ops;
    key.insert(key.end(), (const unsigned char*)&whole_max, (const unsigned char*)&whole_max + sizeof(whole_max));
    for (auto& en : pc.e)
        if (en.key == key) {
            en.last = ++pc.tick;
            if (en.plan.passes.empty()) return AQSG_OK;
            return run_encoded(st, en.plan, en.dev);
        }
    std::vector<LOp> ops;
    if (int rc = lower(&ops)) return rc;
    PlanCache::Entry fresh;
    fresh.key = key;
    if (int rc = encode_tiled(st->n, st->dtype, ops, c->tensor_cores != 0, &fresh.plan, true, whole_max)) return rc;
    // the slot: a free one, else the least recently used (its device table
    // is reused when large enough)
    PlanCache::Entry* slot = nullptr;
    if (pc.e.size() < kPlanCacheEntries) {
        pc.e.emplace_back();
        slot = &pc.e.back();
    } else {
        slot = &pc.e[0];
        for (auto& en : pc.e)
            if (en.last < slot->last) slot = &en;
    }
    const size_t poff = fresh.plan.pool_offset();
    const size_t bytes = poff + fresh.plan.pool.size() + 16;
    void* dev = slot->dev;
    size_t dev_bytes = slot->dev_bytes;
    slot->key.clear();  // the slot is invalid until the new table is in place
    if (dev_bytes < bytes) {
        if (dev) {
            AQSG_CUDA_TRY(cudaStreamSynchronize(c->stream));  // the old table may still be in use
            AQSG_CUDA_TRY(cudaFree(dev));
            dev = nullptr;
            dev_bytes = 0;
        }
        AQSG_CUDA_TRY(cudaMalloc(&dev, bytes));
        dev_bytes = bytes;
    }
    slot->dev = dev;
    slot->dev_bytes = dev_bytes;
    if (!fresh.plan.passes.empty()) {
        AQSG_CUDA_TRY(cudaMemcpyAsync(dev, fresh.plan.table.data(), fresh.plan.table.size(), cudaMemcpyHostToDevice,
                                      c->stream));
        if (!fresh.plan.pool.empty())
            AQSG_CUDA_TRY(cudaMemcpyAsync((char*)dev + poff, fresh.plan.pool.data(), fresh.plan.pool.size(),
                                          cudaMemcpyHostToDevice, c->stream));
    }
    slot->plan = std::move(fresh.plan);
    slot->key = key;
    slot->last = ++pc.tick;
    if (slot->plan.passes.empty()) return AQSG_OK;
    return run_encoded(st, slot->plan, slot->dev);
}

int run_plan_async(aqsg_state_s* st, const TilePlan& plan, const void* dev_table, double* d_norms) {
    if (plan.passes.empty()) return AQSG_OK;
    return launch_plan_renorm(st, plan, dev_table, d_norms);
}

}  // namespace aqsg

// ---- testing aid ----------------------------------------------------------------------

#include "../../include/aqsg_debug.h"

extern "C" int aqsg_debug_tile_plan(int n, int dtype, const aqsg_op* ops, int count, int fuse_qubits,
                                    int whole_tile_max, int tensor_cores, aqsg_tile_pass* passes, int pass_capacity,
                                    int* pass_count,
                                    void* table, size_t table_capacity, size_t* table_bytes, void* pool,
                                    size_t pool_capacity, size_t* pool_bytes) {
    using namespace aqsg;
    if (n < 1 || n > AQSG_MAX_QUBITS) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Invalid qubit count");
    if (dtype != AQSG_C64 && dtype != AQSG_C128) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown dtype");
    std::vector<LOp> low;
    if (fuse_qubits > 0) {
        aqsg_program p = nullptr;
        if (int rc = aqsg_compile(n, dtype, ops, count, fuse_qubits, &p)) return rc;
        low = program_ops(p);
        aqsg_program_free(p);
    } else {
        if (int rc = aqsg_check_ops(n, ops, count)) return rc;
        for (int i = 0; i < count; ++i) {
            LOp o;
            if (int rc = lower_op(n, dtype, ops[i], &o)) return rc;
            if (o.cls != L_NOP) low.push_back(std::move(o));
        }
    }
    TilePlan plan;
    if (whole_tile_max < 0) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Negative whole-tile qubit count");
    if (tensor_cores < 0 || tensor_cores > 2) return set_error(AQSG_ERR_INVALID_ARGUMENT, "tensor_cores is 0, 1 or 2");
    // 2: the batched engine's form, where a fused permutation matrix goes to
    // the tensor cores too (the choice depends on the op structure only)
    if (int rc = encode_tiled(n, dtype, low, tensor_cores != 0, &plan, tensor_cores != 2, whole_tile_max)) return rc;
    if (pass_count) *pass_count = (int)plan.passes.size();
    if (table_bytes) *table_bytes = plan.table.size();
    if (pool_bytes) *pool_bytes = plan.pool.size();
    if (passes) {
        if (pass_capacity < (int)plan.passes.size()) return set_error(AQSG_ERR_OUT_OF_RANGE, "Pass buffer too small");
        for (size_t i = 0; i < plan.passes.size(); ++i) {
            const TilePass& p = plan.passes[i];
            aqsg_tile_pass& o = passes[i];
            std::memset(&o, 0, sizeof(o));
            o.m = p.m;
            o.L = p.L;
            o.first = (int32_t)p.first;
            o.count = (int32_t)p.count;
            for (int b = 0; b < p.m && b < 16; ++b) o.tbits[b] = p.tbits[b];
            o.tc = p.tc;
            o.matk = p.matk;
            o.tc_blob = p.tc_blob;
            o.tc_bytes = p.tc_bytes;
        }
    }
    if (table) {
        if (table_capacity < plan.table.size()) return set_error(AQSG_ERR_OUT_OF_RANGE, "Table buffer too small");
        if (!plan.table.empty()) std::memcpy(table, plan.table.data(), plan.table.size());
    }
    if (pool && !plan.pool.empty()) {
        if (pool_capacity < plan.pool.size()) return set_error(AQSG_ERR_OUT_OF_RANGE, "Pool buffer too small");
        std::memcpy(pool, plan.pool.data(), plan.pool.size());
    }
    return AQSG_OK;
}
