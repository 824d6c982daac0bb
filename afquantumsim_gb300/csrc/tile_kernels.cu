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
#include <cstring>

#include "aqsg_internal.h"
#include "common.cuh"

namespace aqsg {

struct TileOp {
    int32_t cls;
    int32_t lt0, lt1;  // local target bits; DIAG2 with an external target: lt0 = -1
    int32_t k;
    int32_t ltb[AQSG_MAX_UNITARY_QUBITS];
    int32_t mat;       // MATK: offset (complex elements) in the matrix pool
    int32_t ext_t;     // DIAG2 external target: global bit, else -1
    int32_t pad;
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

// EPT: elements per thread in register runs; MAXT/MINB: launch bounds (the
// whole-register variant runs up to 512 threads in one CTA, the streaming
// variant 256 threads with several CTAs per SM).
template <typename R, int EPT, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB)
k_tile(typename Cx<R>::T* __restrict__ sv, const TileGeom g, const TileOp* __restrict__ ops,
       int nops, const typename Cx<R>::T* __restrict__ mats) {
    using T = typename Cx<R>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int m = g.m, L = g.L;
    const uint32_t size = 1u << m;
    T* s = reinterpret_cast<T*>(smem_raw);
    uint64_t* rowoff = reinterpret_cast<uint64_t*>(smem_raw + sizeof(T) * size);
    const uint32_t rows = 1u << (m - L), rowlen = 1u << L;
    const int nthr = blockDim.x;

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
            const T* mat = mats + op.mat;
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

template <typename R>
static int run_tiled_t(aqsg_state_s* st, const std::vector<LOp>& ops) {
    using T = typename Cx<R>::T;
    aqsg_ctx_s* c = st->ctx;
    const int n = st->n;
    std::vector<Pass> passes = plan(n, st->dtype, ops);
    if (passes.empty()) return AQSG_OK;

    // op tables and matrix pool of all passes in one upload
    std::vector<TileOp> table;
    std::vector<T> pool;
    std::vector<size_t> first;
    for (const Pass& p : passes) {
        first.push_back(table.size());
        uint64_t S = 0;
        for (int b : p.bits) S |= 1ull << b;
        std::vector<int> local(64, -1);
        for (size_t i = 0; i < p.bits.size(); ++i) local[p.bits[i]] = (int)i;
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
                t.mat = (int32_t)pool.size();
                const int D = 1 << o->k;
                for (int e = 0; e < D * D; ++e) {
                    T v;
                    v.x = (R)o->mk[2 * e];
                    v.y = (R)o->mk[2 * e + 1];
                    pool.push_back(v);
                }
            }
            table.push_back(t);
        }
    }
    const size_t tbytes = sizeof(TileOp) * table.size();
    const size_t pbytes = sizeof(T) * pool.size();
    const size_t poff = (tbytes + 255) & ~size_t(255);
    if (int rc = ensure_scratch(c->ops, poff + pbytes + 16)) return rc;
    AQSG_CUDA_TRY(cudaMemcpyAsync(c->ops.ptr, table.data(), tbytes, cudaMemcpyHostToDevice, c->stream));
    if (pbytes)
        AQSG_CUDA_TRY(cudaMemcpyAsync((char*)c->ops.ptr + poff, pool.data(), pbytes,
                                      cudaMemcpyHostToDevice, c->stream));
    const TileOp* dops = (const TileOp*)c->ops.ptr;
    const T* dmats = (const T*)((char*)c->ops.ptr + poff);

    constexpr int EPT_WHOLE = sizeof(R) == 4 ? 32 : 16;  // 2^14 / 512, 2^13 / 512
    constexpr int EPT_STREAM = sizeof(R) == 4 ? 16 : 8;  // 2^12 / 256, 2^11 / 256
    auto kwhole = k_tile<R, EPT_WHOLE, 512, 1>;
    auto kstream = k_tile<R, EPT_STREAM, 256, 3>;
    // largest tile of this dtype plus its row-offset table
    const int max_shm = (int)(sizeof(T) << tile_max_bits(st->dtype)) + 512 * 8;
    AQSG_CUDA_TRY(cudaFuncSetAttribute(kwhole, cudaFuncAttributeMaxDynamicSharedMemorySize, max_shm));
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
        if (whole) {
            int threads = (int)(size / EPT_WHOLE);
            threads = threads < 32 ? 32 : (threads > 512 ? 512 : threads);
            kwhole<<<grid, threads, shm, c->stream>>>((T*)st->d, geo, dops + first[pi], count, dmats);
        } else {
            kstream<<<grid, 256, shm, c->stream>>>((T*)st->d, geo, dops + first[pi], count, dmats);
        }
        c->launches++;
        AQSG_CUDA_TRY(cudaGetLastError());
    }
    return AQSG_OK;
}

int run_tiled(aqsg_state_s* st, const std::vector<LOp>& ops) {
    return st->dtype == AQSG_C64 ? run_tiled_t<float>(st, ops) : run_tiled_t<double>(st, ops);
}

}  // namespace aqsg
