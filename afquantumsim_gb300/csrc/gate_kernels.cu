// One-gate-per-pass kernels: each launch streams the amplitudes a gate can
// change once through HBM, in place.
//
// A gate with target/control bits F touches the index set
//   { expand(k) : k in [0, 2^(n-|F|)) }
// where expand() inserts the fixed bits of F (targets at 0, controls at their
// required value).  Consecutive k give consecutive indices between fixed bits,
// so whenever bit 0 is free two neighbouring c64 amplitudes share one 128-bit
// access (VEC = 2); c128 amplitudes are 128-bit on their own.
//
// These replace the per-gate operator builds + af::matmul of the reference
// (src/quantum.cpp:540-1950): the operators there are 2^n x 2^n (dense
// Kronecker or CSR); here a gate is a handful of coefficients.
#include <algorithm>
#include <cmath>

#include "aqsg_internal.h"
#include "common.cuh"

namespace aqsg {

constexpr int kThreads = 256;

// P_MAT2R: a 2x2 matrix with real entries (H, RotY, real unitaries): half the
// multiplies of P_MAT2, which matters where arithmetic bounds the pass
// (complex128 on a GPU whose FP64 rate is a small fraction of FP32).
enum PairOp { P_MAT2 = 0, P_DIAG2 = 1, P_PERMX = 2, P_PERMOR = 3, P_MAT2R = 4 };

template <typename R>
struct M2 {
    typename Cx<R>::T m[4];
    DFCoef df[4];  // complex128: the coefficients as double-float parts
    int df_on;     // all coefficients of modulus <= 4: the double-float path may run
};

// ---- unit load / store: VEC consecutive amplitudes starting at index i -----
template <typename R, int VEC>
struct Unit {
    typename Cx<R>::T a[VEC];
};

template <typename R, int VEC>
__device__ __forceinline__ Unit<R, VEC> load_unit(const typename Cx<R>::T* sv, uint64_t i) {
    Unit<R, VEC> u;
    if constexpr (VEC == 2) {
        const float4 f = __ldcs(reinterpret_cast<const float4*>(sv) + (i >> 1));
        u.a[0] = make_float2(f.x, f.y);
        u.a[1] = make_float2(f.z, f.w);
    } else {
        u.a[0] = __ldcs(sv + i);
    }
    return u;
}

template <typename R, int VEC>
__device__ __forceinline__ void store_unit(typename Cx<R>::T* sv, uint64_t i, const Unit<R, VEC>& u) {
    if constexpr (VEC == 2) {
        __stcs(reinterpret_cast<float4*>(sv) + (i >> 1),
               make_float4(u.a[0].x, u.a[0].y, u.a[1].x, u.a[1].y));
    } else {
        __stcs(sv + i, u.a[0]);
    }
}

// FP64 forms of the complex128 gate arithmetic, for elements outside the
// double-float split's range.  Out of line, so that the compiler branches
// around them instead of issuing their FP64 instructions, predicated off,
// for every element (GB300's FP64 pipe would then bound the kernel).
template <typename T, int OP>
__device__ __noinline__ void pair_fp64(const T* m, T& a, T& b) {
    const T x = a, y = b;
    if constexpr (OP == P_DIAG2) {
        a = cmul(m[0], x);
        b = cmul(m[1], y);
    } else {
        a = cmul2(m[0], x, m[1], y);
        b = cmul2(m[2], x, m[3], y);
    }
}

template <typename T>
__device__ __noinline__ void diag_fp64(T ph, T& a) { a = cmul(ph, a); }

// ---- pair kernels: MAT2 / DIAG2 / PERM_X / PERM_OR ---------------------------
// PACKED: c64 with target bit 0 — the pair is one 128-bit access.
template <typename R, int VEC, bool PACKED, int OP, typename FX>
__global__ void __launch_bounds__(kThreads)
k_pair(typename Cx<R>::T* __restrict__ sv, FX fx, uint64_t tmask, uint64_t amask,
       uint64_t units, M2<R> m) {
    using T = typename Cx<R>::T;
    constexpr int IT = 2;
    const uint64_t first = (uint64_t)blockIdx.x * (kThreads * IT) + threadIdx.x;
    Unit<R, VEC> lo[IT], hi[IT];
    uint64_t i0[IT];
    bool ok[IT];
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const uint64_t u = first + (uint64_t)it * kThreads;
        ok[it] = u < units;
        if (ok[it]) {
            if constexpr (PACKED) {
                i0[it] = fx.expand(u);
                const float4 f = __ldcs(reinterpret_cast<const float4*>(sv) + (i0[it] >> 1));
                lo[it].a[0] = make_float2(f.x, f.y);
                hi[it].a[0] = make_float2(f.z, f.w);
            } else {
                i0[it] = fx.expand(u * VEC);
                lo[it] = load_unit<R, VEC>(sv, i0[it]);
                hi[it] = load_unit<R, VEC>(sv, i0[it] | tmask);
            }
        }
    }
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        if (!ok[it]) continue;
        bool changed = true;
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
            const T a = lo[it].a[v], b = hi[it].a[v];
            if constexpr (sizeof(R) == 8 && (OP == P_MAT2 || OP == P_MAT2R || OP == P_DIAG2)) {
                // complex128 on the FP32 pipe (double-float), FP64 only for
                // inputs outside the split's range
                bool wide = !m.df_on;
                const float2 ar = df_split(a.x, wide), ai = df_split(a.y, wide);
                const float2 br = df_split(b.x, wide), bi = df_split(b.y, wide);
                if (__any_sync(__activemask(), wide)) {  // the whole warp takes the FP64 route
                    T x = a, y = b;
                    pair_fp64<T, OP == P_DIAG2 ? P_DIAG2 : P_MAT2>(m.m, x, y);
                    lo[it].a[v] = x;
                    hi[it].a[v] = y;
                } else {
                    T r0, r1;
                    if constexpr (OP == P_MAT2R) {
                        DFAcc x0 = df_mul(ar, m.df[0].re), y0 = df_mul(ai, m.df[0].re);
                        DFAcc x1 = df_mul(ar, m.df[2].re), y1 = df_mul(ai, m.df[2].re);
                        df_madd(x0, br, m.df[1].re);
                        df_madd(y0, bi, m.df[1].re);
                        df_madd(x1, br, m.df[3].re);
                        df_madd(y1, bi, m.df[3].re);
                        r0.x = df_join(x0); r0.y = df_join(y0);
                        r1.x = df_join(x1); r1.y = df_join(y1);
                    } else if constexpr (OP == P_MAT2) {
                        // (m0 a + m1 b) and (m2 a + m3 b), complex
                        DFAcc x0 = df_mul(ar, m.df[0].re), y0 = df_mul(ai, m.df[0].re);
                        df_madd(x0, ai, df_neg(m.df[0].im));
                        df_madd(y0, ar, m.df[0].im);
                        df_madd(x0, br, m.df[1].re);
                        df_madd(y0, bi, m.df[1].re);
                        df_madd(x0, bi, df_neg(m.df[1].im));
                        df_madd(y0, br, m.df[1].im);
                        DFAcc x1 = df_mul(ar, m.df[2].re), y1 = df_mul(ai, m.df[2].re);
                        df_madd(x1, ai, df_neg(m.df[2].im));
                        df_madd(y1, ar, m.df[2].im);
                        df_madd(x1, br, m.df[3].re);
                        df_madd(y1, bi, m.df[3].re);
                        df_madd(x1, bi, df_neg(m.df[3].im));
                        df_madd(y1, br, m.df[3].im);
                        r0.x = df_join(x0); r0.y = df_join(y0);
                        r1.x = df_join(x1); r1.y = df_join(y1);
                    } else {  // P_DIAG2: m0 on t = 0, m1 on t = 1
                        DFAcc x0 = df_mul(ar, m.df[0].re), y0 = df_mul(ai, m.df[0].re);
                        df_madd(x0, ai, df_neg(m.df[0].im));
                        df_madd(y0, ar, m.df[0].im);
                        DFAcc x1 = df_mul(br, m.df[1].re), y1 = df_mul(bi, m.df[1].re);
                        df_madd(x1, bi, df_neg(m.df[1].im));
                        df_madd(y1, br, m.df[1].im);
                        r0.x = df_join(x0); r0.y = df_join(y0);
                        r1.x = df_join(x1); r1.y = df_join(y1);
                    }
                    lo[it].a[v] = r0;
                    hi[it].a[v] = r1;
                }
                continue;
            }
            if constexpr (OP == P_MAT2) {
                lo[it].a[v] = cmul2(m.m[0], a, m.m[1], b);
                hi[it].a[v] = cmul2(m.m[2], a, m.m[3], b);
            } else if constexpr (OP == P_MAT2R) {
                T r0, r1;
                r0.x = m.m[0].x * a.x + m.m[1].x * b.x;
                r0.y = m.m[0].x * a.y + m.m[1].x * b.y;
                r1.x = m.m[2].x * a.x + m.m[3].x * b.x;
                r1.y = m.m[2].x * a.y + m.m[3].x * b.y;
                lo[it].a[v] = r0;
                hi[it].a[v] = r1;
            } else if constexpr (OP == P_DIAG2) {  // m[0] on t=0, m[1] on t=1
                lo[it].a[v] = cmul(m.m[0], a);
                hi[it].a[v] = cmul(m.m[1], b);
            } else if constexpr (OP == P_PERMX) {
                lo[it].a[v] = b;
                hi[it].a[v] = a;
            } else {  // P_PERMOR: flip unless all of amask are 0
                const bool fire = ((i0[it] + v) & amask) != 0;
                lo[it].a[v] = fire ? b : a;
                hi[it].a[v] = fire ? a : b;
            }
        }
        if constexpr (OP == P_PERMOR) {
            changed = ((i0[it] & amask) != 0) || (VEC == 2 && ((i0[it] + 1) & amask) != 0);
        }
        if (!changed) continue;
        if constexpr (PACKED) {
            __stcs(reinterpret_cast<float4*>(sv) + (i0[it] >> 1),
                   make_float4(lo[it].a[0].x, lo[it].a[0].y, hi[it].a[0].x, hi[it].a[0].y));
        } else {
            store_unit<R, VEC>(sv, i0[it], lo[it]);
            store_unit<R, VEC>(sv, i0[it] | tmask, hi[it]);
        }
    }
}

// ---- DIAG1: multiply the amplitudes of one index pattern by a phase --------
template <typename R, int VEC, typename FX>
__global__ void __launch_bounds__(kThreads)
k_diag1(typename Cx<R>::T* __restrict__ sv, FX fx, uint64_t units, typename Cx<R>::T ph, DFCoef phd) {
    constexpr int IT = 4;
    const uint64_t first = (uint64_t)blockIdx.x * (kThreads * IT) + threadIdx.x;
    Unit<R, VEC> a[IT];
    uint64_t idx[IT];
    bool ok[IT];
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const uint64_t u = first + (uint64_t)it * kThreads;
        ok[it] = u < units;
        if (ok[it]) {
            idx[it] = fx.expand(u * VEC);
            a[it] = load_unit<R, VEC>(sv, idx[it]);
        }
    }
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        if (!ok[it]) continue;
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
            if constexpr (sizeof(R) == 8) {  // complex128: double-float on the FP32 pipe
                bool wide = false;
                const float2 xr = df_split(a[it].a[v].x, wide), xi = df_split(a[it].a[v].y, wide);
                if (__any_sync(__activemask(), wide)) {
                    diag_fp64(ph, a[it].a[v]);
                } else {
                    DFAcc re = df_mul(xr, phd.re), im = df_mul(xi, phd.re);
                    df_madd(re, xi, df_neg(phd.im));
                    df_madd(im, xr, phd.im);
                    a[it].a[v].x = df_join(re);
                    a[it].a[v].y = df_join(im);
                }
                continue;
            }
            a[it].a[v] = cmul(ph, a[it].a[v]);
        }
        store_unit<R, VEC>(sv, idx[it], a[it]);
    }
}

// DIAG1 whose pattern fixes index bit 0 or 1 (complex64) / bit 0
// (complex128): the changed amplitudes then fill only part of each 32-byte
// DRAM sector, which is read and written in full all the same.  Each thread
// takes whole aligned blocks of BLK amplitudes (one sector: 4 complex64 / 2
// complex128), multiplies the elements j of the pattern ((j & lowmask) ==
// lowval) by the phase and writes the block back whole, so every access is
// a 16-byte one and every sector write a full one.  fx expands the block's
// index over the pattern's other fixed bits.
template <typename R, int BLK, typename FX>
__global__ void __launch_bounds__(kThreads)
k_diag1_blk(typename Cx<R>::T* __restrict__ sv, FX fx, uint64_t blocks, typename Cx<R>::T ph, DFCoef phd,
            uint32_t lowmask, uint32_t lowval) {
    using T = typename Cx<R>::T;
    constexpr int IT = 2;
    static_assert(BLK * sizeof(T) == 32, "one block is one 32-byte sector");
    const uint64_t first = (uint64_t)blockIdx.x * (kThreads * IT) + threadIdx.x;
    T a[IT][BLK];
    uint64_t idx[IT];
    bool ok[IT];
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const uint64_t u = first + (uint64_t)it * kThreads;
        ok[it] = u < blocks;
        if (ok[it]) {
            idx[it] = fx.expand(u * BLK);
            if constexpr (sizeof(R) == 4) {
                const float4* p = reinterpret_cast<const float4*>(sv) + (idx[it] >> 1);
                const float4 f0 = __ldcs(p), f1 = __ldcs(p + 1);
                a[it][0] = make_float2(f0.x, f0.y);
                a[it][1] = make_float2(f0.z, f0.w);
                a[it][2] = make_float2(f1.x, f1.y);
                a[it][3] = make_float2(f1.z, f1.w);
            } else {
#pragma unroll
                for (int j = 0; j < BLK; ++j) a[it][j] = __ldcs(sv + idx[it] + j);
            }
        }
    }
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        if (!ok[it]) continue;
#pragma unroll
        for (int j = 0; j < BLK; ++j) {
            if (((uint32_t)j & lowmask) != lowval) continue;  // the same j for the whole warp
            if constexpr (sizeof(R) == 8) {
                bool wide = false;
                const float2 xr = df_split(a[it][j].x, wide), xi = df_split(a[it][j].y, wide);
                if (__any_sync(__activemask(), wide)) {
                    diag_fp64(ph, a[it][j]);
                } else {
                    DFAcc re = df_mul(xr, phd.re), im = df_mul(xi, phd.re);
                    df_madd(re, xi, df_neg(phd.im));
                    df_madd(im, xr, phd.im);
                    a[it][j].x = df_join(re);
                    a[it][j].y = df_join(im);
                }
            } else {
                a[it][j] = cmul(ph, a[it][j]);
            }
        }
        if constexpr (sizeof(R) == 4) {
            float4* p = reinterpret_cast<float4*>(sv) + (idx[it] >> 1);
            __stcs(p, make_float4(a[it][0].x, a[it][0].y, a[it][1].x, a[it][1].y));
            __stcs(p + 1, make_float4(a[it][2].x, a[it][2].y, a[it][3].x, a[it][3].y));
        } else {
#pragma unroll
            for (int j = 0; j < BLK; ++j) __stcs(sv + idx[it] + j, a[it][j]);
        }
    }
}

// ---- PERM_SWAP: exchange (a=0,b=1) with (a=1,b=0) ---------------------------
template <typename R, int VEC, typename FX>
__global__ void __launch_bounds__(kThreads)
k_swap(typename Cx<R>::T* __restrict__ sv, FX fx, uint64_t xmask, uint64_t units) {
    constexpr int IT = 2;
    const uint64_t first = (uint64_t)blockIdx.x * (kThreads * IT) + threadIdx.x;
    Unit<R, VEC> p[IT], q[IT];
    uint64_t idx[IT];
    bool ok[IT];
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const uint64_t u = first + (uint64_t)it * kThreads;
        ok[it] = u < units;
        if (ok[it]) {
            idx[it] = fx.expand(u * VEC);
            p[it] = load_unit<R, VEC>(sv, idx[it]);
            q[it] = load_unit<R, VEC>(sv, idx[it] ^ xmask);
        }
    }
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        if (!ok[it]) continue;
        store_unit<R, VEC>(sv, idx[it], q[it]);
        store_unit<R, VEC>(sv, idx[it] ^ xmask, p[it]);
    }
}

// ---- MATK: dense 2^K x 2^K matrix on K target bits ---------------------------
template <typename R, int K>
struct MK {
    typename Cx<R>::T m[(1 << K) * (1 << K)];
    uint64_t off[1 << K];
};

template <typename R, int K, typename FX>
__global__ void __launch_bounds__(kThreads)
k_matk(typename Cx<R>::T* __restrict__ sv, FX fx, uint64_t units, const MK<R, K> mk) {
    using T = typename Cx<R>::T;
    constexpr int D = 1 << K;
    const uint64_t u = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
    if (u >= units) return;
    const uint64_t base = fx.expand(u);
    T v[D];
#pragma unroll
    for (int c = 0; c < D; ++c) v[c] = sv[base + mk.off[c]];
    for (int r = 0; r < D; ++r) {
        T acc;
        acc.x = 0;
        acc.y = 0;
#pragma unroll
        for (int c = 0; c < D; ++c) {
            const T mm = mk.m[r * D + c];
            cmac(acc, mm, v[c]);
        }
        sv[base + mk.off[r]] = acc;
    }
}

// ---- host-side dispatch -----------------------------------------------------------

struct FixedBits {
    int nf = 0;
    uint32_t pos[64];
    uint64_t val = 0;
    uint64_t mask = 0;
};

static FixedBits make_fixed(uint64_t mask, uint64_t val) {
    FixedBits f;
    f.mask = mask;
    f.val = val & mask;
    for (int b = 0; b < 64; ++b)
        if ((mask >> b) & 1ull) f.pos[f.nf++] = (uint32_t)b;
    return f;
}

template <int NF>
static Fix32<NF> to_fix32(const FixedBits& f) {
    Fix32<NF> x;
    for (int i = 0; i < NF; ++i) x.pos[i] = f.pos[i];
    x.val = (uint32_t)f.val;
    return x;
}

static FixN to_fixn(const FixedBits& f) {
    FixN x;
    x.nf = f.nf;
    for (int i = 0; i < f.nf; ++i) x.pos[i] = f.pos[i];
    x.val = f.val;
    return x;
}

static inline unsigned grid_for(uint64_t units, int per_block) {
    return (unsigned)((units + per_block - 1) / per_block);
}

// Calls fn(fixer) with the narrowest fixer type for f.nf: 32-bit index
// arithmetic for registers of up to 32 qubits, 64-bit above.
template <typename Fn>
static void with_fix(const FixedBits& f, int n, Fn&& fn) {
    if (n > 32) {
        fn(to_fixn(f));
        return;
    }
    switch (f.nf) {
        case 0: fn(to_fix32<0>(f)); break;
        case 1: fn(to_fix32<1>(f)); break;
        case 2: fn(to_fix32<2>(f)); break;
        case 3: fn(to_fix32<3>(f)); break;
        case 4: fn(to_fix32<4>(f)); break;
        default: fn(to_fixn(f)); break;
    }
}

template <typename R>
static typename Cx<R>::T cval(double re, double im) {
    typename Cx<R>::T t;
    t.x = (R)re;
    t.y = (R)im;
    return t;
}

// v = hi + lo as floats (hi rounded to nearest, lo the rounded remainder)
static float2 host_df(double v) {
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}

static DFCoef df_coef(double re, double im) {
    DFCoef c;
    c.re = host_df(re);
    c.im = host_df(im);
    return c;
}

template <typename R, int VEC, bool PACKED, int OP>
static void launch_pair_v(aqsg_state_s* st, const FixedBits& f, uint64_t tmask, uint64_t amask,
                          uint64_t units, const M2<R>& m) {
    using T = typename Cx<R>::T;
    const unsigned grid = grid_for(units, kThreads * 2);
    with_fix(f, st->n, [&](auto fx) {
        k_pair<R, VEC, PACKED, OP, decltype(fx)><<<grid, kThreads, 0, st->ctx->stream>>>(
            (T*)st->d, fx, tmask, amask, units, m);
    });
}

template <typename R>
static int launch_typed(aqsg_state_s* st, const LOp& op) {
    using T = typename Cx<R>::T;
    const bool is_f = sizeof(R) == 4;
    const uint64_t N = st->amps;
    switch (op.cls) {
        case L_MAT2: case L_DIAG2: case L_PERM_X: case L_PERM_OR: {
            const uint64_t tmask = 1ull << op.t0;
            FixedBits f = make_fixed(op.cmask | tmask, op.cval);
            M2<R> m;
            m.df_on = 1;
            for (int e = 0; e < 4; ++e) {
                m.m[e] = cval<R>(op.m[2 * e], op.m[2 * e + 1]);
                m.df[e] = df_coef(op.m[2 * e], op.m[2 * e + 1]);
                // user unitaries may hold any values: large ones stay in FP64
                if (!(std::fabs(op.m[2 * e]) <= 4.0 && std::fabs(op.m[2 * e + 1]) <= 4.0)) m.df_on = 0;
            }
            const bool real = op.m[1] == 0.0 && op.m[3] == 0.0 && op.m[5] == 0.0 && op.m[7] == 0.0;
            const int OPK = op.cls == L_MAT2 ? (real ? P_MAT2R : P_MAT2) : op.cls == L_DIAG2 ? P_DIAG2
                          : op.cls == L_PERM_X ? P_PERMX : P_PERMOR;
            uint64_t units = N >> f.nf;
            const bool packed = is_f && op.t0 == 0;
            const bool vec2 = is_f && !packed && (f.mask & 1ull) == 0;
            auto go = [&](auto vec_tag, auto packed_tag) {
                constexpr int V = decltype(vec_tag)::value;
                constexpr bool P = decltype(packed_tag)::value;
                switch (OPK) {
                    case P_MAT2: launch_pair_v<R, V, P, P_MAT2>(st, f, tmask, op.amask, units, m); break;
                    case P_MAT2R: launch_pair_v<R, V, P, P_MAT2R>(st, f, tmask, op.amask, units, m); break;
                    case P_DIAG2: launch_pair_v<R, V, P, P_DIAG2>(st, f, tmask, op.amask, units, m); break;
                    case P_PERMX: launch_pair_v<R, V, P, P_PERMX>(st, f, tmask, op.amask, units, m); break;
                    default: launch_pair_v<R, V, P, P_PERMOR>(st, f, tmask, op.amask, units, m); break;
                }
            };
            if constexpr (sizeof(R) == 4) {
                if (packed) go(std::integral_constant<int, 1>(), std::true_type());
                else if (vec2) { units >>= 1; go(std::integral_constant<int, 2>(), std::false_type()); }
                else go(std::integral_constant<int, 1>(), std::false_type());
            } else {
                go(std::integral_constant<int, 1>(), std::false_type());
            }
            break;
        }
        case L_DIAG1: {
            FixedBits f = make_fixed(op.cmask, op.cval);
            uint64_t units = N >> f.nf;
            const T ph = cval<R>(op.m[0], op.m[1]);
            const DFCoef phd = df_coef(op.m[0], op.m[1]);
            // the index bits inside one 32-byte sector: 0-1 (complex64), 0 (complex128)
            constexpr int BLK = sizeof(R) == 4 ? 4 : 2;
            const uint64_t low = (uint64_t)BLK - 1u;
            if ((f.mask & low) != 0 && N >= (uint64_t)BLK) {
                const FixedBits fb = make_fixed(f.mask & ~low, f.val & ~low);
                const uint64_t blocks = (N >> fb.nf) / BLK;
                const unsigned grid = grid_for(blocks, kThreads * 2);
                with_fix(fb, st->n, [&](auto fx) {
                    k_diag1_blk<R, BLK, decltype(fx)><<<grid, kThreads, 0, st->ctx->stream>>>(
                        (T*)st->d, fx, blocks, ph, phd, (uint32_t)(f.mask & low), (uint32_t)(f.val & low));
                });
                break;
            }
            const bool vec2 = is_f && (f.mask & 1ull) == 0;
            if (vec2) {
                units >>= 1;
                const unsigned grid = grid_for(units, kThreads * 4);
                with_fix(f, st->n, [&](auto fx) {
                    k_diag1<R, (sizeof(R) == 4 ? 2 : 1), decltype(fx)>
                        <<<grid, kThreads, 0, st->ctx->stream>>>((T*)st->d, fx, units, ph, phd);
                });
            } else {
                const unsigned grid = grid_for(units, kThreads * 4);
                with_fix(f, st->n, [&](auto fx) {
                    k_diag1<R, 1, decltype(fx)><<<grid, kThreads, 0, st->ctx->stream>>>(
                        (T*)st->d, fx, units, ph, phd);
                });
            }
            break;
        }
        case L_PERM_SWAP: {
            const uint64_t ma = 1ull << op.t0, mb = 1ull << op.t1;
            FixedBits f = make_fixed(op.cmask | ma | mb, op.cval | mb);
            uint64_t units = N >> f.nf;
            const bool vec2 = is_f && (f.mask & 1ull) == 0;
            if (vec2) {
                units >>= 1;
                const unsigned grid = grid_for(units, kThreads * 2);
                with_fix(f, st->n, [&](auto fx) {
                    k_swap<R, (sizeof(R) == 4 ? 2 : 1), decltype(fx)>
                        <<<grid, kThreads, 0, st->ctx->stream>>>((T*)st->d, fx, ma | mb, units);
                });
            } else {
                const unsigned grid = grid_for(units, kThreads * 2);
                with_fix(f, st->n, [&](auto fx) {
                    k_swap<R, 1, decltype(fx)><<<grid, kThreads, 0, st->ctx->stream>>>(
                        (T*)st->d, fx, ma | mb, units);
                });
            }
            break;
        }
        case L_MATK: {
            uint64_t tm = 0;
            for (int j = 0; j < op.k; ++j) tm |= 1ull << op.tb[j];
            FixedBits f = make_fixed(op.cmask | tm, op.cval);
            const uint64_t units = N >> f.nf;
            const unsigned grid = grid_for(units, kThreads);
            auto go = [&](auto k_tag) {
                constexpr int K = decltype(k_tag)::value;
                constexpr int D = 1 << K;
                auto* mk = new MK<R, K>();
                for (int r = 0; r < D; ++r) {
                    uint64_t off = 0;
                    for (int j = 0; j < K; ++j)
                        if ((r >> (K - 1 - j)) & 1) off |= 1ull << op.tb[j];
                    mk->off[r] = off;
                }
                for (int e = 0; e < D * D; ++e) mk->m[e] = cval<R>(op.mk[2 * e], op.mk[2 * e + 1]);
                with_fix(f, st->n, [&](auto fx) {
                    k_matk<R, K, decltype(fx)><<<grid, kThreads, 0, st->ctx->stream>>>(
                        (T*)st->d, fx, units, *mk);
                });
                delete mk;
            };
            switch (op.k) {
                case 2: go(std::integral_constant<int, 2>()); break;
                case 3: go(std::integral_constant<int, 3>()); break;
                case 4: go(std::integral_constant<int, 4>()); break;
                case 5: go(std::integral_constant<int, 5>()); break;
                default: return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unsupported unitary size");
            }
            break;
        }
        default: return AQSG_OK;
    }
    st->ctx->launches++;
    AQSG_CUDA_TRY(cudaGetLastError());
    return AQSG_OK;
}

int launch_lop(aqsg_state_s* st, const LOp& op) {
    if (op.cls == L_NOP) return AQSG_OK;
    return st->dtype == AQSG_C64 ? launch_typed<float>(st, op) : launch_typed<double>(st, op);
}

}  // namespace aqsg
