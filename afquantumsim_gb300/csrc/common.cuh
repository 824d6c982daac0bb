// Device helpers shared by the kernels of libaqsg.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace aqsg {

template <typename R>
struct Cx;
template <>
struct Cx<float> {
    using T = float2;  // one amplitude
    using V = float4;  // two consecutive amplitudes (128-bit access)
};
template <>
struct Cx<double> {
    using T = double2;  // one amplitude (128-bit access)
    using V = double2;
};

template <typename T>
__device__ __forceinline__ T cmul(T a, T b) {
    T r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}

// m0 * a + m1 * b
template <typename T>
__device__ __forceinline__ T cmul2(T m0, T a, T m1, T b) {
    T r;
    r.x = m0.x * a.x - m0.y * a.y + m1.x * b.x - m1.y * b.y;
    r.y = m0.x * a.y + m0.y * a.x + m1.x * b.y + m1.y * b.x;
    return r;
}

// ---- bounded waits ----------------------------------------------------------------

constexpr uint64_t kWaitNs = 200000000ull;    // 0.2 s of waiting per bounded wait
constexpr uint64_t kWaitStepNs = 1000000ull;  // 1 ms

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Time a bounded wait has spent, from %globaltimer read at each check: a
// step counts at most kWaitStepNs, so a jump of the timer or a spell off
// the SM (a preemption) counts as one step, not as a stall.
struct WaitClock {
    uint64_t last, spent = 0;
    __device__ __forceinline__ WaitClock() : last(globaltimer_ns()) {}
    __device__ __forceinline__ bool expired(uint64_t limit_ns = kWaitNs) {
        const uint64_t now = globaltimer_ns(), dt = now - last;
        last = now;
        spent += dt < kWaitStepNs ? dt : kWaitStepNs;
        return spent > limit_ns;
    }
};

// acc += m * x (complex) as four chained fused multiply-adds (written as
// acc += a*b - c*d the compiler emits a multiply, an FMA and an add per
// component).
__device__ __forceinline__ float fmadd(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmadd(double a, double b, double c) { return __fma_rn(a, b, c); }
template <typename T>
__device__ __forceinline__ void cmac(T& acc, T m, T x) {
    acc.x = fmadd(m.x, x.x, acc.x);
    acc.x = fmadd(-m.y, x.y, acc.x);
    acc.y = fmadd(m.x, x.y, acc.y);
    acc.y = fmadd(m.y, x.x, acc.y);
}

// Compensated sums on the FP32 pipe (GB300's FP64 rate is a small fraction
// of its FP32 rate).  FAcc holds an unevaluated float sum hi + lo: add() is
// Knuth's TwoSum (the rounding error of each addition is kept in lo), and
// add_sq() adds x*x exactly (Dekker's TwoProd via FMA).  Over the few
// hundred terms one thread sums, the result carries ~44 significant bits;
// threads then combine their value() in FP64.  The _rn intrinsics keep the
// compiler from contracting or reassociating the error terms.
struct FAcc {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float v) {
        const float s = __fadd_rn(hi, v);
        const float bp = __fsub_rn(s, hi);
        const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(v, bp));
        hi = s;
        lo = __fadd_rn(lo, e);
    }
    // add an unevaluated sum v + vl
    __device__ __forceinline__ void add(float v, float vl) {
        add(v);
        lo = __fadd_rn(lo, vl);
    }
    __device__ __forceinline__ void add_sq(float x) {
        const float p = __fmul_rn(x, x);
        add(p, __fmaf_rn(x, x, -p));
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// |a|^2 of a c64 amplitude as an unevaluated sum h + l (exact up to one
// rounding of the final sum)
__device__ __forceinline__ void norm2_ff(float x, float y, float& h, float& l) {
    const float px = __fmul_rn(x, x), py = __fmul_rn(y, y);
    const float ex = __fmaf_rn(x, x, -px), ey = __fmaf_rn(y, y, -py);
    h = __fadd_rn(px, py);
    const float bp = __fsub_rn(h, px);
    const float e = __fadd_rn(__fsub_rn(px, __fsub_rn(h, bp)), __fsub_rn(py, bp));
    l = __fadd_rn(__fadd_rn(ex, ey), e);
}

// ---- double-float arithmetic for complex128 gates ----------------------------
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so a complex128
// gate done in FP64 (4-8 FP64 operations per amplitude) is bound by the FP64
// pipe, not by HBM.  The gate kernels instead split each double into two
// floats with integer operations (df_split), form the products and sums as
// unevaluated float pairs on the FP32 pipe (Dekker's TwoProd through an FMA,
// Knuth's TwoSum: DFAcc), and rebuild each output double with one FP64 add
// of the pair's two floats (df_join), whose conversion to double is again
// done with integer operations.  Each output carries about 45 significant
// bits (the split keeps 24 + 23 of the 53 bits of an input; the worst
// relative error of a phase multiply is 2.5e-14).
//
// The split covers inputs of magnitude 2^-80 .. 2^117 (and exact zeros);
// anything else (tiny, huge, inf, nan) sets `wide`, and the kernel computes
// that element's gate in plain FP64 instead.

// x = hi + lo (up to the dropped bits): hi = x truncated to its leading 24
// significant bits, lo = the next 23 bits.  Both carry x's sign.
__device__ __forceinline__ float2 df_split(double x, bool& wide) {
    const uint32_t bh = (uint32_t)__double2hiint(x), bl = (uint32_t)__double2loint(x);
    const uint32_t e = (bh >> 20) & 0x7FFu;  // biased exponent; 0: zero or below 2^-1022
    const uint32_t sign = bh & 0x80000000u;
    const bool in = e - 943u <= 1140u - 943u;
    wide |= !in && e != 0u;
    // the exponent's low 9 bits and the top 23 mantissa bits, then the
    // exponent rebased from 1023 to 127 (e - 896, < 256 in range)
    const uint32_t t = __funnelshift_r(bl, bh, 29);
    const uint32_t hb = ((t + 0x40000000u) & 0x7FFFFFFFu) | sign;
    const float hi = __uint_as_float(in ? hb : 0u);
    // the next 23 mantissa bits as an exact float integer, scaled by
    // 2^(e - 1069)
    const float rf = __fsub_rn(__uint_as_float(0x4B000000u | ((bl >> 6) & 0x7FFFFFu)), 8388608.0f);
    const float scale = __uint_as_float(in ? (hb & 0x7F800000u) - (46u << 23) : 0u);
    const float lo = __uint_as_float(__float_as_uint(__fmul_rn(rf, scale)) | (in ? sign : 0u));
    return make_float2(hi, lo);
}

// A float as a double, by moving its fields (a float below 2^-126 becomes a
// signed zero; the fast path produces no inf or nan).
__device__ __forceinline__ double df_f2d(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xFFu;
    const uint32_t s = u & 0x80000000u;
    // exponent and top mantissa bits moved down by 3, exponent rebased by 896
    const uint32_t hw = e ? ((((u >> 3) & 0x0FFFFFFFu) + 0x38000000u) | s) : s;
    const uint32_t lw = e ? (u << 29) : 0u;
    return __hiloint2double((int)hw, (int)lw);
}

// An unevaluated float sum s + low.
struct DFAcc {
    float s, low;
};

// a * c for a = ah + al and a coefficient c = ch + cl: the exact product of
// the high parts (TwoProd) plus the cross terms.
__device__ __forceinline__ DFAcc df_mul(float2 a, float2 c) {
    const float p = __fmul_rn(a.x, c.x);
    const float e = __fmaf_rn(a.x, c.x, -p);
    const float t = __fmaf_rn(a.x, c.y, __fmul_rn(a.y, c.x));
    return DFAcc{p, __fadd_rn(e, t)};
}

// acc += a * c, the high parts added with TwoSum.
__device__ __forceinline__ void df_madd(DFAcc& acc, float2 a, float2 c) {
    const float p = __fmul_rn(a.x, c.x);
    const float e = __fmaf_rn(a.x, c.x, -p);
    const float t = __fmaf_rn(a.x, c.y, __fmul_rn(a.y, c.x));
    const float s = __fadd_rn(acc.s, p);
    const float bp = __fsub_rn(s, acc.s);
    const float err = __fadd_rn(__fsub_rn(acc.s, __fsub_rn(s, bp)), __fsub_rn(p, bp));
    acc.s = s;
    acc.low = __fadd_rn(acc.low, __fadd_rn(err, __fadd_rn(e, t)));
}

// The double nearest to acc.s + acc.low: one FP64 add.
__device__ __forceinline__ double df_join(const DFAcc& acc) { return __dadd_rn(df_f2d(acc.s), df_f2d(acc.low)); }

__device__ __forceinline__ float2 df_neg(float2 c) { return make_float2(-c.x, -c.y); }

// A complex128 coefficient as double-float parts: (re hi, re lo, im hi, im lo).
struct DFCoef {
    float2 re, im;
};

// Insert NF fixed bits (ascending positions) into a free index, then OR in
// their values.  NF == 0 is the identity.
template <int NF>
struct Fix {
    uint32_t pos[NF > 0 ? NF : 1];
    uint64_t val;
    __device__ __forceinline__ uint64_t expand(uint64_t k) const {
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            const uint64_t lo = k & ((1ull << pos[f]) - 1ull);
            k = ((k - lo) << 1) | lo;
        }
        return k | val;
    }
};

// The same in 32-bit arithmetic, for registers of at most 2^32 amplitudes
// (half the integer instructions of the 64-bit form per index).
template <int NF>
struct Fix32 {
    uint32_t pos[NF > 0 ? NF : 1];
    uint32_t val;
    __device__ __forceinline__ uint64_t expand(uint64_t k64) const {
        uint32_t k = (uint32_t)k64;
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            const uint32_t lo = k & ((1u << pos[f]) - 1u);
            k = ((k - lo) << 1) | lo;
        }
        return (uint64_t)(k | val);
    }
};

// Runtime-count variant for ops with many controls.
struct FixN {
    int nf;
    uint32_t pos[40];
    uint64_t val;
    __device__ __forceinline__ uint64_t expand(uint64_t k) const {
        for (int f = 0; f < nf; ++f) {
            const uint64_t lo = k & ((1ull << pos[f]) - 1ull);
            k = ((k - lo) << 1) | lo;
        }
        return k | val;
    }
};

}  // namespace aqsg
