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
