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
