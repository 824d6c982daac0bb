// State preparation and measurement kernels.
//
// Reductions are FP64 and deterministic (fixed two-level trees, no atomics).
// They replace the ArrayFire reductions of the reference's measurement
// members (src/quantum.cpp:308-531), which sum in FP32.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "aqsg_internal.h"
#include "common.cuh"

namespace aqsg {

constexpr int kRedThreads = 256;

// ---- preparation ---------------------------------------------------------------

template <typename T>
__global__ void k_set_one(T* sv, uint64_t k) {
    T one;
    one.x = 1;
    one.y = 0;
    sv[k] = one;
}

int launch_set_basis(aqsg_state_s* st, uint64_t k) {
    cudaStream_t s = st->ctx->stream;
    AQSG_CUDA_TRY(cudaMemsetAsync(st->d, 0, st->amps * amp_bytes(st->dtype), s));
    if (st->dtype == AQSG_C64)
        k_set_one<float2><<<1, 1, 0, s>>>((float2*)st->d, k);
    else
        k_set_one<double2><<<1, 1, 0, s>>>((double2*)st->d, k);
    st->ctx->launches++;
    AQSG_CUDA_TRY(cudaGetLastError());
    return AQSG_OK;
}

struct QAmps {
    float v[4 * AQSG_MAX_QUBITS];
};

// Product state: the Kronecker chain of generate_statevector
// (quantum.cpp:261-275, tensor_product utils.cpp:16-30): after step i the
// amplitude is q_i[b_i] * (previous), multiplied without contraction so c64
// results equal the reference's float arithmetic bit for bit.
__global__ void k_product_f32(float2* sv, int n, uint64_t N, QAmps q) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    int b = (int)((i >> (n - 1)) & 1);
    float2 acc = make_float2(q.v[2 * b], q.v[2 * b + 1]);
    for (int k = 1; k < n; ++k) {
        b = (int)((i >> (n - 1 - k)) & 1);
        const float ar = q.v[4 * k + 2 * b], ai = q.v[4 * k + 2 * b + 1];
        float2 r;
        r.x = __fsub_rn(__fmul_rn(ar, acc.x), __fmul_rn(ai, acc.y));
        r.y = __fadd_rn(__fmul_rn(ar, acc.y), __fmul_rn(ai, acc.x));
        acc = r;
    }
    sv[i] = acc;
}

__global__ void k_product_f64(double2* sv, int n, uint64_t N, QAmps q) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    int b = (int)((i >> (n - 1)) & 1);
    double2 acc = make_double2(q.v[2 * b], q.v[2 * b + 1]);
    for (int k = 1; k < n; ++k) {
        b = (int)((i >> (n - 1 - k)) & 1);
        const double ar = q.v[4 * k + 2 * b], ai = q.v[4 * k + 2 * b + 1];
        double2 r;
        r.x = __dsub_rn(__dmul_rn(ar, acc.x), __dmul_rn(ai, acc.y));
        r.y = __dadd_rn(__dmul_rn(ar, acc.y), __dmul_rn(ai, acc.x));
        acc = r;
    }
    sv[i] = acc;
}

int launch_set_product(aqsg_state_s* st, const float* amps) {
    QAmps q;
    for (int i = 0; i < 4 * st->n; ++i) q.v[i] = amps[i];
    const unsigned grid = (unsigned)((st->amps + 255) / 256);
    if (st->dtype == AQSG_C64)
        k_product_f32<<<grid, 256, 0, st->ctx->stream>>>((float2*)st->d, st->n, st->amps, q);
    else
        k_product_f64<<<grid, 256, 0, st->ctx->stream>>>((double2*)st->d, st->n, st->amps, q);
    st->ctx->launches++;
    AQSG_CUDA_TRY(cudaGetLastError());
    return AQSG_OK;
}

template <typename T, typename R>
__global__ void k_scale(T* sv, uint64_t N, R s) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (uint64_t)gridDim.x * blockDim.x) {
        T a = sv[i];
        a.x *= s;
        a.y *= s;
        sv[i] = a;
    }
}

static unsigned stream_grid(aqsg_state_s* st, uint64_t items, int threads) {
    uint64_t want = (items + threads - 1) / threads;
    uint64_t cap = (uint64_t)st->ctx->sm_count * 8;
    if (want > cap) want = cap;
    return (unsigned)(want < 1 ? 1 : want);
}

int launch_scale(aqsg_state_s* st, double scale) {
    const unsigned grid = stream_grid(st, st->amps, 256);
    if (st->dtype == AQSG_C64)
        k_scale<float2, float><<<grid, 256, 0, st->ctx->stream>>>((float2*)st->d, st->amps, (float)scale);
    else
        k_scale<double2, double><<<grid, 256, 0, st->ctx->stream>>>((double2*)st->d, st->amps, scale);
    st->ctx->launches++;
    AQSG_CUDA_TRY(cudaGetLastError());
    return AQSG_OK;
}

// component type of an amplitude type (float2 -> float, double2 -> double)
template <typename T>
using a_t = decltype(T{}.x);

// ---- block reduction helpers ---------------------------------------------------

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the block; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double* sh) {
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0;
    if (w == 0) {
        r = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
        r = warp_sum(r);
    }
    __syncthreads();
    return r;
}

// ---- masked probability sum: sum |a_i|^2 over (i & mask) == val --------------

template <typename R, int VEC, typename FX>
__global__ void __launch_bounds__(kRedThreads)
k_prob_partial(const typename Cx<R>::T* __restrict__ sv, FX fx, uint64_t units, double* partial) {
    __shared__ double sh[32];
    double acc = 0;
    if constexpr (sizeof(R) == 4) {
        FAcc fa;  // c64: exact squares, compensated sums on the FP32 pipe
        for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < units;
             u += (uint64_t)gridDim.x * blockDim.x) {
            const uint64_t i = fx.expand(u * VEC);
            if constexpr (VEC == 2) {
                const float4 f = __ldcs(reinterpret_cast<const float4*>(sv) + (i >> 1));
                fa.add_sq(f.x);
                fa.add_sq(f.y);
                fa.add_sq(f.z);
                fa.add_sq(f.w);
            } else {
                const auto a = __ldcs(sv + i);
                fa.add_sq(a.x);
                fa.add_sq(a.y);
            }
        }
        acc = fa.value();
    } else {
        for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < units;
             u += (uint64_t)gridDim.x * blockDim.x) {
            const auto a = __ldcs(sv + fx.expand(u * VEC));
            acc += (double)a.x * a.x + (double)a.y * a.y;
        }
    }
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// Deterministic final sum of `count` partials into out[0].
__global__ void k_sum_partials(const double* partial, int count, double* out) {
    __shared__ double sh[32];
    double acc = 0;
    for (int i = threadIdx.x; i < count; i += blockDim.x) acc += partial[i];
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) out[0] = s;
}

template <typename R>
static int reduce_prob_t(aqsg_state_s* st, uint64_t mask, uint64_t val, double* out) {
    using T = typename Cx<R>::T;
    aqsg_ctx_s* c = st->ctx;
    int nf = __builtin_popcountll(mask);
    uint64_t units = st->amps >> nf;
    const bool vec2 = sizeof(R) == 4 && (mask & 1ull) == 0 && units >= 2;
    if (vec2) units >>= 1;
    const unsigned grid = stream_grid(st, units, kRedThreads);
    if (int rc = ensure_scratch(c->partial, sizeof(double) * (grid + 1))) return rc;
    double* partial = (double*)c->partial.ptr;
    auto go = [&](auto fx) {
        if (vec2) {
            if constexpr (sizeof(R) == 4)
                k_prob_partial<R, 2, decltype(fx)><<<grid, kRedThreads, 0, c->stream>>>(
                    (const T*)st->d, fx, units, partial);
        } else {
            k_prob_partial<R, 1, decltype(fx)><<<grid, kRedThreads, 0, c->stream>>>(
                (const T*)st->d, fx, units, partial);
        }
    };
    if (nf == 0) {
        Fix<0> fx;
        fx.pos[0] = 0;
        fx.val = 0;
        go(fx);
    } else {
        FixN fx;
        fx.nf = 0;
        for (int b = 0; b < 64; ++b)
            if ((mask >> b) & 1ull) fx.pos[fx.nf++] = (uint32_t)b;
        fx.val = val & mask;
        go(fx);
    }
    k_sum_partials<<<1, 256, 0, c->stream>>>(partial, (int)grid, partial + grid);
    c->launches += 2;
    AQSG_CUDA_TRY(cudaGetLastError());
    AQSG_CUDA_TRY(cudaMemcpyAsync(c->host_result, partial + grid, sizeof(double),
                                  cudaMemcpyDeviceToHost, c->stream));
    AQSG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    *out = c->host_result[0];
    return AQSG_OK;
}

int reduce_prob(aqsg_state_s* st, uint64_t mask, uint64_t val, double* out) {
    return st->dtype == AQSG_C64 ? reduce_prob_t<float>(st, mask, val, out)
                                 : reduce_prob_t<double>(st, mask, val, out);
}

// ---- all probabilities ------------------------------------------------------------

// float output follows af::real(sv * af::conjg(sv)) (quantum.cpp:408):
// re*re - im*(-im), uncontracted.
template <typename T>
__global__ void k_probs(const T* __restrict__ sv, uint64_t N, void* out, int out_dtype) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const T a = sv[i];
        if (out_dtype == 0) {
            const float re = (float)a.x, im = (float)a.y;
            ((float*)out)[i] = __fsub_rn(__fmul_rn(re, re), __fmul_rn(im, -im));
        } else {
            ((double*)out)[i] = (double)a.x * (double)a.x + (double)a.y * (double)a.y;
        }
    }
}

int launch_probs(aqsg_state_s* st, void* dev_out, int out_dtype) {
    const unsigned grid = stream_grid(st, st->amps, 256);
    if (st->dtype == AQSG_C64)
        k_probs<float2><<<grid, 256, 0, st->ctx->stream>>>((const float2*)st->d, st->amps, dev_out, out_dtype);
    else
        k_probs<double2><<<grid, 256, 0, st->ctx->stream>>>((const double2*)st->d, st->amps, dev_out, out_dtype);
    st->ctx->launches++;
    AQSG_CUDA_TRY(cudaGetLastError());
    return AQSG_OK;
}

// ---- sampling ----------------------------------------------------------------------
//
// The reference draws u ~ U[0,1) and returns the first index whose inclusive
// cumulative probability exceeds u (af::accum + af::where, quantum.cpp:344-359;
// profile_measure_all repeats this per shot with R x 2^n temporaries,
// quantum.cpp:467-501).  Here: (1) FP64 sums of 2^CB-amplitude chunks,
// (2) an inclusive scan of the chunk sums, (3) one warp per shot: binary
// search over chunks, then a warp-level prefix scan inside the chunk.

constexpr int kChunkBits = 12;

template <typename T>
__global__ void __launch_bounds__(256) k_chunk_sums(const T* __restrict__ sv, int cb, double* sums) {
    __shared__ double sh[32];
    const uint64_t base = (uint64_t)blockIdx.x << cb;
    const uint64_t len = 1ull << cb;
    double acc = 0;
    if constexpr (sizeof(a_t<T>) == 4) {
        FAcc fa;
        for (uint64_t j = threadIdx.x; j < len; j += blockDim.x) {
            const T a = sv[base + j];
            fa.add_sq(a.x);
            fa.add_sq(a.y);
        }
        acc = fa.value();
    } else {
        for (uint64_t j = threadIdx.x; j < len; j += blockDim.x) {
            const T a = sv[base + j];
            acc += (double)a.x * a.x + (double)a.y * a.y;
        }
    }
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) sums[blockIdx.x] = s;
}

// Inclusive scan of `count` values by one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_scan(const double* in, double* out, uint64_t count) {
    __shared__ double sh[1024];
    const uint64_t per = (count + blockDim.x - 1) / blockDim.x;
    const uint64_t b = threadIdx.x * per;
    const uint64_t e = b + per < count ? b + per : count;
    double s = 0;
    for (uint64_t i = b; i < e; ++i) s += in[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    // Hillis-Steele scan over the thread totals
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        double v = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0.0;
        __syncthreads();
        sh[threadIdx.x] += v;
        __syncthreads();
    }
    double run = threadIdx.x ? sh[threadIdx.x - 1] : 0.0;
    for (uint64_t i = b; i < e; ++i) {
        run += in[i];
        out[i] = run;
    }
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): counter (shot, 0, 0, 0), key = seed.
__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
    }
}

__device__ inline double philox_uniform(uint64_t seed, uint64_t shot) {
    uint32_t c[4] = {(uint32_t)shot, (uint32_t)(shot >> 32), 0u, 0u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const uint64_t m = ((uint64_t)(c[0] >> 5) << 26) | (uint64_t)(c[1] >> 6);
    return (double)m * (1.0 / 9007199254740992.0);
}

template <typename T>
__device__ __forceinline__ double pr(const T a) {
    return (double)a.x * a.x + (double)a.y * a.y;
}

template <typename T>
__global__ void __launch_bounds__(256)
k_sample(const T* __restrict__ sv, int cb, uint64_t nchunks, const double* __restrict__ prefix,
         const double* __restrict__ us, uint64_t seed, int seeded, uint64_t count, int rule,
         uint64_t* out) {
    const uint64_t shot = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (shot >= count) return;
    const double u = seeded ? philox_uniform(seed, shot) : us[shot];
    const double total = prefix[nchunks - 1];
    const uint64_t clen = 1ull << cb;
    uint64_t result = 0;
    if (u < total) {
        // first chunk with inclusive prefix > u
        uint64_t lo = 0, hi = nchunks - 1;
        while (lo < hi) {
            const uint64_t mid = (lo + hi) >> 1;
            if (prefix[mid] > u) hi = mid; else lo = mid + 1;
        }
        const uint64_t c = lo;
        double run = c ? prefix[c - 1] : 0.0;
        const uint64_t base = c << cb;
        uint64_t found = base + clen - 1;  // rounding fallback: chunk's last index
        for (uint64_t s = 0; s < clen; s += 64) {
            // lane holds amplitudes base+s+2*lane and +1 (chunks have >= 2 amps)
            const uint64_t j = base + s + 2 * lane;
            const bool in = s + 2 * lane < clen;
            const double p0 = in ? pr(sv[j]) : 0.0;
            const double p1 = (in && s + 2 * lane + 1 < clen) ? pr(sv[j + 1]) : 0.0;
            double incl = p0 + p1;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            const unsigned hit = __ballot_sync(0xffffffffu, run + incl > u);
            if (hit) {
                const int L = __ffs(hit) - 1;
                const double excl = __shfl_sync(0xffffffffu, incl - p0 - p1, L);
                const double q0 = __shfl_sync(0xffffffffu, p0, L);
                found = base + s + 2 * L + ((run + excl + q0 > u) ? 0 : 1);
                break;
            }
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
        result = found;
    } else if (rule == AQSG_SAMPLE_CLAMP) {
        // last index of non-zero probability: first chunk reaching the total
        uint64_t lo = 0, hi = nchunks - 1;
        while (lo < hi) {
            const uint64_t mid = (lo + hi) >> 1;
            if (prefix[mid] >= total) hi = mid; else lo = mid + 1;
        }
        const uint64_t base = lo << cb;
        uint64_t last = base;
        for (uint64_t s = 0; s < clen; s += 32) {
            const uint64_t j = base + s + lane;
            const bool nz = (s + lane < clen) && pr(sv[j]) > 0.0;
            const unsigned m = __ballot_sync(0xffffffffu, nz);
            if (m) last = base + s + (31 - __clz(m));
        }
        result = last;
    }
    if (lane == 0) out[shot] = result;
}

template <typename T>
static int sample_t(aqsg_state_s* st, const double* host_u, uint64_t seed, bool seeded,
                    uint64_t count, int rule, uint64_t* host_out) {
    aqsg_ctx_s* c = st->ctx;
    const int cb = st->n < kChunkBits ? st->n : kChunkBits;
    const uint64_t nchunks = st->amps >> cb;
    if (int rc = ensure_scratch(c->partial, sizeof(double) * nchunks)) return rc;
    if (int rc = ensure_scratch(c->prefix, sizeof(double) * nchunks)) return rc;
    if (int rc = ensure_scratch(c->sample_o, sizeof(uint64_t) * count)) return rc;
    if (!seeded) {
        if (int rc = ensure_scratch(c->sample_u, sizeof(double) * count)) return rc;
        AQSG_CUDA_TRY(cudaMemcpyAsync(c->sample_u.ptr, host_u, sizeof(double) * count,
                                      cudaMemcpyHostToDevice, c->stream));
    }
    k_chunk_sums<T><<<(unsigned)nchunks, 256, 0, c->stream>>>((const T*)st->d, cb, (double*)c->partial.ptr);
    k_scan<<<1, 1024, 0, c->stream>>>((const double*)c->partial.ptr, (double*)c->prefix.ptr, nchunks);
    const uint64_t threads = count * 32;
    const unsigned grid = (unsigned)((threads + 255) / 256);
    k_sample<T><<<grid, 256, 0, c->stream>>>((const T*)st->d, cb, nchunks, (const double*)c->prefix.ptr,
                                              seeded ? nullptr : (const double*)c->sample_u.ptr, seed,
                                              seeded ? 1 : 0, count, rule, (uint64_t*)c->sample_o.ptr);
    c->launches += 3;
    AQSG_CUDA_TRY(cudaGetLastError());
    AQSG_CUDA_TRY(cudaMemcpyAsync(host_out, c->sample_o.ptr, sizeof(uint64_t) * count,
                                  cudaMemcpyDeviceToHost, c->stream));
    AQSG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return AQSG_OK;
}

int sample(aqsg_state_s* st, const double* host_u, uint64_t seed, bool seeded, uint64_t count,
           int rule, uint64_t* host_out) {
    return st->dtype == AQSG_C64 ? sample_t<float2>(st, host_u, seed, seeded, count, rule, host_out)
                                 : sample_t<double2>(st, host_u, seed, seeded, count, rule, host_out);
}

// ---- allocation-free sampling ----------------------------------------------------
//
// aqsg_sample_noalloc runs the three sampling kernels above on scratch carved
// from one static device array instead of context buffers grown with
// cudaMalloc.  Layout: chunk sums and chunk prefix sums (2^(30-12) doubles
// each), then the call's uniforms and outcomes (AQSG_NOALLOC_MAX_SHOTS each).
// Every buffer is fully written before it is read within a call, so nothing
// has to be cleared between calls.

constexpr uint64_t kNoallocChunks = 1ull << (AQSG_NOALLOC_MAX_QUBITS - kChunkBits);
static_assert(AQSG_NOALLOC_SCRATCH_BYTES ==
                  2 * sizeof(double) * kNoallocChunks + 16 * (size_t)AQSG_NOALLOC_MAX_SHOTS,
              "scratch layout");

static __device__ __align__(256) unsigned char g_noalloc_scratch[AQSG_NOALLOC_SCRATCH_BYTES];

constexpr int kNoallocMaxDevices = 256;
static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[kNoallocMaxDevices];

// Device address of the static scratch on `device`, looked up once per device
// with that device current.  (In host code g_noalloc_scratch names a host-side
// stand-in, not device memory, so only the looked-up address is passed on.)
// aqsg_init calls this for its device, so the module that holds the array is
// loaded, and the array resident, before any sampling call; a sampling call
// then only reads the cached address.
static int noalloc_scratch(int device, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (device < 0 || device >= kNoallocMaxDevices)
        return set_error(AQSG_ERR_OUT_OF_RANGE, "Device index beyond the allocation-free table");
    if (!g_noalloc_addr[device]) {
        AQSG_ON_DEVICE(device);
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(allocation-free scratch)");
        g_noalloc_addr[device] = p;
    }
    *out = (unsigned char*)g_noalloc_addr[device];
    return AQSG_OK;
}

int noalloc_prepare(int device) {
    unsigned char* p = nullptr;
    return noalloc_scratch(device, &p);
}

template <typename T>
static int sample_noalloc_t(aqsg_state_s* st, const double* host_u, uint64_t count, int rule,
                            uint64_t* host_out) {
    aqsg_ctx_s* c = st->ctx;
    unsigned char* base = nullptr;
    if (int rc = noalloc_scratch(c->device, &base)) return rc;
    const int cb = st->n < kChunkBits ? st->n : kChunkBits;
    const uint64_t nchunks = st->amps >> cb;
    double* sums = (double*)base;
    double* prefix = sums + kNoallocChunks;
    double* us = prefix + kNoallocChunks;
    uint64_t* outs = (uint64_t*)(us + AQSG_NOALLOC_MAX_SHOTS);
    AQSG_CUDA_TRY(cudaMemcpyAsync(us, host_u, sizeof(double) * count, cudaMemcpyHostToDevice, c->stream));
    k_chunk_sums<T><<<(unsigned)nchunks, 256, 0, c->stream>>>((const T*)st->d, cb, sums);
    k_scan<<<1, 1024, 0, c->stream>>>(sums, prefix, nchunks);
    const unsigned grid = (unsigned)((count * 32 + 255) / 256);
    k_sample<T><<<grid, 256, 0, c->stream>>>((const T*)st->d, cb, nchunks, prefix, us, 0, 0, count,
                                              rule, outs);
    c->launches += 3;
    AQSG_CUDA_TRY(cudaGetLastError());
    AQSG_CUDA_TRY(cudaMemcpyAsync(host_out, outs, sizeof(uint64_t) * count, cudaMemcpyDeviceToHost,
                                  c->stream));
    AQSG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return AQSG_OK;
}

}  // namespace aqsg

extern "C" int aqsg_sample_noalloc(aqsg_state st, const double* u, uint64_t count, int rule,
                                   uint64_t* out) {
    using namespace aqsg;
    if (!st || !st->d) return set_error(AQSG_ERR_NULL, "NULL state");
    if (count == 0) return AQSG_OK;
    if (!u || !out) return set_error(AQSG_ERR_NULL, "NULL buffer");
    if (rule != AQSG_SAMPLE_REFERENCE && rule != AQSG_SAMPLE_CLAMP)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown sampling rule");
    if (st->n > AQSG_NOALLOC_MAX_QUBITS)
        return set_error(AQSG_ERR_INVALID_ARGUMENT,
                         "Allocation-free sampling supports at most " +
                             std::to_string(AQSG_NOALLOC_MAX_QUBITS) + " qubits, register has " +
                             std::to_string(st->n));
    if (count > AQSG_NOALLOC_MAX_SHOTS)
        return set_error(AQSG_ERR_INVALID_ARGUMENT,
                         "Allocation-free sampling takes at most " +
                             std::to_string(AQSG_NOALLOC_MAX_SHOTS) + " shots per call, got " +
                             std::to_string(count));
    AQSG_ON_DEVICE(st->ctx->device);
    return st->dtype == AQSG_C64 ? sample_noalloc_t<float2>(st, u, count, rule, out)
                                 : sample_noalloc_t<double2>(st, u, count, rule, out);
}

namespace aqsg {

// ---- collapse of one qubit: one pass, reads only the kept branch -------------------

template <typename T, typename R>
__global__ void k_collapse(T* sv, uint64_t units, int bitpos, int outcome, R scale) {
    for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < units;
         u += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t lo = u & ((1ull << bitpos) - 1ull);
        const uint64_t i0 = ((u - lo) << 1) | lo;  // bit = 0
        const uint64_t keep = outcome ? (i0 | (1ull << bitpos)) : i0;
        const uint64_t drop = outcome ? i0 : (i0 | (1ull << bitpos));
        T a = sv[keep];
        a.x *= scale;
        a.y *= scale;
        sv[keep] = a;
        T z;
        z.x = 0;
        z.y = 0;
        sv[drop] = z;
    }
}

int launch_collapse_qubit(aqsg_state_s* st, uint64_t mask, int outcome, double scale) {
    int bitpos = 0;
    while (!((mask >> bitpos) & 1ull)) ++bitpos;
    const uint64_t units = st->amps >> 1;
    const unsigned grid = stream_grid(st, units, 256);
    if (st->dtype == AQSG_C64)
        k_collapse<float2, float><<<grid, 256, 0, st->ctx->stream>>>((float2*)st->d, units, bitpos,
                                                                     outcome, (float)scale);
    else
        k_collapse<double2, double><<<grid, 256, 0, st->ctx->stream>>>((double2*)st->d, units, bitpos,
                                                                       outcome, scale);
    st->ctx->launches++;
    AQSG_CUDA_TRY(cudaGetLastError());
    return AQSG_OK;
}

// ---- <Z_q> and <Z_q Z_q+1> in one pass -----------------------------------------------
//
// Block b owns the contiguous range [b 2^RB, (b+1) 2^RB).  Thread t reads
// j = s * nthreads + t, so index bits below TB = log2(nthreads) are the
// thread's own (constant), bits TB..RB-1 are the loop counter s, bits >= RB
// are the block's.  Per thread: total T, per-s-bit sums S and neighbour-pair
// parity sums X (at most 12 + 11 doubles).  Each block writes
// [T, S1[0..RB), X[0..RB-1)] over its bits; a final kernel folds in the block
// bits and sums blocks in a fixed order.

constexpr int kZMaxS = 12;
constexpr int kZMaxRB2 = 40;  // 2 x amplitude bits per block, at most (rb <= 20)

size_t expz_partial_doubles(int n);
int launch_expz_raw(const void* sv, int n, int dtype, double* partial, double* out_raw, cudaStream_t stream);

template <typename T>
__global__ void __launch_bounds__(256)
k_expz_partial(const T* __restrict__ sv, int tb, int rb, double* partial, uint64_t reg_stride = 0,
               uint64_t partial_stride = 0) {
    __shared__ double sh[32];
    sv += (uint64_t)blockIdx.y * reg_stride;  // grouped registers: one per blockIdx.y
    partial += (uint64_t)blockIdx.y * partial_stride;
    const int sb = rb - tb;
    const uint64_t base = (uint64_t)blockIdx.x << rb;
    const uint64_t nt = 1ull << tb;  // threads that own indices (<= blockDim.x)
    double tot = 0, S[kZMaxS], X[kZMaxS];
#pragma unroll
    for (int i = 0; i < kZMaxS; ++i) { S[i] = 0; X[i] = 0; }
    const uint64_t iters = threadIdx.x < nt ? (1ull << sb) : 0;
    if constexpr (sizeof(a_t<T>) == 4) {
        // c64: exact |a|^2 and compensated sums on the FP32 pipe
        FAcc ft, fs[kZMaxS], fx[kZMaxS];
        for (uint64_t s = 0; s < iters; ++s) {
            const T a = sv[base + s * nt + threadIdx.x];
            float h, l;
            norm2_ff(a.x, a.y, h, l);
            ft.add(h, l);
#pragma unroll
            for (int i = 0; i < kZMaxS; ++i) {
                if (i < sb) {
                    const uint64_t bi = (s >> i) & 1ull;
                    if (bi) fs[i].add(h, l);
                    if (i + 1 < sb && (bi ^ ((s >> (i + 1)) & 1ull))) fx[i].add(h, l);
                }
            }
        }
        tot = ft.value();
#pragma unroll
        for (int i = 0; i < kZMaxS; ++i) {
            S[i] = fs[i].value();
            X[i] = fx[i].value();
        }
    } else {
        for (uint64_t s = 0; s < iters; ++s) {
            const double p = pr(sv[base + s * nt + threadIdx.x]);
            tot += p;
#pragma unroll
            for (int i = 0; i < kZMaxS; ++i) {
                if (i < sb) {
                    const uint64_t bi = (s >> i) & 1ull;
                    if (bi) S[i] += p;
                    if (i + 1 < sb && (bi ^ ((s >> (i + 1)) & 1ull))) X[i] += p;
                }
            }
        }
    }
    const int stride = 2 * rb;
    double* out = partial + (uint64_t)blockIdx.x * stride;
    if constexpr (sizeof(a_t<T>) == 4) {
        // c64: every block sum in float-float on the FP32 pipe (warp
        // butterflies, then across the <= 8 warps); FP64 only for the
        // block's results
        __shared__ float ffh[8][kZMaxRB2], ffl[8][kZMaxRB2];
        const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const FAcc ftot = [&] { FAcc t; t.hi = (float)tot; t.lo = (float)(tot - (double)(float)tot); return t; }();
        for (int v = 0; v < stride; ++v) {
            FAcc c;  // this thread's share of value v
            if (v == 0) {
                c = ftot;
            } else if (v <= rb) {  // S1[q]
                const int q = v - 1;
                if (q < tb) {
                    if ((threadIdx.x >> q) & 1) c = ftot;
                } else {
                    const double d = S[q - tb < kZMaxS ? q - tb : 0];
                    c.hi = (float)d;
                    c.lo = (float)(d - (double)c.hi);
                }
            } else {  // X[q], pair (q, q+1)
                const int q = v - 1 - rb;
                double d = 0;
                if (q + 1 < tb) d = (((threadIdx.x >> q) ^ (threadIdx.x >> (q + 1))) & 1) ? tot : 0.0;
                else if (q + 1 == tb) d = ((threadIdx.x >> q) & 1) ? tot - S[0] : S[0];
                else d = X[q - tb < kZMaxS ? q - tb : 0];
                c.hi = (float)d;
                c.lo = (float)(d - (double)c.hi);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float h = __shfl_xor_sync(0xffffffffu, c.hi, o);
                const float l = __shfl_xor_sync(0xffffffffu, c.lo, o);
                c.add(h, l);
            }
            if (lane == 0) {
                ffh[w][v] = c.hi;
                ffl[w][v] = c.lo;
            }
        }
        __syncthreads();
        if ((int)threadIdx.x < stride) {
            FAcc r;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) r.add(ffh[q][threadIdx.x], ffl[q][threadIdx.x]);
            out[threadIdx.x] = r.value();
        }
        return;
    }
    const double btot = block_sum(tot, sh);
    if (threadIdx.x == 0) out[0] = btot;
    // S1[q] for q < rb
    for (int q = 0; q < rb; ++q) {
        double v;
        if (q < tb) v = ((threadIdx.x >> q) & 1) ? tot : 0.0;
        else v = S[q - tb < kZMaxS ? q - tb : 0];
        const double r = block_sum(v, sh);
        if (threadIdx.x == 0) out[1 + q] = r;
    }
    // X[q] for pairs (q, q+1), q < rb - 1
    for (int q = 0; q + 1 < rb; ++q) {
        double v;
        if (q + 1 < tb) v = (((threadIdx.x >> q) ^ (threadIdx.x >> (q + 1))) & 1) ? tot : 0.0;
        else if (q + 1 == tb) v = ((threadIdx.x >> q) & 1) ? tot - S[0] : S[0];
        else v = X[q - tb < kZMaxS ? q - tb : 0];
        const double r = block_sum(v, sh);
        if (threadIdx.x == 0) out[1 + rb + q] = r;
    }
}

// One thread per output value: threads [0, n) -> S1 over index bits,
// [n, 2n-1) -> X over neighbour bit pairs, thread 2n-1 -> total.
__global__ void k_expz_final(const double* partial, int n, int rb, uint64_t nblocks, double* res,
                             uint64_t partial_stride = 0, const uint64_t* res_off = nullptr) {
    partial += (uint64_t)blockIdx.x * partial_stride;  // grouped registers: one block each
    if (res_off) res += res_off[blockIdx.x];
    const int t = threadIdx.x;
    if (t >= 2 * n) return;
    const int stride = 2 * rb;
    double acc = 0;
    for (uint64_t b = 0; b < nblocks; ++b) {
        const double* p = partial + b * stride;
        const uint64_t base = b << rb;
        const double T = p[0];
        if (t < n) {
            const int q = t;
            acc += q < rb ? p[1 + q] : (((base >> q) & 1ull) ? T : 0.0);
        } else if (t < 2 * n - 1) {
            const int q = t - n;
            if (q + 1 < rb) acc += p[1 + rb + q];
            else if (q + 1 == rb) acc += ((base >> rb) & 1ull) ? T - p[1 + q] : p[1 + q];
            else acc += ((((base >> q) ^ (base >> (q + 1))) & 1ull) ? T : 0.0);
        } else {
            acc += T;
        }
    }
    res[t] = acc;
}

template <typename T>
static int expect_z_t(aqsg_state_s* st, double* z, double* zz) {
    aqsg_ctx_s* c = st->ctx;
    const int n = st->n;
    const size_t pd = expz_partial_doubles(n);
    if (int rc = ensure_scratch(c->partial, sizeof(double) * (pd + 2 * n + 1))) return rc;
    double* partial = (double*)c->partial.ptr;
    double* res = partial + pd;
    if (int rc = launch_expz_raw(st->d, n, st->dtype, partial, res, c->stream)) return rc;
    c->launches += 2;
    std::vector<double> h(2 * n);
    AQSG_CUDA_TRY(cudaMemcpyAsync(h.data(), res, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, c->stream));
    AQSG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    const double tot = h[2 * n - 1];
    for (int q = 0; q < n; ++q) {
        const int bq = n - 1 - q;
        if (z) z[q] = tot - 2.0 * h[bq];
        if (zz && q + 1 < n) zz[q] = tot - 2.0 * h[n + (n - 2 - q)];
    }
    return AQSG_OK;
}

int expect_z(aqsg_state_s* st, double* z, double* zz) {
    return st->dtype == AQSG_C64 ? expect_z_t<float2>(st, z, zz) : expect_z_t<double2>(st, z, zz);
}

}  // namespace aqsg

// ---- comparison of two registers ------------------------------------------------

namespace aqsg {

template <typename TA, typename TB>
__global__ void __launch_bounds__(256)
k_compare(const TA* __restrict__ a, const TB* __restrict__ b, uint64_t N, double* partial) {
    __shared__ double sh[32];
    double mx = 0, ore = 0, oim = 0, na = 0, nb = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const TA x = __ldcs(a + i);
        const TB y = __ldcs(b + i);
        const double xr = x.x, xi = x.y, yr = y.x, yi = y.y;
        const double dr = xr - yr, di = xi - yi;
        mx = fmax(mx, sqrt(dr * dr + di * di));
        ore += xr * yr + xi * yi;  // conj(x) * y
        oim += xr * yi - xi * yr;
        na += xr * xr + xi * xi;
        nb += yr * yr + yi * yi;
    }
    // block max of mx through shared memory, sums through block_sum
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __shared__ double shm[32];
    if ((threadIdx.x & 31) == 0) shm[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0;
        for (unsigned w = 0; w < (blockDim.x >> 5); ++w) m = fmax(m, shm[w]);
        partial[5 * blockIdx.x] = m;
    }
    const double s1 = block_sum(ore, sh), s2 = block_sum(oim, sh), s3 = block_sum(na, sh),
                 s4 = block_sum(nb, sh);
    if (threadIdx.x == 0) {
        partial[5 * blockIdx.x + 1] = s1;
        partial[5 * blockIdx.x + 2] = s2;
        partial[5 * blockIdx.x + 3] = s3;
        partial[5 * blockIdx.x + 4] = s4;
    }
}

}  // namespace aqsg

extern "C" int aqsg_state_compare(aqsg_state a, aqsg_state b, double* max_abs_diff, double* overlap_re,
                                  double* overlap_im, double* norm2_a, double* norm2_b) {
    using namespace aqsg;
    if (!a || !a->d || !b || !b->d) return set_error(AQSG_ERR_NULL, "NULL state");
    if (a->n != b->n) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Registers differ in qubit count");
    if (a->ctx != b->ctx) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Registers belong to different contexts");
    aqsg_ctx_s* c = a->ctx;
    AQSG_ON_DEVICE(c->device);
    const unsigned grid = stream_grid(a, a->amps, 256);
    if (int rc = ensure_scratch(c->partial, sizeof(double) * 5 * grid)) return rc;
    double* part = (double*)c->partial.ptr;
    const bool a64 = a->dtype == AQSG_C64, b64 = b->dtype == AQSG_C64;
    if (a64 && b64)
        k_compare<float2, float2><<<grid, 256, 0, c->stream>>>((const float2*)a->d, (const float2*)b->d, a->amps, part);
    else if (a64)
        k_compare<float2, double2><<<grid, 256, 0, c->stream>>>((const float2*)a->d, (const double2*)b->d, a->amps, part);
    else if (b64)
        k_compare<double2, float2><<<grid, 256, 0, c->stream>>>((const double2*)a->d, (const float2*)b->d, a->amps, part);
    else
        k_compare<double2, double2><<<grid, 256, 0, c->stream>>>((const double2*)a->d, (const double2*)b->d, a->amps, part);
    c->launches++;
    AQSG_CUDA_TRY(cudaGetLastError());
    std::vector<double> h(5 * grid);
    AQSG_CUDA_TRY(cudaMemcpyAsync(h.data(), part, sizeof(double) * 5 * grid, cudaMemcpyDeviceToHost, c->stream));
    AQSG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    double r[5] = {0, 0, 0, 0, 0};
    for (unsigned i = 0; i < grid; ++i) {
        r[0] = h[5 * i] > r[0] ? h[5 * i] : r[0];
        for (int j = 1; j < 5; ++j) r[j] += h[5 * i + j];
    }
    if (max_abs_diff) *max_abs_diff = r[0];
    if (overlap_re) *overlap_re = r[1];
    if (overlap_im) *overlap_im = r[2];
    if (norm2_a) *norm2_a = r[3];
    if (norm2_b) *norm2_b = r[4];
    return AQSG_OK;
}

// ---- raw <Z> sums without a host read (the batched engine) -----------------------

namespace aqsg {

// Amplitudes per block of the expectation reduction: 2^12 (at most 2^16
// blocks), the whole register when smaller.
static int expz_rb(int n) {
    int rb = n < 12 ? n : 12;
    if (n - rb > 16) rb = n - 16;
    return rb;
}

size_t expz_partial_doubles(int n) {
    const int rb = expz_rb(n);
    return ((size_t)1 << (n - rb)) * 2 * (size_t)rb;
}

// Writes the 2n raw sums (S over index bits, X over neighbour bit pairs, then
// the total) of register sv to out_raw, on `stream`, without synchronising.
int launch_expz_raw(const void* sv, int n, int dtype, double* partial, double* out_raw, cudaStream_t stream) {
    const int rb = expz_rb(n);
    int tb = rb < 8 ? rb : 8;
    if (rb - tb > kZMaxS) tb = rb - kZMaxS;
    const uint64_t nblocks = (1ull << n) >> rb;
    const int threads = (1 << tb) < 32 ? 32 : (1 << tb);
    if (dtype == AQSG_C64)
        k_expz_partial<float2><<<(unsigned)nblocks, threads, 0, stream>>>((const float2*)sv, tb, rb, partial);
    else
        k_expz_partial<double2><<<(unsigned)nblocks, threads, 0, stream>>>((const double2*)sv, tb, rb, partial);
    k_expz_final<<<1, 128, 0, stream>>>(partial, n, rb, nblocks, out_raw);
    AQSG_CUDA_TRY(cudaGetLastError());
    return AQSG_OK;
}

// The raw sums of `members` c64 registers reg_stride amplitudes apart; the
// sums of register j go to out_base + out_off[j] (device array).  partial
// holds members x expz_partial_doubles(n) doubles.
int launch_expz_raw_multi(const void* sv0, uint64_t reg_stride, int members, int n, double* partial,
                          const uint64_t* out_off, double* out_base, cudaStream_t stream) {
    const int rb = expz_rb(n);
    int tb = rb < 8 ? rb : 8;
    if (rb - tb > kZMaxS) tb = rb - kZMaxS;
    const uint64_t nblocks = (1ull << n) >> rb;
    const int threads = (1 << tb) < 32 ? 32 : (1 << tb);
    const uint64_t pd = expz_partial_doubles(n);
    k_expz_partial<float2><<<dim3((unsigned)nblocks, (unsigned)members), threads, 0, stream>>>(
        (const float2*)sv0, tb, rb, partial, reg_stride, pd);
    k_expz_final<<<(unsigned)members, 128, 0, stream>>>(partial, n, rb, nblocks, out_base, pd, out_off);
    AQSG_CUDA_TRY(cudaGetLastError());
    return AQSG_OK;
}

}  // namespace aqsg

// ---- asynchronous variants (no host read) for the serving runtime -------------------

namespace aqsg {

int launch_sum_partials(aqsg_ctx_s* c, const double* parts, int count, double* out) {
    k_sum_partials<<<1, 256, 0, c->stream>>>(parts, count, out);
    c->launches++;
    AQSG_CUDA_TRY(cudaGetLastError());
    return AQSG_OK;
}

// FP64 sum of |a|^2 into d_out (device), on the context stream.
int launch_norm_to_device(aqsg_state_s* st, double* d_out) {
    aqsg_ctx_s* c = st->ctx;
    uint64_t units = st->amps;
    const bool vec2 = st->dtype == AQSG_C64 && units >= 2;
    if (vec2) units >>= 1;
    const unsigned grid = stream_grid(st, units, kRedThreads);
    if (c->partial.bytes < sizeof(double) * (grid + 1))
        return set_error(AQSG_ERR_RUNTIME, "Reduction scratch not reserved");
    double* partial = (double*)c->partial.ptr;
    Fix<0> fx;
    fx.pos[0] = 0;
    fx.val = 0;
    if (st->dtype == AQSG_C64) {
        if (vec2)
            k_prob_partial<float, 2, Fix<0>><<<grid, kRedThreads, 0, c->stream>>>((const float2*)st->d, fx, units, partial);
        else
            k_prob_partial<float, 1, Fix<0>><<<grid, kRedThreads, 0, c->stream>>>((const float2*)st->d, fx, units, partial);
    } else {
        k_prob_partial<double, 1, Fix<0>><<<grid, kRedThreads, 0, c->stream>>>((const double2*)st->d, fx, units, partial);
    }
    k_sum_partials<<<1, 256, 0, c->stream>>>(partial, (int)grid, d_out);
    c->launches += 2;
    AQSG_CUDA_TRY(cudaGetLastError());
    return AQSG_OK;
}

template <typename T, typename R>
__global__ void k_scale_dev(T* sv, uint64_t N, const double* n_before, const double* n_after) {
    const double nb = *n_before, na = *n_after;
    const R s = (na > 0 && nb > 0) ? (R)sqrt(nb / na) : (R)1;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (uint64_t)gridDim.x * blockDim.x) {
        T a = sv[i];
        a.x *= s;
        a.y *= s;
        sv[i] = a;
    }
}

// Scale the register by sqrt(*n_before / *n_after), both read on the device.
int launch_renorm_device(aqsg_state_s* st, const double* n_before, const double* n_after) {
    const unsigned grid = stream_grid(st, st->amps, 256);
    if (st->dtype == AQSG_C64)
        k_scale_dev<float2, float><<<grid, 256, 0, st->ctx->stream>>>((float2*)st->d, st->amps, n_before, n_after);
    else
        k_scale_dev<double2, double><<<grid, 256, 0, st->ctx->stream>>>((double2*)st->d, st->amps, n_before, n_after);
    st->ctx->launches++;
    AQSG_CUDA_TRY(cudaGetLastError());
    return AQSG_OK;
}

// Reserve the context scratch a register of n qubits and `shots` samples
// need, so the asynchronous calls below never allocate.
int reserve_scratch(aqsg_ctx_s* c, int n, uint64_t shots) {
    const uint64_t nchunks = (1ull << n) >> (n < kChunkBits ? n : kChunkBits);
    const size_t red = sizeof(double) * ((size_t)c->sm_count * 8 + 1);
    size_t need = sizeof(double) * nchunks;
    if (red > need) need = red;
    if (int rc = ensure_scratch(c->partial, need + 64)) return rc;
    if (int rc = ensure_scratch(c->prefix, sizeof(double) * nchunks)) return rc;
    if (int rc = ensure_scratch(c->sample_o, sizeof(uint64_t) * (shots ? shots : 1))) return rc;
    return AQSG_OK;
}

// Seeded sampling whose outcomes land in pinned host memory when the
// context stream reaches that point; nothing waits.
int sample_seeded_async(aqsg_state_s* st, uint64_t seed, uint64_t count, int rule, uint64_t* pinned_out) {
    aqsg_ctx_s* c = st->ctx;
    const int cb = st->n < kChunkBits ? st->n : kChunkBits;
    const uint64_t nchunks = st->amps >> cb;
    if (c->partial.bytes < sizeof(double) * nchunks || c->prefix.bytes < sizeof(double) * nchunks ||
        c->sample_o.bytes < sizeof(uint64_t) * count)
        return set_error(AQSG_ERR_RUNTIME, "Sampling scratch not reserved");
    if (st->dtype == AQSG_C64) {
        k_chunk_sums<float2><<<(unsigned)nchunks, 256, 0, c->stream>>>((const float2*)st->d, cb, (double*)c->partial.ptr);
    } else {
        k_chunk_sums<double2><<<(unsigned)nchunks, 256, 0, c->stream>>>((const double2*)st->d, cb, (double*)c->partial.ptr);
    }
    k_scan<<<1, 1024, 0, c->stream>>>((const double*)c->partial.ptr, (double*)c->prefix.ptr, nchunks);
    const unsigned grid = (unsigned)((count * 32 + 255) / 256);
    if (st->dtype == AQSG_C64)
        k_sample<float2><<<grid, 256, 0, c->stream>>>((const float2*)st->d, cb, nchunks, (const double*)c->prefix.ptr,
                                                       nullptr, seed, 1, count, rule, (uint64_t*)c->sample_o.ptr);
    else
        k_sample<double2><<<grid, 256, 0, c->stream>>>((const double2*)st->d, cb, nchunks, (const double*)c->prefix.ptr,
                                                        nullptr, seed, 1, count, rule, (uint64_t*)c->sample_o.ptr);
    c->launches += 3;
    AQSG_CUDA_TRY(cudaGetLastError());
    AQSG_CUDA_TRY(cudaMemcpyAsync(pinned_out, c->sample_o.ptr, sizeof(uint64_t) * count, cudaMemcpyDeviceToHost,
                                  c->stream));
    return AQSG_OK;
}

}  // namespace aqsg

// ---- Pauli-string expectation values -----------------------------------------------
//
// P = P_0 (x) ... (x) P_{n-1} with P_j in {I, X, Y, Z} on qubit j (index bit
// n-1-j).  With Y = i X Z, P = i^{#Y} X^x Z^z where x marks the X/Y qubits and
// z the Y/Z qubits, so P|k> = i^{#Y} (-1)^{|k & z|} |k ^ x> and
//   <psi|P|psi> = i^{#Y} sum_k (-1)^{|k & z|} conj(psi[k ^ x]) psi[k].
// The sums run in FP64, kPauliChunk strings per pass over the register.

namespace aqsg {

constexpr int kPauliChunk = 8;
constexpr int kPauliThreads = 256;

struct PauliChunk {
    uint64_t x[kPauliChunk];
    uint64_t z[kPauliChunk];
    int count;
};

template <typename T>
__global__ void __launch_bounds__(kPauliThreads)
k_pauli_partial(const T* __restrict__ sv, uint64_t N, PauliChunk pc, double* partial) {
    __shared__ double sh[32];
    double re[kPauliChunk], im[kPauliChunk];
#pragma unroll
    for (int s = 0; s < kPauliChunk; ++s) re[s] = im[s] = 0.0;
    if constexpr (sizeof(a_t<T>) == 4) {
        // c64: exact products (TwoProd), compensated sums on the FP32 pipe
        FAcc fr[kPauliChunk], fi[kPauliChunk];
        auto prod = [](FAcc& acc, float x, float y, bool neg) {
            const float p = __fmul_rn(x, y);
            const float e = __fmaf_rn(x, y, -p);
            if (neg) acc.add(-p, -e);
            else acc.add(p, e);
        };
        for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < N;
             k += (uint64_t)gridDim.x * blockDim.x) {
            const T a = sv[k];
#pragma unroll
            for (int s = 0; s < kPauliChunk; ++s) {
                if (s < pc.count) {
                    const T b = sv[k ^ pc.x[s]];
                    const bool neg = __popcll(k & pc.z[s]) & 1;
                    // conj(b) a = (br ar + bi ai) + i (br ai - bi ar)
                    prod(fr[s], b.x, a.x, neg);
                    prod(fr[s], b.y, a.y, neg);
                    prod(fi[s], b.x, a.y, neg);
                    prod(fi[s], b.y, a.x, !neg);
                }
            }
        }
#pragma unroll
        for (int s = 0; s < kPauliChunk; ++s) {
            re[s] = fr[s].value();
            im[s] = fi[s].value();
        }
    } else {
        for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < N;
             k += (uint64_t)gridDim.x * blockDim.x) {
            const T a = sv[k];
            const double ar = a.x, ai = a.y;
#pragma unroll
            for (int s = 0; s < kPauliChunk; ++s) {
                if (s < pc.count) {
                    const T b = sv[k ^ pc.x[s]];
                    const double br = b.x, bi = b.y;
                    double pr = br * ar + bi * ai, pi = br * ai - bi * ar;
                    if (__popcll(k & pc.z[s]) & 1) {
                        pr = -pr;
                        pi = -pi;
                    }
                    re[s] += pr;
                    im[s] += pi;
                }
            }
        }
    }
    for (int s = 0; s < kPauliChunk; ++s) {
        if (s >= pc.count) break;
        const double r = block_sum(re[s], sh);
        const double q = block_sum(im[s], sh);
        if (threadIdx.x == 0) {
            partial[(uint64_t)blockIdx.x * 2 * kPauliChunk + 2 * s] = r;
            partial[(uint64_t)blockIdx.x * 2 * kPauliChunk + 2 * s + 1] = q;
        }
    }
}

// out[c] = sum over blocks of partial[b * cols + c]; one warp per column.
__global__ void k_pauli_final(const double* partial, int blocks, int cols, double* out) {
    const int c = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (c >= cols) return;
    double acc = 0;
    for (int b = l; b < blocks; b += 32) acc += partial[(uint64_t)b * 2 * kPauliChunk + c];
    acc = warp_sum(acc);
    if (l == 0) out[c] = acc;
}

static int pauli_masks(int n, const char* s, uint64_t* x, uint64_t* z, int* ny) {
    *x = *z = 0;
    *ny = 0;
    for (int j = 0; j < n; ++j) {
        const uint64_t bit = 1ull << (n - 1 - j);
        switch (s[j]) {
            case 'i': case 'I': break;
            case 'x': case 'X': *x |= bit; break;
            case 'y': case 'Y': *x |= bit; *z |= bit; ++*ny; break;
            case 'z': case 'Z': *z |= bit; break;
            default:
                return set_error(AQSG_ERR_INVALID_ARGUMENT,
                                 std::string("Pauli strings take the letters i, x, y, z; got '") + s[j] + "'");
        }
    }
    return AQSG_OK;
}

template <typename T>
static int expect_pauli_t(aqsg_state_s* st, const char* paulis, int count, double* out) {
    aqsg_ctx_s* c = st->ctx;
    const int n = st->n;
    struct Item {
        uint64_t x, z;
        int ny, idx;
    };
    std::vector<Item> items(count);
    for (int s = 0; s < count; ++s) {
        items[s].idx = s;
        if (int rc = pauli_masks(n, paulis + (size_t)s * n, &items[s].x, &items[s].z, &items[s].ny)) return rc;
    }
    // strings with the same x read the same partner amplitudes: keep them together
    std::stable_sort(items.begin(), items.end(), [](const Item& a, const Item& b) { return a.x < b.x; });
    const unsigned grid = stream_grid(st, st->amps, kPauliThreads);
    const size_t chunk_doubles = (size_t)grid * 2 * kPauliChunk;
    const int chunks = (count + kPauliChunk - 1) / kPauliChunk;
    if (int rc = ensure_scratch(c->partial, sizeof(double) * (chunk_doubles + 2 * kPauliChunk * (size_t)chunks)))
        return rc;
    double* partial = (double*)c->partial.ptr;
    double* results = partial + chunk_doubles;
    for (int ch = 0; ch < chunks; ++ch) {
        PauliChunk pc;
        std::memset(&pc, 0, sizeof(pc));
        pc.count = std::min(kPauliChunk, count - ch * kPauliChunk);
        for (int s = 0; s < pc.count; ++s) {
            pc.x[s] = items[ch * kPauliChunk + s].x;
            pc.z[s] = items[ch * kPauliChunk + s].z;
        }
        k_pauli_partial<T><<<grid, kPauliThreads, 0, c->stream>>>((const T*)st->d, st->amps, pc, partial);
        k_pauli_final<<<1, 32 * 2 * kPauliChunk, 0, c->stream>>>(partial, (int)grid, 2 * pc.count,
                                                                  results + (size_t)ch * 2 * kPauliChunk);
        c->launches += 2;
        AQSG_CUDA_TRY(cudaGetLastError());
    }
    std::vector<double> host((size_t)chunks * 2 * kPauliChunk);
    AQSG_CUDA_TRY(cudaMemcpyAsync(host.data(), results, sizeof(double) * host.size(), cudaMemcpyDeviceToHost,
                                  c->stream));
    AQSG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    for (int j = 0; j < count; ++j) {
        const Item& it = items[j];
        double r = host[2 * (size_t)j], q = host[2 * (size_t)j + 1];
        // multiply by i^{ny}
        for (int t = 0; t < (it.ny & 3); ++t) {
            const double nr = -q;
            q = r;
            r = nr;
        }
        out[2 * (size_t)it.idx] = r;
        out[2 * (size_t)it.idx + 1] = q;
    }
    return AQSG_OK;
}

}  // namespace aqsg

extern "C" int aqsg_expect_pauli(aqsg_state st, const char* paulis, int count, double* out) {
    using namespace aqsg;
    if (!st || !st->d) return set_error(AQSG_ERR_NULL, "NULL state");
    if (count < 0) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Negative string count");
    if (count == 0) return AQSG_OK;
    if (!paulis || !out) return set_error(AQSG_ERR_NULL, "NULL argument");
    AQSG_ON_DEVICE(st->ctx->device);
    return st->dtype == AQSG_C64 ? expect_pauli_t<float2>(st, paulis, count, out)
                                 : expect_pauli_t<double2>(st, paulis, count, out);
}

// ---- bounded-wait check ------------------------------------------------------------
//
// One thread waits on an mbarrier that nothing arrives at, with the same
// bounded-wait loop the tile kernels use (here with a caller-chosen limit),
// and reports whether it gave up.  Used to test that a wait that runs out
// ends with an error status the host reads while the context stays usable.

namespace aqsg {

__global__ void k_wait_selftest(uint64_t limit_ns, int* timed_out) {
    __shared__ uint64_t bar;
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(&bar);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(1) : "memory");
    WaitClock clk;
    uint32_t ok = 0;
    for (uint32_t it = 0;; ++it) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok) : "r"(a), "r"(0u) : "memory");
        if (ok) break;
        if ((it & 63u) == 63u && clk.expired(limit_ns)) break;
    }
    *timed_out = ok ? 0 : 1;
}

}  // namespace aqsg

extern "C" int aqsg_selftest_bounded_wait(aqsg_ctx ctx, uint32_t limit_us, int* timed_out) {
    using namespace aqsg;
    if (!ctx || !timed_out) return set_error(AQSG_ERR_NULL, "NULL argument");
    if (limit_us < 1 || limit_us > 100000) return set_error(AQSG_ERR_OUT_OF_RANGE, "Limit must be 1 us to 0.1 s");
    AQSG_ON_DEVICE(ctx->device);
    if (int rc = ensure_scratch(ctx->partial, 64)) return rc;
    int* d_flag = reinterpret_cast<int*>(ctx->partial.ptr);
    k_wait_selftest<<<1, 1, 0, ctx->stream>>>((uint64_t)limit_us * 1000ull, d_flag);
    ctx->launches++;
    AQSG_CUDA_TRY(cudaGetLastError());
    int h = -1;
    AQSG_CUDA_TRY(cudaMemcpyAsync(&h, d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    AQSG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    *timed_out = h;
    return h == 1 ? set_error(AQSG_ERR_TIMEOUT, "Bounded wait ran out (as intended)") : AQSG_OK;
}
