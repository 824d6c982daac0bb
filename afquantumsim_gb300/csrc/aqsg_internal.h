// Internal declarations of libaqsg: context/state objects, the lowered gate
// form the kernels consume, and the kernel launchers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <functional>
#include <vector>

#include "../../include/aqsg.h"

namespace aqsg {

// ---- errors ---------------------------------------------------------------
int set_error(int code, const std::string& msg);
std::string last_error_message();  // this thread's last set_error text
int cuda_error(cudaError_t e, const char* where);
#define AQSG_CUDA_TRY(expr)                                     \
    do {                                                        \
        cudaError_t e__ = (expr);                               \
        if (e__ != cudaSuccess) return ::aqsg::cuda_error(e__, #expr); \
    } while (0)

// Makes a context's device current for the duration of an entry point and
// gives the calling thread back the device it had current on the way out,
// so that one host thread can drive contexts on several GPUs in any order.
class DeviceScope {
  public:
    explicit DeviceScope(int device) {
        if (cudaGetDevice(&prev_) != cudaSuccess) prev_ = -1;
        if (prev_ != device) {
            err_ = cudaSetDevice(device);
            switched_ = err_ == cudaSuccess && prev_ >= 0;
        }
    }
    ~DeviceScope() {
        if (switched_) cudaSetDevice(prev_);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
    cudaError_t error() const { return err_; }

  private:
    int prev_ = -1;
    bool switched_ = false;
    cudaError_t err_ = cudaSuccess;
};
#define AQSG_ON_DEVICE(dev)                                                   \
    ::aqsg::DeviceScope aqsg_device_scope__(dev);                             \
    if (aqsg_device_scope__.error() != cudaSuccess)                           \
        return ::aqsg::cuda_error(aqsg_device_scope__.error(), "cudaSetDevice")

// ---- lowered gate form ------------------------------------------------------
// Every reference gate lowers to one of these classes acting on index bits
// (bit = n-1-qubit).  Coefficients for c64 are float values (computed with
// float trig exactly as src/quantum.cpp does) stored in double; for c128
// they are the double-precision values of the same formulas.
enum LCls : int {
    L_NOP = 0,
    L_PERM_X = 1,    // swap the pair (t=0, t=1) where the condition holds
    L_PERM_OR = 2,   // as PERM_X, condition: (i & amask) != 0
    L_PERM_SWAP = 3, // swap (a=0,b=1) <-> (a=1,b=0) where the condition holds
    L_DIAG1 = 4,     // multiply amplitudes with (i & pmask) == pval by m[0]
    L_DIAG2 = 5,     // target t: multiply t=0 by m[0], t=1 by m[1] (complex slots)
    L_MAT2 = 6,      // 2x2 matrix on target t
    L_MATK = 7       // 2^k x 2^k matrix on bits tb[0..k) (tb[0] = MSB)
};

struct LOp {
    int cls = L_NOP;
    int t0 = -1, t1 = -1;       // target bits
    int k = 0;                  // MATK
    int tb[AQSG_MAX_UNITARY_QUBITS] = {0, 0, 0, 0, 0};
    uint64_t cmask = 0, cval = 0;  // all-of condition on other bits
    uint64_t amask = 0;            // any-of condition (Or)
    double m[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // complex coefficients (re, im)
    std::vector<double> mk;        // MATK: row-major complex matrix
    // diagonal ops do not force their bits into a tile
    bool diagonal() const { return cls == L_DIAG1 || cls == L_DIAG2; }
};

// Number of target qubits of a gate kind (0 for a barrier, -1 if unknown;
// unitaries carry theirs in num_qubits).
int op_arity(int kind);
// Validate one op against an n-qubit register with the reference's check()
// messages; returns AQSG_OK or an error code (message set).
int check_op(int n, const aqsg_op& op);
// Lower one op (already checked).  dtype selects the coefficient precision.
int lower_op(int n, int dtype, const aqsg_op& op, LOp* out);

// ---- objects ------------------------------------------------------------------
struct Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
};

}  // namespace aqsg

namespace aqsg {
struct PlanCache;
}

struct aqsg_ctx_s {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    int exec_mode = AQSG_EXEC_AUTO;
    uint64_t launches = 0;
    int live_states = 0;
    aqsg::Scratch partial;   // FP64 partial sums of reductions
    aqsg::Scratch tcnorm;    // per-CTA norm partials of the first / last tensor-core pass
    aqsg::Scratch prefix;    // FP64 chunk prefix sums for sampling
    aqsg::Scratch sample_u;  // uniforms of one sampling call
    aqsg::Scratch sample_o;  // outcomes of one sampling call
    aqsg::Scratch ops;       // device copy of tile-pass op tables
    aqsg::Scratch probs;     // probability download staging
    double* host_result = nullptr;  // pinned FP64 results
    int* d_err = nullptr;           // device flag: a bounded kernel wait gave up
    int tensor_cores = 1;           // fused unitaries on tcgen05 (c64 tiles)
    int whole_tile_max = 0;         // largest register run as one tile (0: the dtype's maximum)
    cudaEvent_t order = nullptr;    // marks this stream's queue for aqsg_ctx_after
    aqsg::PlanCache* plans = nullptr;  // recently run tile plans (host + device copies)
};

struct aqsg_state_s {
    aqsg_ctx ctx = nullptr;
    int n = 0;
    int dtype = AQSG_C64;
    uint64_t amps = 0;
    void* d = nullptr;
};

namespace aqsg {

int ensure_scratch(Scratch& s, size_t bytes);
inline size_t amp_bytes(int dtype) { return dtype == AQSG_C128 ? 16 : 8; }

// ---- kernel launchers (gate_kernels.cu) -------------------------------------
int launch_lop(aqsg_state_s* st, const LOp& op);

// ---- tile passes (tile_kernels.cu) ---------------------------------------------
// One pass of a tile plan: its m tile bits (ascending; the first L are the
// row bits) and its ops table[first, first+count).
struct TilePass {
    int m, L;
    int tbits[16];
    uint32_t first, count;
    int tc;              // uses the tensor-core kernel
    int matk;            // has dense k-qubit ops run on CUDA cores
    uint32_t tc_blob;    // pool offset of the pass's tensor-core operands (1 KiB aligned)
    uint32_t tc_bytes;   // their size: loaded into shared memory once per CTA
};
// Encoded passes of an op list: op table (device TileOp records, as bytes)
// and operand pool (matrices / tensor-core operands) to upload together,
// table first and the pool at pool_offset().
struct TilePlan {
    int n = 0, dtype = AQSG_C64;
    std::vector<unsigned char> table;
    std::vector<unsigned char> pool;
    std::vector<TilePass> passes;
    bool any_tc = false;
    bool any_stream = false;  // a pass runs bounded waits that may set the error flag
    size_t pool_offset() const;
};
// exact_perm: fused permutation matrices stay off the tensor cores (bit-exact
// moves); false makes the choice depend on the op structure only.
bool relocate_tile_matrices(unsigned char* table, size_t count, int32_t delta);
// whole_max: the largest register encoded as one whole-register tile (0: the
// dtype's maximum, tile_max_bits; clamped to [stream_tile_bits, tile_max_bits]).
int encode_tiled(int n, int dtype, const std::vector<LOp>& ops, bool tc_on, TilePlan* plan, bool exact_perm = true,
                 int whole_max = 0);
// Launch the passes on `stream`; dev = device copy of table + pool.
// norm_part (optional, 2 x tc_grid doubles): the first pass, when it runs on
// the tensor cores, writes per-CTA FP64 partial sums of |a|^2 of its input
// to norm_part[0, grid), the last such pass of its output to
// norm_part[grid, 2 grid); *tc_grid = the tensor-core passes' grid.
int launch_tile_plan(void* sv, const TilePlan& plan, const void* dev, cudaStream_t stream, int* d_err,
                     uint64_t* launches, double* norm_part = nullptr, uint32_t* tc_grid = nullptr);
// One FP64 sum of count partials into *out (device), on the context stream.
int launch_sum_partials(aqsg_ctx_s* c, const double* parts, int count, double* out);
// A plain (no tensor-core) complex64 streaming plan over `members` registers
// at reg_stride amplitudes from one another, whose tables (the same geometry,
// their own ops) sit dev_stride bytes apart from dev0: one launch per pass.
int launch_tile_plan_multi(void* sv0, uint64_t reg_stride, int members, const TilePlan& plan, const void* dev0,
                           uint64_t dev_stride, cudaStream_t stream, int* d_err, uint64_t* launches);
// Runs ops through shared-memory tile passes, with the encoded plan and its
// device table cached per context under `key` (bytes that determine the
// plan: the caller's ops, or a program's identity).  On a hit, lower() is
// not called; on a miss it fills the ops to encode.
int run_tiled_cached(aqsg_state_s* st, const std::vector<unsigned char>& key,
                     const std::function<int(std::vector<LOp>*)>& lower);
void plan_cache_free(aqsg_ctx_s* c);
// Largest tile (log2 amplitudes) the tile kernel holds for a dtype.
int tile_max_bits(int dtype);
// Tile of a streaming pass (log2 amplitudes) for a dtype.
int stream_tile_bits(int dtype);
// The whole-register limit a setting of aqsg_set_whole_tile_max gives.
int whole_tile_limit(int dtype, int setting);
// Algorithmic HBM bytes of running a plan once: one read and one write of
// the register per tile pass; with renorm, a run with tensor-core passes
// also reads the register twice for its norms and rescales it once.
// HBM bytes of the plan's passes, with renorm also its renormalisation
// (= plan_run_bytes).
uint64_t plan_hbm_bytes(const TilePlan& plan, bool renorm);
// HBM bytes of one run of the plan: its passes and, for tensor-core runs,
// the scale pass plus a norm read for each end that is not a tensor-core
// pass.
uint64_t plan_run_bytes(const TilePlan& plan);

// ---- init / measurement launchers (measure_kernels.cu) -------------------------
int launch_set_basis(aqsg_state_s* st, uint64_t k);
int launch_set_product(aqsg_state_s* st, const float* amps);
int launch_scale(aqsg_state_s* st, double scale);
// sum of |a_i|^2 over i with (i & mask) == val, FP64; result on host
int reduce_prob(aqsg_state_s* st, uint64_t mask, uint64_t val, double* out);
int launch_probs(aqsg_state_s* st, void* dev_out, int out_dtype);
int sample(aqsg_state_s* st, const double* host_u, uint64_t seed, bool seeded,
           uint64_t count, int rule, uint64_t* host_out);
int launch_collapse_qubit(aqsg_state_s* st, uint64_t mask, int outcome,
                          double scale);
int expect_z(aqsg_state_s* st, double* z, double* zz);
// Looks up (once per device, with that device current) the device address of
// the allocation-free sampler's static scratch, which loads its module.
int noalloc_prepare(int device);
// asynchronous variants (no host read; scratch reserved beforehand)
int reserve_scratch(aqsg_ctx_s* c, int n, uint64_t shots);
int launch_norm_to_device(aqsg_state_s* st, double* d_out);
int launch_renorm_device(aqsg_state_s* st, const double* n_before, const double* n_after);
int sample_seeded_async(aqsg_state_s* st, uint64_t seed, uint64_t count, int rule, uint64_t* pinned_out);
// Tile passes without host synchronisation; dev_table is the device copy of
// plan.table followed by plan.pool at plan.pool_offset().  Tensor-core runs
// renormalise on the device through d_norms (tc_norm_doubles() doubles; the
// context's reduction scratch reserved for read passes).
int run_plan_async(aqsg_state_s* st, const TilePlan& plan, const void* dev_table, double* d_norms);
// Doubles of the renormalisation buffer of a tensor-core run on c.
size_t tc_norm_doubles(const aqsg_ctx_s* c);
// aqsg_autotune, optionally without the one-gate-per-pass candidate.
int autotune_impl(aqsg_ctx ctx, int n, int dtype, const aqsg_op* ops, int count, int reps, bool tiled_only,
                  aqsg_tune_entry* best, aqsg_tune_entry* all, int capacity, int* count_out);
// Fusion width for a batched large register, timed as a group of replicas
// on the CUDA cores (cached per context and structure).
int autotune_grouped(aqsg_ctx ctx, int n, const aqsg_op* ops, int count, int* fuse_out, int* tc_out);
// Drop the autotuner's cached choices of a context (it is shutting down).
void autotune_forget(aqsg_ctx ctx);
// The fused op list of a compiled program.
const std::vector<LOp>& program_ops(aqsg_program p);

}  // namespace aqsg
