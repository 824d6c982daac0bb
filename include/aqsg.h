/*
 * aqsg.h — C ABI of the GB300 state-vector engine (libaqsg.so).
 *
 * This is the drop-in boundary for the hot path of arrayfire/afQuantumSim:
 * `aqs::QSimulator::simulate(const QCircuit&)` (src/quantum.cpp:277-291) and
 * the state / measurement members of QSimulator that read the same state
 * vector (src/quantum.cpp:212-531).  The reference has no C ABI: its callers
 * use the C++ classes of include/quantum.h.  Each entry point below names the
 * reference member it replaces.  The C++ layer `aqs::` (quantum.h of this
 * project) binds these calls exactly as the reference's classes did.
 *
 * Conventions
 *  - Qubit q of an n-qubit state is index bit (n-1-q): qubit 0 is the most
 *    significant bit (src/quantum.cpp:546, :261-275).
 *  - A state holds 2^n interleaved complex amplitudes, {float re, float im}
 *    (AQSG_C64, the reference's c32 dtype, include/quantum.h:107-111) or
 *    {double re, double im} (AQSG_C128).
 *  - Every call returns an aqsg_status; 0 is success.  The negative codes map
 *    one-to-one onto the exception classes the reference throws
 *    (std::out_of_range, std::invalid_argument, std::domain_error,
 *    std::runtime_error); aqsg_last_error() returns the message text.
 *  - The library owns device buffers; the caller owns host buffers.  Work is
 *    ordered on the context's CUDA stream; calls that return host data
 *    synchronise that stream.
 *  - A context and its states are used from one host thread at a time.
 */
#ifndef AQSG_H
#define AQSG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AQSG_VERSION_MAJOR 0
#define AQSG_VERSION_MINOR 1

/* Largest register the engine allocates (c64: 2^34 * 8 B = 128 GiB). The
 * reference caps circuits at 30 qubits (include/quantum.h:122); the C++ layer
 * keeps that cap, the ABI allows a little more. */
#define AQSG_MAX_QUBITS 34
/* Largest dense unitary accepted by AQSG_OP_UNITARY (32 x 32). */
#define AQSG_MAX_UNITARY_QUBITS 5
/* Operand slots of one op. */
#define AQSG_OP_MAX_QUBITS 5
#define AQSG_OP_MAX_CONTROLS 16

typedef enum aqsg_status {
    AQSG_OK = 0,
    AQSG_ERR_OUT_OF_RANGE = -1,     /* std::out_of_range in the reference   */
    AQSG_ERR_INVALID_ARGUMENT = -2, /* std::invalid_argument                */
    AQSG_ERR_DOMAIN = -3,           /* std::domain_error                    */
    AQSG_ERR_RUNTIME = -4,          /* std::runtime_error                   */
    AQSG_ERR_CUDA = -5,             /* CUDA runtime failure                 */
    AQSG_ERR_OUT_OF_MEMORY = -6,    /* device allocation failed             */
    AQSG_ERR_TIMEOUT = -7,          /* a bounded device wait gave up        */
    AQSG_ERR_NULL = -8              /* NULL handle or buffer                */
} aqsg_status;

typedef enum aqsg_dtype {
    AQSG_C64 = 0,  /* complex float32 (af::cfloat, the reference's c32) */
    AQSG_C128 = 1  /* complex float64 */
} aqsg_dtype;

/* Gate kinds.  Values 0..20 follow QGate::GateTypes (include/quantum.h:
 * 776-800) so a gate's type() maps straight onto a kind. */
typedef enum aqsg_op_kind {
    AQSG_OP_BARRIER = 0, /* Barrier          quantum.h:857-876 (no-op)           */
    AQSG_OP_X = 1,       /* X(t)             quantum.cpp:540-562                 */
    AQSG_OP_Y = 2,       /* Y(t)             quantum.cpp:580-609                 */
    AQSG_OP_Z = 3,       /* Z(t)             quantum.cpp:627-653                 */
    AQSG_OP_H = 4,       /* H(t)             quantum.cpp:812-831                 */
    AQSG_OP_PHASE = 5,   /* Phase(t, a)      quantum.cpp:849-877                 */
    AQSG_OP_SWAP = 6,    /* Swap(a, b)       quantum.cpp:912-952                 */
    AQSG_OP_RX = 7,      /* RotX(t, a)       quantum.cpp:671-699                 */
    AQSG_OP_RY = 8,      /* RotY(t, a)       quantum.cpp:718-746                 */
    AQSG_OP_RZ = 9,      /* RotZ(t, a)       quantum.cpp:765-793                 */
    AQSG_OP_CX = 10,     /* CX(c, t)         quantum.cpp:979-1014                */
    AQSG_OP_CY = 11,     /* CY(c, t)         quantum.cpp:1041-1088               */
    AQSG_OP_CZ = 12,     /* CZ(c, t)         quantum.cpp:1115-1152               */
    AQSG_OP_CH = 13,     /* CH(c, t)         quantum.cpp:1342-1400               */
    AQSG_OP_CPHASE = 14, /* CPhase(c, t, a)  quantum.cpp:1179-1218               */
    AQSG_OP_CSWAP = 15,  /* CSwap(c, a, b)   quantum.cpp:1265-1313               */
    AQSG_OP_CRX = 16,    /* CRotX(c, t, a)   quantum.cpp:1424-1436               */
    AQSG_OP_CRY = 17,    /* CRotY(c, t, a)   quantum.cpp:1461-1473               */
    AQSG_OP_CRZ = 18,    /* CRotZ(c, t, a)   quantum.cpp:1498-1510               */
    AQSG_OP_CCX = 19,    /* CCNot(a, b, t)   quantum.cpp:1542-1580               */
    AQSG_OP_OR = 20,     /* Or(a, b, t)      quantum.cpp:1614-1653               */
    /* Dense k-qubit unitary, k = num_qubits <= AQSG_MAX_UNITARY_QUBITS.  The
     * engine's form of Gate / ControlGate (quantum.cpp:1760-1814, 1888-1950):
     * `matrix` is 2^k x 2^k complex, row-major, (re, im) pairs, and qubits[0]
     * is the most significant bit of the matrix index, as in the reference's
     * gen_index embedding (src/utils.cpp:157-167). */
    AQSG_OP_UNITARY = 32
} aqsg_op_kind;

/* One gate application.  Fixed-arity kinds take their operands in the
 * reference constructor's order in qubits[] (e.g. CX: {control, target};
 * CCX: {control_a, control_b, target}; CSwap: {control, a, b}).  Any kind may
 * carry extra controls: the op then acts only on basis states whose
 * controls[i] bit equals bit i of control_values (the lowering of ControlGate
 * and NControl_Gate, src/quantum_gates.cpp:80-182). */
typedef struct aqsg_op {
    int32_t kind;            /* aqsg_op_kind                                   */
    int32_t num_qubits;      /* operands in qubits[] (UNITARY: k)              */
    int32_t num_controls;    /* extra controls in controls[]                   */
    uint32_t control_values; /* bit i: 1 = controls[i] fires on |1>, 0 on |0>  */
    float angle;             /* radians, float like the reference's gates      */
    int32_t qubits[AQSG_OP_MAX_QUBITS];
    int32_t controls[AQSG_OP_MAX_CONTROLS];
    const double* matrix;    /* UNITARY only                                   */
} aqsg_op;

/* Execution modes of aqsg_apply_ops.  All modes give the same results within
 * the precision of the state's dtype. */
typedef enum aqsg_exec_mode {
    AQSG_EXEC_AUTO = 0,     /* planner picks (currently: TILED)               */
    AQSG_EXEC_PER_GATE = 1, /* one kernel pass over HBM per gate               */
    AQSG_EXEC_TILED = 2     /* gate runs staged in shared-memory tiles         */
} aqsg_exec_mode;

/* Sampling rule for aqsg_sample. */
typedef enum aqsg_sample_rule {
    /* First index whose inclusive cumulative probability exceeds u; 0 when no
     * index does (u >= total).  This is peek_measure_all, quantum.cpp:344-359. */
    AQSG_SAMPLE_REFERENCE = 0,
    /* As above but an unmatched u returns the last index of non-zero
     * probability instead of 0. */
    AQSG_SAMPLE_CLAMP = 1
} aqsg_sample_rule;

typedef struct aqsg_ctx_s* aqsg_ctx;
typedef struct aqsg_state_s* aqsg_state;

/* ---- library / context -------------------------------------------------- */

/* Version as major*100 + minor. */
int aqsg_version(void);

/* Copy the calling thread's last error message into buf (NUL-terminated,
 * truncated to len).  Returns the full message length. */
size_t aqsg_last_error(char* buf, size_t len);

/* Open a context on CUDA device `device`, with its own stream.
 * Replaces aqs::initialize(argc, argv, backend): include/quantum.h:138-139,
 * src/quantum.cpp:69-86 (device selection; RNG seeding is explicit here). */
int aqsg_init(int device, aqsg_ctx* out);

/* Release a context.  States of the context must be freed first. */
int aqsg_shutdown(aqsg_ctx ctx);

/* Default execution mode for aqsg_apply_ops on this context. */
int aqsg_set_exec_mode(aqsg_ctx ctx, int mode);

/* Apply fused 3..5-qubit unitaries of c64 tile passes on the tensor cores
 * (tcgen05, split-BF16 three-term products accumulated in FP32) when enable
 * is non-zero (the default); otherwise on the CUDA cores in FP32. */
int aqsg_set_tensor_cores(aqsg_ctx ctx, int enable);

/* Tile shape of the tile passes that aqsg_apply_ops and aqsg_run_program
 * run on this context (batches and servers plan their own).  A register of at most
 * `qubits` qubits runs as ONE tile: one CTA holds the whole register in
 * shared memory and runs every op of the circuit in a single launch.  A
 * larger register streams through tiles of 2^12 (c64) / 2^11 (c128)
 * amplitudes, one CTA per tile and one launch per pass; only streaming
 * tiles of 2^12 c64 amplitudes run fused unitaries on the tensor cores.
 * qubits is clamped at use to [12, 14] for c64 and [11, 13] for c128;
 * 0 restores the default (14 / 13).  Negative: AQSG_ERR_INVALID_ARGUMENT.
 * The reference has no counterpart (it has no tiles). */
int aqsg_set_whole_tile_max(aqsg_ctx ctx, int qubits);

/* Wait for all work queued on the context's stream. */
int aqsg_synchronize(aqsg_ctx ctx);

/* Order two contexts of one device without blocking the host: work queued on
 * ctx after this call starts only once everything queued on other before it
 * has finished.  A pipeline over two registers uses it to keep one step's
 * gates from running alongside the previous step's (HBM-bound passes of two
 * registers interleaved run slower than one after the other) while each
 * step's host copies overlap the other step's gates.  The reference has no
 * counterpart (one simulator, one implicit ArrayFire queue). */
int aqsg_ctx_after(aqsg_ctx ctx, aqsg_ctx other);

/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work or timing events with the engine's. */
int aqsg_ctx_stream(aqsg_ctx ctx, void** stream);

/* Number of kernels this library launched on the context so far. */
int aqsg_launch_count(aqsg_ctx ctx, uint64_t* out);

/* ---- states -------------------------------------------------------------- */

/* Allocate an n-qubit register (uninitialised).  The storage of
 * QSimulator::statevector_ (include/quantum.h:738; quantum.cpp:212-259). */
int aqsg_state_alloc(aqsg_ctx ctx, int n, int dtype, aqsg_state* out);
int aqsg_state_free(aqsg_state st);
int aqsg_state_info(aqsg_state st, int* n, int* dtype);

/* Set the register to basis state |k>.  QSimulator(n, QState::zero()/one()):
 * quantum.cpp:219-222 (zero -> k=0, one -> k=2^n-1). */
int aqsg_state_set_basis_index(aqsg_state st, uint64_t k);

/* Set the register to the product state q_0 (x) q_1 (x) ... (x) q_{n-1}.
 * `amps` holds 4n floats: {re0, im0, re1, im1} per qubit, qubit 0 first.
 * QSimulator::generate_statevector, quantum.cpp:261-275. */
int aqsg_state_set_product(aqsg_state st, const float* amps);

/* Copy 2^n host amplitudes (the state's dtype, interleaved) into the register.
 * normalize != 0 divides by the 2-norm (computed in FP64) and rejects a null
 * vector with AQSG_ERR_INVALID_ARGUMENT, as QSimulator(n, af::array)
 * does (quantum.cpp:242-259). */
int aqsg_state_upload(aqsg_state st, const void* host, int normalize);

/* Copy the register to 2^n host amplitudes (the state's dtype).  Replaces
 * QSimulator::statevector() / state(k) (include/quantum.h:726-734, 694-697). */
int aqsg_state_download(aqsg_state st, void* host);

/* Copy amplitudes [begin, begin+count) to the host. */
int aqsg_state_download_range(aqsg_state st, uint64_t begin, uint64_t count,
                              void* host);

/* As aqsg_state_download, but only enqueued on the context's stream: the
 * host buffer is complete after the next aqsg_synchronize of the context.
 * With pinned host memory this lets a host pipeline registers on several
 * contexts (copies of one overlapping the gates of another).  No reference
 * counterpart (the reference reads the state synchronously). */
int aqsg_state_download_async(aqsg_state st, void* host);

/* Copy src into dst (same n and dtype). */
int aqsg_state_copy(aqsg_state dst, aqsg_state src);

/* Compare two registers with the same qubit count (either dtype) in one
 * FP64 pass: max_i |a_i - b_i|, the overlap <a|b> and both squared norms.
 * Any output pointer may be NULL.  (Parity checks of large registers, e.g. a
 * c64 run against a c128 run of the same circuit.) */
int aqsg_state_compare(aqsg_state a, aqsg_state b, double* max_abs_diff, double* overlap_re,
                       double* overlap_im, double* norm2_a, double* norm2_b);

/* ---- simulation ----------------------------------------------------------- */

/* Validate ops against an n-qubit register without running them.  Returns the
 * status the reference's QGate::check would raise (src/quantum.cpp, the
 * check() of each gate), with its message. */
int aqsg_check_ops(int n, const aqsg_op* ops, int count);

/* Apply ops in order to the register: the gate loop of
 * QSimulator::simulate, quantum.cpp:285-290, with QGate::operator() of every
 * gate class (quantum.cpp:533-1950) replaced by in-place kernels.
 * mode: an aqsg_exec_mode, or -1 for the context default. */
int aqsg_apply_ops(aqsg_state st, const aqsg_op* ops, int count, int mode);

/* ---- compiled programs ---------------------------------------------------- */

typedef struct aqsg_program_s* aqsg_program;

/* Compile ops for an n-qubit register of `dtype`: consecutive gates are fused
 * into dense unitaries on at most `max_qubits` (1..5) qubits (diagonal-only
 * groups stay diagonal).  The engine's form of QCircuit::compile
 * (quantum.cpp:199-210), which folds gates into one 2^n x 2^n matrix; here
 * the folded pieces stay small enough for tensor-core tile passes.
 * Validation and messages as aqsg_check_ops. */
int aqsg_compile(int n, int dtype, const aqsg_op* ops, int count, int max_qubits,
                 aqsg_program* out);

/* Number of fused ops and of source ops of a program. */
int aqsg_program_info(aqsg_program prog, int* fused_ops, int* source_ops);

/* The tile plan a tiled run of the program executes (tensor cores on or
 * off): *passes tile passes, *tc_passes of them on the tensor cores, and
 * *hbm_bytes = the HBM bytes of one run (one read and one write of the
 * register per pass, plus the renormalisation of a run with tensor-core
 * passes: a scale pass, and a read pass for each end of the run that is not
 * a tensor-core pass).  Host-side only; any output may be NULL. */
int aqsg_program_plan(aqsg_program prog, int tensor_cores, int* passes, int* tc_passes, uint64_t* hbm_bytes);

/* Run a compiled program on a register with the program's n and dtype
 * (QSimulator::simulate's compiled prefix, quantum.cpp:283).  mode: an
 * aqsg_exec_mode or -1 for the context default. */
int aqsg_run_program(aqsg_state st, aqsg_program prog, int mode);

/* Copy the program's ops in ABI form into out[0..capacity) (fused groups
 * become AQSG_OP_UNITARY ops whose matrix points into the program, valid
 * until aqsg_program_free); *count receives the op count.  out may be NULL
 * to query the count.  For inspection, serialisation and replay. */
int aqsg_program_export(aqsg_program prog, aqsg_op* out, int capacity, int* count);

int aqsg_program_free(aqsg_program prog);

/* ---- circuit text ------------------------------------------------------------ */

/* Circuits as text: the reference's gate representation ("Name,controls,
 * targets:controls...,targets...;", QGate::to_string, src/quantum.cpp:
 * 569-1662; the layout parse_circuit_representation reads, src/
 * quantum_visuals.cpp:71-80) extended into a replayable wire format for
 * request streams and golden files:
 *   "n;"                      header: the qubit count
 *   "RotX(0.25),0,1:3;"       parameters after the name: an angle (float,
 *                             printed to round-trip exactly), or for "U" the
 *                             2^k x 2^k matrix as (re, im) doubles, row-major
 *   "X,1,1:0,2;" "X,2,1:0,1,2;"  base gate name with its controls first
 *                             (CX, CCNot), as the reference writes them
 *   "Z,1,1:~4,2;"             a control that fires on |0>
 *   "Or,2,1:0,1,2;"  "B;"     Or; a barrier ("P;" reads as one too)
 * Reference names that fix an angle read as their gates: S, S†, T, T†.
 * Written text is canonical (parse, then write, gives the same text). */

/* Write ops as text into buf (len bytes, NUL-terminated); *needed receives
 * the size including the NUL.  buf may be NULL to query the size.  The ops
 * are validated first (aqsg_check_ops). */
int aqsg_circuit_to_text(int n, const aqsg_op* ops, int count, char* buf, size_t len, size_t* needed);

/* Parse text into *n and ops[0 .. *count).  Unitary matrices are copied into
 * matrices (matrix_capacity doubles) and the ops point there; with ops ==
 * NULL only *n, *count and *matrix_count (doubles needed) are set.  Syntax
 * errors return AQSG_ERR_INVALID_ARGUMENT with the offending token in
 * aqsg_last_error; the parsed ops are validated like aqsg_check_ops (the
 * reference's exception classes and messages). */
int aqsg_circuit_from_text(const char* text, int* n, aqsg_op* ops, int capacity, int* count,
                           double* matrices, size_t matrix_capacity, size_t* matrix_count);

/* ---- autotuner ------------------------------------------------------------- */

/* One way of running a circuit and its measured time. */
typedef struct aqsg_tune_entry {
    int32_t exec_mode;     /* AQSG_EXEC_PER_GATE or AQSG_EXEC_TILED            */
    int32_t fuse_qubits;   /* 0 = the gates as they are, else aqsg_compile width */
    int32_t tensor_cores;  /* fused unitaries on the tensor cores (c64)         */
    int32_t ops;           /* ops after fusion                                  */
    double ms;             /* device time of one run                           */
    int32_t tile_bits;     /* tile passes: log2 of the amplitudes one CTA holds
                            * (n = the whole register in one tile; to run this
                            * way set aqsg_set_whole_tile_max below n);
                            * 0 for one gate per pass                          */
    int32_t reserved;      /* 0                                                */
} aqsg_tune_entry;

/* Time the circuit (on a scratch n-qubit register of dtype, from |0...0>)
 * one gate per pass, in tile passes, compiled with fusion width 1 (runs of
 * 1-qubit gates merged) and with widths 2..5 with and without the tensor
 * cores; reps timed runs each after one warm-up.  A register that fits one
 * whole-register tile but is larger than a streaming tile (13-14 qubits
 * c64, 12-13 c128) has every tile-pass candidate timed in both tile shapes.
 * *best receives the fastest.  The choice is cached per context by the
 * circuit's structure (kinds and operands, not angles or matrix entries):
 * with all == NULL a cached choice returns at once.  all (capacity entries,
 * may be NULL) receives every timing, *count_out their number.  The
 * reference has no counterpart: it runs every circuit one way. */
int aqsg_autotune(aqsg_ctx ctx, int n, int dtype, const aqsg_op* ops, int count, int reps,
                  aqsg_tune_entry* best, aqsg_tune_entry* all, int capacity, int* count_out);

/* ---- batched engine (many independent registers) ------------------------ */

/* One circuit of a batch: an n-qubit c64 register, run from |0...0>. */
typedef struct aqsg_circuit {
    int32_t n;
    int32_t count;
    const aqsg_op* ops;
} aqsg_circuit;

typedef struct aqsg_batch_s* aqsg_batch;

/* Plan a batch of independent circuits of uneven size, each ending in
 * <Z_q> and <Z_q Z_q+1> summed in FP64 (divided by the register's FP64
 * norm).  It generalises the reference's VQE cost loop
 * (src/quantum_algo.cpp:412-456: one simulate and one expectation read per
 * parameter set) to a whole sweep.  Registers of up to 14 qubits run
 * entirely in shared memory (a persistent kernel per size class, one CTA per
 * circuit); larger ones (up to 30) run as tile passes over one reused device
 * register, each compiled with the fusion width the autotuner picks for its
 * structure, timed the way the batch runs it: registers of equal structure
 * run as a group, one launch per tile pass for all of them (the choice is
 * cached per structure and timed over a group size that depends on n only,
 * so a circuit runs the same way alone and in any batch).  The whole run is
 * captured once as a CUDA graph.  Create and update lower and encode the
 * circuits on all host threads; the encoded plans are kept in one pinned
 * host image, uploaded with one copy, and the caller's circuits are not
 * retained. */
int aqsg_batch_create(aqsg_ctx ctx, const aqsg_circuit* circuits, int count, aqsg_batch* out);

/* Swap in new parameters (angles, matrices): the same count, qubit counts,
 * gate kinds and operands as at creation; the graph is kept.  Circuits whose
 * encoding changes shape (op records, operand sizes, passes) are refused
 * with AQSG_ERR_INVALID_ARGUMENT and the device copy is left as it was. */
int aqsg_batch_update(aqsg_batch b, const aqsg_circuit* circuits);

/* Replay the graph.  z receives sum_i n_i values (<Z_q> of circuit i at
 * offset sum_{j<i} n_j), zz receives sum_i (n_i - 1) values of <Z_q Z_q+1>;
 * either may be NULL. */
int aqsg_batch_run(aqsg_batch b, double* z, double* zz);

/* Circuits run in shared memory / as tile passes, kernels per replay. */
int aqsg_batch_info(aqsg_batch b, int* small_circuits, int* large_circuits, int* kernels);
/* Algorithmic HBM bytes of one aqsg_batch_run: for each register of more
 * than 14 qubits, its clear to |0...0> (one write), one read and one write
 * per tile pass and the read of the expectation sums; registers of at most
 * 14 qubits live in shared memory and move no state through HBM. */
int aqsg_batch_traffic(aqsg_batch b, uint64_t* hbm_bytes);

/* Fusion width (0 = none) and tensor-core use the autotuner chose for each
 * large register, in circuit order (arrays of large_circuits entries, see
 * aqsg_batch_info; either may be NULL). */
int aqsg_batch_tuning(aqsg_batch b, int* fuse_qubits, int* tensor_cores);

int aqsg_batch_free(aqsg_batch b);

/* ---- noise by trajectories ------------------------------------------------ */

/* A Pauli channel after every gate: each qubit the gate touches (targets and
 * controls) independently gets X, Y or Z with probability p[0], p[1], p[2]
 * (and is left alone with 1 - p[0] - p[1] - p[2]); p1 applies after gates
 * on one qubit, p2 after gates on several.  Depolarizing noise of strength
 * p is p/3 for each.  The reference reserves a class for noise (QNoise,
 * include/quantum.h:475) but leaves it empty; this is the engine's own. */
typedef struct aqsg_noise {
    float p1[3];
    float p2[3];
} aqsg_noise;

/* Trajectory `trajectory` of the noisy circuit: the ops with the Paulis it
 * draws inserted right after the gates they follow.  Each draw is a
 * counter-based function of (seed, trajectory, gate index, qubit), so a
 * trajectory is the same circuit whatever else is drawn.  With out NULL,
 * *out_count receives the trajectory's length; otherwise at most capacity
 * ops are written (AQSG_ERR_OUT_OF_RANGE if they do not fit).  Probabilities
 * must be >= 0 with sums <= 1 (AQSG_ERR_INVALID_ARGUMENT). */
int aqsg_noise_trajectory(int n, const aqsg_op* ops, int count, const aqsg_noise* noise, uint64_t seed,
                          uint64_t trajectory, aqsg_op* out, int capacity, int* out_count);

/* <Z_q> and <Z_q Z_q+1> of the noisy circuit run from |0...0> (n <= 30),
 * estimated by trajectories 0 .. trajectories - 1 of (seed) run as one
 * batch (aqsg_batch_create): z[n], zz[n - 1] are the means over the
 * trajectories, z_err / zz_err (may be NULL) their standard errors
 * (sample standard deviation / sqrt(trajectories)). */
int aqsg_noise_expect_z(aqsg_ctx ctx, int n, const aqsg_op* ops, int count, const aqsg_noise* noise,
                        uint64_t seed, int trajectories, double* z, double* zz, double* z_err, double* zz_err);

/* ---- serving runtime (a stream of independent requests) ------------------ */

/* A request is one circuit run from |0...0> followed by `shots` seeded
 * measure-all draws: QSimulator::simulate (quantum.cpp:277) then repeated
 * peek_measure_all (quantum.cpp:343-358, sample rule AQSG_SAMPLE_REFERENCE,
 * uniforms from aqsg_sample_seeded's generator); profile_measure_all
 * (quantum.cpp:467) is the histogram of such draws.  The reference handles one circuit per
 * QSimulator call; the server keeps a fixed HBM slab and runs many requests
 * at once:
 *  - admission: a request is eligible once its arrival time has passed; it
 *    is admitted when a lane is idle and a 2^n-amplitude block of the slab
 *    (buddy allocator, power-of-two blocks) is free.  Eligible requests are
 *    tried in arrival order and a smaller later one may pass a larger one
 *    that does not fit, unless that one has been passed over 64 times;
 *  - lanes: each lane owns a CUDA stream and reserved scratch, so a running
 *    request never allocates and never blocks the host;
 *  - the register stays in HBM from preparation to sampling; only the op
 *    tables go up and the outcomes come down. */
typedef struct aqsg_server_s* aqsg_server;

typedef struct aqsg_server_done {
    uint64_t ticket;
    int32_t status;   /* aqsg_status of the request */
    int32_t n;
    int32_t lane;
    int32_t fused_ops; /* ops after fusion (or the lowered op count) */
    double arrival_s;  /* seconds since aqsg_server_start */
    double admit_s;
    double done_s;     /* when the worker saw the outcomes on the host */
} aqsg_server_done;

typedef struct aqsg_server_stats {
    uint64_t submitted, completed, failed;
    uint64_t slab_bytes;       /* HBM held for registers */
    uint64_t peak_bytes;       /* most slab bytes in use at once */
    int32_t peak_running;      /* most requests in flight at once */
    int32_t lanes;
    uint64_t launches;         /* kernels launched by all lanes */
    uint64_t hbm_bytes;        /* algorithmic HBM bytes of the completed requests:
                                  register set to |0...0>, one read + one write per
                                  tile pass, the renormalisation's reads and rescale
                                  of tensor-core runs, the sampling reads */
} aqsg_server_stats;

/* Create a server on `device` for registers of dtype and at most max_qubits
 * qubits, holding hbm_budget_bytes of registers (rounded down to a multiple
 * of the largest register), with `lanes` concurrent requests and at most
 * max_shots shots per request. */
int aqsg_server_create(int device, int dtype, uint64_t hbm_budget_bytes, int lanes, int max_qubits,
                       uint32_t max_shots, aqsg_server* out);

/* Queue a request.  The ops are validated (aqsg_check_ops), lowered, fused
 * into unitaries of up to fuse_qubits qubits (0 = no fusion) and planned
 * here, on the caller's thread.  arrival_s is the earliest admission time in
 * seconds after aqsg_server_start (negative = now).  `outcomes` (shots
 * values) must stay valid until the request shows up in aqsg_server_poll.
 * The ops and their matrices may be freed when this returns. */
int aqsg_server_submit(aqsg_server srv, int n, const aqsg_op* ops, int count, int fuse_qubits,
                       uint32_t shots, uint64_t seed, double arrival_s, uint64_t* outcomes,
                       uint64_t* ticket);

/* Start the clock and the worker thread. */
int aqsg_server_start(aqsg_server srv);

/* Move up to `capacity` finished requests into done[]; *count receives how
 * many. */
int aqsg_server_poll(aqsg_server srv, aqsg_server_done* done, int capacity, int* count);

/* Wait until every submitted request has finished (AQSG_ERR_TIMEOUT after
 * timeout_s seconds). */
int aqsg_server_wait_idle(aqsg_server srv, double timeout_s);

int aqsg_server_get_stats(aqsg_server srv, aqsg_server_stats* out);

/* Stop the worker and free the slab: requests in flight finish, queued ones
 * are dropped (they never show up in aqsg_server_poll). */
int aqsg_server_destroy(aqsg_server srv);

/* ---- failure handling -------------------------------------------------------- */

/* Run one thread waiting on a barrier that nothing releases, with the
 * bounded-wait loop the tile kernels use and a limit of limit_us
 * microseconds (1 .. 100000).  *timed_out = 1 when the wait ran out, and the
 * call then returns AQSG_ERR_TIMEOUT; the context stays usable.  Exists to
 * test the engine's failure path without a GPU fault; no reference
 * counterpart. */
int aqsg_selftest_bounded_wait(aqsg_ctx ctx, uint32_t limit_us, int* timed_out);

/* ---- measurement ---------------------------------------------------------- */

/* Probability that `qubit` reads |1>, summed in FP64.
 * QSimulator::qubit_probability_true, quantum.cpp:372-391. */
int aqsg_qubit_prob(aqsg_state st, int qubit, double* out);

/* |a_k|^2.  QSimulator::state_probability, quantum.cpp:393-402. */
int aqsg_state_prob(aqsg_state st, uint64_t k, double* out);

/* All 2^n probabilities |a_k|^2 to the host as float (out_dtype 0) or double
 * (out_dtype 1).  QSimulator::probabilities, quantum.cpp:404-414. */
int aqsg_probs(aqsg_state st, void* host, int out_dtype);

/* Total probability sum_k |a_k|^2 in FP64. */
int aqsg_norm2(aqsg_state st, double* out);

/* Draw `count` outcomes for the uniforms u[0..count) from the FP64
 * cumulative distribution of |a_k|^2 (rule: aqsg_sample_rule).  The index
 * of each outcome goes to out[i].  peek_measure_all (quantum.cpp:344-359)
 * is count = 1 with rule AQSG_SAMPLE_REFERENCE; profile_measure_all
 * (quantum.cpp:467-501) is a histogram of count outcomes. */
int aqsg_sample(aqsg_state st, const double* u, uint64_t count, int rule,
                uint64_t* out);

/* As aqsg_sample with the uniforms drawn on the device by Philox4x32-10
 * from (seed, stream counter 0..count). */
int aqsg_sample_seeded(aqsg_state st, uint64_t seed, uint64_t count, int rule,
                       uint64_t* out);

/* Allocation-free sampling.  No counterpart in the reference: it exists for
 * callers that must not allocate device memory once they are running — for
 * example a serving loop that admits work against a fixed HBM budget, or a
 * host that embeds the engine next to a framework's caching allocator — since
 * cudaMalloc/cudaFree can synchronise the whole device and stall unrelated
 * streams.  Same rule and results as aqsg_sample, but its device scratch is
 * one static array of the library (AQSG_NOALLOC_SCRATCH_BYTES, held on every
 * GPU that loads the library until the process exits) instead of buffers
 * grown on demand.  The register must have at most AQSG_NOALLOC_MAX_QUBITS
 * qubits and count must be at most AQSG_NOALLOC_MAX_SHOTS; larger requests
 * fail with AQSG_ERR_INVALID_ARGUMENT.  aqsg_init looks up the array's
 * device address for its device (which also loads the code that holds the
 * array, so the array is resident before any sampling call); create the
 * context before any stream capture.  Every call makes the context's device
 * current and gives the caller's device back.  All calls on a device share
 * the array: calls whose GPU work overlaps (other threads or streams) race
 * and must be serialised by the caller. */
#define AQSG_NOALLOC_MAX_QUBITS 30
#define AQSG_NOALLOC_MAX_SHOTS 16384
#define AQSG_NOALLOC_SCRATCH_BYTES \
    ((size_t)2 * 8 * ((size_t)1 << (AQSG_NOALLOC_MAX_QUBITS - 12)) + \
     (size_t)16 * AQSG_NOALLOC_MAX_SHOTS)
int aqsg_sample_noalloc(aqsg_state st, const double* u, uint64_t count, int rule,
                        uint64_t* out);

/* Measure `qubit` with uniform u: outcome = (u < p1), then zero the other
 * branch and renormalise the kept one, in one pass.  The outcome goes to
 * *outcome and its probability to *prob.  QSimulator::measure,
 * quantum.cpp:308-342. */
int aqsg_collapse_qubit(aqsg_state st, int qubit, double u, int* outcome,
                        double* prob);

/* Measure all qubits with uniform u (rule AQSG_SAMPLE_REFERENCE) and set the
 * register to the basis state drawn.  QSimulator::measure_all,
 * quantum.cpp:361-370. */
int aqsg_collapse_all(aqsg_state st, double u, uint64_t* outcome);

/* <Z_q> for every qubit q (z[n]) and <Z_q Z_{q+1}> for q = 0..n-2 (zz[n-1]),
 * summed in FP64 in one pass.  Either pointer may be NULL.  <Z_q> is
 * 1 - 2 * qubit_probability_true(q) (quantum.cpp:372-391). */
int aqsg_expect_z(aqsg_state st, double* z, double* zz);

/* <psi|P|psi> for `count` Pauli strings, summed in FP64: out[2s], out[2s+1]
 * = real and imaginary part for string s.  `paulis` holds the strings back
 * to back, n characters each from {i, x, y, z} (either case), character j
 * acting on qubit j: the strings decompose_hamiltonian returns
 * (quantum_algo.cpp:131-190).  A Hamiltonian's energy is sum_s c_s out[s];
 * this replaces the reference's bra-ket product of the state with the
 * evolved state (quantum_algo.cpp:441-450).  Strings with the same X/Y
 * pattern share their reads; each pass over the register serves 8 strings. */
int aqsg_expect_pauli(aqsg_state st, const char* paulis, int count, double* out);

#ifdef __cplusplus
}
#endif

#endif /* AQSG_H */
