// C ABI of libaqsg: contexts, registers, op validation/lowering, dispatch.
//
// The checks below restate the check() members of the reference's gate
// classes (src/quantum.cpp:533-1677) with the same exception classes (as
// status codes) and message texts.
#include <cmath>
#include <cstring>
#include <string>

#include "aqsg_internal.h"
#include "../../include/aqsg_debug.h"

namespace aqsg {

static thread_local std::string g_last_error;

int set_error(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

std::string last_error_message() { return g_last_error; }

int cuda_error(cudaError_t e, const char* where) {
    std::string msg = std::string("CUDA error ") + cudaGetErrorName(e) + " (" +
                      cudaGetErrorString(e) + ") at " + where;
    return set_error(e == cudaErrorMemoryAllocation ? AQSG_ERR_OUT_OF_MEMORY
                                                    : AQSG_ERR_CUDA,
                     msg);
}

int ensure_scratch(Scratch& s, size_t bytes) {
    if (s.bytes >= bytes && s.ptr) return AQSG_OK;
    if (s.ptr) {
        AQSG_CUDA_TRY(cudaFree(s.ptr));
        s.ptr = nullptr;
        s.bytes = 0;
    }
    size_t want = bytes < 4096 ? 4096 : bytes;
    AQSG_CUDA_TRY(cudaMalloc(&s.ptr, want));
    s.bytes = want;
    return AQSG_OK;
}

static const char* kAt = "Cannot add gate at the given qubit position";
static const char* kCtlTgt = "Control qubit cannot be the same as the target qubit";
static const char* kSwapSame = "Cannot use the swap gate on the same target qubits";

int op_arity(int kind) {
    switch (kind) {
        case AQSG_OP_BARRIER: return 0;
        case AQSG_OP_X: case AQSG_OP_Y: case AQSG_OP_Z: case AQSG_OP_H:
        case AQSG_OP_PHASE: case AQSG_OP_RX: case AQSG_OP_RY: case AQSG_OP_RZ:
            return 1;
        case AQSG_OP_SWAP: case AQSG_OP_CX: case AQSG_OP_CY: case AQSG_OP_CZ:
        case AQSG_OP_CH: case AQSG_OP_CPHASE: case AQSG_OP_CRX:
        case AQSG_OP_CRY: case AQSG_OP_CRZ:
            return 2;
        case AQSG_OP_CSWAP: case AQSG_OP_CCX: case AQSG_OP_OR: return 3;
        default: return -1;
    }
}

int check_op(int n, const aqsg_op& op) {
    const int* q = op.qubits;
    auto oob = [n](int x) { return x < 0 || x >= n; };
    switch (op.kind) {
        case AQSG_OP_BARRIER: break;
        case AQSG_OP_X: case AQSG_OP_Y: case AQSG_OP_Z: case AQSG_OP_H:
        case AQSG_OP_PHASE: case AQSG_OP_RX: case AQSG_OP_RY: case AQSG_OP_RZ:
            // X::check quantum.cpp:533-538 (same for Y, Z, H, Phase, RotX/Y/Z)
            if (oob(q[0])) return set_error(AQSG_ERR_OUT_OF_RANGE, kAt);
            break;
        case AQSG_OP_SWAP:  // quantum.cpp:898-910
            if (n < 2) return set_error(AQSG_ERR_DOMAIN, "Gate not supported for given simulation");
            if (oob(q[0]) || oob(q[1])) return set_error(AQSG_ERR_OUT_OF_RANGE, kAt);
            if (q[0] == q[1]) return set_error(AQSG_ERR_INVALID_ARGUMENT, kSwapSame);
            break;
        case AQSG_OP_CX: case AQSG_OP_CY: case AQSG_OP_CZ: case AQSG_OP_CH:
        case AQSG_OP_CPHASE:  // CX::check quantum.cpp:965-977
            if (n < 2) return set_error(AQSG_ERR_DOMAIN, "Gate not supported for given simulation");
            if (oob(q[0]) || oob(q[1])) return set_error(AQSG_ERR_OUT_OF_RANGE, kAt);
            if (q[0] == q[1]) return set_error(AQSG_ERR_INVALID_ARGUMENT, kCtlTgt);
            break;
        case AQSG_OP_CRX: case AQSG_OP_CRY: case AQSG_OP_CRZ:  // quantum.cpp:1413-1422
            if (oob(q[0]) || oob(q[1])) return set_error(AQSG_ERR_OUT_OF_RANGE, kAt);
            if (q[0] == q[1]) return set_error(AQSG_ERR_INVALID_ARGUMENT, kCtlTgt);
            break;
        case AQSG_OP_CSWAP:  // quantum.cpp:1245-1263
            if (n < 3) return set_error(AQSG_ERR_DOMAIN, "Gate not supported for given circuit");
            if (oob(q[1]) || oob(q[2]) || oob(q[0])) return set_error(AQSG_ERR_OUT_OF_RANGE, kAt);
            if (q[0] == q[1] || q[0] == q[2]) return set_error(AQSG_ERR_INVALID_ARGUMENT, kCtlTgt);
            if (q[1] == q[2]) return set_error(AQSG_ERR_INVALID_ARGUMENT, kSwapSame);
            break;
        case AQSG_OP_CCX: case AQSG_OP_OR:  // quantum.cpp:1524-1540, 1596-1612
            if (n < 3) return set_error(AQSG_ERR_DOMAIN, "Gate not supported for given simulation");
            if (oob(q[0]) || oob(q[1]) || oob(q[2])) return set_error(AQSG_ERR_OUT_OF_RANGE, kAt);
            if (q[0] == q[2] || q[1] == q[2]) return set_error(AQSG_ERR_INVALID_ARGUMENT, kCtlTgt);
            break;
        case AQSG_OP_UNITARY: {
            int k = op.num_qubits;
            if (k < 1 || k > AQSG_MAX_UNITARY_QUBITS)
                return set_error(AQSG_ERR_INVALID_ARGUMENT,
                                 "Unitary gate must act on 1 to 5 qubits");
            if (!op.matrix) return set_error(AQSG_ERR_NULL, "Unitary gate has no matrix");
            if (k > n) return set_error(AQSG_ERR_INVALID_ARGUMENT,
                                        "Cannot add a bigger gate to the circuit");
            for (int i = 0; i < k; ++i) {
                if (oob(q[i])) return set_error(AQSG_ERR_OUT_OF_RANGE, kAt);
                for (int j = 0; j < i; ++j)
                    if (q[i] == q[j])
                        return set_error(AQSG_ERR_INVALID_ARGUMENT,
                                         "Unitary gate targets must be distinct");
            }
            break;
        }
        default:
            return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown gate kind " + std::to_string(op.kind));
    }
    if (op.num_controls < 0 || op.num_controls > AQSG_OP_MAX_CONTROLS)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Too many control qubits");
    if (op.num_controls > 0) {
        int na = op.kind == AQSG_OP_UNITARY ? op.num_qubits : op_arity(op.kind);
        for (int i = 0; i < op.num_controls; ++i) {
            int c = op.controls[i];
            // ControlGate::check, quantum.cpp:1871-1886
            if (oob(c)) return set_error(AQSG_ERR_OUT_OF_RANGE,
                                         "Control qubit must be inside the circuit qubit range");
            for (int j = 0; j < na; ++j)
                if (q[j] == c)
                    return set_error(AQSG_ERR_OUT_OF_RANGE,
                                     "Control qubit cannot be one of the target qubits of the gate");
            for (int j = 0; j < i; ++j)
                if (op.controls[j] == c)
                    return set_error(AQSG_ERR_INVALID_ARGUMENT, "Control qubits must be distinct");
        }
    }
    return AQSG_OK;
}

// Coefficients of the reference's gate matrices.  For c64 they are computed in
// float as src/quantum.cpp does (std::cos(angle / 2.0f) on a float, the
// literal 0.70710678118f for H, quantum.cpp:46-49); for c128 in double.
struct Coef {
    double c2, s2, c1, s1, h;
};

static Coef coefs(int dtype, float angle) {
    Coef c;
    if (dtype == AQSG_C64) {
        c.c2 = std::cos(angle / 2.0f);
        c.s2 = std::sin(angle / 2.0f);
        c.c1 = std::cos(angle);
        c.s1 = std::sin(angle);
        c.h = 0.70710678118f;
    } else {
        double a = (double)angle;
        c.c2 = std::cos(a / 2.0);
        c.s2 = std::sin(a / 2.0);
        c.c1 = std::cos(a);
        c.s1 = std::sin(a);
        c.h = 0.70710678118654752440;
    }
    return c;
}

static void set2(LOp* o, double a, double ai, double b, double bi, double c, double ci,
                 double d, double di) {
    o->m[0] = a; o->m[1] = ai; o->m[2] = b; o->m[3] = bi;
    o->m[4] = c; o->m[5] = ci; o->m[6] = d; o->m[7] = di;
}

int lower_op(int n, int dtype, const aqsg_op& op, LOp* o) {
    *o = LOp();
    const int* q = op.qubits;
    auto bit = [n](int qq) { return n - 1 - qq; };
    auto bm = [n](int qq) { return 1ull << (n - 1 - qq); };
    const Coef cf = coefs(dtype, op.angle);
    int base = op.kind;
    uint64_t cm = 0;
    int t = -1;
    switch (op.kind) {
        case AQSG_OP_BARRIER: o->cls = L_NOP; return AQSG_OK;
        case AQSG_OP_X: case AQSG_OP_Y: case AQSG_OP_Z: case AQSG_OP_H:
        case AQSG_OP_PHASE: case AQSG_OP_RX: case AQSG_OP_RY: case AQSG_OP_RZ:
            t = q[0]; break;
        case AQSG_OP_SWAP: break;
        case AQSG_OP_CX: base = AQSG_OP_X; cm = bm(q[0]); t = q[1]; break;
        case AQSG_OP_CY: base = AQSG_OP_Y; cm = bm(q[0]); t = q[1]; break;
        case AQSG_OP_CZ: base = AQSG_OP_Z; cm = bm(q[0]); t = q[1]; break;
        case AQSG_OP_CH: base = AQSG_OP_H; cm = bm(q[0]); t = q[1]; break;
        case AQSG_OP_CPHASE: base = AQSG_OP_PHASE; cm = bm(q[0]); t = q[1]; break;
        case AQSG_OP_CRX: base = AQSG_OP_RX; cm = bm(q[0]); t = q[1]; break;
        case AQSG_OP_CRY: base = AQSG_OP_RY; cm = bm(q[0]); t = q[1]; break;
        case AQSG_OP_CRZ: base = AQSG_OP_RZ; cm = bm(q[0]); t = q[1]; break;
        case AQSG_OP_CSWAP: base = AQSG_OP_SWAP; cm = bm(q[0]); break;
        case AQSG_OP_CCX: base = AQSG_OP_X; cm = bm(q[0]) | bm(q[1]); t = q[2]; break;
        case AQSG_OP_OR: base = AQSG_OP_OR; t = q[2]; break;
        case AQSG_OP_UNITARY: break;
        default: return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown gate kind");
    }
    uint64_t cval = cm;
    for (int i = 0; i < op.num_controls; ++i) {
        uint64_t b = bm(op.controls[i]);
        cm |= b;
        if ((op.control_values >> i) & 1u) cval |= b;
    }
    o->cmask = cm;
    o->cval = cval;

    if (op.kind == AQSG_OP_UNITARY) {
        const int k = op.num_qubits, dim = 1 << k;
        if (k == 1) {
            o->cls = L_MAT2;
            o->t0 = bit(q[0]);
            for (int e = 0; e < 8; ++e)
                o->m[e] = dtype == AQSG_C64 ? (double)(float)op.matrix[e] : op.matrix[e];
            return AQSG_OK;
        }
        o->cls = L_MATK;
        o->k = k;
        for (int j = 0; j < k; ++j) o->tb[j] = bit(q[j]);
        o->mk.resize(2 * dim * dim);
        for (int e = 0; e < 2 * dim * dim; ++e)
            o->mk[e] = dtype == AQSG_C64 ? (double)(float)op.matrix[e] : op.matrix[e];
        return AQSG_OK;
    }
    if (base == AQSG_OP_SWAP) {
        int a = op.kind == AQSG_OP_SWAP ? q[0] : q[1];
        int b = op.kind == AQSG_OP_SWAP ? q[1] : q[2];
        o->cls = L_PERM_SWAP;
        o->t0 = bit(a);
        o->t1 = bit(b);
        return AQSG_OK;
    }
    o->t0 = bit(t);
    switch (base) {
        case AQSG_OP_X: o->cls = L_PERM_X; break;
        case AQSG_OP_OR:
            o->cls = L_PERM_OR;
            o->amask = bm(q[0]) | bm(q[1]);
            break;
        case AQSG_OP_Y: o->cls = L_MAT2; set2(o, 0, 0, 0, -1, 0, 1, 0, 0); break;
        case AQSG_OP_Z:
            o->cls = L_DIAG1;
            o->m[0] = -1; o->m[1] = 0;
            break;
        case AQSG_OP_PHASE:
            o->cls = L_DIAG1;
            o->m[0] = cf.c1; o->m[1] = cf.s1;
            break;
        case AQSG_OP_H: o->cls = L_MAT2; set2(o, cf.h, 0, cf.h, 0, cf.h, 0, -cf.h, 0); break;
        case AQSG_OP_RX: o->cls = L_MAT2; set2(o, cf.c2, 0, 0, -cf.s2, 0, -cf.s2, cf.c2, 0); break;
        case AQSG_OP_RY: o->cls = L_MAT2; set2(o, cf.c2, 0, -cf.s2, 0, cf.s2, 0, cf.c2, 0); break;
        case AQSG_OP_RZ:
            o->cls = L_DIAG2;
            o->m[0] = cf.c2; o->m[1] = -cf.s2; o->m[2] = cf.c2; o->m[3] = cf.s2;
            break;
        default: return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown gate kind");
    }
    if (o->cls == L_DIAG1) {
        // the phase applies where the target bit is 1 and the controls hold
        o->cmask |= 1ull << o->t0;
        o->cval |= 1ull << o->t0;
    }
    return AQSG_OK;
}

static int check_state(aqsg_state st) {
    if (!st || !st->d) return set_error(AQSG_ERR_NULL, "NULL state");
    return AQSG_OK;
}

}  // namespace aqsg

using namespace aqsg;

extern "C" {

int aqsg_version(void) { return AQSG_VERSION_MAJOR * 100 + AQSG_VERSION_MINOR; }

size_t aqsg_last_error(char* buf, size_t len) {
    const std::string& e = g_last_error;
    if (buf && len > 0) {
        size_t c = e.size() < len - 1 ? e.size() : len - 1;
        memcpy(buf, e.data(), c);
        buf[c] = 0;
    }
    return e.size();
}

int aqsg_init(int device, aqsg_ctx* out) {
    if (!out) return set_error(AQSG_ERR_NULL, "NULL output handle");
    *out = nullptr;
    int count = 0;
    AQSG_CUDA_TRY(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count)
        return set_error(AQSG_ERR_OUT_OF_RANGE, "No CUDA device " + std::to_string(device));
    AQSG_ON_DEVICE(device);
    auto* c = new aqsg_ctx_s();
    c->device = device;
    cudaError_t e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&c->host_result, 4096);
    if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_err, 256);
    if (e == cudaSuccess) e = cudaMemset(c->d_err, 0, 256);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->order, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        if (c->order) cudaEventDestroy(c->order);
        if (c->d_err) cudaFree(c->d_err);
        if (c->host_result) cudaFreeHost(c->host_result);
        if (c->stream) cudaStreamDestroy(c->stream);
        delete c;
        return cuda_error(e, "aqsg_init");
    }
    // the allocation-free sampler's static scratch becomes resident on this
    // device now, not inside a caller's loop (lazy module loading)
    if (int rc = noalloc_prepare(device)) {
        cudaEventDestroy(c->order);
        cudaFree(c->d_err);
        cudaFreeHost(c->host_result);
        cudaStreamDestroy(c->stream);
        delete c;
        return rc;
    }
    *out = c;
    return AQSG_OK;
}

int aqsg_shutdown(aqsg_ctx ctx) {
    if (!ctx) return set_error(AQSG_ERR_NULL, "NULL context");
    if (ctx->live_states != 0)
        return set_error(AQSG_ERR_RUNTIME, "Context still owns live states");
    DeviceScope scope(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    Scratch* all[] = {&ctx->partial, &ctx->tcnorm, &ctx->prefix, &ctx->sample_u, &ctx->sample_o,
                      &ctx->ops, &ctx->probs};
    for (Scratch* s : all)
        if (s->ptr) cudaFree(s->ptr);
    if (ctx->host_result) cudaFreeHost(ctx->host_result);
    if (ctx->d_err) cudaFree(ctx->d_err);
    if (ctx->order) cudaEventDestroy(ctx->order);
    plan_cache_free(ctx);
    cudaStreamDestroy(ctx->stream);
    autotune_forget(ctx);
    delete ctx;
    return AQSG_OK;
}

int aqsg_set_exec_mode(aqsg_ctx ctx, int mode) {
    if (!ctx) return set_error(AQSG_ERR_NULL, "NULL context");
    if (mode < AQSG_EXEC_AUTO || mode > AQSG_EXEC_TILED)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown execution mode");
    ctx->exec_mode = mode;
    return AQSG_OK;
}

int aqsg_set_tensor_cores(aqsg_ctx ctx, int enable) {
    if (!ctx) return set_error(AQSG_ERR_NULL, "NULL context");
    ctx->tensor_cores = enable ? 1 : 0;
    return AQSG_OK;
}

int aqsg_set_whole_tile_max(aqsg_ctx ctx, int qubits) {
    if (!ctx) return set_error(AQSG_ERR_NULL, "NULL context");
    if (qubits < 0) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Negative whole-tile qubit count");
    ctx->whole_tile_max = qubits;
    return AQSG_OK;
}

int aqsg_synchronize(aqsg_ctx ctx) {
    if (!ctx) return set_error(AQSG_ERR_NULL, "NULL context");
    AQSG_ON_DEVICE(ctx->device);
    AQSG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return AQSG_OK;
}

int aqsg_ctx_after(aqsg_ctx ctx, aqsg_ctx other) {
    if (!ctx || !other) return set_error(AQSG_ERR_NULL, "NULL context");
    if (ctx == other) return AQSG_OK;  // a stream is already ordered with itself
    if (ctx->device != other->device)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Contexts on different devices");
    AQSG_ON_DEVICE(ctx->device);
    AQSG_CUDA_TRY(cudaEventRecord(other->order, other->stream));
    AQSG_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, other->order, 0));
    return AQSG_OK;
}

int aqsg_debug_ctx_scratch(aqsg_ctx ctx, size_t* bytes, int capacity, int* count) {
    if (!ctx || !count) return set_error(AQSG_ERR_NULL, "NULL argument");
    const Scratch* all[] = {&ctx->partial, &ctx->tcnorm, &ctx->prefix, &ctx->sample_u,
                            &ctx->sample_o,  &ctx->ops,    &ctx->probs};
    *count = 6;
    for (int i = 0; i < 6 && i < capacity && bytes; ++i) bytes[i] = all[i]->ptr ? all[i]->bytes : 0;
    return AQSG_OK;
}

int aqsg_ctx_stream(aqsg_ctx ctx, void** stream) {
    if (!ctx || !stream) return set_error(AQSG_ERR_NULL, "NULL argument");
    *stream = (void*)ctx->stream;
    return AQSG_OK;
}

int aqsg_launch_count(aqsg_ctx ctx, uint64_t* out) {
    if (!ctx || !out) return set_error(AQSG_ERR_NULL, "NULL argument");
    *out = ctx->launches;
    return AQSG_OK;
}

int aqsg_state_alloc(aqsg_ctx ctx, int n, int dtype, aqsg_state* out) {
    if (!ctx || !out) return set_error(AQSG_ERR_NULL, "NULL argument");
    *out = nullptr;
    if (n < 1) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Circuit must contain at least 1 qubit");
    if (n > AQSG_MAX_QUBITS)
        return set_error(AQSG_ERR_INVALID_ARGUMENT,
                         "Maximum qubit count supported is " + std::to_string(AQSG_MAX_QUBITS));
    if (dtype != AQSG_C64 && dtype != AQSG_C128)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown dtype");
    AQSG_ON_DEVICE(ctx->device);
    auto* s = new aqsg_state_s();
    s->ctx = ctx;
    s->n = n;
    s->dtype = dtype;
    s->amps = 1ull << n;
    cudaError_t e = cudaMalloc(&s->d, s->amps * amp_bytes(dtype));
    if (e != cudaSuccess) {
        delete s;
        return cuda_error(e, "aqsg_state_alloc");
    }
    ctx->live_states++;
    *out = s;
    return AQSG_OK;
}

int aqsg_state_free(aqsg_state st) {
    if (!st) return set_error(AQSG_ERR_NULL, "NULL state");
    DeviceScope scope(st->ctx->device);
    cudaStreamSynchronize(st->ctx->stream);
    if (st->d) cudaFree(st->d);
    st->ctx->live_states--;
    delete st;
    return AQSG_OK;
}

int aqsg_state_info(aqsg_state st, int* n, int* dtype) {
    if (int rc = check_state(st)) return rc;
    if (n) *n = st->n;
    if (dtype) *dtype = st->dtype;
    return AQSG_OK;
}

int aqsg_state_set_basis_index(aqsg_state st, uint64_t k) {
    if (int rc = check_state(st)) return rc;
    AQSG_ON_DEVICE(st->ctx->device);
    if (k >= st->amps) return set_error(AQSG_ERR_OUT_OF_RANGE, "Basis index out of range");
    return launch_set_basis(st, k);
}

int aqsg_state_set_product(aqsg_state st, const float* amps) {
    if (int rc = check_state(st)) return rc;
    AQSG_ON_DEVICE(st->ctx->device);
    if (!amps) return set_error(AQSG_ERR_NULL, "NULL qubit amplitudes");
    return launch_set_product(st, amps);
}

int aqsg_state_upload(aqsg_state st, const void* host, int normalize) {
    if (int rc = check_state(st)) return rc;
    AQSG_ON_DEVICE(st->ctx->device);
    if (!host) return set_error(AQSG_ERR_NULL, "NULL host buffer");
    AQSG_CUDA_TRY(cudaMemcpyAsync(st->d, host, st->amps * amp_bytes(st->dtype),
                                  cudaMemcpyHostToDevice, st->ctx->stream));
    if (normalize) {
        double s = 0;
        if (int rc = reduce_prob(st, 0, 0, &s)) return rc;
        if (!(s > 0.0)) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Cannot have a null statevector");
        if (int rc = launch_scale(st, 1.0 / std::sqrt(s))) return rc;
    }
    return AQSG_OK;
}

int aqsg_state_download(aqsg_state st, void* host) {
    if (int rc = check_state(st)) return rc;
    AQSG_ON_DEVICE(st->ctx->device);
    if (!host) return set_error(AQSG_ERR_NULL, "NULL host buffer");
    AQSG_CUDA_TRY(cudaMemcpyAsync(host, st->d, st->amps * amp_bytes(st->dtype),
                                  cudaMemcpyDeviceToHost, st->ctx->stream));
    AQSG_CUDA_TRY(cudaStreamSynchronize(st->ctx->stream));
    return AQSG_OK;
}

int aqsg_state_download_async(aqsg_state st, void* host) {
    if (int rc = check_state(st)) return rc;
    AQSG_ON_DEVICE(st->ctx->device);
    if (!host) return set_error(AQSG_ERR_NULL, "NULL host buffer");
    AQSG_CUDA_TRY(cudaMemcpyAsync(host, st->d, st->amps * amp_bytes(st->dtype),
                                  cudaMemcpyDeviceToHost, st->ctx->stream));
    return AQSG_OK;
}

int aqsg_state_download_range(aqsg_state st, uint64_t begin, uint64_t count, void* host) {
    if (int rc = check_state(st)) return rc;
    AQSG_ON_DEVICE(st->ctx->device);
    if (!host) return set_error(AQSG_ERR_NULL, "NULL host buffer");
    if (begin > st->amps || count > st->amps - begin)
        return set_error(AQSG_ERR_OUT_OF_RANGE, "Range outside the register");
    const size_t b = amp_bytes(st->dtype);
    AQSG_CUDA_TRY(cudaMemcpyAsync(host, (char*)st->d + begin * b, count * b,
                                  cudaMemcpyDeviceToHost, st->ctx->stream));
    AQSG_CUDA_TRY(cudaStreamSynchronize(st->ctx->stream));
    return AQSG_OK;
}

int aqsg_state_copy(aqsg_state dst, aqsg_state src) {
    if (int rc = check_state(dst)) return rc;
    if (int rc = check_state(src)) return rc;
    if (dst->n != src->n || dst->dtype != src->dtype)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Registers differ in size or dtype");
    AQSG_ON_DEVICE(src->ctx->device);
    AQSG_CUDA_TRY(cudaMemcpyAsync(dst->d, src->d, src->amps * amp_bytes(src->dtype),
                                  cudaMemcpyDeviceToDevice, src->ctx->stream));
    if (dst->ctx != src->ctx) AQSG_CUDA_TRY(cudaStreamSynchronize(src->ctx->stream));
    return AQSG_OK;
}

int aqsg_check_ops(int n, const aqsg_op* ops, int count) {
    if (count < 0) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Negative op count");
    if (count > 0 && !ops) return set_error(AQSG_ERR_NULL, "NULL op list");
    for (int i = 0; i < count; ++i)
        if (int rc = check_op(n, ops[i])) return rc;
    return AQSG_OK;
}

// Bytes that determine the tile plan of ops on a register of st's shape:
// the ops (matrix pointers replaced by the matrices' contents) and the
// settings the encoding depends on.
static std::vector<unsigned char> plan_key(const aqsg_state_s* st, const aqsg_op* ops, int count) {
    std::vector<unsigned char> k;
    const int32_t head[4] = {'A', st->n, st->dtype, st->ctx->tensor_cores};
    k.insert(k.end(), (const unsigned char*)head, (const unsigned char*)head + sizeof(head));
    for (int i = 0; i < count; ++i) {
        aqsg_op o = ops[i];
        o.matrix = nullptr;
        k.insert(k.end(), (const unsigned char*)&o, (const unsigned char*)&o + sizeof(o));
        if (ops[i].kind == AQSG_OP_UNITARY && ops[i].matrix) {
            const size_t d = (size_t)1 << ops[i].num_qubits;
            k.insert(k.end(), (const unsigned char*)ops[i].matrix,
                     (const unsigned char*)(ops[i].matrix + 2 * d * d));
        }
    }
    return k;
}

int aqsg_apply_ops(aqsg_state st, const aqsg_op* ops, int count, int mode) {
    if (int rc = check_state(st)) return rc;
    if (mode < 0) mode = st->ctx->exec_mode;
    if (mode < AQSG_EXEC_AUTO || mode > AQSG_EXEC_TILED)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown execution mode");
    if (mode != AQSG_EXEC_PER_GATE) {
        if (count > 0 && !ops) return set_error(AQSG_ERR_NULL, "NULL op list");
        if (count < 0) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Negative op count");
        AQSG_ON_DEVICE(st->ctx->device);
        // a circuit run before on this context reuses its checked, lowered,
        // encoded and uploaded plan
        return run_tiled_cached(st, plan_key(st, ops, count), [&](std::vector<LOp>* low) {
            if (int rc = aqsg_check_ops(st->n, ops, count)) return rc;
            low->reserve(count);
            for (int i = 0; i < count; ++i) {
                LOp o;
                if (int rc = lower_op(st->n, st->dtype, ops[i], &o)) return rc;
                if (o.cls != L_NOP) low->push_back(std::move(o));
            }
            return (int)AQSG_OK;
        });
    }
    if (int rc = aqsg_check_ops(st->n, ops, count)) return rc;
    std::vector<LOp> low;
    low.reserve(count);
    for (int i = 0; i < count; ++i) {
        LOp o;
        if (int rc = lower_op(st->n, st->dtype, ops[i], &o)) return rc;
        if (o.cls != L_NOP) low.push_back(std::move(o));
    }
    AQSG_ON_DEVICE(st->ctx->device);
    for (const LOp& o : low)
        if (int rc = launch_lop(st, o)) return rc;
    return AQSG_OK;
}

int aqsg_qubit_prob(aqsg_state st, int qubit, double* out) {
    if (int rc = check_state(st)) return rc;
    AQSG_ON_DEVICE(st->ctx->device);
    if (!out) return set_error(AQSG_ERR_NULL, "NULL output");
    if (qubit < 0 || qubit >= st->n)
        return set_error(AQSG_ERR_OUT_OF_RANGE, "Cannot obtain probability of the given qubit");
    uint64_t m = 1ull << (st->n - 1 - qubit);
    return reduce_prob(st, m, m, out);
}

int aqsg_state_prob(aqsg_state st, uint64_t k, double* out) {
    if (int rc = check_state(st)) return rc;
    if (!out) return set_error(AQSG_ERR_NULL, "NULL output");
    if (k >= st->amps) return set_error(AQSG_ERR_OUT_OF_RANGE, "Cannot obtain probability of the given state");
    if (st->dtype == AQSG_C64) {
        float a[2];
        if (int rc = aqsg_state_download_range(st, k, 1, a)) return rc;
        *out = (double)a[0] * a[0] + (double)a[1] * a[1];
    } else {
        double a[2];
        if (int rc = aqsg_state_download_range(st, k, 1, a)) return rc;
        *out = a[0] * a[0] + a[1] * a[1];
    }
    return AQSG_OK;
}

int aqsg_probs(aqsg_state st, void* host, int out_dtype) {
    if (int rc = check_state(st)) return rc;
    AQSG_ON_DEVICE(st->ctx->device);
    if (!host) return set_error(AQSG_ERR_NULL, "NULL host buffer");
    if (out_dtype != 0 && out_dtype != 1)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "out_dtype must be 0 (float) or 1 (double)");
    const size_t bytes = st->amps * (out_dtype ? 8 : 4);
    if (int rc = ensure_scratch(st->ctx->probs, bytes)) return rc;
    if (int rc = launch_probs(st, st->ctx->probs.ptr, out_dtype)) return rc;
    AQSG_CUDA_TRY(cudaMemcpyAsync(host, st->ctx->probs.ptr, bytes, cudaMemcpyDeviceToHost,
                                  st->ctx->stream));
    AQSG_CUDA_TRY(cudaStreamSynchronize(st->ctx->stream));
    return AQSG_OK;
}

int aqsg_norm2(aqsg_state st, double* out) {
    if (int rc = check_state(st)) return rc;
    AQSG_ON_DEVICE(st->ctx->device);
    if (!out) return set_error(AQSG_ERR_NULL, "NULL output");
    return reduce_prob(st, 0, 0, out);
}

int aqsg_sample(aqsg_state st, const double* u, uint64_t count, int rule, uint64_t* out) {
    if (int rc = check_state(st)) return rc;
    AQSG_ON_DEVICE(st->ctx->device);
    if (count == 0) return AQSG_OK;
    if (!u || !out) return set_error(AQSG_ERR_NULL, "NULL buffer");
    if (rule != AQSG_SAMPLE_REFERENCE && rule != AQSG_SAMPLE_CLAMP)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown sampling rule");
    return sample(st, u, 0, false, count, rule, out);
}

int aqsg_sample_seeded(aqsg_state st, uint64_t seed, uint64_t count, int rule, uint64_t* out) {
    if (int rc = check_state(st)) return rc;
    AQSG_ON_DEVICE(st->ctx->device);
    if (count == 0) return AQSG_OK;
    if (!out) return set_error(AQSG_ERR_NULL, "NULL buffer");
    if (rule != AQSG_SAMPLE_REFERENCE && rule != AQSG_SAMPLE_CLAMP)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown sampling rule");
    return sample(st, nullptr, seed, true, count, rule, out);
}

int aqsg_collapse_qubit(aqsg_state st, int qubit, double u, int* outcome, double* prob) {
    if (int rc = check_state(st)) return rc;
    AQSG_ON_DEVICE(st->ctx->device);
    if (qubit < 0 || qubit >= st->n)
        return set_error(AQSG_ERR_OUT_OF_RANGE, "Cannot measure the state of the given qubit");
    uint64_t m = 1ull << (st->n - 1 - qubit);
    double p1 = 0;
    if (int rc = reduce_prob(st, m, m, &p1)) return rc;
    // quantum.cpp:333-339: outcome 1 when u < p1; renormalise the kept branch
    int r = u < p1 ? 1 : 0;
    double p = r ? p1 : 1.0 - p1;
    double scale = p > 0 ? 1.0 / std::sqrt(p) : 0.0;
    if (int rc = launch_collapse_qubit(st, m, r, scale)) return rc;
    if (outcome) *outcome = r;
    if (prob) *prob = p;
    return AQSG_OK;
}

int aqsg_collapse_all(aqsg_state st, double u, uint64_t* outcome) {
    if (int rc = check_state(st)) return rc;
    AQSG_ON_DEVICE(st->ctx->device);
    uint64_t k = 0;
    if (int rc = sample(st, &u, 0, false, 1, AQSG_SAMPLE_REFERENCE, &k)) return rc;
    if (int rc = launch_set_basis(st, k)) return rc;
    if (outcome) *outcome = k;
    return AQSG_OK;
}

int aqsg_expect_z(aqsg_state st, double* z, double* zz) {
    if (int rc = check_state(st)) return rc;
    AQSG_ON_DEVICE(st->ctx->device);
    return expect_z(st, z, zz);
}

}  // extern "C"
