/*
 * aqs_oracle.c — CPU oracle for the GB300 state-vector engine.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py (results are compared with it; the
 * CPU-baseline leg times it as the CPU arm).  The product never links it.
 *
 * Built with -ffp-contract=off so x86-64 and aarch64 hosts round alike.
 * See aqs_oracle.h for what each family restates.
 */
#include "aqs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* H entries of the reference (src/quantum.cpp:46-49) */
#define REF_H_F32 0.70710678118f

static int g_threads = 0;

void orc_set_threads(int threads) {
    g_threads = threads;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
}

int orc_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* per-gate oracle                                                          */
/* ------------------------------------------------------------------------ */

typedef struct orc_gate {
    int k;             /* target count, matrix is 2^k x 2^k; 0 = no-op      */
    int tbit[AQSG_MAX_UNITARY_QUBITS];
    uint64_t cmask;    /* all-of condition: (i & cmask) == cval             */
    uint64_t cval;
    uint64_t amask;    /* any-of condition (Or gate): (i & amask) != 0      */
    double m[2 * 32 * 32];
} orc_gate;

static inline uint64_t qbit(int n, int q) { return 1ull << (n - 1 - q); }

static void set_m(orc_gate* g, int r, int c, double re, double im) {
    int dim = 1 << g->k;
    g->m[2 * (r * dim + c)] = re;
    g->m[2 * (r * dim + c) + 1] = im;
}

static void set_2x2(orc_gate* g, double a_re, double a_im, double b_re,
                    double b_im, double c_re, double c_im, double d_re,
                    double d_im) {
    set_m(g, 0, 0, a_re, a_im);
    set_m(g, 0, 1, b_re, b_im);
    set_m(g, 1, 0, c_re, c_im);
    set_m(g, 1, 1, d_re, d_im);
}

/* Mathematical matrix of each gate.  p32 != 0 computes the coefficients in
 * float the way src/quantum.cpp does (std::cos(angle / 2.0f) on a float,
 * 0.70710678118f for H); p32 == 0 computes them in double from the float
 * angle. */
static int build_gate(const aqsg_op* op, int n, int p32, orc_gate* g) {
    memset(g, 0, sizeof(*g));
    const int* q = op->qubits;
    double c2, s2, c1, s1;
    if (p32) {
        float a = op->angle;
        c2 = (double)cosf(a / 2.0f);
        s2 = (double)sinf(a / 2.0f);
        c1 = (double)cosf(a);
        s1 = (double)sinf(a);
    } else {
        double a = (double)op->angle;
        c2 = cos(a / 2.0);
        s2 = sin(a / 2.0);
        c1 = cos(a);
        s1 = sin(a);
    }
    const double h = p32 ? (double)REF_H_F32 : 0.70710678118654752440;
    int base = op->kind;
    int ctrl0 = -1, ctrl1 = -1, t0 = -1, t1 = -1;
    switch (op->kind) {
        case AQSG_OP_BARRIER: g->k = 0; return 0;
        case AQSG_OP_X: case AQSG_OP_Y: case AQSG_OP_Z: case AQSG_OP_H:
        case AQSG_OP_PHASE: case AQSG_OP_RX: case AQSG_OP_RY: case AQSG_OP_RZ:
            t0 = q[0];
            break;
        case AQSG_OP_SWAP: t0 = q[0]; t1 = q[1]; break;
        case AQSG_OP_CX: base = AQSG_OP_X; ctrl0 = q[0]; t0 = q[1]; break;
        case AQSG_OP_CY: base = AQSG_OP_Y; ctrl0 = q[0]; t0 = q[1]; break;
        case AQSG_OP_CZ: base = AQSG_OP_Z; ctrl0 = q[0]; t0 = q[1]; break;
        case AQSG_OP_CH: base = AQSG_OP_H; ctrl0 = q[0]; t0 = q[1]; break;
        case AQSG_OP_CPHASE: base = AQSG_OP_PHASE; ctrl0 = q[0]; t0 = q[1]; break;
        case AQSG_OP_CRX: base = AQSG_OP_RX; ctrl0 = q[0]; t0 = q[1]; break;
        case AQSG_OP_CRY: base = AQSG_OP_RY; ctrl0 = q[0]; t0 = q[1]; break;
        case AQSG_OP_CRZ: base = AQSG_OP_RZ; ctrl0 = q[0]; t0 = q[1]; break;
        case AQSG_OP_CSWAP: base = AQSG_OP_SWAP; ctrl0 = q[0]; t0 = q[1]; t1 = q[2]; break;
        case AQSG_OP_CCX: base = AQSG_OP_X; ctrl0 = q[0]; ctrl1 = q[1]; t0 = q[2]; break;
        case AQSG_OP_OR: base = AQSG_OP_X; t0 = q[2];
            g->amask = qbit(n, q[0]) | qbit(n, q[1]);
            break;
        case AQSG_OP_UNITARY: break;
        default: return AQSG_ERR_INVALID_ARGUMENT;
    }
    if (ctrl0 >= 0) { g->cmask |= qbit(n, ctrl0); g->cval |= qbit(n, ctrl0); }
    if (ctrl1 >= 0) { g->cmask |= qbit(n, ctrl1); g->cval |= qbit(n, ctrl1); }
    for (int i = 0; i < op->num_controls; ++i) {
        uint64_t b = qbit(n, op->controls[i]);
        g->cmask |= b;
        if ((op->control_values >> i) & 1u) g->cval |= b;
    }
    if (op->kind == AQSG_OP_UNITARY) {
        g->k = op->num_qubits;
        int dim = 1 << g->k;
        for (int j = 0; j < g->k; ++j) g->tbit[j] = n - 1 - q[j];
        for (int e = 0; e < 2 * dim * dim; ++e)
            g->m[e] = p32 ? (double)(float)op->matrix[e] : op->matrix[e];
        return 0;
    }
    if (base == AQSG_OP_SWAP) {
        g->k = 2;
        g->tbit[0] = n - 1 - t0;
        g->tbit[1] = n - 1 - t1;
        set_m(g, 0, 0, 1, 0);
        set_m(g, 1, 2, 1, 0);
        set_m(g, 2, 1, 1, 0);
        set_m(g, 3, 3, 1, 0);
        return 0;
    }
    g->k = 1;
    g->tbit[0] = n - 1 - t0;
    switch (base) {
        case AQSG_OP_X: set_2x2(g, 0, 0, 1, 0, 1, 0, 0, 0); break;
        case AQSG_OP_Y: set_2x2(g, 0, 0, 0, -1, 0, 1, 0, 0); break;
        case AQSG_OP_Z: set_2x2(g, 1, 0, 0, 0, 0, 0, -1, 0); break;
        case AQSG_OP_H: set_2x2(g, h, 0, h, 0, h, 0, -h, 0); break;
        case AQSG_OP_PHASE: set_2x2(g, 1, 0, 0, 0, 0, 0, c1, s1); break;
        case AQSG_OP_RX: set_2x2(g, c2, 0, 0, -s2, 0, -s2, c2, 0); break;
        case AQSG_OP_RY: set_2x2(g, c2, 0, -s2, 0, s2, 0, c2, 0); break;
        case AQSG_OP_RZ: set_2x2(g, c2, -s2, 0, 0, 0, 0, c2, s2); break;
        default: return AQSG_ERR_INVALID_ARGUMENT;
    }
    return 0;
}

#define DEFINE_APPLY(T, SUFFIX)                                               \
    static void apply_gate_##SUFFIX(T* sv, int n, const orc_gate* g) {        \
        if (g->k == 0) return;                                                \
        const int64_t N = (int64_t)1 << n;                                    \
        const int k = g->k, dim = 1 << k;                                     \
        uint64_t tmask = 0, off[32];                                          \
        T m[2 * 32 * 32];                                                     \
        for (int j = 0; j < k; ++j) tmask |= 1ull << g->tbit[j];              \
        for (int r = 0; r < dim; ++r) {                                       \
            off[r] = 0;                                                       \
            for (int j = 0; j < k; ++j)                                       \
                if ((r >> (k - 1 - j)) & 1) off[r] |= 1ull << g->tbit[j];     \
        }                                                                     \
        for (int e = 0; e < 2 * dim * dim; ++e) m[e] = (T)g->m[e];            \
        _Pragma("omp parallel for schedule(static)")                          \
        for (int64_t b = 0; b < N; ++b) {                                     \
            const uint64_t base = (uint64_t)b;                                \
            if (base & tmask) continue;                                       \
            if ((base & g->cmask) != g->cval) continue;                       \
            if (g->amask && !(base & g->amask)) continue;                     \
            T vr[32], vi[32];                                                 \
            for (int r = 0; r < dim; ++r) {                                   \
                vr[r] = sv[2 * (base + off[r])];                              \
                vi[r] = sv[2 * (base + off[r]) + 1];                          \
            }                                                                 \
            for (int r = 0; r < dim; ++r) {                                   \
                T ar = 0, ai = 0;                                             \
                for (int c = 0; c < dim; ++c) {                               \
                    const T mr = m[2 * (r * dim + c)];                        \
                    const T mi = m[2 * (r * dim + c) + 1];                    \
                    ar += mr * vr[c] - mi * vi[c];                            \
                    ai += mr * vi[c] + mi * vr[c];                            \
                }                                                             \
                sv[2 * (base + off[r])] = ar;                                 \
                sv[2 * (base + off[r]) + 1] = ai;                             \
            }                                                                 \
        }                                                                     \
    }

DEFINE_APPLY(double, f64)
DEFINE_APPLY(float, f32)

int orc_apply_ops_f64(double* sv, int n, const aqsg_op* ops, int count) {
    orc_gate* g = (orc_gate*)malloc(sizeof(orc_gate));
    if (!g) return AQSG_ERR_OUT_OF_MEMORY;
    for (int i = 0; i < count; ++i) {
        int rc = build_gate(&ops[i], n, 0, g);
        if (rc) { free(g); return rc; }
        apply_gate_f64(sv, n, g);
    }
    free(g);
    return 0;
}

int orc_apply_ops_f32(float* sv, int n, const aqsg_op* ops, int count) {
    orc_gate* g = (orc_gate*)malloc(sizeof(orc_gate));
    if (!g) return AQSG_ERR_OUT_OF_MEMORY;
    for (int i = 0; i < count; ++i) {
        int rc = build_gate(&ops[i], n, 1, g);
        if (rc) { free(g); return rc; }
        apply_gate_f32(sv, n, g);
    }
    free(g);
    return 0;
}

void orc_probs_f64(const double* sv, int n, double* out) {
    const int64_t N = (int64_t)1 << n;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i)
        out[i] = sv[2 * i] * sv[2 * i] + sv[2 * i + 1] * sv[2 * i + 1];
}

void orc_probs_f32(const float* sv, int n, double* out) {
    const int64_t N = (int64_t)1 << n;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
        double re = sv[2 * i], im = sv[2 * i + 1];
        out[i] = re * re + im * im;
    }
}

int64_t orc_first_index(const double* p, int n, double u) {
    const int64_t N = (int64_t)1 << n;
    double acc = 0.0;
    for (int64_t i = 0; i < N; ++i) {
        acc += p[i];
        if (acc > u) return i;
    }
    return -1;
}

double orc_qubit_prob_f64(const double* sv, int n, int qubit) {
    const int64_t N = (int64_t)1 << n;
    const uint64_t m = qbit(n, qubit);
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t i = 0; i < N; ++i)
        if ((uint64_t)i & m) s += sv[2 * i] * sv[2 * i] + sv[2 * i + 1] * sv[2 * i + 1];
    return s;
}

/* ------------------------------------------------------------------------ */
/* faithful FP32 restatement of the reference algorithm                     */
/* ------------------------------------------------------------------------ */

typedef struct cf { float re, im; } cf;

static inline cf cmul(cf a, cf b) {
    cf r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static inline cf cadd(cf a, cf b) {
    cf r = {a.re + b.re, a.im + b.im};
    return r;
}
static const cf C1 = {1.f, 0.f};

int ref32_qstate_normalize(float* q) {
    /* QState::force_normalize, quantum.cpp:145-157 */
    float mag2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    if (mag2 == 0.f) return -1;
    float mag = sqrtf(mag2);
    for (int i = 0; i < 4; ++i) q[i] = q[i] / mag;
    return 0;
}

void ref32_product_state(int n, const float* q, float* sv) {
    /* generate_statevector, quantum.cpp:261-275: sv = q0; sv = sv (x) q_i.
     * tensor_product (utils.cpp:16-30, 169-194) multiplies the tiled right
     * operand by the resized left one: new[2a + b] = q_i[b] * sv[a]. */
    const int64_t N = (int64_t)1 << n;
    cf* cur = (cf*)sv;
    cur[0].re = q[0]; cur[0].im = q[1];
    cur[1].re = q[2]; cur[1].im = q[3];
    for (int i = 1; i < n; ++i) {
        const int64_t len = (int64_t)1 << i;
        cf b0 = {q[4 * i], q[4 * i + 1]}, b1 = {q[4 * i + 2], q[4 * i + 3]};
        for (int64_t a = len - 1; a >= 0; --a) {
            cf s = cur[a];
            cur[2 * a] = cmul(b0, s);
            cur[2 * a + 1] = cmul(b1, s);
        }
    }
    (void)N;
}

/* X (N x cols) <- G X for a dense N x N G (row-major complex). */
static void dense_apply(cf* x, int64_t N, int cols, const cf* G) {
    cf* y = (cf*)malloc(sizeof(cf) * (size_t)N * cols);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
        for (int c = 0; c < cols; ++c) {
            cf acc = {0.f, 0.f};
            for (int64_t j = 0; j < N; ++j)
                acc = cadd(acc, cmul(G[i * N + j], x[j * cols + c]));
            y[i * cols + c] = acc;
        }
    }
    memcpy(x, y, sizeof(cf) * (size_t)N * cols);
    free(y);
}

/* X <- S X for CSR S with `per_row` entries per row. */
static void csr_apply(cf* x, int64_t N, int cols, int per_row,
                      const int32_t* col, const cf* val) {
    cf* y = (cf*)malloc(sizeof(cf) * (size_t)N * cols);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
        for (int c = 0; c < cols; ++c) {
            cf acc = {0.f, 0.f};
            for (int e = 0; e < per_row; ++e) {
                int32_t j = col[i * per_row + e];
                if (j >= N) continue; /* unreachable: see CH below */
                cf t = cmul(val[i * per_row + e], x[(int64_t)j * cols + c]);
                acc = (e == 0) ? t : cadd(acc, t);
            }
            y[i * cols + c] = acc;
        }
    }
    memcpy(x, y, sizeof(cf) * (size_t)N * cols);
    free(y);
}

/* Dense I(2^t) (x) U (x) I(2^(n-t-1)) (RotX/RotY/RotZ/H, quantum.cpp:671-831) */
static cf* kron_1q(int n, int t, const cf U[4]) {
    const int64_t N = (int64_t)1 << n;
    cf* G = (cf*)calloc((size_t)N * N, sizeof(cf));
    const int64_t m = (int64_t)1 << (n - t - 1);
    for (int64_t i = 0; i < N; ++i) {
        int bi = (i & m) ? 1 : 0;
        int64_t j0 = i & ~m;
        G[i * N + j0] = U[bi * 2 + 0];
        G[i * N + (j0 | m)] = U[bi * 2 + 1];
    }
    return G;
}

/* Dense identity with U scattered onto the controlled subspace of the target
 * bits — the gate_matrix of Gate / ControlGate (quantum.cpp:1778-1806,
 * 1907-1943). */
static cf* scatter_dense(int n, int k, const int* tbit, uint64_t cmask,
                         uint64_t cval, const cf* U) {
    const int64_t N = (int64_t)1 << n;
    const int dim = 1 << k;
    cf* G = (cf*)calloc((size_t)N * N, sizeof(cf));
    uint64_t tmask = 0, off[32];
    for (int j = 0; j < k; ++j) tmask |= 1ull << tbit[j];
    for (int r = 0; r < dim; ++r) {
        off[r] = 0;
        for (int j = 0; j < k; ++j)
            if ((r >> (k - 1 - j)) & 1) off[r] |= 1ull << tbit[j];
    }
    for (int64_t i = 0; i < N; ++i) G[i * N + i] = C1;
    for (int64_t b = 0; b < N; ++b) {
        if ((uint64_t)b & tmask) continue;
        if (((uint64_t)b & cmask) != cval) continue;
        for (int r = 0; r < dim; ++r)
            for (int c = 0; c < dim; ++c)
                G[(b + off[r]) * N + (b + off[c])] = U[r * dim + c];
    }
    return G;
}

static int ref32_apply_one(cf* x, int n, int cols, const aqsg_op* op) {
    const int64_t N = (int64_t)1 << n;
    const int* q = op->qubits;
    const float a = op->angle;
    const float c2 = cosf(a / 2.0f), s2 = sinf(a / 2.0f);
    const cf ph = {cosf(a), sinf(a)};
    const float h = REF_H_F32;

    /* A gate with extra controls comes from ControlGate / NControl_Gate,
     * which the reference always lowers to a dense scatter of the compiled
     * sub-circuit (quantum.cpp:1888-1950).  The per-gate oracle builds that
     * sub-circuit's matrix. */
    if (op->num_controls > 0 || op->kind == AQSG_OP_UNITARY ||
        op->kind == AQSG_OP_CRX || op->kind == AQSG_OP_CRY ||
        op->kind == AQSG_OP_CRZ) {
        orc_gate* g = (orc_gate*)malloc(sizeof(orc_gate));
        int rc = build_gate(op, n, 1, g);
        if (rc) { free(g); return rc; }
        if (g->k == 0) { free(g); return 0; }
        if (g->amask) {
            /* Or with extra controls: fold into a dense permutation */
            cf* G = (cf*)calloc((size_t)N * N, sizeof(cf));
            uint64_t tm = 1ull << g->tbit[0];
            for (int64_t i = 0; i < N; ++i) {
                int fire = ((uint64_t)i & g->amask) && (((uint64_t)i & g->cmask) == g->cval);
                G[i * N + (fire ? (int64_t)((uint64_t)i ^ tm) : i)] = C1;
            }
            dense_apply(x, N, cols, G);
            free(G);
            free(g);
            return 0;
        }
        const int dim = 1 << g->k;
        cf U[32 * 32];
        for (int e = 0; e < dim * dim; ++e) {
            U[e].re = (float)g->m[2 * e];
            U[e].im = (float)g->m[2 * e + 1];
        }
        cf* G = scatter_dense(n, g->k, g->tbit, g->cmask, g->cval, U);
        dense_apply(x, N, cols, G);
        free(G);
        free(g);
        return 0;
    }

    const int32_t nn = n;
    switch (op->kind) {
        case AQSG_OP_BARRIER: return 0;
        case AQSG_OP_H: case AQSG_OP_RX: case AQSG_OP_RY: case AQSG_OP_RZ: {
            cf U[4];
            if (op->kind == AQSG_OP_H) {
                cf t[4] = {{h, 0}, {h, 0}, {h, 0}, {-h, 0}};
                memcpy(U, t, sizeof(U));
            } else if (op->kind == AQSG_OP_RX) {
                cf t[4] = {{c2, 0}, {0, -s2}, {0, -s2}, {c2, 0}};
                memcpy(U, t, sizeof(U));
            } else if (op->kind == AQSG_OP_RY) {
                cf t[4] = {{c2, 0}, {-s2, 0}, {s2, 0}, {c2, 0}};
                memcpy(U, t, sizeof(U));
            } else {
                cf t[4] = {{c2, -s2}, {0, 0}, {0, 0}, {c2, s2}};
                memcpy(U, t, sizeof(U));
            }
            cf* G = kron_1q(n, q[0], U);
            dense_apply(x, N, cols, G);
            free(G);
            return 0;
        }
        default: break;
    }

    /* CSR gates: one entry per row (two for CH), built as quantum.cpp does */
    const int per_row = (op->kind == AQSG_OP_CH) ? 2 : 1;
    int32_t* col = (int32_t*)malloc(sizeof(int32_t) * (size_t)N * per_row);
    cf* val = (cf*)malloc(sizeof(cf) * (size_t)N * per_row);
    for (int32_t i = 0; i < (int32_t)N; ++i) {
        int32_t c = i;
        cf v = C1;
        switch (op->kind) {
            case AQSG_OP_X: { /* :546-555 */
                int32_t m = 1 << (nn - q[0] - 1);
                c = i ^ m;
                break;
            }
            case AQSG_OP_Y: { /* :586-602 */
                int32_t m = 1 << (nn - q[0] - 1);
                c = i ^ m;
                v.re = 0.f; v.im = (i & m) ? 1.f : -1.f;
                break;
            }
            case AQSG_OP_Z: { /* :633-643 */
                int32_t m = 1 << (nn - q[0] - 1);
                v.re = (i & m) ? -1.f : 1.f; v.im = 0.f;
                break;
            }
            case AQSG_OP_PHASE: { /* :855-866 */
                int32_t m = 1 << (nn - q[0] - 1);
                if (i & m) v = ph;
                break;
            }
            case AQSG_OP_SWAP: { /* :925-938 */
                int32_t pa = nn - 1 - q[0], pb = nn - 1 - q[1];
                int32_t t = ((i >> pa) ^ (i >> pb)) & 1;
                c = i ^ ((t << pa) | (t << pb));
                break;
            }
            case AQSG_OP_CX: { /* :992-1002 */
                int32_t cm = 1 << (nn - 1 - q[0]), tm = 1 << (nn - 1 - q[1]);
                c = ((i ^ cm) & cm) ? i : (i ^ tm);
                break;
            }
            case AQSG_OP_CY: { /* :1054-1077 */
                int32_t cm = 1 << (nn - 1 - q[0]), tm = 1 << (nn - 1 - q[1]);
                int32_t mask = cm | tm, opi = i & mask;
                c = ((i ^ cm) & cm) ? i : (i ^ tm);
                if (opi == mask) { v.re = 0.f; v.im = 1.f; }
                if (opi == cm) { v.re = 0.f; v.im = -1.f; }
                break;
            }
            case AQSG_OP_CZ: { /* :1128-1141 */
                int32_t mask = (1 << (nn - 1 - q[0])) | (1 << (nn - 1 - q[1]));
                if ((i & mask) == mask) { v.re = -1.f; v.im = 0.f; }
                break;
            }
            case AQSG_OP_CPHASE: { /* :1192-1207 */
                int32_t mask = (1 << (nn - 1 - q[0])) | (1 << (nn - 1 - q[1]));
                if ((i & mask) == mask) v = ph;
                break;
            }
            case AQSG_OP_CSWAP: { /* :1284-1301 */
                int32_t pa = nn - 1 - q[1], pb = nn - 1 - q[2];
                int32_t ctl = 1 << (nn - q[0] - 1);
                int32_t t = ((i >> pa) ^ (i >> pb)) & 1;
                int32_t rv = i ^ ((t << pa) | (t << pb));
                c = ((i & ctl) == ctl) ? rv : i;
                break;
            }
            case AQSG_OP_CCX: { /* :1558-1568 */
                int32_t cm = (1 << (nn - 1 - q[0])) | (1 << (nn - 1 - q[1]));
                int32_t tm = 1 << (nn - 1 - q[2]);
                c = ((i ^ cm) & cm) ? i : (i ^ tm);
                break;
            }
            case AQSG_OP_OR: { /* :1630-1641 */
                int32_t cm = (1 << (nn - 1 - q[0])) | (1 << (nn - 1 - q[1]));
                int32_t tm = 1 << (nn - 1 - q[2]);
                c = ((i & cm) == 0) ? i : (i ^ tm);
                break;
            }
            case AQSG_OP_CH: { /* :1355-1389, two entries per row */
                int32_t tm = 1 << (nn - q[1] - 1);
                int32_t cm = 1 << (nn - q[0] - 1);
                int32_t lo = i & ~tm;
                cf e0 = C1, e1 = {0.f, 0.f};
                int32_t c0 = i, c1 = i + 1;
                if (i & cm) {
                    c0 = lo;
                    c1 = lo + tm;
                    e0.re = h; e0.im = 0.f;
                    e1.re = (i & tm) ? -h : h; e1.im = 0.f;
                }
                col[2 * (int64_t)i] = c0;
                col[2 * (int64_t)i + 1] = c1;
                val[2 * (int64_t)i] = e0;
                val[2 * (int64_t)i + 1] = e1;
                continue;
            }
            default:
                free(col);
                free(val);
                return AQSG_ERR_INVALID_ARGUMENT;
        }
        col[i] = c;
        val[i] = v;
    }
    csr_apply(x, N, cols, per_row, col, val);
    free(col);
    free(val);
    return 0;
}

int ref32_apply_ops(float* x, int n, int cols, const aqsg_op* ops,
                    int count) {
    for (int i = 0; i < count; ++i) {
        int rc = ref32_apply_one((cf*)x, n, cols, &ops[i]);
        if (rc) return rc;
    }
    return 0;
}

static float* ref32_cdf(const float* sv, int n) {
    const int64_t N = (int64_t)1 << n;
    float* cdf = (float*)malloc(sizeof(float) * (size_t)N);
    float acc = 0.f;
    for (int64_t i = 0; i < N; ++i) {
        /* af::real(sv * af::conjg(sv)) */
        float re = sv[2 * i], im = sv[2 * i + 1];
        float p = re * re - im * (-im);
        acc = acc + p;
        cdf[i] = acc;
    }
    return cdf;
}

uint32_t ref32_peek_measure_all(const float* sv, int n, float u) {
    const int64_t N = (int64_t)1 << n;
    float* cdf = ref32_cdf(sv, n);
    uint32_t state = 0;
    for (int64_t i = 0; i < N; ++i) {
        if (ceilf(cdf[i] - u) != 0.f) { state = (uint32_t)i; break; }
    }
    free(cdf);
    return state;
}

void ref32_profile_measure_all(const float* sv, int n, uint32_t R,
                               const float* u, uint32_t* counts,
                               uint32_t* unmatched) {
    const int64_t N = (int64_t)1 << n;
    float* cdf = ref32_cdf(sv, n);
    memset(counts, 0, sizeof(uint32_t) * (size_t)N);
    uint32_t un = 0;
    for (uint32_t r = 0; r < R; ++r) {
        /* sum over states of ceil(cdf - u): the number of states whose
         * cumulative probability exceeds u; the sample is N - that count */
        float s = 0.f;
        for (int64_t i = 0; i < N; ++i) s += ceilf(cdf[i] - u[r]);
        uint32_t t = (uint32_t)s;
        if (t == 0) { ++un; continue; }
        counts[N - t] += 1;
    }
    if (unmatched) *unmatched = un;
    free(cdf);
}

float ref32_qubit_probability_true(const float* sv, int n, int qubit) {
    const int64_t N = (int64_t)1 << n;
    const int64_t m = (int64_t)1 << (n - qubit - 1);
    float s = 0.f;
    for (int64_t i = 0; i < N; ++i) {
        if (!(i & m)) continue;
        float re = sv[2 * i], im = sv[2 * i + 1];
        s += re * re - im * (-im);
    }
    return s;
}

/* ------------------------------------------------------------------------ */
/* change of measurement basis, QSimulator::set_basis                      */
/* ------------------------------------------------------------------------ */

/* The 2x2 change of basis the reference applies to every qubit
 * (src/quantum.cpp:416-465), in float.  z_to_x and z_to_y are read
 * row-major (af::array(2, 2, vals).T(), :433-434); the matrix from the
 * current basis to Z is the identity for Z and x_to_z = inverse(z_to_x) for
 * X and -- through the missing break at :443 -- also for Y; the target
 * basis then multiplies z_to_y or z_to_x on the left (:454-458).  The
 * inverse is adj/det in float (af::inverse calls LAPACK; its rounding may
 * differ in the last place). */
static void ref32_basis_matrix(int from, int to, cf out[4]) {
    const float h = REF_H_F32;
    const cf z_to_x[4] = {{h, 0.f}, {h, 0.f}, {h, 0.f}, {-h, 0.f}};
    const cf z_to_y[4] = {{h, 0.f}, {h, 0.f}, {0.f, -h}, {0.f, h}};
    cf m[4] = {{1.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {1.f, 0.f}};
    switch (from) {
        case ORC_BASIS_Z: break;
        case ORC_BASIS_Y: /* falls through, as the reference's switch does */
        case ORC_BASIS_X: {
            const cf* a = z_to_x;
            const cf det = cadd(cmul(a[0], a[3]), cmul((cf){-a[1].re, -a[1].im}, a[2]));
            const float dd = det.re * det.re + det.im * det.im;
            const cf inv = {det.re / dd, -det.im / dd};
            m[0] = cmul(a[3], inv);
            m[1] = cmul((cf){-a[1].re, -a[1].im}, inv);
            m[2] = cmul((cf){-a[2].re, -a[2].im}, inv);
            m[3] = cmul(a[0], inv);
            break;
        }
        default: break;
    }
    const cf* l = to == ORC_BASIS_Y ? z_to_y : to == ORC_BASIS_X ? z_to_x : NULL;
    if (l) {
        const cf t[4] = {cadd(cmul(l[0], m[0]), cmul(l[1], m[2])), cadd(cmul(l[0], m[1]), cmul(l[1], m[3])),
                         cadd(cmul(l[2], m[0]), cmul(l[3], m[2])), cadd(cmul(l[2], m[1]), cmul(l[3], m[3]))};
        memcpy(m, t, sizeof(m));
    }
    memcpy(out, m, sizeof(m));
}

void ref32_basis_matrix_f(int from, int to, float* out) { ref32_basis_matrix(from, to, (cf*)out); }

int ref32_set_basis(float* sv, int n, int from, int to) {
    if (from == to) return 0;
    if (n < 1 || n > 12) return -1;
    cf m[4];
    ref32_basis_matrix(from, to, m);
    /* gen_tensor_matrix (:446-451): out = m; out = m (x) out, n - 1 times,
     * then one dense product with the state (:461) */
    cf* out = (cf*)malloc(sizeof(cf) * 4);
    memcpy(out, m, sizeof(m));
    int64_t d = 2;
    for (int i = 0; i < n - 1; ++i) {
        const int64_t e = 2 * d;
        cf* k = (cf*)malloc(sizeof(cf) * (size_t)e * e);
        for (int64_t r = 0; r < e; ++r)
            for (int64_t c = 0; c < e; ++c)
                k[r * e + c] = cmul(out[(r % d) * d + (c % d)], m[(r / d) * 2 + (c / d)]);
        free(out);
        out = k;
        d = e;
    }
    dense_apply((cf*)sv, d, 1, out);
    free(out);
    return 0;
}

void orc_set_basis_f64(double* sv, int n, int from, int to) {
    if (from == to) return;
    /* the same construction in exact FP64 arithmetic: x_to_z is the inverse
     * of z_to_x with h = 1/sqrt(2), i.e. z_to_x itself */
    const double h = 0.70710678118654752440;
    double m[8] = {1, 0, 0, 0, 0, 0, 1, 0};
    if (from == ORC_BASIS_Y || from == ORC_BASIS_X) {
        const double x[8] = {h, 0, h, 0, h, 0, -h, 0};
        memcpy(m, x, sizeof(m));
    }
    if (to == ORC_BASIS_Y || to == ORC_BASIS_X) {
        const double zy[8] = {h, 0, h, 0, 0, -h, 0, h};
        const double zx[8] = {h, 0, h, 0, h, 0, -h, 0};
        const double* l = to == ORC_BASIS_Y ? zy : zx;
        double t[8];
        for (int r = 0; r < 2; ++r)
            for (int c = 0; c < 2; ++c) {
                double re = 0, im = 0;
                for (int k = 0; k < 2; ++k) {
                    const double ar = l[2 * (2 * r + k)], ai = l[2 * (2 * r + k) + 1];
                    const double br = m[2 * (2 * k + c)], bi = m[2 * (2 * k + c) + 1];
                    re += ar * br - ai * bi;
                    im += ar * bi + ai * br;
                }
                t[2 * (2 * r + c)] = re;
                t[2 * (2 * r + c) + 1] = im;
            }
        memcpy(m, t, sizeof(m));
    }
    const int64_t N = (int64_t)1 << n;
    for (int q = 0; q < n; ++q) {
        const int64_t bm = (int64_t)1 << (n - 1 - q);
        for (int64_t i = 0; i < N; ++i) {
            if (i & bm) continue;
            const double ar = sv[2 * i], ai = sv[2 * i + 1];
            const double br = sv[2 * (i | bm)], bi = sv[2 * (i | bm) + 1];
            sv[2 * i] = m[0] * ar - m[1] * ai + m[2] * br - m[3] * bi;
            sv[2 * i + 1] = m[0] * ai + m[1] * ar + m[2] * bi + m[3] * br;
            sv[2 * (i | bm)] = m[4] * ar - m[5] * ai + m[6] * br - m[7] * bi;
            sv[2 * (i | bm) + 1] = m[4] * ai + m[5] * ar + m[6] * bi + m[7] * br;
        }
    }
}
