/*
 * aqs_oracle.h — CPU oracle for the GB300 state-vector engine.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links, loads or calls
 * this code: tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg compare results with it (the last also times it as the CPU arm).
 *
 * Two restatements of arrayfire/afQuantumSim's QSimulator::simulate
 * (src/quantum.cpp:277-291):
 *
 *  orc_*   per-gate oracle.  Each gate is applied in place by its
 *          mathematical definition (FP64: orc_apply_ops_f64; an FP32 twin,
 *          orc_apply_ops_f32, computes gate coefficients exactly as the
 *          reference does — cosf(angle/2.0f), 0.70710678118f — and does the
 *          arithmetic in float).  Ground truth at every size.
 *
 *  ref32_* faithful FP32 restatement of the reference ALGORITHM: every gate
 *          builds its full 2^n x 2^n operator the way src/quantum.cpp does —
 *          dense Kronecker I(x)U(x)I for H/RotX/RotY/RotZ, one- or two-entry
 *          CSR rows for the sparse gates, dense scatter for ControlGate/Gate —
 *          and multiplies it into the state (or, for compile(), into the
 *          circuit matrix).  Feasible to ~14 qubits; it stands in for the
 *          reference's ArrayFire CPU backend, which is not installed here.
 *
 * Parity is pinned by the known answers of the reference's test/tests.cpp
 * (tests/golden/reference_kat.json, tests/test_oracle_golden.py).
 */
#ifndef AQS_ORACLE_H
#define AQS_ORACLE_H

#include <stdint.h>

#include "../include/aqsg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* number of OpenMP threads the oracle uses (0 = all) */
void orc_set_threads(int threads);
int orc_get_threads(void);

/* per-gate oracle, in place on 2^n interleaved complex amplitudes */
int orc_apply_ops_f64(double* sv, int n, const aqsg_op* ops, int count);
int orc_apply_ops_f32(float* sv, int n, const aqsg_op* ops, int count);

/* |a_k|^2 in FP64 */
void orc_probs_f64(const double* sv, int n, double* out);
void orc_probs_f32(const float* sv, int n, double* out);
/* first index whose inclusive FP64 cumulative sum of p exceeds u; -1 if none */
int64_t orc_first_index(const double* p, int n, double u);
/* FP64 marginal P(qubit = 1) */
double orc_qubit_prob_f64(const double* sv, int n, int qubit);

/* ---- faithful FP32 restatement of the reference algorithm ------------- */

/* Product state q_0 (x) ... (x) q_{n-1} by the Kronecker chain of
 * QSimulator::generate_statevector (quantum.cpp:261-275). q: 4n floats. */
void ref32_product_state(int n, const float* q, float* sv);
/* QState::force_normalize (quantum.cpp:145-157) on {re0, im0, re1, im1};
 * returns -1 for a null state. */
int ref32_qstate_normalize(float* q);
/* Apply ops to an N x cols matrix X (row-major, interleaved complex),
 * X <- G X for each gate G, building G as src/quantum.cpp does.
 * cols = 1 is simulate(); cols = N starting from the identity is compile(). */
int ref32_apply_ops(float* x, int n, int cols, const aqsg_op* ops, int count);
/* peek_measure_all with uniform u (quantum.cpp:344-359): float |a|^2, float
 * inclusive scan, first index with cdf - u > 0, 0 if none. */
uint32_t ref32_peek_measure_all(const float* sv, int n, float u);
/* profile_measure_all with R given uniforms (quantum.cpp:467-501).  counts
 * has 2^n entries; samples that no state matches (u above the total
 * probability) are counted in *unmatched instead of overflowing the output
 * as the reference does. */
void ref32_profile_measure_all(const float* sv, int n, uint32_t R,
                               const float* u, uint32_t* counts,
                               uint32_t* unmatched);
/* qubit_probability_true (quantum.cpp:372-391) in float */
float ref32_qubit_probability_true(const float* sv, int n, int qubit);

/* ---- change of measurement basis (QSimulator::set_basis) -------------- */

/* Basis values of QSimulator::Basis (include/quantum.h:489-500). */
#define ORC_BASIS_Z 0
#define ORC_BASIS_Y 1
#define ORC_BASIS_X 2
/* The 2x2 matrix (row-major interleaved complex, 8 floats) set_basis
 * applies to every qubit to go from basis `from` to `to`
 * (quantum.cpp:416-465), with the fall-through of the missing break at
 * :443: leaving Y uses the X-to-Z matrix. */
void ref32_basis_matrix_f(int from, int to, float* out);
/* set_basis as the reference computes it: the n-fold Kronecker product of
 * that matrix as a dense 2^n x 2^n operator times the state, in float
 * (n <= 12).  Returns -1 for other n. */
int ref32_set_basis(float* sv, int n, int from, int to);
/* The same change of basis (same fall-through) in FP64, one 2x2 per qubit. */
void orc_set_basis_f64(double* sv, int n, int from, int to);

#ifdef __cplusplus
}
#endif

#endif
