// quantum_algo.h — circuit generators of arrayfire/afQuantumSim on the hot
// path (include/quantum_algo.h): the quantum Fourier transform and its inverse.
#pragma once

#include "quantum.h"

namespace aqs {

// For i = n-1..0: H(i), then CPhase(j, i, pi / 2^(i-j)) for j < i; no final
// swaps (src/quantum_algo.cpp:103-114).
QCircuit fourier_transform(uint32_t qubits, bool compile = false);

// The mirror sequence with negated angles (src/quantum_algo.cpp:116-129).
QCircuit inverse_fourier_transform(uint32_t qubits, bool compile = false);

// Pauli decomposition of a 2^n x 2^n matrix (row-major): every string P of
// n letters i/x/y/z (letter j on qubit j, string k's letter j = bits 2j..2j+1
// of k, 0..3 = i, x, y, z) whose trace product t = Tr(P^dagger H) has
// |t|^2 > 1e-8, with coefficient t / 2^n, in the order of k
// (src/quantum_algo.cpp:131-190).  Traces are summed in FP64 on the host
// from the structure of P (one non-zero per row) instead of dense products.
std::vector<std::pair<std::string, cfloat>> decompose_hamiltonian(const std::vector<std::complex<float>>& hamiltonian,
                                                                  uint32_t qubits);

// sum_s c_s P_s as a dense 2^n x 2^n row-major matrix (src/quantum_algo.cpp:192-231).
std::vector<std::complex<float>> compose_hamiltonian(const std::vector<std::pair<std::string, cfloat>>& description);

}  // namespace aqs
