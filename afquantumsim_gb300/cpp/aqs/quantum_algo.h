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

}  // namespace aqs
