// quantum_algo.cpp — QFT generators (arrayfire/afQuantumSim
// src/quantum_algo.cpp:103-129 behaviour).
#include "aqs/quantum_algo.h"

namespace aqs {

QCircuit fourier_transform(uint32_t qubits, bool compile) {
    QCircuit qc(qubits);
    for (int32_t i = (int32_t)qubits - 1; i >= 0; --i) {
        qc << H{(uint32_t)i};
        for (uint32_t j = 0; j < (uint32_t)i; ++j)
            qc << CPhase{j, (uint32_t)i, pi / (float)(1u << (i - j))};
    }
    if (compile) qc.compile();
    return qc;
}

QCircuit inverse_fourier_transform(uint32_t qubits, bool compile) {
    QCircuit qc(qubits);
    for (uint32_t i = 0; i < qubits; ++i) {
        for (int32_t j = (int32_t)i - 1; j >= 0; --j)
            qc << CPhase{(uint32_t)j, i, -pi / (float)(1u << (i - j))};
        qc << H{i};
    }
    if (compile) qc.compile();
    return qc;
}

}  // namespace aqs
