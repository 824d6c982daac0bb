// quantum_gates.h — composite-gate builders of arrayfire/afQuantumSim
// (include/quantum_gates.h) over the aqs:: API.  Host-side circuit builders;
// the circuits they return lower to multi-controlled engine ops.
#pragma once

#include "quantum.h"

namespace aqs {

// One 1-qubit gate on every listed qubit (quantum_gates.cpp:16-34).
QCircuit Group_Gate(uint32_t qubits, std::vector<uint32_t> target_qubits, QCircuit gate,
                    bool compile = false);

// One 1-qubit gate on every listed qubit, all controlled by one qubit
// (quantum_gates.cpp:36-78).
QCircuit Control_Group_Gate(uint32_t qubits, uint32_t control_qubit, std::vector<uint32_t> target_qubits,
                            const QCircuit& gate, bool compile = false);

// `gate` controlled by the contiguous qubits [control_qubit_begin,
// +control_qubit_count) (quantum_gates.cpp:80-114).
QCircuit NControl_Gate(uint32_t qubits, uint32_t control_qubit_begin, uint32_t control_qubit_count,
                       uint32_t target_qubit_begin, const QCircuit& gate, bool compile = false);

// `gate` controlled by an arbitrary qubit list (quantum_gates.cpp:116-182).
QCircuit NControl_Gate(uint32_t qubits, std::vector<uint32_t> control_qubits, uint32_t target_qubit_begin,
                       const QCircuit& gate, bool compile = false);

// `gate` with its qubits moved to new positions by a swap network
// (quantum_gates.cpp:184-231).
QCircuit Rewire_Gate(uint32_t qubits, const std::vector<uint32_t>& new_qubit_positions, const QCircuit& gate,
                     bool compile = false);

// The adjoint circuit: gates in reverse order with negated angles
// (quantum_gates.cpp:233-338).  New gate objects are made, so `gate` is left
// unchanged (the reference edits the gates it shares with its argument).
QCircuit Adjoint_Gate(const QCircuit& gate);

}  // namespace aqs
