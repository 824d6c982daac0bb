// quantum_gates.cpp — composite-gate builders (arrayfire/afQuantumSim
// src/quantum_gates.cpp behaviour, restated over the aqs:: API).
#include "aqs/quantum_gates.h"

#include <algorithm>
#include <unordered_set>

namespace aqs {

QCircuit Group_Gate(uint32_t qubits, std::vector<uint32_t> targets, QCircuit gate, bool compile) {
    if (gate.qubit_count() != 1) throw std::invalid_argument{"Gate not supported"};
    std::sort(targets.begin(), targets.end());
    if (targets.size() > qubits)
        throw std::invalid_argument{"Cannot add more target qubits than there are total qubits"};
    gate.compile();
    QCircuit qc{qubits};
    for (uint32_t t : targets) qc << Gate{gate, t};
    if (compile) qc.compile();
    return qc;
}

// As in the reference, the targets on each side of the control are packed
// into one consecutive block that starts at that side's first target.
QCircuit Control_Group_Gate(uint32_t qubits, uint32_t control, std::vector<uint32_t> targets,
                            const QCircuit& gate, bool compile) {
    if (control >= qubits) throw std::invalid_argument{"Invalid control qubit position"};
    if (gate.qubit_count() != 1) throw std::invalid_argument{"Gate not supported"};
    std::sort(targets.begin(), targets.end());
    if (targets.size() >= qubits)
        throw std::invalid_argument{"Cannot add control gate at the given position"};
    const auto pivot = std::lower_bound(targets.cbegin(), targets.cend(), control);
    if (pivot != targets.cend() && *pivot == control)
        throw std::invalid_argument{"Cannot add control gate at the target qubit positions"};
    QCircuit qc(qubits);
    const auto above = std::distance(targets.cbegin(), pivot);
    const auto below = std::distance(pivot, targets.cend());
    if (above) {
        QCircuit block((uint32_t)above);
        for (uint32_t i = 0; i < (uint32_t)above; ++i) block << Gate(gate, i);
        qc << ControlGate(block, control, targets.front());
    }
    if (below) {
        QCircuit block((uint32_t)below);
        for (uint32_t i = 0; i < (uint32_t)below; ++i) block << Gate(gate, i);
        qc << ControlGate(block, control, *pivot);
    }
    if (compile) qc.compile();
    return qc;
}

QCircuit NControl_Gate(uint32_t qubits, uint32_t control_begin, uint32_t control_count,
                       uint32_t target_begin, const QCircuit& gate, bool compile) {
    if (gate.qubit_count() >= qubits) throw std::invalid_argument{"Gate not supported"};
    if (control_count == 0)
        throw std::invalid_argument{"The number of control qubits must be at least 1"};
    if (target_begin + gate.qubit_count() > qubits)
        throw std::invalid_argument{"Invalid target qubit_begin position"};
    if (control_begin + control_count > target_begin)
        throw std::invalid_argument{"Invalid control_qubit position"};
    QCircuit qc(qubits);
    if (control_count == 1) {
        qc << ControlGate(gate, control_begin, target_begin);
    } else {
        // innermost: gate controlled by the last control; each wrap adds the
        // next control in front
        const uint32_t gap = target_begin - control_begin - control_count;
        QCircuit cur(gate.qubit_count() + 1 + gap);
        cur << ControlGate(gate, 0, gap + 1);
        for (uint32_t i = 0; i + 1 < control_count; ++i) {
            QCircuit wrap(cur.qubit_count() + 1);
            wrap << ControlGate(cur, 0, 1);
            cur = std::move(wrap);
        }
        qc << Gate(cur, control_begin);
    }
    if (compile) qc.compile();
    return qc;
}

QCircuit NControl_Gate(uint32_t qubits, std::vector<uint32_t> controls, uint32_t target_begin,
                       const QCircuit& gate, bool compile) {
    if (controls.empty()) throw std::invalid_argument{"Number of control qubits must be at least one"};
    if (gate.qubit_count() + controls.size() > qubits)
        throw std::invalid_argument{"Invalid number of qubits for number of control of qubits and gate count"};
    if (target_begin + gate.qubit_count() > qubits)
        throw std::invalid_argument{"Invalid target qubit begin position"};
    std::sort(controls.begin(), controls.end());
    if (controls.back() >= qubits) throw std::invalid_argument{"Cannot add control gate at the given position"};
    const auto pivot = std::lower_bound(controls.begin(), controls.end(), target_begin);
    if (pivot != controls.end() && *pivot < target_begin + gate.qubit_count())
        throw std::invalid_argument{"Cannot add control gate at the target qubit positions"};
    const std::vector<uint32_t> above(controls.begin(), pivot), below(pivot, controls.end());

    QCircuit cur = gate;
    // controls below the gate: grow the circuit downward one control at a time
    for (std::size_t i = 0; i < below.size(); ++i) {
        const uint32_t c = below[i];
        const bool last = i + 1 == below.size();
        QCircuit wrap(last ? qubits - target_begin : c - target_begin + 1);
        wrap << ControlGate(cur, c - target_begin, 0);
        cur = std::move(wrap);
    }
    // controls above the gate: grow upward, nearest control first
    if (!above.empty()) {
        uint32_t prev = target_begin;
        for (std::size_t i = above.size(); i-- > 1;) {
            const uint32_t c = above[i];
            QCircuit wrap(qubits - c);
            wrap << ControlGate{cur, 0, prev - c};
            prev = c;
            cur = std::move(wrap);
        }
        QCircuit wrap(qubits);
        wrap << ControlGate(cur, above.front(), qubits - cur.qubit_count());
        cur = std::move(wrap);
    }
    if (compile) cur.compile();
    return cur;
}

QCircuit Rewire_Gate(uint32_t qubits, const std::vector<uint32_t>& positions, const QCircuit& gate,
                     bool compile) {
    if (positions.size() != gate.qubit_count())
        throw std::invalid_argument{"New qubit positions must map all the qubits in the gate"};
    if (gate.qubit_count() > qubits) throw std::domain_error{"Cannot rewire circuit to a lower number of qubits"};
    std::vector<uint32_t> sorted = positions;
    std::sort(sorted.begin(), sorted.end());
    for (std::size_t i = 1; i < sorted.size(); ++i)
        if (sorted[i - 1] == sorted[i])
            throw std::invalid_argument{"Cannot rewire multiple qubits to the same qubit"};

    // walk each permutation cycle with swaps, apply the gate, undo the swaps
    QCircuit qc{qubits};
    std::unordered_set<uint32_t> seen;
    std::vector<Swap> swaps;
    for (uint32_t i = 0; i < positions.size(); ++i) {
        if (!seen.insert(i).second) continue;
        uint32_t cur = i;
        while (positions[cur] != i) {
            swaps.emplace_back(cur, positions[cur]);
            qc << swaps.back();
            cur = positions[cur];
            seen.insert(cur);
        }
    }
    qc << Gate{gate, 0};
    for (auto it = swaps.rbegin(); it != swaps.rend(); ++it) qc << *it;
    if (compile) qc.compile();
    return qc;
}

static std::shared_ptr<QGate> adjoint_of(const std::shared_ptr<QGate>& g) {
    switch (g->type()) {
        case Barrier::static_type(): case X::static_type(): case Y::static_type():
        case Z::static_type(): case H::static_type(): case Swap::static_type():
        case CSwap::static_type(): case CX::static_type(): case CY::static_type():
        case CZ::static_type(): case CCNot::static_type(): case Or::static_type():
            return g;  // self-adjoint: the gate object can be shared
        case RotX::static_type(): { auto c = *std::static_pointer_cast<RotX>(g); c.angle = -c.angle; return std::make_shared<RotX>(c); }
        case RotY::static_type(): { auto c = *std::static_pointer_cast<RotY>(g); c.angle = -c.angle; return std::make_shared<RotY>(c); }
        case RotZ::static_type(): { auto c = *std::static_pointer_cast<RotZ>(g); c.angle = -c.angle; return std::make_shared<RotZ>(c); }
        case Phase::static_type(): { auto c = *std::static_pointer_cast<Phase>(g); c.angle = -c.angle; return std::make_shared<Phase>(c); }
        case CRotX::static_type(): { auto c = *std::static_pointer_cast<CRotX>(g); c.angle = -c.angle; return std::make_shared<CRotX>(c); }
        case CRotY::static_type(): { auto c = *std::static_pointer_cast<CRotY>(g); c.angle = -c.angle; return std::make_shared<CRotY>(c); }
        case CRotZ::static_type(): { auto c = *std::static_pointer_cast<CRotZ>(g); c.angle = -c.angle; return std::make_shared<CRotZ>(c); }
        case CPhase::static_type(): { auto c = *std::static_pointer_cast<CPhase>(g); c.angle = -c.angle; return std::make_shared<CPhase>(c); }
        case Gate::static_type(): {
            auto c = *std::static_pointer_cast<Gate>(g);
            c.internal_circuit = std::make_shared<QCircuit>(Adjoint_Gate(*c.internal_circuit));
            return std::make_shared<Gate>(c);
        }
        case ControlGate::static_type(): {
            auto c = *std::static_pointer_cast<ControlGate>(g);
            c.internal_circuit = std::make_shared<QCircuit>(Adjoint_Gate(*c.internal_circuit));
            return std::make_shared<ControlGate>(c);
        }
        default: throw std::runtime_error{"Unknown unsupported gate cannot be adjoint"};
    }
}

QCircuit Adjoint_Gate(const QCircuit& gate) {
    QCircuit qc = gate;
    qc.clear_cache();
    auto& list = qc.gate_list();
    std::reverse(list.begin(), list.end());
    for (auto& g : list) g = adjoint_of(g);
    // reverse the order of the ';'-terminated records of the representation
    const std::string& rep = qc.representation();
    std::string reversed;
    std::size_t prev = 0;
    for (std::size_t mark = rep.find(';'); mark != std::string::npos; mark = rep.find(';', prev)) {
        reversed = rep.substr(prev, mark - prev + 1) + reversed;
        prev = mark + 1;
    }
    qc.representation() = reversed;
    qc.compile();
    return qc;
}

}  // namespace aqs
