// quantum_algo.cpp — QFT generators (arrayfire/afQuantumSim
// src/quantum_algo.cpp:103-129 behaviour).
#include "aqs/quantum_algo.h"

#include <stdexcept>

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

namespace {

// P|k> = phase(k) |k ^ x>: x marks the X/Y letters, z the Y/Z letters
// (index bit n-1-j for letter j), phase = i^{#Y} (-1)^{|k & z|}.
struct PauliMasks {
    uint64_t x = 0, z = 0;
    int ny = 0;
};

PauliMasks masks_of(const std::string& s) {
    PauliMasks m;
    const std::size_t n = s.size();
    for (std::size_t j = 0; j < n; ++j) {
        const uint64_t bit = 1ull << (n - 1 - j);
        switch (s[j]) {
            case 'i': case 'I': break;
            case 'x': case 'X': m.x |= bit; break;
            case 'y': case 'Y': m.x |= bit; m.z |= bit; ++m.ny; break;
            case 'z': case 'Z': m.z |= bit; break;
            default: throw std::invalid_argument{"Pauli strings take the letters i, x, y, z"};
        }
    }
    return m;
}

std::complex<double> phase_of(const PauliMasks& m, uint64_t k) {
    static const std::complex<double> ipow[4] = {{1, 0}, {0, 1}, {-1, 0}, {0, -1}};
    const double sign = (__builtin_popcountll(k & m.z) & 1) ? -1.0 : 1.0;
    return ipow[m.ny & 3] * sign;
}

}  // namespace

std::vector<std::pair<std::string, cfloat>> decompose_hamiltonian(const std::vector<std::complex<float>>& hamiltonian,
                                                                  uint32_t qubits) {
    if (qubits < 1 || qubits > 12) throw std::invalid_argument{"decompose_hamiltonian takes 1 to 12 qubits"};
    const uint64_t N = 1ull << qubits;
    if (hamiltonian.size() != N * N) throw std::invalid_argument{"Hamiltonian must be 2^n x 2^n"};
    static const char letters[4] = {'i', 'x', 'y', 'z'};
    std::vector<std::pair<std::string, cfloat>> out;
    std::string str(qubits, 'i');
    for (uint64_t code = 0; code < (1ull << (2 * qubits)); ++code) {
        for (uint32_t j = 0; j < qubits; ++j) str[j] = letters[(code >> (2 * j)) & 3];
        const PauliMasks m = masks_of(str);
        // column k of P holds phase(k) in row k ^ x, so
        // Tr(P^dagger H) = sum_k conj(phase(k)) H[k ^ x][k]
        std::complex<double> t = 0;
        for (uint64_t k = 0; k < N; ++k) {
            const std::complex<float> h = hamiltonian[(k ^ m.x) * N + k];
            t += std::conj(phase_of(m, k)) * std::complex<double>(h.real(), h.imag());
        }
        if (std::norm(t) > 1e-8) {
            const std::complex<double> c = t / (double)N;
            out.push_back({str, cfloat{(float)c.real(), (float)c.imag()}});
        }
    }
    return out;
}

std::vector<std::complex<float>> compose_hamiltonian(const std::vector<std::pair<std::string, cfloat>>& description) {
    if (description.empty()) return {};
    const std::size_t n = description[0].first.size();
    if (n < 1 || n > 12) throw std::invalid_argument{"compose_hamiltonian takes 1 to 12 qubits"};
    const uint64_t N = 1ull << n;
    std::vector<std::complex<double>> acc(N * N, 0.0);
    for (const auto& term : description) {
        if (term.first.size() != n) throw std::invalid_argument{"Invalid Pauli-description"};
        const PauliMasks m = masks_of(term.first);
        const std::complex<double> c(term.second.real, term.second.imag);
        for (uint64_t k = 0; k < N; ++k) acc[(k ^ m.x) * N + k] += c * phase_of(m, k);
    }
    std::vector<std::complex<float>> out(N * N);
    for (uint64_t i = 0; i < N * N; ++i) out[i] = {(float)acc[i].real(), (float)acc[i].imag()};
    return out;
}

}  // namespace aqs
