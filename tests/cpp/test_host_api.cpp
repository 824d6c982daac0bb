// Host-side checks of the aqs:: C++ layer that need no GPU: QState, the
// single-qubit *_op helpers, representation strings, check() exceptions, and
// the lowering of every builder (Gate, ControlGate, NControl_Gate,
// Control_Group_Gate, Group_Gate, Rewire_Gate, Adjoint_Gate, QFT) — the
// lowered engine ops are executed by the CPU oracle and compared with the
// circuits the reference's test/tests.cpp equates them to.
#include <complex>
#include <vector>

#include "aqs/quantum.h"
#include "aqs/quantum_algo.h"
#include "aqs/quantum_gates.h"
#include "aqs_oracle.h"
#include "check.h"

using namespace aqs;
using cd = std::complex<double>;

static std::vector<cd> run(const QCircuit& qc, std::vector<cd> v) {
    auto ops = qc.lower(0, qc.gate_list().size());
    orc_apply_ops_f64(reinterpret_cast<double*>(v.data()), (int)qc.qubit_count(), ops.data(), (int)ops.size());
    return v;
}

static std::vector<cd> matrix_of(const QCircuit& qc) {
    const uint32_t N = qc.state_count();
    std::vector<cd> M(N * N);
    for (uint32_t k = 0; k < N; ++k) {
        std::vector<cd> e(N, 0.0);
        e[k] = 1.0;
        auto col = run(qc, e);
        for (uint32_t i = 0; i < N; ++i) M[i * N + k] = col[i];
    }
    return M;
}

static double maxdiff(const std::vector<cd>& a, const std::vector<cd>& b) {
    double m = 0;
    for (size_t i = 0; i < a.size(); ++i) m = std::max(m, std::abs(a[i] - b[i]));
    return m;
}

static uint32_t basis_index_after(const QCircuit& qc, uint32_t start) {
    std::vector<cd> v(qc.state_count(), 0.0);
    v[start] = 1.0;
    v = run(qc, v);
    for (uint32_t i = 0; i < v.size(); ++i)
        if (std::abs(v[i]) > 0.5) return i;
    return ~0u;
}

// tests.cpp:42-154
static void qstate_tests() {
    QState q1;
    CHECK(q1[0] == (cfloat{1.f, 0.f}) && q1[1] == (cfloat{0.f, 0.f}));
    QState q2({0.6f, 0.f}, {0.f, 0.8f});
    CHECK(q2[0] == (cfloat{0.6f, 0.f}) && q2[1] == (cfloat{0.f, 0.8f}));
    QState q3(q2);
    CHECK(q3 == q2);
    QState n1({3.f, 0.f}, {4.f, 0.f});
    CHECK(n1[0] == (cfloat{0.6f, 0.f}) && n1[1] == (cfloat{0.8f, 0.f}));
    QState n2({1.f, 2.f}, {3.f, 4.f});
    const float mag = std::sqrt(1.f * 1.f + 2.f * 2.f + 3.f * 3.f + 4.f * 4.f);
    CHECK(n2[0] == (cfloat{1.f / mag, 2.f / mag}) && n2[1] == (cfloat{3.f / mag, 4.f / mag}));
    CHECK_THROWS(QState(0.f, 0.f), std::invalid_argument);
    const float diff = 1e-4f;
    CHECK(QState(1.f, 0.f).probability_false() == 1.f);
    CHECK(QState({0.f, 1.f}, {0.f, 0.f}).probability_true() == 0.f);
    CHECK(QState(0.f, 1.f).probability_true() == 1.f);
    CHECK(fequal(QState({0.f, 1.f}, {0.f, 1.f}).probability_true(), 0.5f, diff));
    CHECK(fequal(QState({0.6f, 0.f}, {0.f, 0.8f}).probability_true(), 0.64f, diff));
    CHECK(fequal(QState({0.6f, 0.f}, {0.f, 0.8f}).probability_false(), 0.36f, diff));
}

// tests.cpp:213-245
static void qstate_op_tests() {
    const QState qref({0.5f, -0.5f}, {0.7f, 0.1f});
    QState a = X_op(qref);
    CHECK(a[0] == (cfloat{0.7f, 0.1f}) && a[1] == (cfloat{0.5f, -0.5f}));
    QState b = Y_op(qref);
    CHECK(b[0] == (cfloat{0.1f, -0.7f}) && b[1] == (cfloat{0.5f, 0.5f}));
    QState c = Z_op(qref);
    CHECK(c[0] == (cfloat{0.5f, -0.5f}) && c[1] == (cfloat{-0.7f, -0.1f}));
    QState h = Hadamard_op(qref);
    QState hh({1.2f, -0.4f}, {-0.2f, -0.6f});
    CHECK(fequal(h[0].real, hh[0].real, 1e-4f) && fequal(h[0].imag, hh[0].imag, 1e-4f) &&
          fequal(h[1].real, hh[1].real, 1e-4f) && fequal(h[1].imag, hh[1].imag, 1e-4f));
}

static void representation_tests() {
    QCircuit qc(4);
    qc << X{2} << CSwap{0, 2, 3} << Phase{1, pi / 2} << CPhase{0, 1, 0.3f};
    CHECK(qc.representation() == "X,0,1:2;Swap,1,2:0,23;S,0,1:1;Phase,1,1:0,1;");
    CHECK(Or(0, 1, 2).to_string() == "P;X,0,1:0;X,0,1:1;X,0,1:2;X,2,1:0,1,2;X,0,1:0;X,0,1:1;P;");
    QCircuit temp(2);
    temp << H{0} << CX{0, 1};
    CHECK(Gate(temp, 1).to_string() == "H,0,1:1;X,1,1:1,2;");
    CHECK(ControlGate(temp, 0, 2).to_string() == "H,1,1:0,2;X,2,1:0,2,3;");
    CHECK(Gate(temp, 1, "Bell").to_string() == "Bell,0,2:1,2;");
    CHECK(ControlGate(temp, 3, 0, "Bell").to_string() == "Bell,1,2:3,0,1;");
    CHECK_THROWS(Gate(temp, 1, "a,b"), std::invalid_argument);
    // Gate / ControlGate share sub-circuits through the cache (quantum.cpp:1710-1724)
    CHECK(Gate(temp, 1) == Gate(temp, 1));
}

static void check_tests() {
    QCircuit q1(1), q3(3);
    CHECK_THROWS(q3 << X{3}, std::out_of_range);
    CHECK_THROWS(q1 << Swap(0, 1), std::domain_error);
    CHECK_THROWS(q3 << Swap(1, 1), std::invalid_argument);
    CHECK_THROWS(q3 << CX(1, 1), std::invalid_argument);
    CHECK_THROWS(q3 << CRotY(0, 4, 0.1f), std::out_of_range);
    QCircuit q2(2);
    CHECK_THROWS(q2 << CSwap(0, 1, 2), std::domain_error);
    CHECK_THROWS(q3 << CCNot(0, 2, 2), std::invalid_argument);
    CHECK_THROWS(QCircuit(0), std::invalid_argument);
    CHECK_THROWS(QCircuit(31), std::invalid_argument);
    QCircuit temp(2);
    temp << H{0};
    CHECK_THROWS(q3 << ControlGate(temp, 1, 0), std::out_of_range);
    CHECK_THROWS(q3 << ControlGate(temp, 0, 2), std::out_of_range);
    CHECK_THROWS(q2 << ControlGate(temp, 0, 0), std::out_of_range);
    CHECK_THROWS(q3 << Gate(temp, 2), std::out_of_range);
}

// tests.cpp:909-961 and 1011-1132, through the oracle
static void builder_tests() {
    QCircuit temp(2);
    temp << H{0} << CNot{0, 1} << Z{0} << Swap{0, 1};
    {
        QCircuit qc(4), ref(4);
        qc << ControlGate(temp, 0, 2);
        ref << CH{0, 2} << CCNot{0, 2, 3} << CZ{0, 2} << CSwap{0, 2, 3};
        CHECK(maxdiff(matrix_of(qc), matrix_of(ref)) == 0.0);
        QCircuit qc2(4), ref2(4);
        qc2 << ControlGate(temp, 2, 0);
        ref2 << CH{2, 0} << CCNot{0, 2, 1} << CZ{2, 0} << CSwap{2, 0, 1};
        CHECK(maxdiff(matrix_of(qc2), matrix_of(ref2)) == 0.0);
    }
    {
        QCircuit t2(2), qc(4), ref(4);
        t2 << H{0} << CPhase{0, 1, 1.0f} << X{1} << Swap{0, 1};
        qc << Gate(t2, 1);
        ref << H{1} << CPhase{1, 2, 1.0f} << X{2} << Swap{1, 2};
        CHECK(maxdiff(matrix_of(qc), matrix_of(ref)) == 0.0);
    }
    {
        QCircuit qc(6);
        qc << Gate(NControl_Gate(6, {0, 2, 4, 5}, 3, X::gate()), 0);
        CHECK(basis_index_after(qc, 0b111111) == 0b111011u);
        CHECK(basis_index_after(qc, 0b111011) == 0b111111u);
        CHECK(basis_index_after(qc, 0b101011) == 0b101111u);
        CHECK(basis_index_after(qc, 0b101111) == 0b101011u);
    }
    {
        QCircuit qc(4), ref(4);
        qc << Gate(NControl_Gate(4, {3}, 0, X::gate()), 0);
        ref << CX(3, 0);
        CHECK(maxdiff(matrix_of(qc), matrix_of(ref)) == 0.0);
        QCircuit qc2(4), ref2(4);
        qc2 << Gate(NControl_Gate(4, {0, 3}, 2, X::gate()), 0);
        ref2 << CCNot(0, 3, 2);
        CHECK(maxdiff(matrix_of(qc2), matrix_of(ref2)) == 0.0);
        // contiguous-control overload: controls 0..2 on target 3
        QCircuit qc3(5), ref3(5);
        qc3 << Gate(NControl_Gate(5, 0, 3, 3, X::gate()), 0);
        QCircuit inner(5);
        inner << Gate(NControl_Gate(5, {0, 1, 2}, 3, X::gate()), 0);
        CHECK(maxdiff(matrix_of(qc3), matrix_of(inner)) == 0.0);
    }
    {
        QCircuit qc(4), ref(4);
        qc << Gate(Control_Group_Gate(4, 1, {0, 2, 3}, X::gate()), 0);
        ref << CX{1, 0} << CX{1, 2} << CX{1, 3};
        CHECK(maxdiff(matrix_of(qc), matrix_of(ref)) == 0.0);
    }
    {
        QCircuit qc = Group_Gate(4, {0, 2, 3}, X::gate(), true);
        QCircuit ref{4};
        ref << X{0} << X{2} << X{3};
        CHECK(maxdiff(matrix_of(qc), matrix_of(ref)) == 0.0);
    }
    {
        QCircuit circuit{4};
        circuit << H{0} << CX{0, 2} << H{1} << Z{3};
        QCircuit qc = Rewire_Gate(4, {2, 1, 3, 0}, circuit, true);
        QCircuit ref{4};
        ref << H{2} << CX{2, 3} << H{1} << Z{0};
        CHECK(maxdiff(matrix_of(qc), matrix_of(ref)) < 1e-15);
    }
    {
        QCircuit ref{4};
        ref << CRotY{3, 0, pi / 2.f} << X{0} << CRotX{1, 3, -pi / 4.f} << CPhase{2, 1, pi / 3.f} << Swap{1, 2};
        QCircuit circuit{4};
        circuit << Swap{1, 2} << CPhase{2, 1, -pi / 3.f} << CRotX{1, 3, pi / 4.f} << X{0} << CRotY{3, 0, -pi / 2.f};
        const std::string before = circuit.representation();
        QCircuit qc = Adjoint_Gate(circuit);
        CHECK(maxdiff(matrix_of(qc), matrix_of(ref)) < 1e-5);
        CHECK(circuit.representation() == before);
        CHECK(static_cast<const CRotY&>(*circuit.gate_list().back()).angle == -pi / 2.f);
        CHECK(qc.representation().rfind("Swap,0,2:1,2;") == qc.representation().size() - 13);
    }
    {
        QCircuit f = fourier_transform(4), inv = inverse_fourier_transform(4);
        QCircuit both(4);
        both << Gate(f, 0) << Gate(inv, 0);
        auto M = matrix_of(both);
        std::vector<cd> I(M.size(), 0.0);
        for (int k = 0; k < 16; ++k) I[k * 16 + k] = 1.0;
        CHECK(maxdiff(M, I) < 1e-6);
        CHECK(f.gate_list().size() == 4 + 6);
    }
}

// decompose_hamiltonian / compose_hamiltonian (quantum_algo.cpp:131-231)
static void hamiltonian_tests() {
    using cf = std::complex<float>;
    // Z (x) I on two qubits: letter 0 = qubit 0 = the first Kronecker factor
    std::vector<cf> zi(16, 0.f);
    for (int k = 0; k < 4; ++k) zi[k * 4 + k] = (k & 2) ? -1.f : 1.f;
    auto d = decompose_hamiltonian(zi, 2);
    CHECK(d.size() == 1 && d[0].first == "zi" && d[0].second == cfloat(1.f, 0.f));
    // a Hermitian 3-qubit matrix: compose(decompose(H)) == H, strings in code order
    std::vector<cf> H(64);
    for (int r = 0; r < 8; ++r)
        for (int c = 0; c <= r; ++c) {
            const cf v((float)((r * 7 + c * 3) % 5) - 2.f, r == c ? 0.f : (float)((r + 2 * c) % 3) - 1.f);
            H[r * 8 + c] = v;
            H[c * 8 + r] = std::conj(v);
        }
    auto desc = decompose_hamiltonian(H, 3);
    CHECK(!desc.empty());
    auto back = compose_hamiltonian(desc);
    double mx = 0;
    for (int i = 0; i < 64; ++i) mx = std::max(mx, (double)std::abs(back[i] - H[i]));
    CHECK(mx < 1e-5);
    for (const auto& t : desc) CHECK(std::abs(t.second.imag) < 1e-6);  // Hermitian: real coefficients
    CHECK_THROWS((compose_hamiltonian({{"xi", cfloat(1.f, 0.f)}, {"x", cfloat(1.f, 0.f)}})), std::invalid_argument);
    CHECK_THROWS((decompose_hamiltonian(H, 2)), std::invalid_argument);
}

int main() {
    hamiltonian_tests();
    qstate_tests();
    qstate_op_tests();
    representation_tests();
    check_tests();
    builder_tests();
    return finish("test_host_api");
}
