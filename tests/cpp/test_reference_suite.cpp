// The assertions of arrayfire/afQuantumSim test/tests.cpp, restated against
// the aqs:: C++ layer running on the GB300 engine.  Each block cites the
// line range of the reference test it restates.  The measurement RNG is
// seeded so the statistical checks are reproducible.
#include <cmath>
#include <complex>
#include <vector>

#include "aqs/quantum.h"
#include "aqs/quantum_algo.h"
#include "aqs/quantum_gates.h"
#include "check.h"

using namespace aqs;

static bool cfequal(const cfloat& a, const cfloat& b, float diff) {
    return fequal(a.real, b.real, diff) && fequal(a.imag, b.imag, diff);
}

static bool matrix_equal(const QCircuit& a, const QCircuit& b, float tol) {
    const auto& x = a.circuit();
    const auto& y = b.circuit();
    if (x.size() != y.size()) return false;
    for (size_t i = 0; i < x.size(); ++i)
        if (std::abs(x[i] - y[i]) > tol) return false;
    return true;
}

static std::pair<int, int> band(float p, int reps) {  // 99.9% interval, tests.cpp:167-174
    const float sd = std::sqrt(p * (1.f - p));
    const int expected = (int)(reps * p);
    const int d = (int)(std::sqrt((float)reps) * 3.291f * sd);
    return {expected - d, expected + d};
}

// tests.cpp:160-207
static void qubit_profile_measure() {
    const int reps = 10000;
    const QState qs[] = {QState({1.f, 0.f}, {0.f, 0.f}), QState({0.f, 1.f}, {0.f, 0.f}),
                         QState({0.f, 0.f}, {1.f, 0.f}), QState({0.f, 0.f}, {0.f, 1.f}),
                         QState({0.f, 1.f}, {0.f, 1.f}), QState({0.6f, 0.f}, {0.f, 0.8f})};
    for (const QState& q : qs) {
        auto prof = q.profile_measure(reps);
        auto r = band(q.probability_true(), reps);
        CHECK(r.first <= (int)prof[1] && (int)prof[1] <= r.second);
    }
}

// tests.cpp:253-268
static void qsim_constructor() {
    QState state{{0.6f, 0.0f}, {0.0f, 0.8f}};
    QSimulator qs(3, state);
    CHECK(qs.qubit_count() == 3);
    for (int i = 0; i < 3; ++i) CHECK(qs.qubit(i) == state);
}

// tests.cpp:274-336
static void qsim_measurement() {
    const int count = 3;
    QSimulator qs(count, QState::zero());
    qs.generate_statevector();
    CHECK(qs.peek_measure_all() == 0);
    for (int i = 0; i < count; ++i) CHECK(qs.peek_measure(i) == false);
    qs.qubit(0) = QState::one();
    qs.qubit(count - 1) = QState::one();
    qs.generate_statevector();
    CHECK(qs.peek_measure_all() == ((1u << (count - 1)) | 1u));
    CHECK(qs.peek_measure(0) == true);
    CHECK(qs.peek_measure(count - 1) == true);
    CHECK(qs.peek_measure(1) == false);

    qs.qubit(0) = QState({0.0f, 1.0f}, {-1.0f, 0.0f});
    qs.qubit(count - 1) = QState({0.6f, 0.0f}, {0.0f, 0.8f});
    qs.generate_statevector();
    auto sv = qs.measure_all();
    CHECK((qs.state(sv) == cfloat{1.0f, 0.0f}));

    qs.qubit(0) = QState({0.0f, 1.0f}, {-1.0f, 0.0f});
    qs.qubit(count - 1) = QState({0.6f, 0.0f}, {0.0f, 0.8f});
    qs.generate_statevector();
    const float diff = 1e-4f;
    const bool q0 = qs.measure(0);
    sv = qs.peek_measure_all();
    CHECK(q0 == static_cast<bool>(sv & (1u << (qs.qubit_count() - 1))));
    if (q0) {
        CHECK(cfequal(qs.state(0b100), cfloat{-0.6f, 0.0f}, diff));
        CHECK(cfequal(qs.state(0b101), cfloat{0.0f, -0.8f}, diff));
    } else {
        CHECK(cfequal(qs.state(0b000), cfloat{0.0f, 0.6f}, diff));
        CHECK(cfequal(qs.state(0b001), cfloat{-0.8f, 0.0f}, diff));
    }
}

// tests.cpp:343-406
static void qsim_profile_measure() {
    const int reps = 10000, qcount = 5;
    QSimulator qs(qcount);
    qs.qubit(3) = QState::one();
    qs.generate_statevector();
    auto profile = qs.profile_measure_all(reps);
    for (uint32_t i = 0; i < profile.size(); ++i) {
        auto r = band(qs.state_probability(i), reps);
        CHECK(r.first <= (int)profile[i] && (int)profile[i] <= r.second);
    }
    qs.qubit(0) = QState(1.0f, 1.0f);
    qs.qubit(1) = QState(-2.0f, 3.0f);
    qs.qubit(4) = QState({0.0f, 0.6f}, {0.8f, 0.0f});
    qs.generate_statevector();
    profile = qs.profile_measure_all(reps);
    for (uint32_t i = 0; i < profile.size(); ++i) {
        auto r = band(qs.state_probability(i), reps);
        CHECK(r.first <= (int)profile[i] && (int)profile[i] <= r.second);
    }
    for (int i = 0; i < qcount; ++i) {
        auto prof = qs.profile_measure(i, reps);
        auto r = band(qs.qubit(i).probability_true(), reps);
        CHECK(r.first <= (int)prof[1] && (int)prof[1] <= r.second);
    }
}

// tests.cpp:414-1005
static void qsim_gates() {
    const float diff = 1e-4f;
    QSimulator qs(4);
    QCircuit qc(4);
    qs.qubit(3) = QState::one();
    auto run = [&](auto... gates) {
        qs.generate_statevector();
        qc.clear();
        (void)std::initializer_list<int>{((qc << gates), 0)...};
        qc.compile();
        qs.simulate(qc);
    };
    run(X(2), X(3));
    CHECK((qs.state(0b0010) == cfloat{1.0f, 0.f}));
    {
        std::vector<X> xg = {X{2}, X{3}};
        qs.generate_statevector();
        qc.clear();
        qc << xg;
        qc.compile();
        qs.simulate(qc);
        CHECK((qs.state(0b0010) == cfloat{1.0f, 0.f}));
    }
    qs.qubit(2) = QState::zero();
    qs.qubit(3) = QState::one();
    run(Y(2), Y(3));
    CHECK((qs.state(0b0010) == cfloat{1.0f, 0.f}));
    run(Z(2), Z(3));
    CHECK((qs.state(0b0001) == cfloat{-1.0f, 0.f}));
    run(Not(2), Not(3));
    CHECK((qs.state(0b0010) == cfloat{1.0f, 0.f}));
    run(H(2), H(3));
    CHECK(cfequal(qs.state(0b0000), cfloat{0.5f, 0.f}, diff));
    CHECK(cfequal(qs.state(0b0001), cfloat{-0.5f, 0.f}, diff));
    CHECK(cfequal(qs.state(0b0010), cfloat{0.5f, 0.f}, diff));
    CHECK(cfequal(qs.state(0b0011), cfloat{-0.5f, 0.f}, diff));

    qs.qubit(2) = QState({0.6f, 0.0f}, {0.0f, 0.8f});
    qs.qubit(3) = QState::zero();
    run(Phase(2, std::atan(0.75f)), Phase(3, std::atan(1.f)));
    CHECK(cfequal(qs.state(0b0000), cfloat{0.6f, 0.f}, diff));
    CHECK(cfequal(qs.state(0b0001), cfloat{0.f, 0.f}, diff));
    CHECK(cfequal(qs.state(0b0010), cfloat{-0.48f, 0.64f}, diff));
    CHECK(cfequal(qs.state(0b0011), cfloat{0.f, 0.f}, diff));

    qs.qubit(0) = QState::zero();
    qs.qubit(1) = QState::zero();
    qs.qubit(2) = QState::minus();
    qs.qubit(3) = QState::zero();
    run(RotX(2, pi / 2.f));
    CHECK(cfequal(qs.state(0b0000), cfloat{0.5f, 0.5f}, diff));
    CHECK(cfequal(qs.state(0b0010), cfloat{-0.5f, -0.5f}, diff));
    qs.qubit(2) = QState::one();
    run(RotY(2, std::acos(0.6f) * 2.f));
    CHECK(cfequal(qs.state(0b0000), cfloat{-0.8f, 0.0f}, diff));
    CHECK(cfequal(qs.state(0b0010), cfloat{0.6f, 0.0f}, diff));
    qs.qubit(2) = QState::minus();
    run(RotZ(2, -pi / 2.f));
    CHECK(cfequal(qs.state(0b0000), cfloat{0.5f, 0.5f}, diff));
    CHECK(cfequal(qs.state(0b0010), cfloat{-0.5f, 0.5f}, diff));

    const QState q68({0.6f, 0.0f}, {0.0f, 0.8f});
    qs.qubit(0) = QState::zero();
    qs.qubit(1) = QState::one();
    qs.qubit(2) = q68;
    qs.qubit(3) = q68;
    auto cx_expect = [&]() {
        CHECK(cfequal(qs.state(0b0100), cfloat{0.0f, 0.48f}, diff));
        CHECK(cfequal(qs.state(0b0101), cfloat{0.36f, 0.f}, diff));
        CHECK(cfequal(qs.state(0b0110), cfloat{-0.64f, 0.f}, diff));
        CHECK(cfequal(qs.state(0b0111), cfloat{0.f, 0.48f}, diff));
    };
    run(Xor(0, 2), Xor(1, 3));
    cx_expect();
    run(CNot(0, 2), CNot(1, 3));
    cx_expect();
    run(CX(0, 2), CX(1, 3));
    cx_expect();
    run(CY(0, 2), CY(1, 3));
    CHECK(cfequal(qs.state(0b0100), cfloat{0.48f, 0.0f}, diff));
    CHECK(cfequal(qs.state(0b0101), cfloat{0.0f, 0.36f}, diff));
    CHECK(cfequal(qs.state(0b0110), cfloat{0.0f, 0.64f}, diff));
    CHECK(cfequal(qs.state(0b0111), cfloat{-0.48f, 0.0f}, diff));
    run(CZ(0, 2), CZ(1, 3));
    CHECK(cfequal(qs.state(0b0100), cfloat{0.36f, 0.0f}, diff));
    CHECK(cfequal(qs.state(0b0101), cfloat{0.0f, -0.48f}, diff));
    CHECK(cfequal(qs.state(0b0110), cfloat{0.0f, 0.48f}, diff));
    CHECK(cfequal(qs.state(0b0111), cfloat{0.64f, 0.0f}, diff));
    run(CPhase(0, 2, std::atan(0.75f)), CPhase(1, 3, std::atan(0.75f)));
    CHECK(cfequal(qs.state(0b0100), cfloat{0.36f, 0.f}, diff));
    CHECK(cfequal(qs.state(0b0101), cfloat{-0.288f, 0.384f}, diff));
    CHECK(cfequal(qs.state(0b0110), cfloat{0.0f, 0.48f}, diff));
    CHECK(cfequal(qs.state(0b0111), cfloat{-0.512f, -0.384f}, diff));

    // the swap test's register (tests.cpp:621-637)
    qs.qubit(3) = QState({0.0f, 0.8f}, {0.6f, 0.0f});
    run(Swap(0, 2), Swap(1, 3));
    CHECK(cfequal(qs.state(0b0001), cfloat{0.0f, 0.48f}, diff));
    CHECK(cfequal(qs.state(0b0101), cfloat{0.36f, 0.0f}, diff));
    CHECK(cfequal(qs.state(0b1001), cfloat{-0.64f, 0.0f}, diff));
    CHECK(cfequal(qs.state(0b1101), cfloat{0.0f, 0.48f}, diff));
    run(CSwap(0, 2, 3));
    CHECK(cfequal(qs.state(0b0100), cfloat{0.0f, 0.48f}, diff));
    CHECK(cfequal(qs.state(0b0101), cfloat{0.36f, 0.0f}, diff));
    CHECK(cfequal(qs.state(0b0110), cfloat{-0.64f, 0.0f}, diff));
    CHECK(cfequal(qs.state(0b0111), cfloat{0.0f, 0.48f}, diff));
    run(CSwap(1, 2, 3));
    CHECK(cfequal(qs.state(0b0101), cfloat{-0.64f, 0.0f}, diff));
    CHECK(cfequal(qs.state(0b0110), cfloat{0.36f, 0.0f}, diff));

    const float s8 = 0.3535533906f;
    qs.qubit(0) = QState::zero();
    qs.qubit(1) = QState::one();
    qs.qubit(2) = QState::minus();
    qs.qubit(3) = QState::minus();
    run(CRotX(0, 2, pi / 2.f), CRotX(1, 3, pi / 2.f));
    CHECK(cfequal(qs.state(0b0100), cfloat{s8, s8}, diff));
    CHECK(cfequal(qs.state(0b0101), cfloat{-s8, -s8}, diff));
    CHECK(cfequal(qs.state(0b0110), cfloat{-s8, -s8}, diff));
    CHECK(cfequal(qs.state(0b0111), cfloat{s8, s8}, diff));
    run(CRotZ(0, 2, -pi / 2.f), CRotZ(1, 3, -pi / 2.f));
    CHECK(cfequal(qs.state(0b0100), cfloat{s8, s8}, diff));
    CHECK(cfequal(qs.state(0b0101), cfloat{-s8, s8}, diff));
    CHECK(cfequal(qs.state(0b0110), cfloat{-s8, -s8}, diff));
    CHECK(cfequal(qs.state(0b0111), cfloat{s8, -s8}, diff));
    qs.qubit(2) = QState::one();
    qs.qubit(3) = QState::one();
    run(CRotY(0, 2, std::acos(0.6f) * 2.f), CRotY(1, 3, std::acos(0.6f) * 2.f));
    CHECK(cfequal(qs.state(0b0110), cfloat{-0.8f, 0.0f}, diff));
    CHECK(cfequal(qs.state(0b0111), cfloat{0.6f, 0.0f}, diff));

    // Or / And / CCNot (tests.cpp:800-907): compiled circuit reused
    for (int kind = 0; kind < 2; ++kind) {
        qs.qubit(0) = QState::zero();
        qs.qubit(1) = QState::one();
        qs.qubit(2) = QState::zero();
        qs.qubit(3) = QState::zero();
        if (kind == 0) run(Or(0, 1, 2), Or(1, 0, 3));
        else run(And(0, 1, 2), And(1, 0, 3));
        CHECK(cfequal(qs.state(kind == 0 ? 0b0111 : 0b0100), cfloat{1.0f, 0.0f}, diff));
        qs.qubit(0) = QState::one();
        qs.generate_statevector();
        qc.compile();
        qs.simulate(qc);
        CHECK(cfequal(qs.state(0b1111), cfloat{1.0f, 0.0f}, diff));
        qs.qubit(0) = QState::zero();
        qs.qubit(1) = QState::zero();
        qs.generate_statevector();
        qc.compile();
        qs.simulate(qc);
        CHECK(cfequal(qs.state(0b0000), cfloat{1.0f, 0.0f}, diff));
    }

    // custom control gate / custom gate (tests.cpp:909-961): exact matrices
    QCircuit temp(2);
    temp << H(0) << CNot(0, 1) << Z(0) << Swap(0, 1);
    QCircuit cg(4), ref(4);
    cg << ControlGate(temp, 0, 2);
    ref << CH(0, 2) << CCNot(0, 2, 3) << CZ(0, 2) << CSwap(0, 2, 3);
    cg.compile();
    ref.compile();
    CHECK(matrix_equal(cg, ref, 0.f));
    QCircuit cg2(4), ref2(4);
    cg2 << ControlGate(temp, 2, 0);
    ref2 << CH(2, 0) << CCNot(0, 2, 1) << CZ(2, 0) << CSwap(2, 0, 1);
    cg2.compile();
    ref2.compile();
    CHECK(matrix_equal(cg2, ref2, 0.f));
    temp.clear();
    temp << H(0) << CPhase(0, 1, 1.0f) << X(1) << Swap(0, 1);
    QCircuit g(4), ref3(4);
    g << Gate(temp, 1);
    ref3 << H(1) << CPhase(1, 2, 1.0f) << X(2) << Swap(1, 2);
    g.compile();
    ref3.compile();
    CHECK(matrix_equal(g, ref3, 0.f));

    // CHadamard (tests.cpp:963-1002).  The reference asserts exact equality;
    // whether QState{r, r} renormalises to r depends on FMA contraction of
    // its float norm, so this compares within 2e-7.
    QSimulator reference(4);
    reference.qubit(2) = QState::one();
    reference.generate_statevector();
    qs.qubit(0) = QState::zero();
    qs.qubit(1) = QState::zero();
    qs.qubit(2) = QState::one();
    qs.qubit(3) = QState::zero();
    run(CH(0, 1), CH(3, 2));
    {
        auto a = reference.statevector(), b = qs.statevector();
        bool eq = true;
        for (size_t i = 0; i < a.size(); ++i) eq = eq && a[i] == b[i];
        CHECK(eq);
    }
    const float r2 = std::sqrt(1.0f / 2.0f);
    reference.qubit(0) = QState::one();
    reference.qubit(3) = QState::one();
    reference.qubit(1) = QState{r2, r2};
    reference.qubit(2) = QState{r2, -r2};
    reference.generate_statevector();
    qs.qubit(0) = QState::one();
    qs.qubit(3) = QState::one();
    qs.qubit(1) = QState::zero();
    qs.qubit(2) = QState::one();
    qs.generate_statevector();
    qc.compile();
    qs.simulate(qc);
    {
        auto a = reference.statevector(), b = qs.statevector();
        float m = 0;
        for (size_t i = 0; i < a.size(); ++i) m = std::max(m, std::abs(a[i] - b[i]));
        CHECK(m <= 2e-7f);
    }
}

// tests.cpp:1011-1135
static void special_gates() {
    {
        QCircuit qc(6);
        QSimulator qs(6);
        const uint32_t target = 3;
        qc << Gate(NControl_Gate(6, {0, 2, 4, 5}, target, X::gate()), 0);
        for (uint32_t i = 0; i < qs.qubit_count(); ++i) qs.qubit(i) = QState::one();
        qc.compile();
        qs.generate_statevector();
        qs.simulate(qc);
        CHECK(qs.peek_measure_all() == 0b111011u);
        qs.qubit(target) = QState::zero();
        qs.generate_statevector();
        qs.simulate(qc);
        CHECK(qs.peek_measure_all() == 0b111111u);
        qs.qubit(1) = QState::zero();
        qs.qubit(target) = QState::zero();
        qs.generate_statevector();
        qs.simulate(qc);
        CHECK(qs.peek_measure_all() == 0b101111u);
        qs.qubit(1) = QState::zero();
        qs.qubit(target) = QState::one();
        qs.generate_statevector();
        qs.simulate(qc);
        CHECK(qs.peek_measure_all() == 0b101011u);
    }
    {
        QCircuit qc(4), ref(4);
        qc << Gate(NControl_Gate(4, {3}, 0, X::gate()), 0);
        ref << CX(3, 0);
        qc.compile();
        ref.compile();
        CHECK(matrix_equal(qc, ref, 0.f));
        qc.clear();
        ref.clear();
        qc << Gate(NControl_Gate(4, {0, 3}, 2, X::gate()), 0);
        ref << CCNot(0, 3, 2);
        qc.compile();
        ref.compile();
        CHECK(matrix_equal(qc, ref, 0.f));
    }
    {
        QCircuit qc(4), ref(4);
        qc << Gate(Control_Group_Gate(4, 1, {0, 2, 3}, X::gate()), 0);
        ref << CX{1, 0} << CX{1, 2} << CX{1, 3};
        qc.compile();
        ref.compile();
        CHECK(matrix_equal(qc, ref, 0.f));
    }
    {
        QCircuit qc = Group_Gate(4, {0, 2, 3}, X::gate(), true);
        QCircuit ref{4};
        ref << X{0} << X{2} << X{3};
        ref.compile();
        CHECK(matrix_equal(qc, ref, 0.f));
    }
    {
        QCircuit circuit{4};
        circuit << H{0} << CX{0, 2} << H{1} << Z{3};
        circuit.compile();
        QCircuit qc = Rewire_Gate(4, {2, 1, 3, 0}, circuit, true);
        QCircuit ref{4};
        ref << H{2} << CX{2, 3} << H{1} << Z{0};
        ref.compile();
        CHECK(matrix_equal(qc, ref, 0.f));
    }
    {
        QCircuit ref{4};
        ref << CRotY{3, 0, pi / 2.f} << X{0} << CRotX{1, 3, -pi / 4.f} << CPhase{2, 1, pi / 3.f} << Swap{1, 2};
        ref.compile();
        QCircuit circuit{4};
        circuit << Swap{1, 2} << CPhase{2, 1, -pi / 3.f} << CRotX{1, 3, pi / 4.f} << X{0} << CRotY{3, 0, -pi / 2.f};
        circuit.compile();
        QCircuit qc = Adjoint_Gate(circuit);
        CHECK(matrix_equal(qc, ref, 1e-5f));
    }
}

// tests.cpp:1141-1194
static void qsim_probability() {
    const int qcount = 4;
    const float diff = 1e-4f;
    QSimulator qs(4);
    qs.generate_statevector();
    for (int i = 0; i < qcount; ++i) {
        CHECK(qs.qubit_probability_true(i) == 0.f);
        CHECK(qs.qubit_probability_false(i) == 1.f);
    }
    qs.qubit(qcount - 1) = QState{0.f, 1.f};
    qs.generate_statevector();
    for (int i = 0; i < qcount - 1; ++i) CHECK(qs.qubit_probability_true(i) == 0.f);
    CHECK(qs.qubit_probability_true(qcount - 1) == 1.f);
    CHECK(qs.qubit_probability_false(qcount - 1) == 0.f);
    qs.qubit(qcount - 1) = QState{1.f, 1.f};
    qs.generate_statevector();
    CHECK(fequal(qs.qubit_probability_true(qcount - 1), 0.5f, diff));
    qs.qubit(0) = QState{{0.6f, 0.0f}, {0.f, 0.8f}};
    qs.generate_statevector();
    CHECK(fequal(qs.qubit_probability_true(0), 0.64f, diff));
    CHECK(fequal(qs.qubit_probability_false(0), 0.36f, diff));
    CHECK(fequal(qs.qubit_probability_true(qcount - 1), 0.5f, diff));
}

// engine-level extras: compile() and simulate() agree; errors keep the
// reference's exception classes; the 12-qubit plain workload's statevector
// sums to one
static void extras() {
    QCircuit a = fourier_transform(10), b = fourier_transform(10);
    b.compile();
    QSimulator s1(10, QState::plus()), s2(10, QState::plus());
    s1.simulate(a);
    s2.simulate(b);
    auto x = s1.statevector(), y = s2.statevector();
    float m = 0;
    for (size_t i = 0; i < x.size(); ++i) m = std::max(m, std::abs(x[i] - y[i]));
    CHECK(m < 1e-6f);
    QCircuit c3(3);
    CHECK_THROWS(s1.simulate(c3), std::invalid_argument);
    CHECK_THROWS(s1.qubit_probability_true(10), std::out_of_range);
    CHECK_THROWS(s1.measure(12), std::out_of_range);
    std::vector<std::complex<float>> zero(8, 0.f);
    CHECK_THROWS(QSimulator(3, zero), std::invalid_argument);
    std::vector<std::complex<float>> v(8, 2.f);
    QSimulator s3(3, v);
    CHECK(fequal(s3.state_probability(5), 0.125f, 1e-6f));
    // set_basis Z -> X on |0...0> gives the uniform superposition
    QSimulator s4(3);
    s4.set_basis(QSimulator::Basis::X);
    CHECK(fequal(s4.state_probability(6), 0.125f, 1e-5f));
    CHECK(s4.get_basis() == QSimulator::Basis::X);
    // compiled circuits run fused (default width 5) or gate by gate (width 0)
    for (int k : {0, 2, 5}) {
        set_fusion_qubits(k);
        QCircuit f = fourier_transform(10);
        f.compile();
        QSimulator s5(10, QState::plus());
        s5.simulate(f);
        auto z = s5.statevector();
        float d = 0;
        for (size_t i = 0; i < x.size(); ++i) d = std::max(d, std::abs(x[i] - z[i]));
        CHECK(d < 1e-5f);
    }
    set_fusion_qubits(5);
    CHECK_THROWS(set_fusion_qubits(6), std::invalid_argument);
    // Pauli expectations on a Bell pair; a Hamiltonian's energy
    QSimulator bell(2);
    QCircuit bc(2);
    bc << H(0) << CNot(0, 1);
    bell.simulate(bc);
    auto e = bell.pauli_expectations({"zz", "xx", "yy", "zi", "ii"});
    CHECK(std::abs(e[0] - 1.0) < 1e-6 && std::abs(e[1] - 1.0) < 1e-6 && std::abs(e[2] + 1.0) < 1e-6);
    CHECK(std::abs(e[3]) < 1e-6 && std::abs(e[4] - 1.0) < 1e-6);
    auto energy = bell.expectation({{"zz", cfloat(0.5f, 0.f)}, {"xx", cfloat(-2.f, 0.f)}});
    CHECK(std::abs(energy - std::complex<double>(-1.5, 0.0)) < 1e-6);
    CHECK_THROWS(bell.pauli_expectations({"zzz"}), std::invalid_argument);
}

int main(int argc, char** argv) {
    aqs::initialize(argc, argv);
    aqs::seed(20240607u);
    qubit_profile_measure();
    qsim_constructor();
    qsim_measurement();
    qsim_profile_measure();
    qsim_gates();
    qsim_probability();
    special_gates();
    extras();
    clear_circuit_cache();
    return finish("test_reference_suite");
}
