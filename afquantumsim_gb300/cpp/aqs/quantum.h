// quantum.h — the aqs:: C++ API of arrayfire/afQuantumSim (include/quantum.h)
// on the GB300 engine (libaqsg.so, include/aqsg.h).
//
// Same class names, constructors, member functions, exception classes and
// messages as the reference.  Deliberate differences (no ArrayFire):
//  - af::cfloat is aqs::cfloat (same {real, imag} layout and operators);
//  - QSimulator::statevector() and QCircuit::circuit() return host copies
//    (std::vector<std::complex<float>>, the matrix row-major) instead of
//    af::array references; QSimulator(n, statevector) takes such a vector;
//  - a plugin gate (QGate subclass) emits engine ops in lower() instead of
//    multiplying an af::array in operator();
//  - aqs::seed() makes the measurement RNG reproducible (the reference's is
//    seeded from std::random_device only).
#pragma once

#include <aqsg.h>

#include <array>
#include <cassert>
#include <complex>
#include <cstdint>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace aqs {

static constexpr float pi = 3.14159265358979323846f;   // quantum.h:121
static constexpr uint32_t max_qubit_count = 30;        // quantum.h:122

class QGate;
class QState;
class QCircuit;
class QSimulator;

inline uint32_t fast_pow2(uint32_t p) { return 1u << p; }

// {real, imag} float pair with the arithmetic af::cfloat offers.
struct cfloat {
    float real = 0.f, imag = 0.f;
    cfloat() = default;
    cfloat(float r) : real(r), imag(0.f) {}
    cfloat(float r, float i) : real(r), imag(i) {}
    friend bool operator==(const cfloat& a, const cfloat& b) { return a.real == b.real && a.imag == b.imag; }
    friend bool operator!=(const cfloat& a, const cfloat& b) { return !(a == b); }
    friend cfloat operator+(const cfloat& a, const cfloat& b) { return {a.real + b.real, a.imag + b.imag}; }
    friend cfloat operator*(const cfloat& a, const cfloat& b) {
        return {a.real * b.real - a.imag * b.imag, a.real * b.imag + a.imag * b.real};
    }
    friend cfloat operator*(const cfloat& a, float s) { return {a.real * s, a.imag * s}; }
    friend cfloat operator/(const cfloat& a, float s) { return {a.real / s, a.imag / s}; }
};

// Open the engine on device argv[1] (default 0).  quantum.h:138-139.
void initialize(int argc = 0, char** argv = nullptr);
// Release the engine context (registers must be gone).
void shutdown();
// Drop the Gate/ControlGate sub-circuit cache.  quantum.h:140.
void clear_circuit_cache();
// Seed the measurement RNG (extension; see header comment).
void seed(uint64_t s);
// The engine context, opened on first use.
aqsg_ctx engine();
// Width (qubits) of the dense unitaries QCircuit::compile() folds gate
// windows into when a circuit is simulated: 1..5, or 0 to apply the compiled
// gates one by one.  Default 5.  (Extension: the reference folds the whole
// circuit into one 2^n x 2^n matrix, quantum.cpp:199-210.)
void set_fusion_qubits(int k);
int fusion_qubits();

// Throws the reference's exception class for an engine status.
void throw_status(int rc);

// ---- QState (quantum.h:151-342) ------------------------------------------------
class QState {
   public:
    QState() = default;
    QState(const std::complex<float>& zero_state, const std::complex<float>& one_state);
    QState(const std::array<std::complex<float>, 2>& states);

    static std::array<std::complex<float>, 2> create_state(float polar_angle, float azimuthal_angle) {
        return {std::cos(polar_angle / 2.f),
                std::complex<float>{std::cos(azimuthal_angle), std::sin(azimuthal_angle)} *
                    std::sin(polar_angle / 2.f)};
    }

    QState& set(const std::complex<float>& zero_state, const std::complex<float>& one_state);
    bool peek_measure() const;
    bool measure();
    std::array<uint32_t, 2> profile_measure(uint32_t rep_count) const;
    float probability_true() const noexcept {
        return state_[1].real * state_[1].real + state_[1].imag * state_[1].imag;
    }
    float probability_false() const noexcept { return 1.f - probability_true(); }
    const cfloat& operator[](bool index) const noexcept { return state_[static_cast<int>(index)]; }
    bool operator!=(const QState& o) const noexcept { return state_[0] != o.state_[0] || state_[1] != o.state_[1]; }
    bool operator==(const QState& o) const noexcept { return !(*this != o); }
    cfloat* data() noexcept { return state_; }
    const cfloat* data() const noexcept { return state_; }
    std::array<std::complex<float>, 2> to_array() const {
        return {std::complex<float>{state_[0].real, state_[0].imag},
                std::complex<float>{state_[1].real, state_[1].imag}};
    }

    static const QState& zero() { static const QState s{1.0f, 0.0f}; return s; }
    static const QState& one() { static const QState s{0.0f, 1.0f}; return s; }
    static const QState& plus() { static const QState s{0.70710678118f, 0.70710678118f}; return s; }
    static const QState& minus() { static const QState s{0.70710678118f, -0.70710678118f}; return s; }

   private:
    cfloat state_[2]{{1.0f, 0.0f}, {0.0f, 0.0f}};
    void force_normalize();
};

// ---- lowering context ----------------------------------------------------------------
// Offset and extra controls accumulated while a Gate / ControlGate is flattened.
struct LowerCtx {
    uint32_t offset = 0;
    std::vector<int32_t> controls;
};
void push_op(std::vector<aqsg_op>& out, const LowerCtx& lc, aqsg_op op);

// ---- QCircuit (quantum.h:350-469) --------------------------------------------------------
class QCircuit {
   public:
    friend class QSimulator;
    QCircuit() = delete;
    QCircuit(const QCircuit&) = default;
    QCircuit(QCircuit&&) = default;
    QCircuit& operator=(const QCircuit&) = default;
    QCircuit& operator=(QCircuit&&) = default;
    explicit QCircuit(uint32_t qubit_count);

    template <typename T>
    friend QCircuit& operator<<(QCircuit& qc, const T& gate);
    template <typename T>
    friend QCircuit& operator<<(QCircuit& qc, const std::vector<T>& gates);

    uint32_t qubit_count() const noexcept { return qubits_; }
    uint32_t state_count() const noexcept { return fast_pow2(qubits_); }
    // The 2^n x 2^n circuit matrix (row-major) of the compiled gates, built by
    // the engine on request for n <= 13 (quantum.h:403-411).
    const std::vector<std::complex<float>>& circuit() const;
    auto& gate_list() noexcept { return gate_list_; }
    const auto& gate_list() const noexcept { return gate_list_; }
    std::string& representation() noexcept { return representation_; }
    const std::string& representation() const noexcept { return representation_; }
    std::size_t cached_index() const noexcept { return cached_index_; }

    // Fold gates [cached_index, end) into the compiled program (quantum.cpp:199-210).
    void compile();
    void clear();
    void clear_cache();
    friend bool operator==(const QCircuit& lhs, const QCircuit& rhs);

    // Engine ops of gates [begin, end).
    std::vector<aqsg_op> lower(std::size_t begin, std::size_t end, const LowerCtx& lc = {}) const;
    // Engine ops of the compiled prefix.
    const std::vector<aqsg_op>& program() const { return program_; }
    // Fold one gate into the compiled program without listing it (what a
    // gate's operator()(QCircuit&) does in the reference).
    void apply_to_program(const QGate& gate);

   private:
    std::vector<std::shared_ptr<QGate>> gate_list_;
    std::string representation_;
    uint32_t qubits_ = 0;
    std::size_t cached_index_ = 0;
    std::vector<aqsg_op> program_;
    // program_ fused into <= fused_k_-qubit unitaries (aqsg_compile), built on
    // the first simulate after a change
    mutable std::shared_ptr<aqsg_program_s> fused_;
    mutable std::size_t fused_len_ = 0;
    mutable int fused_k_ = 0;
    mutable std::vector<std::complex<float>> matrix_;
    mutable bool matrix_valid_ = false;
};

class QNoise {};

// ---- QSimulator (quantum.h:482-742) --------------------------------------------------------
class QSimulator {
   public:
    enum class Basis : int8_t { Z, Y, X };

    explicit QSimulator(uint32_t qubit_count, const QState& initial_state = QState::zero(),
                        const QNoise& noise_generator = QNoise{});
    explicit QSimulator(uint32_t qubit_count, std::vector<QState> initial_states,
                        const QNoise& noise_generator = QNoise{});
    explicit QSimulator(uint32_t qubit_count, const std::vector<std::complex<float>>& statevector,
                        const QNoise& noise_generator = QNoise{});
    QSimulator(const QSimulator&) = delete;
    QSimulator& operator=(const QSimulator&) = delete;
    ~QSimulator();

    void generate_statevector();
    void simulate(const QCircuit& circuit);
    bool peek_measure(uint32_t qubit) const;
    bool measure(uint32_t qubit);
    uint32_t measure_all();
    uint32_t peek_measure_all() const;
    std::array<uint32_t, 2> profile_measure(uint32_t qubit, uint32_t rep_count) const;
    std::vector<uint32_t> profile_measure_all(uint32_t rep_count) const;

    QState& qubit(uint32_t index) noexcept { assert(index < qubit_count()); return states_[index]; }
    const QState& qubit(uint32_t index) const noexcept { assert(index < qubit_count()); return states_[index]; }
    cfloat state(uint32_t state) const;
    float qubit_probability_true(uint32_t qubit) const;
    float qubit_probability_false(uint32_t qubit) const { return 1.f - qubit_probability_true(qubit); }
    float state_probability(uint32_t state) const;
    std::vector<float> probabilities() const;
    uint32_t qubit_count() const noexcept { return qubits_; }
    uint32_t state_count() const noexcept { return fast_pow2(qubits_); }
    Basis get_basis() const noexcept { return basis_; }
    void set_basis(Basis basis);
    // Host copy of the register (replaces the af::array reference).
    std::vector<std::complex<float>> statevector() const;
    // The engine register.
    aqsg_state handle() const noexcept { return sv_; }
    // <psi|P|psi> for Pauli strings of qubit_count() letters from i/x/y/z,
    // letter j on qubit j (the strings decompose_hamiltonian returns), summed
    // in FP64 on the device.  (Extension.)
    std::vector<std::complex<double>> pauli_expectations(const std::vector<std::string>& paulis) const;
    // sum_s c_s <psi|P_s|psi> for a decomposed Hamiltonian.  (Extension.)
    std::complex<double> expectation(const std::vector<std::pair<std::string, cfloat>>& hamiltonian) const;

   private:
    std::vector<QState> states_;
    aqsg_state sv_ = nullptr;
    QNoise noise_;
    uint32_t qubits_;
    Basis basis_ = Basis::Z;
};

// ---- QGate plugin interface (quantum.h:748-824) ----------------------------------------------
class QGate {
   public:
    virtual ~QGate() = default;
    // Left-multiply the circuit's compiled matrix by this gate.
    virtual QCircuit& operator()(QCircuit& qc) const;
    virtual std::string to_string() const = 0;
    virtual uint32_t type() const noexcept = 0;
    virtual bool check(const QCircuit& qc) const = 0;
    virtual bool operator==(const QGate& rhs) const noexcept = 0;
    // Emit this gate's engine ops (the engine's replacement of operator()).
    virtual void lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const = 0;

   protected:
    enum class GateTypes : uint32_t {
        Barrier, X, Y, Z, Hadamard, Phase, Swap, RotX, RotY, RotZ, CX, CY, CZ, CHadamard,
        CPhase, CSwap, CRotX, CRotY, CRotZ, CCX, Or, Circuit, ControlCircuit
    };
};

template <typename T>
QCircuit& operator<<(QCircuit& qc, const T& gate) {
    static_assert(std::is_base_of<QGate, T>::value, "Gate must inherit from QGate class");
    if (gate.check(qc)) {
        qc.representation_.append(gate.to_string());
        qc.gate_list().push_back(std::make_shared<T>(gate));
        qc.matrix_valid_ = false;
    }
    return qc;
}

template <typename T>
QCircuit& operator<<(QCircuit& qc, const std::vector<T>& gates) {
    static_assert(std::is_base_of<QGate, T>::value, "Gate must inherit from QGate class");
    for (const auto& gate : gates) qc << gate;
    return qc;
}

#define AQS_GATE_COMMON(NAME, TYPE)                                                    \
    std::string to_string() const override;                                            \
    bool check(const QCircuit&) const override;                                        \
    uint32_t type() const noexcept override { return static_cast<uint32_t>(GateTypes::TYPE); } \
    bool operator==(const QGate& rhs) const noexcept override;                         \
    void lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const override;          \
    static constexpr uint32_t static_type() noexcept { return static_cast<uint32_t>(GateTypes::TYPE); }

class Barrier : public QGate {
   public:
    Barrier(bool visible_ = true) noexcept : visible{visible_} {}
    std::string to_string() const override { return visible ? "B;" : "P;"; }
    bool check(const QCircuit&) const override { return true; }
    uint32_t type() const noexcept override { return static_cast<uint32_t>(GateTypes::Barrier); }
    bool operator==(const QGate& rhs) const noexcept override { return type() == rhs.type(); }
    void lower(std::vector<aqsg_op>&, const LowerCtx&) const override {}
    static constexpr uint32_t static_type() noexcept { return static_cast<uint32_t>(GateTypes::Barrier); }
    bool visible = true;
};

class X : public QGate {
   public:
    X(uint32_t target_qubit_) noexcept : target_qubit{target_qubit_} {}
    AQS_GATE_COMMON(X, X)
    static const QCircuit& gate();
    uint32_t target_qubit;
};
using Not = X;

class Y : public QGate {
   public:
    Y(uint32_t target_qubit_) noexcept : target_qubit{target_qubit_} {}
    AQS_GATE_COMMON(Y, Y)
    static const QCircuit& gate();
    uint32_t target_qubit;
};

class Z : public QGate {
   public:
    Z(uint32_t target_qubit_) noexcept : target_qubit{target_qubit_} {}
    AQS_GATE_COMMON(Z, Z)
    static const QCircuit& gate();
    uint32_t target_qubit;
};

class RotX : public QGate {
   public:
    RotX(uint32_t target_qubit_, float angle_) noexcept : target_qubit{target_qubit_}, angle{angle_} {}
    AQS_GATE_COMMON(RotX, RotX)
    static QCircuit gate(float angle);
    uint32_t target_qubit;
    float angle;
};

class RotY : public QGate {
   public:
    RotY(uint32_t target_qubit_, float angle_) noexcept : target_qubit{target_qubit_}, angle{angle_} {}
    AQS_GATE_COMMON(RotY, RotY)
    static QCircuit gate(float angle);
    uint32_t target_qubit;
    float angle;
};

class RotZ : public QGate {
   public:
    RotZ(uint32_t target_qubit_, float angle_) noexcept : target_qubit{target_qubit_}, angle{angle_} {}
    AQS_GATE_COMMON(RotZ, RotZ)
    static QCircuit gate(float angle);
    uint32_t target_qubit;
    float angle;
};

class H : public QGate {
   public:
    H(uint32_t target_qubit_) noexcept : target_qubit{target_qubit_} {}
    AQS_GATE_COMMON(H, Hadamard)
    static const QCircuit& gate();
    uint32_t target_qubit;
};

class Phase : public QGate {
   public:
    Phase(uint32_t target_qubit_, float angle_) noexcept : target_qubit{target_qubit_}, angle{angle_} {}
    AQS_GATE_COMMON(Phase, Phase)
    static QCircuit gate(float angle);
    uint32_t target_qubit;
    float angle;
};

class Swap : public QGate {
   public:
    Swap(uint32_t a, uint32_t b) noexcept : target_qubit_A{a}, target_qubit_B{b} {}
    AQS_GATE_COMMON(Swap, Swap)
    uint32_t target_qubit_A;
    uint32_t target_qubit_B;
};

#define AQS_CTRL_GATE(NAME, TYPE)                                                              \
    class NAME : public QGate {                                                                \
       public:                                                                                 \
        NAME(uint32_t control_qubit_, uint32_t target_qubit_) noexcept                         \
            : control_qubit{control_qubit_}, target_qubit{target_qubit_} {}                    \
        AQS_GATE_COMMON(NAME, TYPE)                                                            \
        uint32_t control_qubit;                                                                \
        uint32_t target_qubit;                                                                 \
    };

AQS_CTRL_GATE(CX, CX)
AQS_CTRL_GATE(CY, CY)
AQS_CTRL_GATE(CZ, CZ)
AQS_CTRL_GATE(CH, CHadamard)
using CNot = CX;
using Xor = CX;

#define AQS_CTRL_ANGLE_GATE(NAME, TYPE)                                                        \
    class NAME : public QGate {                                                                \
       public:                                                                                 \
        NAME(uint32_t control_qubit_, uint32_t target_qubit_, float angle_) noexcept           \
            : control_qubit{control_qubit_}, target_qubit{target_qubit_}, angle{angle_} {}     \
        AQS_GATE_COMMON(NAME, TYPE)                                                            \
        uint32_t control_qubit;                                                                \
        uint32_t target_qubit;                                                                 \
        float angle;                                                                           \
    };

AQS_CTRL_ANGLE_GATE(CPhase, CPhase)
AQS_CTRL_ANGLE_GATE(CRotX, CRotX)
AQS_CTRL_ANGLE_GATE(CRotY, CRotY)
AQS_CTRL_ANGLE_GATE(CRotZ, CRotZ)

class CSwap : public QGate {
   public:
    CSwap(uint32_t c, uint32_t a, uint32_t b) noexcept : control_qubit{c}, target_qubit_A{a}, target_qubit_B{b} {}
    AQS_GATE_COMMON(CSwap, CSwap)
    uint32_t control_qubit;
    uint32_t target_qubit_A;
    uint32_t target_qubit_B;
};

class CCNot : public QGate {
   public:
    CCNot(uint32_t a, uint32_t b, uint32_t t) noexcept : control_qubit_A{a}, control_qubit_B{b}, target_qubit{t} {}
    AQS_GATE_COMMON(CCNot, CCX)
    uint32_t control_qubit_A;
    uint32_t control_qubit_B;
    uint32_t target_qubit;
};
using And = CCNot;

class Or : public QGate {
   public:
    Or(uint32_t a, uint32_t b, uint32_t t) noexcept : control_qubit_A{a}, control_qubit_B{b}, target_qubit{t} {}
    AQS_GATE_COMMON(Or, Or)
    uint32_t control_qubit_A;
    uint32_t control_qubit_B;
    uint32_t target_qubit;
};

// Embeds a sub-circuit at qubits [target_qubit_begin, +qubit_count).
// quantum.h:1522-1553, quantum.cpp:1705-1821.
class Gate : public QGate {
   public:
    Gate(const QCircuit& circuit_, uint32_t target_qubit_begin_, std::string name = "");
    AQS_GATE_COMMON(Gate, Circuit)
    std::shared_ptr<QCircuit> internal_circuit;
    std::string representation;
    uint32_t qubit_count;
    uint32_t target_qubit_begin;
};

// As Gate, acting only where control_qubit is |1>.  quantum.h:1555-1589,
// quantum.cpp:1823-1960.
class ControlGate : public QGate {
   public:
    ControlGate(const QCircuit& circuit_, uint32_t control_qubit_, uint32_t target_qubit_begin_,
                std::string name = "");
    AQS_GATE_COMMON(ControlGate, ControlCircuit)
    std::shared_ptr<QCircuit> internal_circuit;
    std::string representation;
    uint32_t qubit_count;
    uint32_t control_qubit;
    uint32_t target_qubit_begin;
};

// 2x2 operations on a single QState (quantum.h:1597-1653), in float.
QState X_op(const QState& state);
QState Y_op(const QState& state);
QState Z_op(const QState& state);
QState RotateX_op(const QState& state, float angle);
QState RotateY_op(const QState& state, float angle);
QState RotateZ_op(const QState& state, float angle);
QState Hadamard_op(const QState& state);
QState Phase_op(const QState& state, float angle);

}  // namespace aqs
