// quantum.cpp — the aqs:: C++ API on the GB300 engine.
//
// Host logic mirrors arrayfire/afQuantumSim src/quantum.cpp (validation,
// messages, representation strings, measurement rules); every state-vector
// computation goes through the C ABI of libaqsg.so.
#include "aqs/quantum.h"

#include <cmath>
#include <cstring>
#include <mutex>
#include <sstream>
#include <unordered_map>

namespace aqs {

namespace {

std::mutex g_mu;
aqsg_ctx g_ctx = nullptr;
int g_device = 0;
std::mt19937 g_rng{std::random_device{}()};
int g_fusion = 5;
std::uniform_real_distribution<float> g_lin{0.0f, 1.0f};
std::unordered_map<std::string, std::shared_ptr<QCircuit>> g_cache;

const char* kAt = "Cannot add gate at the given qubit position";
const char* kCtlTgt = "Control qubit cannot be the same as the target qubit";
const char* kSwapSame = "Cannot use the swap gate on the same target qubits";
const char* kNotSupported = "Gate not supported for given simulation";

float uniform() {
    std::lock_guard<std::mutex> lock(g_mu);
    return g_lin(g_rng);
}

aqsg_op make(int kind, std::initializer_list<uint32_t> qubits, float angle = 0.f) {
    aqsg_op op;
    std::memset(&op, 0, sizeof(op));
    op.kind = kind;
    int i = 0;
    for (uint32_t q : qubits) op.qubits[i++] = (int32_t)q;
    op.num_qubits = i;
    op.angle = angle;
    return op;
}

void check_call(int rc) {
    if (rc != AQSG_OK) throw_status(rc);
}

}  // namespace

void throw_status(int rc) {
    char buf[512];
    aqsg_last_error(buf, sizeof(buf));
    switch (rc) {
        case AQSG_ERR_OUT_OF_RANGE: throw std::out_of_range{buf};
        case AQSG_ERR_INVALID_ARGUMENT:
        case AQSG_ERR_NULL: throw std::invalid_argument{buf};
        case AQSG_ERR_DOMAIN: throw std::domain_error{buf};
        default: throw std::runtime_error{buf};
    }
}

void initialize(int argc, char** argv) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_device = (argc > 1 && argv) ? std::stoi(argv[1]) : 0;
    if (g_ctx) {
        aqsg_shutdown(g_ctx);
        g_ctx = nullptr;
    }
    check_call(aqsg_init(g_device, &g_ctx));
}

void shutdown() {
    std::lock_guard<std::mutex> lock(g_mu);
    if (g_ctx) check_call(aqsg_shutdown(g_ctx));
    g_ctx = nullptr;
}

aqsg_ctx engine() {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_ctx) check_call(aqsg_init(g_device, &g_ctx));
    return g_ctx;
}

void clear_circuit_cache() { g_cache.clear(); }

void set_fusion_qubits(int k) {
    if (k < 0 || k > AQSG_MAX_UNITARY_QUBITS)
        throw std::invalid_argument{"Fusion width must be 0 to 5 qubits"};
    std::lock_guard<std::mutex> lock(g_mu);
    g_fusion = k;
}

int fusion_qubits() {
    std::lock_guard<std::mutex> lock(g_mu);
    return g_fusion;
}

void seed(uint64_t s) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_rng.seed((std::mt19937::result_type)s);
}

// ---- QState ------------------------------------------------------------------------

QState::QState(const std::complex<float>& zero_state, const std::complex<float>& one_state)
    : state_{cfloat{zero_state.real(), zero_state.imag()}, cfloat{one_state.real(), one_state.imag()}} {
    force_normalize();
}

QState::QState(const std::array<std::complex<float>, 2>& s) : QState(s[0], s[1]) {}

QState& QState::set(const std::complex<float>& zero_state, const std::complex<float>& one_state) {
    state_[0] = cfloat{zero_state.real(), zero_state.imag()};
    state_[1] = cfloat{one_state.real(), one_state.imag()};
    force_normalize();
    return *this;
}

bool QState::peek_measure() const { return uniform() < probability_true(); }

bool QState::measure() {
    const bool m = peek_measure();
    state_[m] = cfloat{1.f};
    state_[!m] = cfloat{0.f};
    return m;
}

std::array<uint32_t, 2> QState::profile_measure(uint32_t rep_count) const {
    uint32_t ones = 0;
    for (uint32_t i = 0; i < rep_count; ++i) ones += peek_measure() ? 1u : 0u;
    return {rep_count - ones, ones};
}

// quantum.cpp:145-157: float norm, throws on a null state
void QState::force_normalize() {
    const float mag2 = state_[0].real * state_[0].real + state_[0].imag * state_[0].imag +
                       state_[1].real * state_[1].real + state_[1].imag * state_[1].imag;
    if (mag2 == 0.f) throw std::invalid_argument{"Cannot normalize a null state"};
    const float mag = std::sqrt(mag2);
    state_[0] = state_[0] / mag;
    state_[1] = state_[1] / mag;
}

// ---- lowering ------------------------------------------------------------------------

static int arity(int kind) {
    switch (kind) {
        case AQSG_OP_BARRIER: return 0;
        case AQSG_OP_X: case AQSG_OP_Y: case AQSG_OP_Z: case AQSG_OP_H: case AQSG_OP_PHASE:
        case AQSG_OP_RX: case AQSG_OP_RY: case AQSG_OP_RZ: return 1;
        case AQSG_OP_CSWAP: case AQSG_OP_CCX: case AQSG_OP_OR: return 3;
        case AQSG_OP_UNITARY: return -1;
        default: return 2;
    }
}

void push_op(std::vector<aqsg_op>& out, const LowerCtx& lc, aqsg_op op) {
    const int na = op.kind == AQSG_OP_UNITARY ? op.num_qubits : arity(op.kind);
    for (int i = 0; i < na; ++i) op.qubits[i] += (int32_t)lc.offset;
    for (int i = 0; i < op.num_controls; ++i) op.controls[i] += (int32_t)lc.offset;
    for (int32_t c : lc.controls) {
        if (op.num_controls >= AQSG_OP_MAX_CONTROLS)
            throw std::invalid_argument{"Too many nested control qubits"};
        op.controls[op.num_controls] = c;
        op.control_values |= 1u << op.num_controls;
        op.num_controls++;
    }
    out.push_back(op);
}

// ---- QCircuit ------------------------------------------------------------------------

QCircuit::QCircuit(uint32_t qubit_count) : qubits_{qubit_count} {
    if (qubit_count < 1) throw std::invalid_argument{"Circuit must contain at least 1 qubit"};
    if (qubit_count > max_qubit_count)
        throw std::invalid_argument{"Maximum qubit count supported is " + std::to_string(max_qubit_count)};
}

void QCircuit::clear() {
    clear_cache();
    gate_list_.clear();
}

void QCircuit::clear_cache() {
    cached_index_ = 0;
    program_.clear();
    fused_.reset();
    matrix_valid_ = false;
}

bool operator==(const QCircuit& lhs, const QCircuit& rhs) {
    if (lhs.qubit_count() != rhs.qubit_count()) return false;
    if (lhs.gate_list().size() != rhs.gate_list().size()) return false;
    if (lhs.representation() != rhs.representation()) return false;
    for (std::size_t i = 0; i < lhs.gate_list().size(); ++i)
        if (lhs.gate_list()[i] != rhs.gate_list()[i]) return false;
    return true;
}

std::vector<aqsg_op> QCircuit::lower(std::size_t begin, std::size_t end, const LowerCtx& lc) const {
    std::vector<aqsg_op> out;
    for (std::size_t i = begin; i < end && i < gate_list_.size(); ++i) gate_list_[i]->lower(out, lc);
    return out;
}

void QCircuit::compile() {
    if (cached_index_ != gate_list_.size()) {
        auto ops = lower(cached_index_, gate_list_.size());
        program_.insert(program_.end(), ops.begin(), ops.end());
        cached_index_ = gate_list_.size();
        matrix_valid_ = false;
    }
}

void QCircuit::apply_to_program(const QGate& gate) {
    gate.lower(program_, {});
    matrix_valid_ = false;
}

const std::vector<std::complex<float>>& QCircuit::circuit() const {
    if (matrix_valid_) return matrix_;
    if (qubits_ > 13)
        throw std::runtime_error{"Circuit matrix is only built for up to 13 qubits"};
    // U (x) I applied to sum_k |k>|k> leaves U_ik at index i * 2^n + k: one
    // 2n-qubit register holds the whole matrix, row-major.
    const uint64_t N = state_count();
    std::vector<std::complex<float>> eye(N * N, {0.f, 0.f});
    for (uint64_t k = 0; k < N; ++k) eye[k * N + k] = 1.f;
    aqsg_state st = nullptr;
    check_call(aqsg_state_alloc(engine(), (int)(2 * qubits_), AQSG_C64, &st));
    int rc = aqsg_state_upload(st, eye.data(), 0);
    if (rc == AQSG_OK && !program_.empty())
        rc = aqsg_apply_ops(st, program_.data(), (int)program_.size(), -1);
    if (rc == AQSG_OK) rc = aqsg_state_download(st, eye.data());
    aqsg_state_free(st);
    check_call(rc);
    matrix_ = std::move(eye);
    matrix_valid_ = true;
    return matrix_;
}

QCircuit& QGate::operator()(QCircuit& qc) const {
    if (check(qc)) qc.apply_to_program(*this);
    return qc;
}

// ---- QSimulator ------------------------------------------------------------------------

QSimulator::QSimulator(uint32_t qubit_count, const QState& initial_state, const QNoise& noise)
    : states_(qubit_count, initial_state), noise_{noise}, qubits_{qubit_count} {
    check_call(aqsg_state_alloc(engine(), (int)qubit_count, AQSG_C64, &sv_));
    if (initial_state == QState::zero())
        check_call(aqsg_state_set_basis_index(sv_, 0));
    else if (initial_state == QState::one())
        check_call(aqsg_state_set_basis_index(sv_, state_count() - 1));
    else
        generate_statevector();
}

QSimulator::QSimulator(uint32_t qubit_count, std::vector<QState> initial_states, const QNoise& noise)
    : states_(std::move(initial_states)), noise_{noise}, qubits_{qubit_count} {
    if (qubit_count != states_.size())
        throw std::invalid_argument{
            "The number of initial states must match the number of qubits in the circuit"};
    check_call(aqsg_state_alloc(engine(), (int)qubit_count, AQSG_C64, &sv_));
    generate_statevector();
}

QSimulator::QSimulator(uint32_t qubit_count, const std::vector<std::complex<float>>& statevector,
                       const QNoise& noise)
    : states_(qubit_count), noise_{noise}, qubits_{qubit_count} {
    if (statevector.size() != fast_pow2(qubit_count))
        throw std::invalid_argument{"Invalid initial statevector shape"};
    check_call(aqsg_state_alloc(engine(), (int)qubit_count, AQSG_C64, &sv_));
    const int rc = aqsg_state_upload(sv_, statevector.data(), 1);
    if (rc != AQSG_OK) {
        aqsg_state_free(sv_);
        sv_ = nullptr;
        if (rc == AQSG_ERR_INVALID_ARGUMENT) throw std::invalid_argument{"Cannot have a null statevector"};
        throw_status(rc);
    }
}

QSimulator::~QSimulator() {
    if (sv_) aqsg_state_free(sv_);
}

void QSimulator::generate_statevector() {
    std::vector<float> amps(4 * qubits_);
    for (uint32_t i = 0; i < qubits_; ++i) {
        amps[4 * i] = states_[i][0].real;
        amps[4 * i + 1] = states_[i][0].imag;
        amps[4 * i + 2] = states_[i][1].real;
        amps[4 * i + 3] = states_[i][1].imag;
    }
    check_call(aqsg_state_set_product(sv_, amps.data()));
}

// quantum.cpp:277-291: compiled prefix, then the remaining gates in order.
// The compiled prefix runs as fused unitaries of fusion_qubits() qubits.
void QSimulator::simulate(const QCircuit& circuit) {
    if (circuit.qubit_count() != qubits_)
        throw std::invalid_argument{"Number of qubit states and circuit input qubit states do not match"};
    const auto& prog = circuit.program();
    auto rest = circuit.lower(circuit.cached_index(), circuit.gate_list().size());
    const int k = fusion_qubits();
    if (k > 0 && !prog.empty()) {
        if (!circuit.fused_ || circuit.fused_len_ != prog.size() || circuit.fused_k_ != k) {
            aqsg_program p = nullptr;
            check_call(aqsg_compile((int)qubits_, AQSG_C64, prog.data(), (int)prog.size(), k, &p));
            circuit.fused_.reset(p, [](aqsg_program q) { aqsg_program_free(q); });
            circuit.fused_len_ = prog.size();
            circuit.fused_k_ = k;
        }
        check_call(aqsg_run_program(sv_, circuit.fused_.get(), -1));
    } else if (!prog.empty()) {
        check_call(aqsg_apply_ops(sv_, prog.data(), (int)prog.size(), -1));
    }
    if (!rest.empty()) check_call(aqsg_apply_ops(sv_, rest.data(), (int)rest.size(), -1));
}

bool QSimulator::peek_measure(uint32_t qubit) const {
    if (qubit >= qubit_count()) throw std::out_of_range{"Cannot measure the state of the given qubit"};
    const float prob = qubit_probability_true(qubit);
    return uniform() < prob;
}

bool QSimulator::measure(uint32_t qubit) {
    if (qubit >= qubit_count()) throw std::out_of_range{"Cannot measure the state of the given qubit"};
    int outcome = 0;
    check_call(aqsg_collapse_qubit(sv_, (int)qubit, (double)uniform(), &outcome, nullptr));
    return outcome != 0;
}

uint32_t QSimulator::peek_measure_all() const {
    const double u = uniform();
    uint64_t k = 0;
    check_call(aqsg_sample(sv_, &u, 1, AQSG_SAMPLE_REFERENCE, &k));
    return (uint32_t)k;
}

uint32_t QSimulator::measure_all() {
    const uint32_t k = peek_measure_all();
    check_call(aqsg_state_set_basis_index(sv_, k));
    return k;
}

float QSimulator::qubit_probability_true(uint32_t qubit) const {
    if (qubit >= qubit_count()) throw std::out_of_range{"Cannot obtain probability of the given qubit"};
    double p = 0;
    check_call(aqsg_qubit_prob(sv_, (int)qubit, &p));
    return (float)p;
}

float QSimulator::state_probability(uint32_t state) const {
    if (state >= state_count()) throw std::out_of_range{"Cannot obtain probability of the given state"};
    const cfloat v = this->state(state);
    return v.real * v.real + v.imag * v.imag;
}

cfloat QSimulator::state(uint32_t k) const {
    float a[2];
    check_call(aqsg_state_download_range(sv_, k, 1, a));
    return {a[0], a[1]};
}

std::vector<float> QSimulator::probabilities() const {
    std::vector<float> out(state_count());
    check_call(aqsg_probs(sv_, out.data(), 0));
    return out;
}

std::vector<std::complex<double>> QSimulator::pauli_expectations(const std::vector<std::string>& paulis) const {
    std::string all;
    all.reserve(paulis.size() * qubits_);
    for (const auto& p : paulis) {
        if (p.size() != qubits_)
            throw std::invalid_argument{"Pauli string length does not match the qubit count"};
        all += p;
    }
    std::vector<double> raw(2 * paulis.size());
    if (!paulis.empty()) check_call(aqsg_expect_pauli(sv_, all.data(), (int)paulis.size(), raw.data()));
    std::vector<std::complex<double>> out(paulis.size());
    for (std::size_t i = 0; i < out.size(); ++i) out[i] = {raw[2 * i], raw[2 * i + 1]};
    return out;
}

std::complex<double> QSimulator::expectation(const std::vector<std::pair<std::string, cfloat>>& hamiltonian) const {
    std::vector<std::string> strings;
    strings.reserve(hamiltonian.size());
    for (const auto& term : hamiltonian) strings.push_back(term.first);
    const auto vals = pauli_expectations(strings);
    std::complex<double> e = 0;
    for (std::size_t i = 0; i < vals.size(); ++i)
        e += std::complex<double>(hamiltonian[i].second.real, hamiltonian[i].second.imag) * vals[i];
    return e;
}

std::vector<std::complex<float>> QSimulator::statevector() const {
    std::vector<std::complex<float>> out(state_count());
    check_call(aqsg_state_download(sv_, out.data()));
    return out;
}

std::vector<uint32_t> QSimulator::profile_measure_all(uint32_t rep_count) const {
    std::vector<double> u(rep_count);
    for (auto& x : u) x = uniform();
    std::vector<uint64_t> k(rep_count);
    if (rep_count) check_call(aqsg_sample(sv_, u.data(), rep_count, AQSG_SAMPLE_REFERENCE, k.data()));
    // a draw above the total probability matches no state; the reference
    // writes it past the end of its output (quantum.cpp:494-498), here it is
    // dropped
    std::vector<double> total(1);
    check_call(aqsg_norm2(sv_, total.data()));
    std::vector<uint32_t> count(state_count(), 0);
    for (uint32_t i = 0; i < rep_count; ++i)
        if (u[i] < total[0]) count[k[i]]++;
    return count;
}

std::array<uint32_t, 2> QSimulator::profile_measure(uint32_t qubit, uint32_t rep_count) const {
    if (qubit >= qubit_count()) throw std::out_of_range{"Cannot profile measurement of the given qubit"};
    const float p1 = qubit_probability_true(qubit);
    uint32_t ones = 0;
    for (uint32_t i = 0; i < rep_count; ++i) ones += (uniform() < p1) ? 1u : 0u;
    return {rep_count - ones, ones};
}

// quantum.cpp:416-465.  The change of basis is a 2x2 matrix on every qubit;
// as in the reference, leaving the Y basis uses the X-to-Z matrix (the Y case
// of its switch falls through).
void QSimulator::set_basis(Basis basis) {
    if (basis == basis_) return;
    using C = std::complex<double>;
    const double h = 0.70710678118;
    const C z_to_x[4] = {h, h, h, -h};
    const C z_to_y[4] = {h, h, C(0, -h), C(0, h)};
    auto inv2 = [](const C* m, C* out) {
        const C det = m[0] * m[3] - m[1] * m[2];
        out[0] = m[3] / det;
        out[1] = -m[1] / det;
        out[2] = -m[2] / det;
        out[3] = m[0] / det;
    };
    auto mul2 = [](const C* a, const C* b, C* out) {
        out[0] = a[0] * b[0] + a[1] * b[2];
        out[1] = a[0] * b[1] + a[1] * b[3];
        out[2] = a[2] * b[0] + a[3] * b[2];
        out[3] = a[2] * b[1] + a[3] * b[3];
    };
    C m[4] = {1, 0, 0, 1};
    if (basis_ != Basis::Z) inv2(z_to_x, m);  // Y and X both take x_to_z
    C t[4];
    if (basis == Basis::Y) { mul2(z_to_y, m, t); std::copy(t, t + 4, m); }
    if (basis == Basis::X) { mul2(z_to_x, m, t); std::copy(t, t + 4, m); }
    double mat[8];
    for (int i = 0; i < 4; ++i) { mat[2 * i] = m[i].real(); mat[2 * i + 1] = m[i].imag(); }
    std::vector<aqsg_op> ops;
    for (uint32_t q = 0; q < qubits_; ++q) {
        aqsg_op op = make(AQSG_OP_UNITARY, {q});
        op.matrix = mat;
        ops.push_back(op);
    }
    check_call(aqsg_apply_ops(sv_, ops.data(), (int)ops.size(), -1));
    basis_ = basis;
}

// ---- gates: representation strings (quantum.cpp:569-1677) ----------------------------------

#define Q(x) std::to_string(x)
std::string X::to_string() const { return "X,0,1:" + Q(target_qubit) + ";"; }
std::string Y::to_string() const { return "Y,0,1:" + Q(target_qubit) + ";"; }
std::string Z::to_string() const { return "Z,0,1:" + Q(target_qubit) + ";"; }
std::string RotX::to_string() const { return "RotX,0,1:" + Q(target_qubit) + ";"; }
std::string RotY::to_string() const { return "RotY,0,1:" + Q(target_qubit) + ";"; }
std::string RotZ::to_string() const { return "RotZ,0,1:" + Q(target_qubit) + ";"; }
std::string H::to_string() const { return "H,0,1:" + Q(target_qubit) + ";"; }
static std::string phase_name(float angle) {
    if (angle == pi / 2) return "S";
    if (angle == -pi / 2) return "S†";
    if (angle == pi / 4) return "T";
    if (angle == -pi / 4) return "T†";
    return "Phase";
}
std::string Phase::to_string() const { return phase_name(angle) + ",0,1:" + Q(target_qubit) + ";"; }
std::string Swap::to_string() const { return "Swap,0,2:" + Q(target_qubit_A) + "," + Q(target_qubit_B) + ";"; }
std::string CX::to_string() const { return "X,1,1:" + Q(control_qubit) + "," + Q(target_qubit) + ";"; }
std::string CY::to_string() const { return "Y,1,1:" + Q(control_qubit) + "," + Q(target_qubit) + ";"; }
std::string CZ::to_string() const { return "Z,1,1:" + Q(control_qubit) + "," + Q(target_qubit) + ";"; }
std::string CH::to_string() const { return "H,1,1:" + Q(control_qubit) + "," + Q(target_qubit) + ";"; }
std::string CPhase::to_string() const {
    return phase_name(angle) + ",1,1:" + Q(control_qubit) + "," + Q(target_qubit) + ";";
}
// the reference writes the two swap targets without a separator (quantum.cpp:1322-1326)
std::string CSwap::to_string() const {
    return "Swap,1,2:" + Q(control_qubit) + "," + Q(target_qubit_A) + Q(target_qubit_B) + ";";
}
std::string CRotX::to_string() const { return "RotX,1,1:" + Q(control_qubit) + "," + Q(target_qubit) + ";"; }
std::string CRotY::to_string() const { return "RotY,1,1:" + Q(control_qubit) + "," + Q(target_qubit) + ";"; }
std::string CRotZ::to_string() const { return "RotZ,1,1:" + Q(control_qubit) + "," + Q(target_qubit) + ";"; }
std::string CCNot::to_string() const {
    return "X,2,1:" + Q(control_qubit_A) + "," + Q(control_qubit_B) + "," + Q(target_qubit) + ";";
}
// Or is drawn as its equivalent X / Toffoli / X network (quantum.cpp:1662-1677)
std::string Or::to_string() const {
    const std::string a = Q(control_qubit_A), b = Q(control_qubit_B), t = Q(target_qubit);
    return "P;X,0,1:" + a + ";X,0,1:" + b + ";X,0,1:" + t + ";X,2,1:" + a + "," + b + "," + t +
           ";X,0,1:" + a + ";X,0,1:" + b + ";P;";
}
#undef Q

// ---- gates: check() (quantum.cpp:533-1677) -----------------------------------------------

static void need_in(uint32_t q, uint32_t n) {
    if (q >= n) throw std::out_of_range{kAt};
}
#define ONE_QUBIT_CHECK(G) \
    bool G::check(const QCircuit& qc) const { need_in(target_qubit, qc.qubit_count()); return true; }
ONE_QUBIT_CHECK(X)
ONE_QUBIT_CHECK(Y)
ONE_QUBIT_CHECK(Z)
ONE_QUBIT_CHECK(RotX)
ONE_QUBIT_CHECK(RotY)
ONE_QUBIT_CHECK(RotZ)
ONE_QUBIT_CHECK(H)
ONE_QUBIT_CHECK(Phase)
#undef ONE_QUBIT_CHECK

bool Swap::check(const QCircuit& qc) const {
    const uint32_t n = qc.qubit_count();
    if (n < 2) throw std::domain_error{kNotSupported};
    need_in(target_qubit_A, n);
    need_in(target_qubit_B, n);
    if (target_qubit_A == target_qubit_B) throw std::invalid_argument{kSwapSame};
    return true;
}

#define TWO_QUBIT_CHECK(G)                                                \
    bool G::check(const QCircuit& qc) const {                            \
        const uint32_t n = qc.qubit_count();                              \
        if (n < 2) throw std::domain_error{kNotSupported};                \
        need_in(control_qubit, n);                                        \
        need_in(target_qubit, n);                                         \
        if (control_qubit == target_qubit) throw std::invalid_argument{kCtlTgt}; \
        return true;                                                      \
    }
TWO_QUBIT_CHECK(CX)
TWO_QUBIT_CHECK(CY)
TWO_QUBIT_CHECK(CZ)
TWO_QUBIT_CHECK(CH)
TWO_QUBIT_CHECK(CPhase)
#undef TWO_QUBIT_CHECK

#define CROT_CHECK(G)                                                                   \
    bool G::check(const QCircuit& qc) const {                                          \
        const uint32_t n = qc.qubit_count();                                            \
        if (target_qubit >= n || control_qubit >= n) throw std::out_of_range{kAt};      \
        if (target_qubit == control_qubit) throw std::invalid_argument{kCtlTgt};        \
        return true;                                                                    \
    }
CROT_CHECK(CRotX)
CROT_CHECK(CRotY)
CROT_CHECK(CRotZ)
#undef CROT_CHECK

bool CSwap::check(const QCircuit& qc) const {
    const uint32_t n = qc.qubit_count();
    if (n < 3) throw std::domain_error{"Gate not supported for given circuit"};
    need_in(target_qubit_A, n);
    need_in(target_qubit_B, n);
    need_in(control_qubit, n);
    if (control_qubit == target_qubit_A || control_qubit == target_qubit_B)
        throw std::invalid_argument{kCtlTgt};
    if (target_qubit_A == target_qubit_B) throw std::invalid_argument{kSwapSame};
    return true;
}

#define TOFFOLI_CHECK(G)                                                                    \
    bool G::check(const QCircuit& qc) const {                                              \
        const uint32_t n = qc.qubit_count();                                                \
        if (n < 3) throw std::domain_error{kNotSupported};                                  \
        need_in(control_qubit_A, n);                                                        \
        need_in(control_qubit_B, n);                                                        \
        need_in(target_qubit, n);                                                           \
        if (control_qubit_A == target_qubit || control_qubit_B == target_qubit)            \
            throw std::invalid_argument{kCtlTgt};                                           \
        return true;                                                                        \
    }
TOFFOLI_CHECK(CCNot)
TOFFOLI_CHECK(Or)
#undef TOFFOLI_CHECK

// ---- gates: equality ------------------------------------------------------------------------

#define EQ1(G, ...)                                                        \
    bool G::operator==(const QGate& rhs) const noexcept {                 \
        if (type() != rhs.type()) return false;                           \
        const auto& o = static_cast<const G&>(rhs);                       \
        (void)o;                                                           \
        return __VA_ARGS__;                                                \
    }
EQ1(X, target_qubit == o.target_qubit)
EQ1(Y, target_qubit == o.target_qubit)
EQ1(Z, target_qubit == o.target_qubit)
EQ1(H, target_qubit == o.target_qubit)
EQ1(RotX, target_qubit == o.target_qubit && angle == o.angle)
EQ1(RotY, target_qubit == o.target_qubit && angle == o.angle)
EQ1(RotZ, target_qubit == o.target_qubit && angle == o.angle)
EQ1(Phase, target_qubit == o.target_qubit && angle == o.angle)
EQ1(Swap, target_qubit_A == o.target_qubit_A && target_qubit_B == o.target_qubit_B)
EQ1(CX, target_qubit == o.target_qubit && control_qubit == o.control_qubit)
EQ1(CY, target_qubit == o.target_qubit && control_qubit == o.control_qubit)
EQ1(CZ, target_qubit == o.target_qubit && control_qubit == o.control_qubit)
EQ1(CH, target_qubit == o.target_qubit && control_qubit == o.control_qubit)
EQ1(CPhase, target_qubit == o.target_qubit && control_qubit == o.control_qubit && angle == o.angle)
EQ1(CRotX, target_qubit == o.target_qubit && control_qubit == o.control_qubit && angle == o.angle)
EQ1(CRotY, target_qubit == o.target_qubit && control_qubit == o.control_qubit && angle == o.angle)
EQ1(CRotZ, target_qubit == o.target_qubit && control_qubit == o.control_qubit && angle == o.angle)
EQ1(CSwap, target_qubit_A == o.target_qubit_A && target_qubit_B == o.target_qubit_B &&
               control_qubit == o.control_qubit)
EQ1(CCNot, target_qubit == o.target_qubit && control_qubit_A == o.control_qubit_A &&
               control_qubit_B == o.control_qubit_B)
EQ1(Or, target_qubit == o.target_qubit && control_qubit_A == o.control_qubit_A &&
            control_qubit_B == o.control_qubit_B)
EQ1(Gate, target_qubit_begin == o.target_qubit_begin && internal_circuit == o.internal_circuit)
EQ1(ControlGate, target_qubit_begin == o.target_qubit_begin && control_qubit == o.control_qubit &&
                     internal_circuit == o.internal_circuit)
#undef EQ1

// ---- gates: lowering to engine ops -------------------------------------------------------------

void X::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const { push_op(out, lc, make(AQSG_OP_X, {target_qubit})); }
void Y::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const { push_op(out, lc, make(AQSG_OP_Y, {target_qubit})); }
void Z::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const { push_op(out, lc, make(AQSG_OP_Z, {target_qubit})); }
void H::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const { push_op(out, lc, make(AQSG_OP_H, {target_qubit})); }
void RotX::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const { push_op(out, lc, make(AQSG_OP_RX, {target_qubit}, angle)); }
void RotY::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const { push_op(out, lc, make(AQSG_OP_RY, {target_qubit}, angle)); }
void RotZ::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const { push_op(out, lc, make(AQSG_OP_RZ, {target_qubit}, angle)); }
void Phase::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const { push_op(out, lc, make(AQSG_OP_PHASE, {target_qubit}, angle)); }
void Swap::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const {
    push_op(out, lc, make(AQSG_OP_SWAP, {target_qubit_A, target_qubit_B}));
}
void CX::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const { push_op(out, lc, make(AQSG_OP_CX, {control_qubit, target_qubit})); }
void CY::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const { push_op(out, lc, make(AQSG_OP_CY, {control_qubit, target_qubit})); }
void CZ::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const { push_op(out, lc, make(AQSG_OP_CZ, {control_qubit, target_qubit})); }
void CH::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const { push_op(out, lc, make(AQSG_OP_CH, {control_qubit, target_qubit})); }
void CPhase::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const {
    push_op(out, lc, make(AQSG_OP_CPHASE, {control_qubit, target_qubit}, angle));
}
void CRotX::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const {
    push_op(out, lc, make(AQSG_OP_CRX, {control_qubit, target_qubit}, angle));
}
void CRotY::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const {
    push_op(out, lc, make(AQSG_OP_CRY, {control_qubit, target_qubit}, angle));
}
void CRotZ::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const {
    push_op(out, lc, make(AQSG_OP_CRZ, {control_qubit, target_qubit}, angle));
}
void CSwap::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const {
    push_op(out, lc, make(AQSG_OP_CSWAP, {control_qubit, target_qubit_A, target_qubit_B}));
}
void CCNot::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const {
    push_op(out, lc, make(AQSG_OP_CCX, {control_qubit_A, control_qubit_B, target_qubit}));
}
void Or::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const {
    push_op(out, lc, make(AQSG_OP_OR, {control_qubit_A, control_qubit_B, target_qubit}));
}

// Gate / ControlGate: the sub-circuit's gates, shifted by target_qubit_begin
// (and, for ControlGate, with one more control).  The reference multiplies by
// the sub-circuit's compiled matrix scattered into a 2^n x 2^n operator
// (quantum.cpp:1760-1814, 1888-1950); both give the same unitary.
void Gate::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const {
    LowerCtx sub{lc.offset + target_qubit_begin, lc.controls};
    auto ops = internal_circuit->lower(0, internal_circuit->gate_list().size(), sub);
    out.insert(out.end(), ops.begin(), ops.end());
}

void ControlGate::lower(std::vector<aqsg_op>& out, const LowerCtx& lc) const {
    LowerCtx sub{lc.offset + target_qubit_begin, lc.controls};
    sub.controls.push_back((int32_t)(lc.offset + control_qubit));
    auto ops = internal_circuit->lower(0, internal_circuit->gate_list().size(), sub);
    out.insert(out.end(), ops.begin(), ops.end());
}

// ---- static single-gate circuits (quantum.h X::gate() ...) ----------------------------------

template <typename G, typename... A>
static QCircuit one_gate(A... a) {
    QCircuit qc(1);
    qc << G(0, a...);
    qc.compile();
    return qc;
}
const QCircuit& X::gate() { static QCircuit qc = one_gate<X>(); return qc; }
const QCircuit& Y::gate() { static QCircuit qc = one_gate<Y>(); return qc; }
const QCircuit& Z::gate() { static QCircuit qc = one_gate<Z>(); return qc; }
const QCircuit& H::gate() { static QCircuit qc = one_gate<H>(); return qc; }
QCircuit RotX::gate(float angle) { return one_gate<RotX>(angle); }
QCircuit RotY::gate(float angle) { return one_gate<RotY>(angle); }
QCircuit RotZ::gate(float angle) { return one_gate<RotZ>(angle); }
QCircuit Phase::gate(float angle) { return one_gate<Phase>(angle); }

// ---- Gate / ControlGate ------------------------------------------------------------------------

// The global sub-circuit cache keyed by representation (quantum.cpp:64-65,
// 1710-1724): equal circuits share one stored copy.
static std::shared_ptr<QCircuit> cached(const QCircuit& c) {
    auto it = g_cache.find(c.representation());
    if (it == g_cache.end() || !(c == *it->second))
        g_cache[c.representation()] = std::make_shared<QCircuit>(c);
    return g_cache[c.representation()];
}

// Parse "name,controls,targets:q0,q1,...;" records and rewrite their qubit
// lists: controls shifted by `ctl_shift` with `extra_control` prepended when
// >= 0, targets shifted by `offset` (quantum.cpp:2034-2148).  Records without
// a qubit list ("P;", "B;") are kept as they are.
static std::string shift_representation(const std::string& rep, uint32_t offset, int64_t extra_control) {
    std::ostringstream out;
    std::size_t begin = 0;
    for (std::size_t end = rep.find(';', begin); end != std::string::npos; end = rep.find(';', begin)) {
        const std::string rec = rep.substr(begin, end - begin);
        begin = end + 1;
        const std::size_t comma = rec.find(',');
        const std::size_t colon = rec.find(':');
        if (comma == std::string::npos) {
            out << rec << ";";
            continue;
        }
        out << rec.substr(0, comma) << ",";
        std::string qubits;
        if (colon != std::string::npos) {
            const std::string counts = rec.substr(comma + 1, colon - comma - 1);  // "c,t"
            const std::size_t c2 = counts.find(',');
            if (extra_control >= 0)
                out << std::stoi(counts.substr(0, c2)) + 1 << counts.substr(c2) << ":";
            else
                out << counts << ":";
            qubits = rec.substr(colon + 1);
        } else {
            qubits = rec.substr(comma + 1);
        }
        if (extra_control >= 0) out << extra_control << ",";
        std::size_t qb = 0;
        bool first = true;
        while (qb <= qubits.size()) {
            std::size_t qe = qubits.find(',', qb);
            if (qe == std::string::npos) qe = qubits.size();
            if (!first) out << ",";
            out << std::stoi(qubits.substr(qb, qe - qb)) + (int)offset;
            first = false;
            qb = qe + 1;
        }
        out << ";";
    }
    return out.str();
}

static std::string named_representation(const std::string& name, uint32_t nq, uint32_t begin,
                                        int64_t control) {
    if (name.find_first_of(",;:") != std::string::npos)
        throw std::invalid_argument{"Name cannot contain commas, colons, nor semicolons"};
    std::ostringstream b;
    b << name << "," << (control >= 0 ? 1 : 0) << "," << nq << ":";
    if (control >= 0) b << control << ",";
    b << begin;
    for (uint32_t i = 1; i < nq; ++i) b << "," << i + begin;
    b << ";";
    return b.str();
}

Gate::Gate(const QCircuit& circuit_, uint32_t target_qubit_begin_, std::string name)
    : internal_circuit{cached(circuit_)},
      qubit_count{circuit_.qubit_count()},
      target_qubit_begin{target_qubit_begin_} {
    representation = name.empty() ? shift_representation(circuit_.representation(), target_qubit_begin_, -1)
                                  : named_representation(name, qubit_count, target_qubit_begin_, -1);
}

bool Gate::check(const QCircuit& qc) const {
    const uint32_t n = qc.qubit_count();
    if (target_qubit_begin >= n) throw std::out_of_range{kAt};
    if (target_qubit_begin + qubit_count > n) throw std::out_of_range{kAt};
    return true;
}

std::string Gate::to_string() const { return representation; }

ControlGate::ControlGate(const QCircuit& circuit_, uint32_t control_qubit_, uint32_t target_qubit_begin_,
                         std::string name)
    : internal_circuit{cached(circuit_)},
      qubit_count{circuit_.qubit_count()},
      control_qubit{control_qubit_},
      target_qubit_begin{target_qubit_begin_} {
    representation = name.empty()
                         ? shift_representation(circuit_.representation(), target_qubit_begin_, control_qubit_)
                         : named_representation(name, qubit_count, target_qubit_begin_, control_qubit_);
}

// quantum.cpp:1871-1886
bool ControlGate::check(const QCircuit& qc) const {
    const uint32_t n = qc.qubit_count();
    if (target_qubit_begin + qubit_count > n)
        throw std::out_of_range{"Gate must fit inside the circuit qubit count"};
    if (target_qubit_begin <= control_qubit && control_qubit < target_qubit_begin + qubit_count)
        throw std::out_of_range{"Control qubit cannot be one of the target qubits of the gate"};
    if (qubit_count >= n) throw std::invalid_argument{"Cannot add a bigger gate to the circuit"};
    if (control_qubit >= n) throw std::out_of_range{"Control qubit must be inside the circuit qubit range"};
    return true;
}

std::string ControlGate::to_string() const { return representation; }

// ---- single-QState operations (quantum.cpp:1962-2032) -------------------------------------------

static QState from2(const cfloat& a, const cfloat& b) {
    return QState{std::complex<float>{a.real, a.imag}, std::complex<float>{b.real, b.imag}};
}
static const float kH = 0.70710678118f;

QState X_op(const QState& s) { return from2(s[1], s[0]); }
QState Y_op(const QState& s) {
    return from2(cfloat{0.f, -1.f} * s[1], cfloat{0.f, 1.f} * s[0]);
}
QState Z_op(const QState& s) { return from2(s[0], cfloat{-1.f} * s[1]); }
QState RotateX_op(const QState& s, float angle) {
    const float c = std::cos(angle / 2.f), sn = std::sin(angle / 2.f);
    return from2(s[0] * c + s[1] * cfloat{0.f, -sn}, s[0] * cfloat{0.f, -sn} + s[1] * c);
}
QState RotateY_op(const QState& s, float angle) {
    const float c = std::cos(angle / 2.f), sn = std::sin(angle / 2.f);
    return from2(s[0] * c + s[1] * -sn, s[0] * sn + s[1] * c);
}
QState RotateZ_op(const QState& s, float angle) {
    const float c = std::cos(angle / 2.f), sn = std::sin(angle / 2.f);
    return from2(s[0] * cfloat{c, -sn}, s[1] * cfloat{c, sn});
}
QState Hadamard_op(const QState& s) {
    return from2(cfloat{kH} * s[0] + cfloat{kH} * s[1], cfloat{kH} * s[0] + cfloat{-kH} * s[1]);
}
QState Phase_op(const QState& s, float angle) {
    return from2(s[0], s[1] * cfloat{std::cos(angle), std::sin(angle)});
}

}  // namespace aqs
