// QSimulator::set_basis on the GPU against the oracle's restatement of the
// reference (src/quantum.cpp:416-465), full state vector, for the six
// changes between distinct bases: Z->X, Z->Y, X->Z, Y->Z (which, through the
// reference's missing break at :443, applies the X-to-Z matrix), X->Y and
// Y->X, each from a seeded random product state.
#include <complex>
#include <random>
#include <vector>

#include "aqs/quantum.h"
#include "aqs_oracle.h"
#include "check.h"

using namespace aqs;
using B = QSimulator::Basis;

static int code(B b) { return b == B::Z ? ORC_BASIS_Z : b == B::Y ? ORC_BASIS_Y : ORC_BASIS_X; }

int main(int argc, char** argv) {
    aqs::initialize(argc, argv);
    const uint32_t n = 6;
    const std::pair<B, B> changes[] = {{B::Z, B::X}, {B::Z, B::Y}, {B::X, B::Z},
                                       {B::Y, B::Z}, {B::X, B::Y}, {B::Y, B::X}};
    std::mt19937_64 rng(20241204u);
    std::normal_distribution<float> gauss(0.f, 1.f);
    double worst32 = 0, worst64 = 0;
    for (auto [from, to] : changes) {
        std::vector<QState> qs;
        std::vector<float> q(4 * n);
        for (uint32_t i = 0; i < n; ++i) {
            QState s({gauss(rng), gauss(rng)}, {gauss(rng), gauss(rng)});
            qs.push_back(s);
            q[4 * i] = s[0].real;
            q[4 * i + 1] = s[0].imag;
            q[4 * i + 2] = s[1].real;
            q[4 * i + 3] = s[1].imag;
        }
        QSimulator sim(n, qs);
        sim.set_basis(from);
        sim.set_basis(to);
        CHECK(sim.get_basis() == to);
        const auto got = sim.statevector();

        // the reference's algorithm in float: product state, Z -> from, from -> to
        std::vector<float> ref(2u << n);
        ref32_product_state((int)n, q.data(), ref.data());
        std::vector<double> f64(ref.begin(), ref.end());
        CHECK(ref32_set_basis(ref.data(), (int)n, ORC_BASIS_Z, code(from)) == 0);
        CHECK(ref32_set_basis(ref.data(), (int)n, code(from), code(to)) == 0);
        orc_set_basis_f64(f64.data(), (int)n, ORC_BASIS_Z, code(from));
        orc_set_basis_f64(f64.data(), (int)n, code(from), code(to));

        double d32 = 0, d64 = 0;
        for (size_t k = 0; k < got.size(); ++k) {
            d32 = std::max(d32, (double)std::abs(got[k] - std::complex<float>(ref[2 * k], ref[2 * k + 1])));
            d64 = std::max(d64, std::abs(std::complex<double>(got[k]) -
                                         std::complex<double>(f64[2 * k], f64[2 * k + 1])));
        }
        std::printf("set_basis %d -> %d: max |diff| vs float reference algorithm %.3g, vs FP64 %.3g\n",
                    code(from), code(to), d32, d64);
        CHECK(d32 < 1e-6);
        CHECK(d64 < 1e-6);
        worst32 = std::max(worst32, d32);
        worst64 = std::max(worst64, d64);
    }
    // Y -> Z is not the inverse of Z -> Y (the fall-through): the round trip
    // through Y changes |0...0> (each qubit ends as (1 - i, 1 + i) / 2), a
    // round trip through X does not
    for (B via : {B::Y, B::X}) {
        QSimulator sim(n, QState::zero());
        const auto before = sim.statevector();
        sim.set_basis(via);
        sim.set_basis(B::Z);
        const auto after = sim.statevector();
        double d = 0;
        for (size_t k = 0; k < after.size(); ++k) d = std::max(d, (double)std::abs(after[k] - before[k]));
        if (via == B::X) CHECK(d < 1e-6);
        else CHECK(d > 1e-2);
    }
    std::printf("worst: %.3g (float reference algorithm), %.3g (FP64)\n", worst32, worst64);
    return finish("test_set_basis");
}
