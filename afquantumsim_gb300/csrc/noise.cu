// Noise by trajectories: a Pauli channel after every gate, unravelled into
// circuits with Paulis inserted at random (seeded), each run exactly; a
// quantity's mean over trajectories estimates its value under the channel.
// The batched engine runs the trajectories side by side.  The reference
// declares a noise class (QNoise, include/quantum.h:475) without any member.
#include <cmath>
#include <cstring>
#include <vector>

#include "aqsg_internal.h"

namespace aqsg {

// SplitMix64's finaliser (Steele, Lea, Flood, OOPSLA 2014): a bijective
// 64-bit mix, used as a counter-based generator.
static inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Uniform in [0, 1) for (seed, trajectory, gate, slot): the top 53 bits of
// a mix of a mix, so that neighbouring counters are unrelated.
static inline double draw(uint64_t seed, uint64_t trajectory, uint64_t gate, uint64_t slot) {
    uint64_t h = mix64(seed ^ 0x243F6A8885A308D3ull);
    h = mix64(h ^ trajectory);
    h = mix64(h ^ (gate << 8 | slot));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

static int check_noise(const aqsg_noise* nz) {
    if (!nz) return set_error(AQSG_ERR_NULL, "NULL noise model");
    for (const float* p : {nz->p1, nz->p2}) {
        double s = 0;
        for (int i = 0; i < 3; ++i) {
            if (!(p[i] >= 0.f)) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Noise probabilities must be >= 0");
            s += p[i];
        }
        if (s > 1.0) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Noise probabilities must sum to at most 1");
    }
    return AQSG_OK;
}

// Appends trajectory t of ops to out (the ops were checked).
static void build_trajectory(const aqsg_op* ops, int count, const aqsg_noise& nz, uint64_t seed, uint64_t t,
                             std::vector<aqsg_op>& out) {
    for (int g = 0; g < count; ++g) {
        const aqsg_op& op = ops[g];
        out.push_back(op);
        if (op.kind == AQSG_OP_BARRIER) continue;
        int touched[AQSG_OP_MAX_QUBITS + AQSG_OP_MAX_CONTROLS];
        int m = 0;
        const int na = op.kind == AQSG_OP_UNITARY ? op.num_qubits : op_arity(op.kind);
        for (int i = 0; i < na; ++i) touched[m++] = op.qubits[i];
        for (int i = 0; i < op.num_controls; ++i) touched[m++] = op.controls[i];
        const float* p = m == 1 ? nz.p1 : nz.p2;
        for (int s = 0; s < m; ++s) {
            const double u = draw(seed, t, (uint64_t)g, (uint64_t)s);
            int kind = -1;
            if (u < p[0]) kind = AQSG_OP_X;
            else if (u < (double)p[0] + p[1]) kind = AQSG_OP_Y;
            else if (u < (double)p[0] + p[1] + p[2]) kind = AQSG_OP_Z;
            if (kind < 0) continue;
            aqsg_op e;
            std::memset(&e, 0, sizeof(e));
            e.kind = kind;
            e.num_qubits = 1;
            e.qubits[0] = touched[s];
            out.push_back(e);
        }
    }
}

}  // namespace aqsg

using namespace aqsg;

extern "C" {

int aqsg_noise_trajectory(int n, const aqsg_op* ops, int count, const aqsg_noise* noise, uint64_t seed,
                          uint64_t trajectory, aqsg_op* out, int capacity, int* out_count) {
    if (!out_count) return set_error(AQSG_ERR_NULL, "NULL output count");
    if (int rc = check_noise(noise)) return rc;
    if (int rc = aqsg_check_ops(n, ops, count)) return rc;
    std::vector<aqsg_op> t;
    t.reserve((size_t)count * 2);
    build_trajectory(ops, count, *noise, seed, trajectory, t);
    *out_count = (int)t.size();
    if (!out) return AQSG_OK;
    if ((int)t.size() > capacity) return set_error(AQSG_ERR_OUT_OF_RANGE, "Trajectory longer than the output buffer");
    if (!t.empty()) std::memcpy(out, t.data(), sizeof(aqsg_op) * t.size());
    return AQSG_OK;
}

int aqsg_noise_expect_z(aqsg_ctx ctx, int n, const aqsg_op* ops, int count, const aqsg_noise* noise,
                        uint64_t seed, int trajectories, double* z, double* zz, double* z_err, double* zz_err) {
    if (!ctx || !z || !zz) return set_error(AQSG_ERR_NULL, "NULL argument");
    if (trajectories < 1) return set_error(AQSG_ERR_INVALID_ARGUMENT, "At least one trajectory");
    if (n < 2 || n > 30) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Noisy expectations take 2 to 30 qubits");
    if (int rc = check_noise(noise)) return rc;
    if (int rc = aqsg_check_ops(n, ops, count)) return rc;
    AQSG_ON_DEVICE(ctx->device);
    std::vector<std::vector<aqsg_op>> traj((size_t)trajectories);
    std::vector<aqsg_circuit> circ((size_t)trajectories);
    for (int t = 0; t < trajectories; ++t) {
        traj[t].reserve((size_t)count * 2);
        build_trajectory(ops, count, *noise, seed, (uint64_t)t, traj[t]);
        circ[t].n = n;
        circ[t].count = (int32_t)traj[t].size();
        circ[t].ops = traj[t].data();
    }
    aqsg_batch b = nullptr;
    if (int rc = aqsg_batch_create(ctx, circ.data(), trajectories, &b)) return rc;
    std::vector<double> zs((size_t)trajectories * n), zzs((size_t)trajectories * (n - 1));
    int rc = aqsg_batch_run(b, zs.data(), zzs.data());
    aqsg_batch_free(b);
    if (rc) return rc;
    // means and standard errors over the trajectories (two passes, FP64)
    auto reduce = [trajectories](const std::vector<double>& v, int width, double* mean, double* err) {
        for (int q = 0; q < width; ++q) {
            double s = 0;
            for (int t = 0; t < trajectories; ++t) s += v[(size_t)t * width + q];
            const double m = s / trajectories;
            double d2 = 0;
            for (int t = 0; t < trajectories; ++t) {
                const double d = v[(size_t)t * width + q] - m;
                d2 += d * d;
            }
            mean[q] = m;
            if (err) err[q] = trajectories > 1 ? std::sqrt(d2 / (trajectories - 1) / trajectories) : 0.0;
        }
    };
    reduce(zs, n, z, z_err);
    reduce(zzs, n - 1, zz, zz_err);
    return AQSG_OK;
}

}  // extern "C"
