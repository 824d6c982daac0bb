// Gate fusion: the engine's compile().
//
// The reference folds every gate of a circuit into one dense 2^n x 2^n
// matrix (QCircuit::compile, src/quantum.cpp:199-210); that is O(8^n) work
// and O(4^n) memory.  Here consecutive gates are folded into dense unitaries
// on at most K <= 5 qubits (32 x 32), which the tile engine then applies as
// one operation each (tensor-core contractions on the tile).
//
// Greedy in-order grouping.  A group may absorb the next gate when (1) no
// later group touches any of the gate's qubits — then moving the gate up to
// the group only crosses gates it commutes with — and (2) the union of the
// qubits stays within K.  Afterwards each group may merge whole into the
// previous or next group it shares a qubit with, under the same two rules.
// Each group's unitary is built on the host in FP64 by applying its gates as
// row operations to the 2^k x 2^k identity.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <type_traits>

#include "aqsg_internal.h"

struct aqsg_program_s {
    uint64_t id = 0;  // unique per compiled program (keys the plan cache)
    int n = 0;
    int dtype = AQSG_C64;
    int source_ops = 0;
    std::vector<aqsg::LOp> ops;
    // the same ops in ABI form (fused groups as AQSG_OP_UNITARY whose matrix
    // points into `mats`)
    std::vector<aqsg_op> exported;
    std::vector<std::vector<double>> mats;
};

namespace aqsg {


const std::vector<LOp>& program_ops(aqsg_program p) { return p->ops; }

static uint64_t support(const LOp& o) {
    uint64_t s = o.cmask | o.amask;
    if (o.t0 >= 0) s |= 1ull << o.t0;
    if (o.t1 >= 0) s |= 1ull << o.t1;
    for (int j = 0; j < o.k; ++j) s |= 1ull << o.tb[j];
    return s;
}

// Apply one lowered op to the rows of a D x D matrix U (row-major, real and
// imaginary parts apart) whose row index bits are the op's bits remapped to
// local positions: U <- O U.  Every column sees the same arithmetic as the op
// applied to that column alone; the inner loops run along the contiguous
// columns.
struct RowMat {
    int D = 0;
    std::vector<double> re, im;
    double* r(uint64_t i) { return re.data() + i * (uint64_t)D; }
    double* q(uint64_t i) { return im.data() + i * (uint64_t)D; }
};

static void swap_rows(RowMat& u, uint64_t i, uint64_t j) {
    std::swap_ranges(u.r(i), u.r(i) + u.D, u.r(j));
    std::swap_ranges(u.q(i), u.q(i) + u.D, u.q(j));
}

static void scale_row(RowMat& u, uint64_t i, double cr, double ci) {
    double *xr = u.r(i), *xi = u.q(i);
    for (int c = 0; c < u.D; ++c) {
        const double a = xr[c], b = xi[c];
        xr[c] = cr * a - ci * b;
        xi[c] = cr * b + ci * a;
    }
}

static void host_apply_rows(RowMat& u, const LOp& o) {
    const uint64_t N = (uint64_t)u.D;
    auto ok = [&](uint64_t i) { return (i & o.cmask) == o.cval; };
    switch (o.cls) {
        case L_PERM_X: case L_PERM_OR: case L_MAT2: case L_DIAG2: {
            const uint64_t t = 1ull << o.t0;
            for (uint64_t i = 0; i < N; ++i) {
                if ((i & t) || !ok(i)) continue;
                if (o.cls == L_PERM_X || (o.cls == L_PERM_OR && (i & o.amask))) {
                    swap_rows(u, i, i | t);
                } else if (o.cls == L_MAT2) {
                    double *ar = u.r(i), *ai = u.q(i), *br = u.r(i | t), *bi = u.q(i | t);
                    const double m0r = o.m[0], m0i = o.m[1], m1r = o.m[2], m1i = o.m[3];
                    const double m2r = o.m[4], m2i = o.m[5], m3r = o.m[6], m3i = o.m[7];
                    for (int c = 0; c < u.D; ++c) {
                        const double xr = ar[c], xi = ai[c], yr = br[c], yi = bi[c];
                        ar[c] = (m0r * xr - m0i * xi) + (m1r * yr - m1i * yi);
                        ai[c] = (m0r * xi + m0i * xr) + (m1r * yi + m1i * yr);
                        br[c] = (m2r * xr - m2i * xi) + (m3r * yr - m3i * yi);
                        bi[c] = (m2r * xi + m2i * xr) + (m3r * yi + m3i * yr);
                    }
                } else if (o.cls == L_DIAG2) {
                    scale_row(u, i, o.m[0], o.m[1]);
                    scale_row(u, i | t, o.m[2], o.m[3]);
                }
            }
            break;
        }
        case L_DIAG1:
            for (uint64_t i = 0; i < N; ++i)
                if (ok(i)) scale_row(u, i, o.m[0], o.m[1]);
            break;
        case L_PERM_SWAP: {
            const uint64_t a = 1ull << o.t0, b = 1ull << o.t1;
            for (uint64_t i = 0; i < N; ++i)
                if (!(i & a) && (i & b) && ok(i)) swap_rows(u, i, i ^ (a | b));
            break;
        }
        case L_MATK: {
            const int D = 1 << o.k;
            uint64_t tm = 0, off[32];
            for (int j = 0; j < o.k; ++j) tm |= 1ull << o.tb[j];
            for (int r = 0; r < D; ++r) {
                off[r] = 0;
                for (int j = 0; j < o.k; ++j)
                    if ((r >> (o.k - 1 - j)) & 1) off[r] |= 1ull << o.tb[j];
            }
            std::vector<double> inr((size_t)D * u.D), ini((size_t)D * u.D);
            for (uint64_t i = 0; i < N; ++i) {
                if ((i & tm) || !ok(i)) continue;
                for (int c = 0; c < D; ++c) {
                    std::copy(u.r(i | off[c]), u.r(i | off[c]) + u.D, inr.begin() + (size_t)c * u.D);
                    std::copy(u.q(i | off[c]), u.q(i | off[c]) + u.D, ini.begin() + (size_t)c * u.D);
                }
                for (int r = 0; r < D; ++r) {
                    double *yr = u.r(i | off[r]), *yi = u.q(i | off[r]);
                    std::fill(yr, yr + u.D, 0.0);
                    std::fill(yi, yi + u.D, 0.0);
                    for (int c = 0; c < D; ++c) {
                        const double mr = o.mk[2 * (r * D + c)], mi = o.mk[2 * (r * D + c) + 1];
                        const double* xr = inr.data() + (size_t)c * u.D;
                        const double* xi = ini.data() + (size_t)c * u.D;
                        for (int col = 0; col < u.D; ++col) {
                            yr[col] += mr * xr[col] - mi * xi[col];
                            yi[col] += mr * xi[col] + mi * xr[col];
                        }
                    }
                }
            }
            break;
        }
        default: break;
    }
}

static uint64_t remap_mask(uint64_t m, const int* local) {
    uint64_t r = 0;
    for (; m; m &= m - 1) r |= 1ull << local[__builtin_ctzll(m)];
    return r;
}

static LOp remap(const LOp& o, const int* local) {
    LOp r = o;
    if (r.t0 >= 0) r.t0 = local[r.t0];
    if (r.t1 >= 0) r.t1 = local[r.t1];
    for (int j = 0; j < r.k; ++j) r.tb[j] = local[r.tb[j]];
    r.cmask = remap_mask(o.cmask, local);
    r.cval = remap_mask(o.cval, local);
    r.amask = remap_mask(o.amask, local);
    return r;
}

struct Group {
    uint64_t bits = 0;
    std::vector<int> ops;  // indices into the input
};

// in[i] is the lowering of src[i].  Fills out (lowered) and exported (ABI
// form) in parallel.
static int fuse(int n, const std::vector<LOp>& in, const std::vector<aqsg_op>& src, int K,
                aqsg_program_s* prog) {
    std::vector<LOp>* out = &prog->ops;
    std::vector<Group> groups;
    int last[64];
    std::fill(last, last + 64, -1);
    for (int oi = 0; oi < (int)in.size(); ++oi) {
        const LOp& o = in[oi];
        if (o.cls == L_NOP) continue;
        const uint64_t s = support(o);
        int cand = -1;
        for (uint64_t x = s; x; x &= x - 1) cand = std::max(cand, last[__builtin_ctzll(x)]);
        int g;
        if (cand >= 0 && __builtin_popcountll(groups[cand].bits | s) <= K) {
            g = cand;
        } else {
            g = (int)groups.size();
            groups.emplace_back();
        }
        groups[g].bits |= s;
        groups[g].ops.push_back(oi);
        for (uint64_t x = s; x; x &= x - 1) last[__builtin_ctzll(x)] = g;
    }
    // Merge groups into the previous (else the next) group that shares a
    // qubit with them when the union stays within K qubits.  The groups in
    // between share no qubit with the merged one, so they commute with it.
    // Lone one- and two-qubit groups would otherwise each cost a pass over
    // the tile; diagonal-only groups are cheap and stay.
    auto all_diag_of = [&](const Group& g) {
        for (int oi : g.ops)
            if (!in[oi].diagonal()) return false;
        return true;
    };
    std::vector<char> gone(groups.size(), 0);
    for (size_t g = 0; g < groups.size(); ++g) {
        Group& cur = groups[g];
        if (all_diag_of(cur) || __builtin_popcountll(cur.bits) > K) continue;
        int prev = -1, next = -1;
        for (int q = (int)g - 1; q >= 0; --q)
            if (!gone[q] && (groups[q].bits & cur.bits)) {
                prev = q;
                break;
            }
        if (prev >= 0 && __builtin_popcountll(groups[prev].bits | cur.bits) <= K) {
            groups[prev].bits |= cur.bits;
            groups[prev].ops.insert(groups[prev].ops.end(), cur.ops.begin(), cur.ops.end());
            gone[g] = 1;
            continue;
        }
        for (size_t q = g + 1; q < groups.size(); ++q)
            if (!gone[q] && (groups[q].bits & cur.bits)) {
                next = (int)q;
                break;
            }
        if (next >= 0 && __builtin_popcountll(groups[next].bits | cur.bits) <= K &&
            !all_diag_of(groups[next])) {
            groups[next].bits |= cur.bits;
            groups[next].ops.insert(groups[next].ops.begin(), cur.ops.begin(), cur.ops.end());
            gone[g] = 1;
        }
    }
    out->clear();
    prog->exported.clear();
    prog->mats.clear();
    prog->mats.reserve(groups.size());
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        if (gone[gi]) continue;
        const Group& gr = groups[gi];
        bool all_diag = true;
        for (int oi : gr.ops) all_diag = all_diag && in[oi].diagonal();
        const int k = __builtin_popcountll(gr.bits);
        // keep lone gates, diagonal-only groups and groups too wide to fuse
        // (a gate with many controls) as they are
        if (gr.ops.size() == 1 || all_diag || k > K) {
            for (int oi : gr.ops) {
                out->push_back(in[oi]);
                prog->exported.push_back(src[oi]);
                if (src[oi].kind == AQSG_OP_UNITARY) {  // point at a private copy
                    if (in[oi].cls == L_MATK) prog->mats.push_back(in[oi].mk);
                    else prog->mats.emplace_back(in[oi].m, in[oi].m + 8);
                    prog->exported.back().matrix = prog->mats.back().data();
                }
            }
            continue;
        }
        int local[64];
        std::fill(local, local + 64, 0);
        std::vector<int> bits;  // ascending global bits = local bit positions
        for (int b = 0; b < 64; ++b)
            if ((gr.bits >> b) & 1ull) {
                local[b] = (int)bits.size();
                bits.push_back(b);
            }
        std::vector<LOp> lops;
        for (int oi : gr.ops) lops.push_back(remap(in[oi], local));
        const int D = 1 << k;
        LOp f;
        f.k = k;
        // matrix index MSB = highest global bit
        for (int j = 0; j < k; ++j) f.tb[j] = bits[k - 1 - j];
        f.mk.assign(2 * D * D, 0.0);
        RowMat u;
        u.D = D;
        u.re.assign((size_t)D * D, 0.0);
        u.im.assign((size_t)D * D, 0.0);
        for (int c = 0; c < D; ++c) u.re[(size_t)c * D + c] = 1.0;
        // consecutive uncontrolled 2x2 gates on one qubit (RotY then RotZ, ...)
        // act on the rows as their product: one row pass instead of several
        for (size_t q = 0; q < lops.size();) {
            const LOp& o = lops[q];
            auto single = [](const LOp& x) {
                return (x.cls == L_MAT2 || x.cls == L_DIAG2) && x.cmask == 0 && x.t0 >= 0;
            };
            if (!single(o)) {
                host_apply_rows(u, o);
                ++q;
                continue;
            }
            // product m (row-major 2x2, complex as re/im pairs) of the run
            auto mat_of = [](const LOp& x, double* m) {
                if (x.cls == L_MAT2) {
                    for (int e = 0; e < 8; ++e) m[e] = x.m[e];
                } else {  // diag(m0, m1)
                    m[0] = x.m[0]; m[1] = x.m[1]; m[2] = 0; m[3] = 0;
                    m[4] = 0; m[5] = 0; m[6] = x.m[2]; m[7] = x.m[3];
                }
            };
            double m[8];
            mat_of(o, m);
            size_t r = q + 1;
            for (; r < lops.size() && single(lops[r]) && lops[r].t0 == o.t0; ++r) {
                double b[8], c[8];
                mat_of(lops[r], b);
                for (int i = 0; i < 2; ++i)
                    for (int j = 0; j < 2; ++j) {  // c = b m
                        double re = 0, im = 0;
                        for (int k = 0; k < 2; ++k) {
                            const double br = b[2 * (2 * i + k)], bi = b[2 * (2 * i + k) + 1];
                            const double mr = m[2 * (2 * k + j)], mi = m[2 * (2 * k + j) + 1];
                            re += br * mr - bi * mi;
                            im += br * mi + bi * mr;
                        }
                        c[2 * (2 * i + j)] = re;
                        c[2 * (2 * i + j) + 1] = im;
                    }
                for (int e = 0; e < 8; ++e) m[e] = c[e];
            }
            if (r == q + 1) {
                host_apply_rows(u, o);
            } else {
                LOp p2 = o;
                p2.cls = L_MAT2;
                for (int e = 0; e < 8; ++e) p2.m[e] = m[e];
                host_apply_rows(u, p2);
            }
            q = r;
        }
        // local index i has bit j <-> bits[j]; the matrix index r has
        // bit (k-1-j') <-> tb[j'] = bits[k-1-j'], i.e. r == i
        for (int r = 0; r < D; ++r)
            for (int c = 0; c < D; ++c) {
                f.mk[2 * (r * D + c)] = u.re[(size_t)r * D + c];
                f.mk[2 * (r * D + c) + 1] = u.im[(size_t)r * D + c];
            }
        aqsg_op ex;
        std::memset(&ex, 0, sizeof(ex));
        ex.kind = AQSG_OP_UNITARY;
        ex.num_qubits = k;
        for (int j = 0; j < k; ++j) ex.qubits[j] = n - 1 - f.tb[j];
        if (k == 1) {
            prog->mats.push_back(f.mk);
            ex.matrix = prog->mats.back().data();
            f.cls = L_MAT2;
            f.t0 = bits[0];
            f.k = 0;
            for (int e = 0; e < 8; ++e) f.m[e] = f.mk[e];
            f.mk.clear();
            out->push_back(std::move(f));
        } else {
            // the exported op reads the matrix the lowered op holds (its heap
            // buffer stays put when the op vector grows: ops are moved)
            static_assert(std::is_nothrow_move_constructible<LOp>::value, "fused ops must move on growth");
            f.cls = L_MATK;
            out->push_back(std::move(f));
            ex.matrix = out->back().mk.data();
        }
        prog->exported.push_back(ex);
    }
    return AQSG_OK;
}

}  // namespace aqsg

using namespace aqsg;

extern "C" {

int aqsg_compile(int n, int dtype, const aqsg_op* ops, int count, int max_qubits, aqsg_program* out) {
    if (!out) return set_error(AQSG_ERR_NULL, "NULL output handle");
    *out = nullptr;
    if (n < 1 || n > AQSG_MAX_QUBITS)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Invalid qubit count");
    if (dtype != AQSG_C64 && dtype != AQSG_C128) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown dtype");
    if (max_qubits < 1 || max_qubits > AQSG_MAX_UNITARY_QUBITS)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Fusion width must be 1 to 5 qubits");
    if (int rc = aqsg_check_ops(n, ops, count)) return rc;
    std::vector<LOp> low;
    std::vector<aqsg_op> src;
    low.reserve(count);
    for (int i = 0; i < count; ++i) {
        LOp o;
        if (int rc = lower_op(n, dtype, ops[i], &o)) return rc;
        if (o.cls == L_NOP) continue;
        low.push_back(std::move(o));
        src.push_back(ops[i]);
        src.back().matrix = nullptr;  // the caller's buffer need not outlive the program
    }
    static std::atomic<uint64_t> next_id{1};
    auto* p = new aqsg_program_s();
    p->id = next_id++;
    p->n = n;
    p->dtype = dtype;
    p->source_ops = count;
    // pass-through unitaries keep a private copy of their matrix
    p->mats.reserve(2 * src.size() + 1);
    if (int rc = fuse(n, low, src, max_qubits, p)) {
        delete p;
        return rc;
    }
    *out = p;
    return AQSG_OK;
}

int aqsg_program_info(aqsg_program p, int* fused_ops, int* source_ops) {
    if (!p) return set_error(AQSG_ERR_NULL, "NULL program");
    if (fused_ops) *fused_ops = (int)p->ops.size();
    if (source_ops) *source_ops = p->source_ops;
    return AQSG_OK;
}

int aqsg_program_plan(aqsg_program p, int tensor_cores, int* passes, int* tc_passes, uint64_t* hbm_bytes) {
    if (!p) return set_error(AQSG_ERR_NULL, "NULL program");
    TilePlan plan;
    if (int rc = encode_tiled(p->n, p->dtype, p->ops, tensor_cores != 0, &plan)) return rc;
    int ntc = 0;
    for (const TilePass& tp : plan.passes) ntc += tp.tc ? 1 : 0;
    if (passes) *passes = (int)plan.passes.size();
    if (tc_passes) *tc_passes = ntc;
    if (hbm_bytes) *hbm_bytes = plan_run_bytes(plan);
    return AQSG_OK;
}

int aqsg_run_program(aqsg_state st, aqsg_program p, int mode) {
    if (!st || !st->d) return set_error(AQSG_ERR_NULL, "NULL state");
    if (!p) return set_error(AQSG_ERR_NULL, "NULL program");
    if (p->n != st->n || p->dtype != st->dtype)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Program was compiled for another register size or dtype");
    if (mode < 0) mode = st->ctx->exec_mode;
    if (mode < AQSG_EXEC_AUTO || mode > AQSG_EXEC_TILED)
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown execution mode");
    AQSG_ON_DEVICE(st->ctx->device);
    if (mode == AQSG_EXEC_PER_GATE) {
        for (const LOp& o : p->ops)
            if (int rc = launch_lop(st, o)) return rc;
        return AQSG_OK;
    }
    // the program's plan stays cached on the context while it is in use
    std::vector<unsigned char> key;
    const uint64_t head[4] = {'P', p->id, (uint64_t)st->dtype, (uint64_t)st->ctx->tensor_cores};
    key.insert(key.end(), (const unsigned char*)head, (const unsigned char*)head + sizeof(head));
    return run_tiled_cached(st, key, [&](std::vector<LOp>* low) {
        *low = p->ops;
        return (int)AQSG_OK;
    });
}

int aqsg_program_export(aqsg_program p, aqsg_op* out, int capacity, int* count) {
    if (!p) return set_error(AQSG_ERR_NULL, "NULL program");
    if (count) *count = (int)p->exported.size();
    if (!out) return AQSG_OK;
    if (capacity < (int)p->exported.size())
        return set_error(AQSG_ERR_INVALID_ARGUMENT, "Output holds fewer ops than the program");
    std::copy(p->exported.begin(), p->exported.end(), out);
    return AQSG_OK;
}

int aqsg_program_free(aqsg_program p) {
    if (!p) return set_error(AQSG_ERR_NULL, "NULL program");
    delete p;
    return AQSG_OK;
}

}  // extern "C"
