// Circuit text: the reference's gate representation extended to a complete
// wire format.
//
// The reference writes each gate as "Name,controls,targets:q,...;"
// (QGate::to_string, src/quantum.cpp:569-1662; read back for drawing by
// parse_circuit_representation, src/quantum_visuals.cpp:71-80): the name of
// the base gate (X for X/CX/CCNot, Swap for Swap/CSwap, ...), the number of
// control and target qubits, then the controls followed by the targets.  It
// carries no angles, so it cannot replay a circuit.  This format keeps that
// layout and adds what an aqsg_op holds:
//   - a header "n;" with the qubit count;
//   - parameters after the name in parentheses: the angle of rotations and
//     phases as a float ("%.9g", exact round trip), the 2^k x 2^k matrix of a
//     unitary as (re, im) doubles in row-major order ("%.17g");
//   - a control that fires on |0> written "~q";
//   - "B;" for a barrier ("P;", the reference's invisible barrier, reads as
//     one too).
// Reference names without parameters read as their gates where the name
// fixes the angle: S, S†, T, T† (Phase with ±pi/2, ±pi/4, the float angles
// of include/quantum.h:121).  Written text is canonical: parsing it and
// writing again gives the same text.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "aqsg_internal.h"

namespace aqsg {

namespace {

constexpr float kPiF = 3.14159265358979323846f;

struct Family {
    const char* name;
    int base;        // kind with no fixed control
    int ctl;         // kind with one fixed control (-1: none)
    int ctl2;        // kind with two fixed controls (-1: none)
    int targets;     // target qubits
    bool angle;      // carries an angle
};

const Family kFamilies[] = {
    {"X", AQSG_OP_X, AQSG_OP_CX, AQSG_OP_CCX, 1, false},
    {"Y", AQSG_OP_Y, AQSG_OP_CY, -1, 1, false},
    {"Z", AQSG_OP_Z, AQSG_OP_CZ, -1, 1, false},
    {"H", AQSG_OP_H, AQSG_OP_CH, -1, 1, false},
    {"Phase", AQSG_OP_PHASE, AQSG_OP_CPHASE, -1, 1, true},
    {"RotX", AQSG_OP_RX, AQSG_OP_CRX, -1, 1, true},
    {"RotY", AQSG_OP_RY, AQSG_OP_CRY, -1, 1, true},
    {"RotZ", AQSG_OP_RZ, AQSG_OP_CRZ, -1, 1, true},
    {"Swap", AQSG_OP_SWAP, AQSG_OP_CSWAP, -1, 2, false},
};

// Family of a kind and the number of fixed controls it has.
const Family* family_of(int kind, int* fixed) {
    for (const Family& f : kFamilies) {
        if (kind == f.base) { *fixed = 0; return &f; }
        if (kind == f.ctl) { *fixed = 1; return &f; }
        if (kind == f.ctl2) { *fixed = 2; return &f; }
    }
    return nullptr;
}

void append_fmt(std::string& s, const char* fmt, double v) {
    char b[40];
    std::snprintf(b, sizeof(b), fmt, v);
    s += b;
}

int write_op(const aqsg_op& o, std::string& out) {
    if (o.kind == AQSG_OP_BARRIER) {
        out += "B;";
        return AQSG_OK;
    }
    // controls: the kind's fixed controls (fire on |1>), then the extra ones
    std::vector<std::string> ctl;
    std::vector<int> tgt;
    std::string name, params;
    if (o.kind == AQSG_OP_UNITARY) {
        const int k = o.num_qubits;
        if (k < 1 || k > AQSG_MAX_UNITARY_QUBITS || !o.matrix)
            return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unitary op without a valid matrix");
        name = "U";
        const int entries = 2 * (1 << k) * (1 << k);
        for (int e = 0; e < entries; ++e) {
            if (e) params += ',';
            append_fmt(params, "%.17g", o.matrix[e]);
        }
        for (int i = 0; i < k; ++i) tgt.push_back(o.qubits[i]);
    } else if (o.kind == AQSG_OP_OR) {
        name = "Or";
        ctl.push_back(std::to_string(o.qubits[0]));
        ctl.push_back(std::to_string(o.qubits[1]));
        tgt.push_back(o.qubits[2]);
    } else {
        int fixed = 0;
        const Family* f = family_of(o.kind, &fixed);
        if (!f) return set_error(AQSG_ERR_INVALID_ARGUMENT, "Unknown op kind");
        name = f->name;
        if (f->angle) append_fmt(params, "%.9g", (double)o.angle);
        for (int i = 0; i < fixed; ++i) ctl.push_back(std::to_string(o.qubits[i]));
        for (int i = 0; i < f->targets; ++i) tgt.push_back(o.qubits[fixed + i]);
    }
    for (int i = 0; i < o.num_controls; ++i)
        ctl.push_back(((o.control_values >> i) & 1u) ? std::to_string(o.controls[i])
                                                       : "~" + std::to_string(o.controls[i]));
    out += name;
    if (!params.empty()) out += "(" + params + ")";
    out += "," + std::to_string(ctl.size()) + "," + std::to_string(tgt.size()) + ":";
    bool first = true;
    for (const std::string& c : ctl) {
        out += (first ? "" : ",") + c;
        first = false;
    }
    for (int t : tgt) {
        out += (first ? "" : ",") + std::to_string(t);
        first = false;
    }
    out += ";";
    return AQSG_OK;
}

struct Parsed {
    aqsg_op op;
    std::vector<double> mat;
};

int syntax(const std::string& what) { return set_error(AQSG_ERR_INVALID_ARGUMENT, "Circuit text: " + what); }

bool parse_int(const std::string& s, long* v) {
    if (s.empty() || s.size() > 9) return false;
    for (char c : s)
        if (c < '0' || c > '9') return false;
    *v = std::stol(s);
    return true;
}

bool parse_num(const std::string& s, double* v) {
    if (s.empty()) return false;
    char* end = nullptr;
    *v = std::strtod(s.c_str(), &end);
    return end && *end == '\0';
}

std::vector<std::string> split(const std::string& s, char sep) {
    std::vector<std::string> out;
    std::string cur;
    for (char c : s) {
        if (c == sep) {
            out.push_back(cur);
            cur.clear();
        } else {
            cur += c;
        }
    }
    out.push_back(cur);
    return out;
}

// One "Name[(params)],nc,nt:qubits" token (without its ';').
int parse_op(const std::string& tok, Parsed* p) {
    std::memset(&p->op, 0, sizeof(p->op));
    p->mat.clear();
    if (tok == "B" || tok == "P") {
        p->op.kind = AQSG_OP_BARRIER;
        return AQSG_OK;
    }
    const size_t colon = tok.find(':');
    if (colon == std::string::npos) return syntax("missing ':' in \"" + tok + "\"");
    std::string head = tok.substr(0, colon);
    const std::string qlist = tok.substr(colon + 1);
    // name and parameters
    std::string name, params;
    bool has_params = false;
    const size_t lp = head.find('(');
    size_t rest_at;
    if (lp != std::string::npos) {
        const size_t rp = head.find(')', lp);
        if (rp == std::string::npos) return syntax("unclosed '(' in \"" + tok + "\"");
        name = head.substr(0, lp);
        params = head.substr(lp + 1, rp - lp - 1);
        has_params = true;
        rest_at = rp + 1;
    } else {
        const size_t c = head.find(',');
        name = head.substr(0, c == std::string::npos ? head.size() : c);
        rest_at = name.size();
    }
    const std::vector<std::string> counts = split(head.substr(rest_at), ',');
    long nc = 0, nt = 0;
    if (counts.size() != 3 || !counts[0].empty() || !parse_int(counts[1], &nc) || !parse_int(counts[2], &nt))
        return syntax("expected \",controls,targets\" in \"" + tok + "\"");
    // qubits: controls (optionally "~q") then targets
    const std::vector<std::string> qs = split(qlist, ',');
    if ((long)qs.size() != nc + nt) return syntax("qubit list does not match the counts in \"" + tok + "\"");
    std::vector<int> ctl, tgt;
    uint32_t ctl_values = 0;
    for (long i = 0; i < nc + nt; ++i) {
        std::string q = qs[i];
        bool zero = false;
        if (i < nc && !q.empty() && q[0] == '~') {
            zero = true;
            q = q.substr(1);
        }
        long v = 0;
        if (!parse_int(q, &v)) return syntax("bad qubit \"" + qs[i] + "\"");
        if (i < nc) {
            if (!zero) ctl_values |= 1u << ctl.size();
            ctl.push_back((int)v);
        } else {
            tgt.push_back((int)v);
        }
    }
    std::vector<double> pv;
    if (has_params)
        for (const std::string& s : split(params, ',')) {
            double v = 0;
            if (!parse_num(s, &v)) return syntax("bad parameter \"" + s + "\"");
            pv.push_back(v);
        }
    aqsg_op& o = p->op;
    auto set_extra = [&](size_t fixed) -> int {  // controls past the fixed ones
        for (size_t i = 0; i < fixed; ++i)
            if (!((ctl_values >> i) & 1u)) return syntax("a fixed control cannot fire on |0> in \"" + tok + "\"");
        const size_t extra = ctl.size() - fixed;
        if (extra > AQSG_OP_MAX_CONTROLS) return syntax("too many controls in \"" + tok + "\"");
        o.num_controls = (int)extra;
        o.control_values = ctl_values >> fixed;
        for (size_t i = 0; i < extra; ++i) o.controls[i] = ctl[fixed + i];
        return AQSG_OK;
    };
    if (name == "U") {
        const int k = (int)tgt.size();
        if (k < 1 || k > AQSG_MAX_UNITARY_QUBITS) return syntax("unitary on 1 to 5 qubits");
        if ((long)pv.size() != 2L * (1 << k) * (1 << k)) return syntax("unitary needs 2 x 4^k parameters");
        o.kind = AQSG_OP_UNITARY;
        o.num_qubits = k;
        for (int i = 0; i < k; ++i) o.qubits[i] = tgt[i];
        p->mat = pv;
        return set_extra(0);
    }
    if (name == "Or") {
        if (nc < 2 || nt != 1 || has_params) return syntax("Or takes two controls and one target");
        o.kind = AQSG_OP_OR;
        o.num_qubits = 3;
        o.qubits[0] = ctl[0];
        o.qubits[1] = ctl[1];
        o.qubits[2] = tgt[0];
        return set_extra(2);
    }
    std::string fam = name;
    float fixed_angle = 0.0f;
    bool named_angle = false;
    if (name == "S" || name == "S†" || name == "T" || name == "T†") {
        fam = "Phase";
        named_angle = true;
        const float a = (name[0] == 'S') ? kPiF / 2 : kPiF / 4;
        fixed_angle = (name.size() > 1) ? -a : a;
    }
    const Family* f = nullptr;
    for (const Family& cand : kFamilies)
        if (fam == cand.name) f = &cand;
    if (!f) return syntax("unknown gate \"" + name + "\"");
    if ((int)nt != f->targets) return syntax("wrong number of targets in \"" + tok + "\"");
    if (f->angle) {
        if (named_angle) {
            if (has_params) return syntax("\"" + name + "\" takes no parameter");
            o.angle = fixed_angle;
        } else {
            if (pv.size() != 1) return syntax("\"" + name + "\" needs its angle: " + name + "(angle)");
            o.angle = (float)pv[0];
        }
    } else if (has_params) {
        return syntax("\"" + name + "\" takes no parameter");
    }
    size_t fixed = 0;
    if (ctl.size() >= 2 && f->ctl2 >= 0 && ((ctl_values & 3u) == 3u)) fixed = 2;
    else if (ctl.size() >= 1 && f->ctl >= 0 && (ctl_values & 1u)) fixed = 1;
    o.kind = fixed == 2 ? f->ctl2 : (fixed == 1 ? f->ctl : f->base);
    o.num_qubits = (int)fixed + f->targets;
    for (size_t i = 0; i < fixed; ++i) o.qubits[i] = ctl[i];
    for (int i = 0; i < f->targets; ++i) o.qubits[fixed + i] = tgt[i];
    return set_extra(fixed);
}

}  // namespace

}  // namespace aqsg

using namespace aqsg;

extern "C" {

int aqsg_circuit_to_text(int n, const aqsg_op* ops, int count, char* buf, size_t len, size_t* needed) {
    if (count > 0 && !ops) return set_error(AQSG_ERR_NULL, "NULL op list");
    if (int rc = aqsg_check_ops(n, ops, count)) return rc;
    std::string out = std::to_string(n) + ";";
    for (int i = 0; i < count; ++i)
        if (int rc = write_op(ops[i], out)) return rc;
    if (needed) *needed = out.size() + 1;
    if (buf && len > 0) {
        if (len < out.size() + 1) return set_error(AQSG_ERR_OUT_OF_RANGE, "Text buffer too small");
        std::memcpy(buf, out.c_str(), out.size() + 1);
    }
    return AQSG_OK;
}

int aqsg_circuit_from_text(const char* text, int* n_out, aqsg_op* ops, int capacity, int* count,
                           double* matrices, size_t matrix_capacity, size_t* matrix_count) {
    if (!text || !n_out || !count) return set_error(AQSG_ERR_NULL, "NULL argument");
    std::string s;
    for (const char* c = text; *c; ++c)
        if (*c != ' ' && *c != '\t' && *c != '\n' && *c != '\r') s += *c;
    std::vector<std::string> toks = split(s, ';');
    if (toks.empty() || !toks.back().empty()) return syntax("must end with ';'");
    toks.pop_back();
    long n = 0;
    if (toks.empty() || !parse_int(toks[0], &n)) return syntax("must start with the qubit count, \"n;\"");
    if (n < 1 || n > AQSG_MAX_QUBITS) return set_error(AQSG_ERR_OUT_OF_RANGE, "Circuit exceeds supported max qubit count");
    std::vector<Parsed> parsed(toks.size() - 1);
    size_t doubles = 0;
    for (size_t i = 1; i < toks.size(); ++i) {
        if (int rc = parse_op(toks[i], &parsed[i - 1])) return rc;
        doubles += parsed[i - 1].mat.size();
    }
    // validated before anything is returned, so a size query and the
    // parse proper fail alike
    {
        std::vector<aqsg_op> check(parsed.size());
        for (size_t i = 0; i < parsed.size(); ++i) {
            check[i] = parsed[i].op;
            if (!parsed[i].mat.empty()) check[i].matrix = parsed[i].mat.data();
        }
        if (int rc = aqsg_check_ops((int)n, check.data(), (int)check.size())) return rc;
    }
    *n_out = (int)n;
    *count = (int)parsed.size();
    if (matrix_count) *matrix_count = doubles;
    if (!ops) return AQSG_OK;  // sizes only
    if (capacity < (int)parsed.size()) return set_error(AQSG_ERR_OUT_OF_RANGE, "Op buffer too small");
    if (doubles > 0 && (!matrices || matrix_capacity < doubles))
        return set_error(AQSG_ERR_OUT_OF_RANGE, "Matrix buffer too small");
    size_t at = 0;
    for (size_t i = 0; i < parsed.size(); ++i) {
        ops[i] = parsed[i].op;
        if (!parsed[i].mat.empty()) {
            std::memcpy(matrices + at, parsed[i].mat.data(), sizeof(double) * parsed[i].mat.size());
            ops[i].matrix = matrices + at;
            at += parsed[i].mat.size();
        }
    }
    return AQSG_OK;
}

}  // extern "C"
