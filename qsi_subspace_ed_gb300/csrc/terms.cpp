// Operator-term compiler: the bit-mask algebra of SymbolicPMROperator.
//
// A term is  c * sign * Z X P  with P a projector given by (up, down) masks
// (components/operator/include/operator.hpp:215-347).  Construction walks the
// operator string right to left, exactly as SymbolicPMROperator::_construct
// (operator.hpp:383-466), so term masks match the reference bit for bit.
#include <cctype>
#include <cstdarg>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "qsi_internal.h"

namespace qsi {

static thread_local std::string g_last_error;

qsi_status fail(qsi_status st, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return st;
}

namespace {

struct Masks {
    u128 x = 0, z = 0, up = 0, down = 0;
    int sign = 1;
};

inline bool bit(u128 m, int j) { return (m >> j) & 1; }
inline u128 one(int j) { return (u128)1 << j; }

// One right-to-left pass over (op, spin) pairs; same case analysis as
// operator.hpp:389-463, including the 'p'/'q' projector forms.
void construct(Masks& m, const std::vector<char>& ops, const std::vector<int>& ids) {
    if (ops.size() != ids.size()) throw std::invalid_argument("opstring and spin_ids differ in length");
    for (int i = (int)ops.size() - 1; i >= 0; --i) {
        const int J = ids[i];
        if (J < 0 || J >= 128) throw std::invalid_argument("spin index out of range [0,128)");
        switch (ops[i]) {
            case 'x':
            case 'X':
                m.x ^= one(J);
                if (bit(m.z, J)) m.sign = -m.sign;
                break;
            case 'z':
            case 'Z':
                m.z ^= one(J);
                break;
            case '+':
            case 'q':
            case 'Q':
                // raising (and the 'q' form, which the reference handles as a raise)
                if (bit(m.down & m.x, J)) { m.sign = 0; break; }
                if (bit(m.z, J)) m.sign = -m.sign;
                m.x ^= one(J);
                if (!bit(m.x, J)) m.up |= one(J);
                else m.down |= one(J);
                break;
            case '-':
                if (bit(m.up & m.x, J)) { m.sign = 0; break; }
                if (bit(m.z, J)) m.sign = -m.sign;
                m.x ^= one(J);
                if (!bit(m.x, J)) m.down |= one(J);
                else m.up |= one(J);
                break;
            case 'p':
            case 'P':
                if (bit(m.up & m.x, J)) { m.sign = 0; break; }
                if (!bit(m.x, J)) m.down |= one(J);
                else m.up |= one(J);
                break;
            default: {
                std::string s = "bad operator spec: ";
                for (size_t k = 0; k < ops.size(); ++k) {
                    s += std::to_string(ids[k]);
                    s += ops[k];
                    s += ' ';
                }
                throw std::invalid_argument(s);
            }
        }
    }
}

void to_term(const Masks& m, double c, qsi_term* out) {
    out->c = c;
    out->x[0] = lo64(m.x), out->x[1] = hi64(m.x);
    out->z[0] = lo64(m.z), out->z[1] = hi64(m.z);
    out->up[0] = lo64(m.up), out->up[1] = hi64(m.up);
    out->down[0] = lo64(m.down), out->down[1] = hi64(m.down);
    out->sign = m.sign;
    out->reserved = 0;
}

Masks from_term(const qsi_term* t) {
    Masks m;
    m.x = make_u128(t->x[0], t->x[1]);
    m.z = make_u128(t->z[0], t->z[1]);
    m.up = make_u128(t->up[0], t->up[1]);
    m.down = make_u128(t->down[0], t->down[1]);
    m.sign = t->sign;
    return m;
}

}  // namespace
}  // namespace qsi

using namespace qsi;

extern "C" const char* qsi_version(void) { return "qsi-gb300 0.1.0"; }

extern "C" qsi_status qsi_last_error(char* buf, size_t len) {
    if (!buf || len == 0) return QSI_INVALID_ARG;
    std::snprintf(buf, len, "%s", qsi::g_last_error.c_str());
    return QSI_OK;
}

extern "C" qsi_status qsi_term_compile(const char* ops, const int32_t* spin_ids, int32_t n,
                                       double c, qsi_term* out) {
    return guarded([&]() -> qsi_status {
        if (!out || n < 0 || (n > 0 && (!ops || !spin_ids))) return fail(QSI_INVALID_ARG, "qsi_term_compile: null argument");
        if ((int32_t)std::strlen(ops) != n) return fail(QSI_INVALID_ARG, "qsi_term_compile: ops has %zu chars, n=%d", std::strlen(ops), n);
        std::vector<char> o(ops, ops + n);
        std::vector<int> ids(spin_ids, spin_ids + n);
        Masks m;
        construct(m, o, ids);
        to_term(m, c, out);
        return QSI_OK;
    });
}

// Tokeniser with the acceptance rules of parseSpec (operator.hpp:349-381):
// whitespace-separated "<digits><op>" tokens; the op set is "xyz+-pqXYZPQ"
// ('y' passes the tokeniser and is rejected by construction).
extern "C" qsi_status qsi_term_parse(const char* spec, double c, qsi_term* out) {
    return guarded([&]() -> qsi_status {
        if (!spec || !out) return fail(QSI_INVALID_ARG, "qsi_term_parse: null argument");
        std::vector<char> ops;
        std::vector<int> ids;
        const char* p = spec;
        static const char* valid = "xyz+-pqXYZPQ";
        while (*p) {
            while (*p && std::isspace((unsigned char)*p)) ++p;
            if (!*p) break;
            const char* q = p;
            while (*q && !std::isspace((unsigned char)*q)) ++q;
            std::string tok(p, q);
            p = q;
            if (tok.size() < 2) return fail(QSI_INVALID_ARG, "Invalid token in operator string: %s", tok.c_str());
            size_t i = 0;
            int idx = 0;
            while (i < tok.size() - 1 && std::isdigit((unsigned char)tok[i])) {
                idx = idx * 10 + (tok[i] - '0');
                ++i;
            }
            char op = tok[i];
            if (!std::strchr(valid, op)) return fail(QSI_INVALID_ARG, "Invalid op '%c' in token: %s", op, tok.c_str());
            ops.push_back(op);
            ids.push_back(idx);
        }
        Masks m;
        construct(m, ops, ids);
        to_term(m, c, out);
        return QSI_OK;
    });
}

// operator*= of operator.hpp:312-330.
extern "C" qsi_status qsi_term_mul(qsi_term* a, const qsi_term* b) {
    if (!a || !b) return fail(QSI_INVALID_ARG, "qsi_term_mul: null argument");
    Masks A = from_term(a), B = from_term(b);
    A.sign *= (popc128(A.x & B.z) % 2) ? -1 : 1;
    A.z ^= B.z;
    A.x ^= B.x;
    u128 require_up = (A.down & B.x) | (A.up & ~B.x);
    u128 require_down = (A.up & B.x) | (A.down & ~B.x);
    A.up = B.up | require_up;
    A.down = B.down | require_down;
    if ((A.up & A.down) != 0) A.sign = 0;
    to_term(A, a->c * b->c, a);
    return QSI_OK;
}

// applyState of operator.hpp:232-254.
extern "C" qsi_status qsi_term_apply_state(const qsi_term* t, uint64_t state[2], int32_t* sign) {
    if (!t || !state || !sign) return fail(QSI_INVALID_ARG, "qsi_term_apply_state: null argument");
    Masks m = from_term(t);
    u128 s = make_u128(state[0], state[1]);
    const int ok = ((s & m.down) == 0) && ((s & m.up) == m.up);
    const u128 sel = (u128)0 - (u128)ok;
    s ^= (m.x & sel);
    state[0] = lo64(s);
    state[1] = hi64(s);
    *sign = m.sign * (1 - 2 * (popc128(~s & m.z) % 2)) * ok;
    return QSI_OK;
}
