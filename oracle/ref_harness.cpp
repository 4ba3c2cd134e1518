// ORACLE — test infrastructure.  Harness compiled together with the
// reference's own components/operator/src/operator.cpp (by oracle/build_ref.sh)
// into oracle/_ref/libqsi_ref.so.  It drives the reference's
// SymbolicPMROperator and ZBasisBST unchanged, through the loop of
// LazyOpSum::evaluate_add (components/operator/src/operator_matrix.cpp:28-82)
// and LazyOpSum::toSparseMatrix (operator_matrix.hpp:79-105), which cannot be
// compiled here because they need Eigen.
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <vector>
#include <omp.h>

#include "operator.hpp"

namespace {
struct Peek : SymbolicPMROperator {
    explicit Peek(const SymbolicPMROperator& o) : SymbolicPMROperator(o) {}
    void masks(uint64_t* out, int* sgn) const {
        const ZBasisBase::state_t* m[4] = {&X_mask, &Z_mask, &up_mask, &down_mask};
        for (int k = 0; k < 4; ++k) {
            out[2 * k] = m[k]->uint64[0];
            out[2 * k + 1] = m[k]->uint64[1];
        }
        *sgn = sign;
    }
};

struct RefBasis : ZBasisBST {
    RefBasis(const uint64_t* lohi, int64_t n) {
        states.resize(n);
        for (int64_t i = 0; i < n; ++i) states[i] = Uint128(lohi[2 * i + 1], lohi[2 * i]);
    }
};

// The basis class diag_DOQSI_ham and bench_apply use: high-word buckets (find_bounds) + ZBasisInterp::search.
struct RefInterp : ZBasisInterp {
    RefInterp(const uint64_t* lohi, int64_t n) {
        states.resize(n);
        for (int64_t i = 0; i < n; ++i) states[i] = Uint128(lohi[2 * i + 1], lohi[2 * i]);
        find_bounds();
    }
};

// Terms arrive as (ops string, spin ids, coefficient); split by add_term.
SymbolicOpSum<double> make_sum(const char* const* ops, const int32_t* const* ids, const int32_t* lens,
                               const double* coef, int n_terms) {
    SymbolicOpSum<double> H;
    for (int k = 0; k < n_terms; ++k) {
        std::vector<char> o(ops[k], ops[k] + lens[k]);
        std::vector<int> s(ids[k], ids[k] + lens[k]);
        H.add_term(coef[k], SymbolicPMROperator(o, s));
    }
    return H;
}
}  // namespace

extern "C" {

// masks: X lo,hi, Z lo,hi, up lo,hi, down lo,hi
int ref_term_masks(const char* ops, const int32_t* ids, int n, uint64_t* masks, int* sign) {
    try {
        std::vector<char> o(ops, ops + n);
        std::vector<int> s(ids, ids + n);
        Peek p{SymbolicPMROperator(o, s)};
        p.masks(masks, sign);
        return 0;
    } catch (...) {
        return -1;
    }
}

int ref_apply_state(const char* ops, const int32_t* ids, int n, uint64_t* state) {
    std::vector<char> o(ops, ops + n);
    std::vector<int> s(ids, ids + n);
    SymbolicPMROperator op(o, s);
    ZBasisBase::state_t st(state[1], state[0]);
    int sg = op.applyState(st);
    state[0] = st.uint64[0];
    state[1] = st.uint64[1];
    return sg;
}

int ref_search(const uint64_t* basis, int64_t n, const uint64_t* q, int64_t nq, int64_t* idx) {
    RefBasis B(basis, n);
    for (int64_t k = 0; k < nq; ++k) {
        ZBasisBase::idx_t J = 0;
        int f = B.search(Uint128(q[2 * k + 1], q[2 * k]), J);
        idx[k] = f ? J : -1;
    }
    return 0;
}

// ZBasisInterp::search per query: the index, -1 when absent, -2 when the reference throws (an unseen high word).
int ref_search_interp(const uint64_t* basis, int64_t n, const uint64_t* q, int64_t nq, int64_t* idx) {
    RefInterp B(basis, n);
    for (int64_t k = 0; k < nq; ++k) {
        ZBasisBase::idx_t J = 0;
        try {
            int f = B.search(Uint128(q[2 * k + 1], q[2 * k]), J);
            idx[k] = f ? J : -1;
        } catch (const std::out_of_range&) {
            idx[k] = -2;
        }
    }
    return 0;
}

int ref_evaluate_add(const uint64_t* basis, int64_t n, const char* const* ops, const int32_t* const* ids,
                     const int32_t* lens, const double* coef, int n_terms, const double* x, double* y,
                     int n_threads) {
    RefBasis B(basis, n);
    SymbolicOpSum<double> H = make_sum(ops, ids, lens, coef, n_terms);
    if (n_threads > 0) omp_set_num_threads(n_threads);
    const double APPLY_TOL = 1e-15;
    for (const auto& term : H.off_diag_terms) {
        const auto& c = term.first;
        const auto& op = term.second;
#pragma omp parallel
        {
            ZBasisBase::idx_t J;
            ZBasisBase::state_t state;
            double dy;
#pragma omp for schedule(static)
            for (ZBasisBase::idx_t i = 0; i < B.dim(); ++i) {
                state = B[i];
                int sign = op.applyState(state);
                if (sign != 0 && std::abs(x[i]) > APPLY_TOL) {
                    sign *= B.search(state, J);
                    dy = c * x[i] * sign;
                    if (J < n) {
#pragma omp atomic
                        y[J] += dy;
                    }
                }
            }
        }
    }
    for (const auto& term : H.diagonal_terms) {
        const auto& c = term.first;
        const auto& op = term.second;
#pragma omp parallel for schedule(static)
        for (ZBasisBase::idx_t i = 0; i < B.dim(); ++i) {
            ZBasisBase::state_t psi = B[i];
            double dy = c * x[i] * static_cast<double>(op.applyState(psi));
            y[i] += dy;
        }
    }
    return 0;
}

int64_t ref_triplets(const uint64_t* basis, int64_t n, const char* const* ops, const int32_t* const* ids,
                     const int32_t* lens, const double* coef, int n_terms, double tol, int64_t* rows, int64_t* cols,
                     double* vals) {
    RefBasis B(basis, n);
    SymbolicOpSum<double> H = make_sum(ops, ids, lens, coef, n_terms);
    int64_t w = 0;
    for (ZBasisBase::idx_t j = 0; j < n; ++j) {
        for (auto& [c, op] : H.off_diag_terms) {
            ZBasisBase::idx_t J = j;
            double res = c * op.applyIndex(B, J);
            if (std::abs(res) > tol) {
                if (rows) rows[w] = J, cols[w] = j, vals[w] = res;
                ++w;
            }
        }
        double acc = 0;
        ZBasisBase::idx_t jj = j;
        for (auto& [c, op] : H.diagonal_terms) acc += c * op.applyIndex(B, jj);
        if (rows) rows[w] = j, cols[w] = j, vals[w] = acc;
        ++w;
    }
    return w;
}
}
