// gb300_lazy_op.hpp — the reference-side adaptor: LazyOpSum's contract (evaluate, evaluate_add, rows, cols)
// over the C-ABI of qsi_ed.h.  It belongs beside components/operator/include/operator_matrix.hpp of the
// reference and includes the reference's operator.hpp; nothing in this library includes it.
#pragma once
#include "operator.hpp"
#include "qsi_ed.h"
#include <stdexcept>
#include <vector>

// Reads SymbolicPMROperator's protected fields through a derived view.
struct PMRFields : SymbolicPMROperator {
    explicit PMRFields(const SymbolicPMROperator& o) : SymbolicPMROperator(o) {}
    qsi_term term(double c) const {
        qsi_term t{};
        t.c = c;
        t.x[0] = X_mask.uint64[0];    t.x[1] = X_mask.uint64[1];
        t.z[0] = Z_mask.uint64[0];    t.z[1] = Z_mask.uint64[1];
        t.up[0] = up_mask.uint64[0];  t.up[1] = up_mask.uint64[1];
        t.down[0] = down_mask.uint64[0]; t.down[1] = down_mask.uint64[1];
        t.sign = sign;
        return t;
    }
};

inline void qsi_check(qsi_status s) {
    if (s != QSI_OK) { char b[1024]; qsi_last_error(b, sizeof b); throw std::runtime_error(b); }
}

// Same contract as LazyOpSum<double, B>: evaluate (y = Hx), evaluate_add (y += Hx), rows/cols.
template <Basis B>
struct GB300LazyOpSum {
    GB300LazyOpSum(const B& basis, const SymbolicOpSum<double>& ops) : n(basis.dim()) {
        std::vector<uint64_t> lohi(2 * n);
        for (int64_t i = 0; i < n; ++i) { lohi[2*i] = basis[i].uint64[0]; lohi[2*i+1] = basis[i].uint64[1]; }
        qsi_check(qsi_basis_create(lohi.data(), n, 0, &qb));
        std::vector<qsi_term> t;
        for (auto& [c, op] : ops.off_diag_terms) t.push_back(PMRFields(op).term(c));
        for (auto& [c, op] : ops.diagonal_terms) t.push_back(PMRFields(op).term(c));
        qsi_check(qsi_op_create(qb, t.data(), (int32_t)t.size(), &op));
    }
    ~GB300LazyOpSum() { qsi_op_destroy(op); qsi_basis_destroy(qb); }
    void evaluate(const double* x, double* y) const { qsi_check(qsi_op_apply(op, x, y, 0, QSI_PTR_HOST, nullptr)); }
    void evaluate_add(const double* x, double* y) const { qsi_check(qsi_op_apply(op, x, y, 1, QSI_PTR_HOST, nullptr)); }
    int64_t rows() const { return n; }
    int64_t cols() const { return n; }
    int64_t n; qsi_basis* qb = nullptr; qsi_op* op = nullptr;
};
