// Test driver of the reference-side adaptor include/gb300_lazy_op.hpp, compiled against the reference's own
// operator.hpp / operator.cpp: the way the reference's code would use it.  The basis is loaded into ZBasisBST from
// a CSV file (ZBasisBase::load_from_file, components/operator/src/operator.cpp:146-148), the Hamiltonian is built
// with SymbolicPMROperator(ops, ids) and SymbolicOpSum::add_term, then GB300LazyOpSum's evaluate (y = H x) and
// evaluate_add (y += H x) run, as LazyOpSumProd::perform_op and projED::RealApplyFn call them.
//
// Usage: adaptor_main BASIS.csv TERMS.txt X.bin TERMS_OUT.bin Y_OUT.bin
//   TERMS.txt      one term per line: coefficient, op characters, spin ids (whitespace separated)
//   X.bin          n little-endian doubles
//   TERMS_OUT.bin  the qsi_term array the adaptor hands to qsi_op_create (its PMRFields conversion)
//   Y_OUT.bin      y = H x, then y += H x (2n doubles), when the library's device path runs;
//                  "library error: <text>" on stdout when it reports an error (a machine without a GPU)
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "gb300_lazy_op.hpp"

int main(int argc, char** argv) {
    if (argc != 6) {
        std::cerr << "usage: adaptor_main BASIS.csv TERMS.txt X.bin TERMS_OUT.bin Y_OUT.bin\n";
        return 2;
    }
    ZBasisBST basis;
    basis.load_from_file(argv[1], "basis");
    SymbolicOpSum<double> H;
    std::ifstream tf(argv[2]);
    std::string line;
    while (std::getline(tf, line)) {
        std::istringstream ls(line);
        double c;
        std::string ops;
        if (!(ls >> c >> ops)) continue;
        std::vector<int> ids;
        for (int id; ls >> id;) ids.push_back(id);
        H.add_term(c, SymbolicPMROperator(std::vector<char>(ops.begin(), ops.end()), ids));
    }
    // the conversion GB300LazyOpSum's constructor performs, written out for the checks
    std::vector<qsi_term> t;
    for (auto& [c, op] : H.off_diag_terms) t.push_back(PMRFields(op).term(c));
    for (auto& [c, op] : H.diagonal_terms) t.push_back(PMRFields(op).term(c));
    FILE* f = std::fopen(argv[4], "wb");
    std::fwrite(t.data(), sizeof(qsi_term), t.size(), f);
    std::fclose(f);
    const size_t n = basis.dim();
    std::vector<double> x(n), y(2 * n, 0.0);
    f = std::fopen(argv[3], "rb");
    if (!f || std::fread(x.data(), sizeof(double), n, f) != n) {
        std::cerr << "cannot read " << argv[3] << "\n";
        return 2;
    }
    std::fclose(f);
    try {
        GB300LazyOpSum<ZBasisBST> op(basis, H);
        if ((size_t)op.rows() != n || (size_t)op.cols() != n) return 3;
        op.evaluate(x.data(), y.data());
        for (size_t i = 0; i < n; ++i) y[n + i] = y[i];
        op.evaluate_add(x.data(), y.data() + n);
    } catch (const std::runtime_error& e) {
        std::printf("library error: %s\n", e.what());
        return 0;
    }
    f = std::fopen(argv[5], "wb");
    std::fwrite(y.data(), sizeof(double), 2 * n, f);
    std::fclose(f);
    return 0;
}
