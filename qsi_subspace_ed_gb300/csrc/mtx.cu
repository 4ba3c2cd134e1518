// MatrixMarket export of an operator's connectivity: the file build_hamiltonian writes with
// Eigen::saveMarket(H.toSparseMatrix(), out) (src/build_hamiltonian.cpp:104-111).
//
// The matrix is the one toSparseMatrix assembles (operator_matrix.hpp:79-105): the triplets of
// qsi_op_triplets in their order, duplicates of a (row, col) summed in that order (setFromTriplets), stored
// column by column with rows ascending (Eigen's default column-major SparseMatrix), explicit zeros kept.
// The text follows Eigen's MarketIO writer (Eigen 3.x unsupported/Eigen/src/SparseExtra/MarketIO.h, a
// third-party header absent here, restated): the header line "%%MatrixMarket matrix coordinate  real
// general" (Eigen joins "coordinate " and " real"), then "rows cols nnz", then one "row col value" line per
// stored entry with 1-based indices and the value in scientific notation with 17 digits after the point.
#include <algorithm>
#include <cstdio>
#include <numeric>
#include <vector>

#include "qsi_handles.h"
#include "qsi_internal.h"

using namespace qsi;

extern "C" qsi_status qsi_op_write_mtx(qsi_op* op, const char* path, double tol, int64_t* nnz_out) {
    return guarded([&]() -> qsi_status {
        if (!op || !path) return fail(QSI_INVALID_ARG, "qsi_op_write_mtx: null argument");
        int64_t n_trip = 0;
        qsi_status s = qsi_op_triplets(op, tol, nullptr, nullptr, nullptr, 0, &n_trip);
        if (s != QSI_OK) return s;
        std::vector<int64_t> rows(n_trip), cols(n_trip);
        std::vector<double> vals(n_trip);
        s = qsi_op_triplets(op, tol, rows.data(), cols.data(), vals.data(), n_trip, &n_trip);
        if (s != QSI_OK) return s;
        std::vector<int64_t> order(n_trip);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
            return cols[a] != cols[b] ? cols[a] < cols[b] : rows[a] < rows[b];
        });
        // collapse duplicates (sum in triplet order)
        std::vector<int64_t> er, ec;
        std::vector<double> ev;
        er.reserve(n_trip), ec.reserve(n_trip), ev.reserve(n_trip);
        for (int64_t k = 0; k < n_trip; ++k) {
            const int64_t t = order[k];
            if (!er.empty() && er.back() == rows[t] && ec.back() == cols[t]) ev.back() += vals[t];
            else er.push_back(rows[t]), ec.push_back(cols[t]), ev.push_back(vals[t]);
        }
        FILE* f = std::fopen(path, "w");
        if (!f) return fail(QSI_IO_ERROR, "qsi_op_write_mtx: cannot create %s", path);
        std::vector<char> buf(1 << 20);
        std::setvbuf(f, buf.data(), _IOFBF, buf.size());
        const int64_t N = op->basis->n;
        std::fprintf(f, "%%%%MatrixMarket matrix coordinate  real general\n");
        std::fprintf(f, "%lld %lld %lld\n", (long long)N, (long long)N, (long long)ev.size());
        for (size_t k = 0; k < ev.size(); ++k)
            std::fprintf(f, "%lld %lld %.17e\n", (long long)(er[k] + 1), (long long)(ec[k] + 1), ev[k]);
        const bool ok = std::ferror(f) == 0;
        if (std::fclose(f) != 0 || !ok) return fail(QSI_IO_ERROR, "qsi_op_write_mtx: write failed: %s", path);
        if (nnz_out) *nnz_out = (int64_t)ev.size();
        return QSI_OK;
    });
}
