// Launch-configuration autotuner of the tile apply kernels.
//
// Every candidate computes the same sums in the same order (row-wise pull with
// a fixed term order), so tuning changes only speed, never results.  The tuner
// times real applies of the operator on its own stream with CUDA events and
// keeps, one parameter at a time (coordinate descent), the fastest value of:
//   lookup      hash index, or the bucket table + binary search at several
//               table widths (QSI_TUNE_INDEX; the basis keeps the best table)
//               or at its current width (QSI_TUNE_LOOKUP)
//   vec_chunk   vectors per pass of the 16-byte batched kernel (R FP32 vectors)
//   grid_bps    blocks per SM of the tile kernels
//   list_cap    per-warp hit-list size of the batched kernel (rows per chunk)
#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "qsi_device.cuh"
#include "qsi_handles.h"

namespace qsi {

__global__ void k_fill_uniform(void* v, int64_t n, int is_f32, uint64_t seed) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t z = seed + 0x9E3779B97F4A7C15ULL * (uint64_t)(i + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5;
        if (is_f32) static_cast<float*>(v)[i] = (float)u;
        else static_cast<double*>(v)[i] = u;
    }
}

namespace {

struct Trial {
    qsi_op* op;
    const void* x;
    void* y;
    int R, dtype, reps;
    cudaEvent_t e0, e1;
    std::string log;
    int runs = 0;

    // Best-of-reps milliseconds of one apply at the op's current settings (one untimed warm-up).
    qsi_status time(float& ms) {
        qsi_status s = launch_apply(op, x, y, R, dtype, 0, op->stream);
        if (s != QSI_OK) return s;
        ms = 1e30f;
        for (int r = 0; r < reps; ++r) {
            QSI_CUDA(cudaEventRecord(e0, op->stream));
            s = launch_apply(op, x, y, R, dtype, 0, op->stream);
            if (s != QSI_OK) return s;
            QSI_CUDA(cudaEventRecord(e1, op->stream));
            QSI_CUDA(cudaEventSynchronize(e1));
            float t = 0.f;
            QSI_CUDA(cudaEventElapsedTime(&t, e0, e1));
            ms = std::min(ms, t);
        }
        ++runs;
        return QSI_OK;
    }

    // Tries each value of one parameter, keeps the fastest (set(v) applies a value).
    template <class Set>
    qsi_status sweep(const char* name, const std::vector<int>& values, int& best_value, float& best_ms, Set set) {
        for (int v : values) {
            if (v == best_value) continue;
            qsi_status s = set(v);
            if (s != QSI_OK) return s;
            float ms = 0.f;
            s = time(ms);
            if (s != QSI_OK) return s;
            char line[96];
            std::snprintf(line, sizeof line, "%s=%d %.3f ms\n", name, v, ms);
            log += line;
            if (ms < best_ms) best_ms = ms, best_value = v;
        }
        return set(best_value);
    }
};

}  // namespace
}  // namespace qsi

using namespace qsi;

extern "C" qsi_status qsi_op_set_tuning(qsi_op* op, int32_t which, int32_t grid_bps, int32_t vec_chunk,
                                        int32_t vec_width) {
    if (!op || which < -1 || which > 1 || grid_bps < 0 || grid_bps > 64 ||
        !(vec_chunk == 0 || vec_chunk == 16 || vec_chunk == 32 || vec_chunk == 64 || vec_chunk == 128 ||
          vec_chunk == 256 || vec_chunk == 512) ||
        !(vec_width == 0 || vec_width == 4 || vec_width == 8 || vec_width == 16))
        return fail(QSI_INVALID_ARG, "qsi_op_set_tuning: bad argument");
    for (int c = 0; c < 2; ++c)
        if (which < 0 || which == c) {
            op->tune[c].grid_bps = grid_bps;
            op->tune[c].vec_chunk = vec_chunk;
            op->tune[c].vec_width = vec_width;
        }
    return QSI_OK;
}

extern "C" qsi_status qsi_op_get_tuning(const qsi_op* op, int32_t which, int32_t* kernel, int32_t* use_hash,
                                        int32_t* list_cap, int32_t* grid_bps, int32_t* vec_chunk,
                                        int32_t* vec_width) {
    if (!op || which < 0 || which > 1) return fail(QSI_INVALID_ARG, "qsi_op_get_tuning: bad argument");
    const qsi_tuning& T = op->tune[which];
    if (kernel) *kernel = op->kernel;
    if (use_hash) *use_hash = T.use_hash | (op->ff_accumulate ? 0 : 2);
    if (list_cap) *list_cap = T.list_cap;
    if (grid_bps) *grid_bps = T.grid_bps;
    if (vec_chunk) *vec_chunk = T.vec_chunk;
    if (vec_width) *vec_width = T.vec_width;
    return QSI_OK;
}

extern "C" qsi_status qsi_op_autotune(qsi_op* op, const void* x, void* y, int32_t R, int32_t dtype, int32_t flags,
                                      int32_t reps, char* report, size_t report_len) {
    return guarded([&]() -> qsi_status {
        if (!op || R < 1 || (dtype != QSI_F64 && dtype != QSI_F32) || reps < 0)
            return fail(QSI_INVALID_ARG, "qsi_op_autotune: bad argument");
        if (op->kernel != 1) return fail(QSI_INVALID_ARG, "qsi_op_autotune: tunes the tile kernels (kernel 1)");
        cudaStream_t st = op->stream;
        qsi_tuning& cfg = op->tune[R > 1];  // the settings this tuning run chooses
        const int64_t n = op->basis->n;
        const size_t esz = dtype == QSI_F32 ? 4 : 8;
        void* dx = nullptr;
        void* dy = nullptr;
        if (!x || !y) {  // scratch vectors, filled with uniform values (none below the apply tolerance matters)
            QSI_CUDA(cudaMallocAsync(&dx, (size_t)n * R * esz, st));
            QSI_CUDA(cudaMallocAsync(&dy, (size_t)n * R * esz, st));
            k_fill_uniform<<<grid_for((int64_t)n * R, 256), 256, 0, st>>>(dx, (int64_t)n * R, dtype == QSI_F32, 7);
        }
        Trial T{op, x ? x : dx, y ? y : dy, R, dtype, reps > 0 ? reps : 2, nullptr, nullptr, {}};
        qsi_status s = QSI_OK;
        if (cudaEventCreate(&T.e0) != cudaSuccess || cudaEventCreate(&T.e1) != cudaSuccess)
            s = fail(QSI_CUDA_ERROR, "qsi_op_autotune: event creation failed");
        float best = 0.f;
        if (s == QSI_OK) s = T.time(best);
        if (s == QSI_OK) {
            char line[96];
            std::snprintf(line, sizeof line, "start use_hash=%d grid_bps=%d vec_chunk=%d list_cap=%d %.3f ms\n",
                          cfg.use_hash, cfg.grid_bps, cfg.vec_chunk, cfg.list_cap, best);
            T.log += line;
        }
        // lookup: bisection over the bucket table or the regional hash, whose regions are the table's buckets
        // (QSI_TUNE_INDEX: both at widths around the current one; QSI_TUNE_LOOKUP: at the current width, leaving
        // the basis as it is).  code = 2 * bits + (1 for the hash).
        if (s == QSI_OK && (flags & (QSI_TUNE_INDEX | QSI_TUNE_LOOKUP))) {
            qsi_basis* b = op->basis;
            const int b0 = b->bits;
            const bool can_hash = b->d_hash != nullptr;
            const int hash0 = cfg.use_hash && can_hash ? 1 : 0;
            int best_code = 2 * b0 + hash0;
            std::vector<int> codes;
            for (int d = -4; d <= 4; d += 2) {
                const int bits = b0 + d;
                if (!((flags & QSI_TUNE_INDEX) || d == 0) || bits < 8 || bits > std::min(31, b->hb + 1)) continue;
                codes.push_back(2 * bits);
                if (can_hash) codes.push_back(2 * bits + 1);
            }
            s = T.sweep("index(2*bits+hash)", codes, best_code, best, [&](int code) -> qsi_status {
                cfg.use_hash = code & 1;
                return qsi_basis_index(b, can_hash ? 1 : 0, code >> 1);
            });
        }
        const bool v4 = dtype == QSI_F32 && R > 1 && op->ff_accumulate && R >= 16 && (R & 3) == 0 &&
                        (R <= 128 ? (R & (R - 1)) == 0 : (R & 127) == 0);
        if (s == QSI_OK && v4) {
            // vectors per lane (8 takes R >= 32, powers of two up to 256 or multiples of 256), then per pass
            const bool v8 = R >= 32 && (R <= 256 ? (R & (R - 1)) == 0 : (R & 255) == 0);
            const bool v16 = R >= 64 && (R <= 512 ? (R & (R - 1)) == 0 : (R & 511) == 0);
            if (v8) {
                int cur = cfg.vec_width;
                std::vector<int> widths{4, 8};
                if (v16) widths.push_back(16);
                s = T.sweep("vec_width", widths, cur, best, [&](int v) {
                    cfg.vec_width = v;
                    return QSI_OK;
                });
            }
            std::vector<int> vcs;
            const int vpl = cfg.vec_width >= 8 ? cfg.vec_width : 4;
            for (int v : {16, 32, 64, 128, 256, 512})
                if (v <= R && v >= vpl && v <= 32 * vpl) vcs.push_back(v);
            int cur = cfg.vec_chunk;
            if (s == QSI_OK)
                s = T.sweep("vec_chunk", vcs, cur, best, [&](int v) {
                    cfg.vec_chunk = v;
                    return QSI_OK;
                });
        }
        if (s == QSI_OK) {
            std::vector<int> g = (R == 1) ? std::vector<int>{3, 4, 6, 12, 16} : std::vector<int>{1, 2, 3, 4, 8};
            int cur = cfg.grid_bps;
            s = T.sweep("grid_bps", g, cur, best, [&](int v) {
                cfg.grid_bps = v;
                return QSI_OK;
            });
        }
        if (s == QSI_OK && R > 1) {
            int cur = cfg.list_cap;
            s = T.sweep("list_cap", {128, 192, 256, 384, 512}, cur, best, [&](int v) {
                cfg.list_cap = v;
                return QSI_OK;
            });
        }
        if (s == QSI_OK) {
            char line[128];
            std::snprintf(line, sizeof line,
                          "best use_hash=%d bucket_bits=%d grid_bps=%d vec_width=%d vec_chunk=%d list_cap=%d %.3f ms\n",
                          cfg.use_hash, op->basis->bits, cfg.grid_bps, cfg.vec_width, cfg.vec_chunk, cfg.list_cap, best);
            T.log += line;
        }
        if (T.e0) cudaEventDestroy(T.e0);
        if (T.e1) cudaEventDestroy(T.e1);
        if (dx) cudaFreeAsync(dx, st);
        if (dy) cudaFreeAsync(dy, st);
        cudaStreamSynchronize(st);
        if (report && report_len) {
            std::snprintf(report, report_len, "%s", T.log.c_str());
        }
        return s;
    });
}
