// Operator families and the apply batcher of the request loop (continuous batching).
//
// A family is one basis with one term list whose coefficients vary by class: H(p) = sum_t p[class(t)] term_t
// (ring couplings by hexagon type, Zeeman field by sublattice, ...).  Every parameter point a request asks for is a
// member: an ordinary operator (qsi_op) with the real coefficients, so every solver entry point takes it, plus a
// link to the family.  A member's FP64 single-vector applies are not launched on their own: the member's thread
// queues the apply with the family, and whichever waiting thread finds the queue ready runs all queued applies
// as one batched apply, one column per member with that member's class coefficients (launch_family), then hands
// every member its result.  Requests therefore join the batch at their first apply and leave it when their
// solve ends, at any step of their own solver, with no lockstep between them.
//
// The queue is ready when it holds an apply of every live member (up to max_cols), or when its oldest entry has
// waited a quarter of the last batch's duration (members spend the time between applies in their dot products).
// Bases below kFamilyDirectRows states are not batched: their applies take about a kernel launch, less than the
// queueing would cost, and each member's column runs at once on its own stream.
// One column runs the single-vector family kernel and several the batched one; both sum a row in the same order
// with the same coefficients and diagonal, so a request's results are bitwise the same alone and in any mix.
//
// The template operator holds the term list with coefficient class + 1 on every term, which carries the class
// through qsi_op_create (term pruning, the diagonal's grouping by weight) into the kernels (fam_coef, fam_diag).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <vector>

#include "qsi_device.cuh"
#include "qsi_handles.h"

struct qsi_family {
    qsi_op* tmpl = nullptr;
    qsi_basis* basis = nullptr;
    std::vector<qsi_term> terms;   // the caller's term list (masks and signs)
    std::vector<int32_t> cls;      // class of every term
    int n_cls = 0;
    int max_cols = 8;
    int64_t min_rows = 0;          // bases below this many states run members' applies directly
    // batcher
    std::mutex mu;
    std::condition_variable cv;
    struct Req {
        qsi_op* op;
        const double* x;
        double* y;
        int accumulate;
        bool done = false;
        qsi_status status = QSI_OK;
        std::string error;
        std::chrono::steady_clock::time_point arrival;
    };
    std::deque<Req*> pending;
    bool running = false;
    int members = 0;
    std::chrono::steady_clock::duration window = std::chrono::microseconds(200);
    int64_t batches = 0, served = 0;
    // batch buffers (family stream = the template's stream)
    double* X = nullptr;
    double* Y = nullptr;
    size_t cols_alloc = 0;
    // one device block and its page-locked host image, copied in one transfer per batch:
    // [n_cls][32] class coefficients, 32 x pointers, 32 y pointers, 32 accumulate flags
    unsigned char* dpack = nullptr;
    unsigned char* hpack = nullptr;
    size_t pack_bytes = 0;
    double* fcoef = nullptr;         // views into dpack
    const double** xptr = nullptr;
    double** yptr = nullptr;
    int* accs = nullptr;
};

namespace qsi {
namespace {

constexpr int kMaxFamilyClasses = 16;
constexpr int64_t kFamilyDirectRows = 1 << 17;  // default: bases below this many states are not batched

// X[i][c] = x_c[i] for the batch's columns
__global__ void k_gather_columns(const double* const* __restrict__ xs, int R, int64_t n, double* __restrict__ X) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * R; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e / R;
        const int c = (int)(e - i * R);
        X[e] = xs[c][i];
    }
}

// y_c[i] = Y[i][c] (+ y_c[i] when accumulating), the single-vector kernel's final step
__global__ void k_scatter_columns(const double* __restrict__ Y, int R, int64_t n, double* const* __restrict__ ys,
                                  const int* __restrict__ acc) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * R; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e / R;
        const int c = (int)(e - i * R);
        double v = Y[e];
        if (acc[c]) v += ys[c][i];
        ys[c][i] = v;
    }
}

qsi_status run_batch(qsi_family* f, const std::vector<qsi_family::Req*>& batch) {
    qsi_op* T = f->tmpl;
    cudaStream_t st = T->stream;
    const int R = (int)batch.size();
    const int64_t n = f->basis->n;
    if (R == 1) {
        qsi_family::Req* r = batch[0];
        qsi_status s = launch_family(T, r->x, r->y, 1, r->op->d_fcoef, r->accumulate, st);
        if (s != QSI_OK) return s;
        QSI_CUDA(cudaStreamSynchronize(st));
        return QSI_OK;
    }
    if (f->cols_alloc < (size_t)R) {
        cudaFree(f->X);
        cudaFree(f->Y);
        f->X = f->Y = nullptr;
        f->cols_alloc = 0;
        QSI_CUDA(cudaMalloc(&f->X, (size_t)n * R * sizeof(double)));
        QSI_CUDA(cudaMalloc(&f->Y, (size_t)n * R * sizeof(double)));
        f->cols_alloc = (size_t)R;
    }
    // the batch's coefficients ([class][R]), pointers and flags into the pinned image, then one copy
    double* coef = reinterpret_cast<double*>(f->hpack);
    const double** xs = reinterpret_cast<const double**>(f->hpack + ((unsigned char*)f->xptr - f->dpack));
    double** ys = reinterpret_cast<double**>(f->hpack + ((unsigned char*)f->yptr - f->dpack));
    int* accs = reinterpret_cast<int*>(f->hpack + ((unsigned char*)f->accs - f->dpack));
    for (int c = 0; c < R; ++c) {
        for (int k = 0; k < f->n_cls; ++k) coef[(size_t)k * R + c] = batch[c]->op->fcoef[k];
        xs[c] = batch[c]->x;
        ys[c] = batch[c]->y;
        accs[c] = batch[c]->accumulate;
    }
    QSI_CUDA(cudaMemcpyAsync(f->dpack, f->hpack, f->pack_bytes, cudaMemcpyHostToDevice, st));
    k_gather_columns<<<grid_for(n * R, 256), 256, 0, st>>>(f->xptr, R, n, f->X);
    QSI_CUDA(cudaGetLastError());
    qsi_status s = launch_family(T, f->X, f->Y, R, f->fcoef, 0, st);
    if (s != QSI_OK) return s;
    k_scatter_columns<<<grid_for(n * R, 256), 256, 0, st>>>(f->Y, R, n, f->yptr, f->accs);
    QSI_CUDA(cudaGetLastError());
    QSI_CUDA(cudaStreamSynchronize(st));
    return QSI_OK;
}

}  // namespace

qsi_status family_apply(qsi_op* op, const double* x, double* y, int accumulate, cudaStream_t st) {
    qsi_family* f = op->family;
    if (f->basis->n < f->min_rows) {
        // a small basis: an apply takes about a launch, so waiting for partners would cost more than the
        // lookups a batch shares; the member's own column runs at once on its stream (same kernel, same sums)
        qsi_status s = launch_family(f->tmpl, x, y, 1, op->d_fcoef, accumulate, st);
        if (s != QSI_OK) return s;
        std::lock_guard<std::mutex> lk(f->mu);
        ++f->batches;
        ++f->served;
        return QSI_OK;
    }
    QSI_CUDA(cudaStreamSynchronize(st));  // x (and y when accumulating) are ready
    qsi_family::Req r{op, x, y, accumulate};
    r.arrival = std::chrono::steady_clock::now();
    std::unique_lock<std::mutex> lk(f->mu);
    f->pending.push_back(&r);
    f->cv.notify_all();
    while (!r.done) {
        const auto now = std::chrono::steady_clock::now();
        const bool ready = !f->pending.empty() &&
                           ((int)f->pending.size() >= std::min(f->members, f->max_cols) ||
                            now - f->pending.front()->arrival >= f->window);
        if (!f->running && ready) {
            f->running = true;
            std::vector<qsi_family::Req*> batch;
            while (!f->pending.empty() && (int)batch.size() < f->max_cols) {
                batch.push_back(f->pending.front());
                f->pending.pop_front();
            }
            lk.unlock();
            const auto t0 = std::chrono::steady_clock::now();
            const qsi_status s = run_batch(f, batch);
            std::string err;
            if (s != QSI_OK) {
                char buf[512];
                qsi_last_error(buf, sizeof buf);
                err = buf;
            }
            const auto dt = std::chrono::steady_clock::now() - t0;
            lk.lock();
            f->window = std::min<std::chrono::steady_clock::duration>(
                std::max<std::chrono::steady_clock::duration>(dt / 4, std::chrono::microseconds(5)),
                std::chrono::milliseconds(20));
            ++f->batches;
            f->served += (int64_t)batch.size();
            for (qsi_family::Req* q : batch) {
                q->status = s;
                q->error = err;
                q->done = true;
            }
            f->running = false;
            f->cv.notify_all();
        } else if (!f->running && !f->pending.empty()) {
            f->cv.wait_until(lk, f->pending.front()->arrival + f->window);  // until the oldest entry's window ends
        } else {
            f->cv.wait_for(lk, std::chrono::milliseconds(5));  // a batch runs, or this entry was taken: notified
        }
    }
    if (r.status != QSI_OK) return fail(r.status, "family batch: %s", r.error.c_str());
    return QSI_OK;
}

void family_release_member(qsi_op* op) {
    qsi_family* f = op->family;
    std::lock_guard<std::mutex> lk(f->mu);
    --f->members;
    f->cv.notify_all();
}

}  // namespace qsi

using namespace qsi;

extern "C" qsi_status qsi_family_create(qsi_basis* b, const qsi_term* terms, int32_t n_terms, const int32_t* term_class,
                                        int32_t n_classes, int32_t max_cols, qsi_family** out) {
    return guarded([&]() -> qsi_status {
        if (!b || !out || n_terms < 1 || !terms || !term_class || n_classes < 1 || n_classes > kMaxFamilyClasses ||
            max_cols < 1 || max_cols > 32)
            return fail(QSI_INVALID_ARG, "qsi_family_create: bad argument (1..%d classes, 1..32 columns)",
                        kMaxFamilyClasses);
        auto* f = new qsi_family();
        f->basis = b;
        f->terms.assign(terms, terms + n_terms);
        f->cls.assign(term_class, term_class + n_terms);
        f->n_cls = n_classes;
        f->max_cols = max_cols;
        f->min_rows = kFamilyDirectRows;
        std::vector<qsi_term> tt(f->terms);
        for (int t = 0; t < n_terms; ++t) {
            if (f->cls[t] < 0 || f->cls[t] >= n_classes) {
                delete f;
                return fail(QSI_INVALID_ARG, "qsi_family_create: term %d has class %d", t, f->cls[t]);
            }
            tt[t].c = (double)(f->cls[t] + 1);
        }
        qsi_status s = qsi_op_create(b, tt.data(), n_terms, &f->tmpl);
        if (s != QSI_OK) {
            delete f;
            return s;
        }
        // the diagonal must be single-site z terms only (grouped by class in the template's diagonal), each class
        // one weight: two terms on a site, or other diagonal terms, are not supported in a family
        if (f->tmpl->n_diag_generic > 0) {
            qsi_op_destroy(f->tmpl);
            delete f;
            return fail(QSI_INVALID_ARG, "qsi_family_create: diagonal terms other than single-site z");
        }
        const size_t coef_b = (size_t)n_classes * 32 * sizeof(double), ptr_b = 32 * sizeof(double*);
        f->pack_bytes = coef_b + 2 * ptr_b + 32 * sizeof(int);
        cudaError_t e = cudaMalloc(&f->dpack, f->pack_bytes);
        if (e == cudaSuccess) e = cudaMallocHost(&f->hpack, f->pack_bytes);
        if (e == cudaSuccess) {
            f->fcoef = reinterpret_cast<double*>(f->dpack);
            f->xptr = reinterpret_cast<const double**>(f->dpack + coef_b);
            f->yptr = reinterpret_cast<double**>(f->dpack + coef_b + ptr_b);
            f->accs = reinterpret_cast<int*>(f->dpack + coef_b + 2 * ptr_b);
        }
        if (e != cudaSuccess) {
            qsi_family_destroy(f);
            return fail(QSI_OOM, "qsi_family_create: %s", cudaGetErrorString(e));
        }
        *out = f;
        return QSI_OK;
    });
}

extern "C" qsi_status qsi_family_set_min_rows(qsi_family* f, int64_t min_rows) {
    if (!f || min_rows < 0) return fail(QSI_INVALID_ARG, "qsi_family_set_min_rows: bad argument");
    std::lock_guard<std::mutex> lk(f->mu);
    f->min_rows = min_rows;
    return QSI_OK;
}

extern "C" qsi_status qsi_family_destroy(qsi_family* f) {
    if (!f) return QSI_OK;
    if (f->tmpl) qsi_op_destroy(f->tmpl);
    cudaFree(f->X);
    cudaFree(f->Y);
    cudaFree(f->dpack);
    if (f->hpack) cudaFreeHost(f->hpack);
    delete f;
    return QSI_OK;
}

extern "C" qsi_status qsi_family_member(qsi_family* f, const double* p, qsi_op** out) {
    return guarded([&]() -> qsi_status {
        if (!f || !p || !out) return fail(QSI_INVALID_ARG, "qsi_family_member: null argument");
        std::vector<qsi_term> tt(f->terms);
        for (size_t t = 0; t < tt.size(); ++t) tt[t].c = p[f->cls[t]];
        qsi_op* op = nullptr;
        qsi_status s = qsi_op_create(f->basis, tt.data(), (int32_t)tt.size(), &op);
        if (s != QSI_OK) return s;
        op->fcoef.assign(p, p + f->n_cls);
        cudaError_t e = cudaMalloc(&op->d_fcoef, (size_t)f->n_cls * sizeof(double));
        if (e == cudaSuccess) e = cudaMemcpy(op->d_fcoef, p, (size_t)f->n_cls * sizeof(double), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            qsi_op_destroy(op);
            return fail(QSI_OOM, "qsi_family_member: %s", cudaGetErrorString(e));
        }
        {
            std::lock_guard<std::mutex> lk(f->mu);
            op->family = f;
            ++f->members;
        }
        *out = op;
        return QSI_OK;
    });
}

extern "C" qsi_status qsi_family_stats(const qsi_family* f, int64_t* batches, int64_t* applies) {
    if (!f) return fail(QSI_INVALID_ARG, "qsi_family_stats: null family");
    auto* ff = const_cast<qsi_family*>(f);
    std::lock_guard<std::mutex> lk(ff->mu);
    if (batches) *batches = f->batches;
    if (applies) *applies = f->served;
    return QSI_OK;
}
