// Host-buffer apply that allocates no device memory.
//
// qsi_op_apply with host pointers stages x and y in device buffers that it
// allocates (once per operator, then reuses).  Some callers cannot allow
// that: a process whose GPU memory is owned by another allocator (a
// framework's caching pool or a per-process quota that is already fully
// reserved), where a new cudaMalloc fails or is forbidden by policy after
// start-up.  qsi_op_apply_static stages through two fixed arrays compiled
// into this library instead, so a call performs only copies and the kernel
// launch.
//
// Limits and sharing:
//  * at most kStaticMaxStates basis states (262,144, i.e. 2 MiB per vector);
//    larger bases are rejected with QSI_INVALID_ARG;
//  * the arrays live on every GPU that loads the library, for the life of the
//    process (4 MiB per GPU);
//  * every call on a device uses the same two arrays, which keep the previous
//    call's contents; each call overwrites x (and y when accumulating) before
//    the kernel reads them, so nothing has to start at zero.  Calls that
//    overlap on the GPU (from several host threads, or on several streams)
//    race on the arrays; calls from one thread, one after another, do not,
//    because every call returns only after its result is copied back;
//  * the first call on a device looks the arrays' device addresses up
//    (cudaGetSymbolAddress) with that device current, so make that first call
//    before any stream capture.  The caller's current device must be the one
//    the operator was created on.
#include <mutex>

#include "qsi_device.cuh"
#include "qsi_handles.h"

namespace qsi {
namespace {

constexpr int64_t kStaticMaxStates = 1 << 18;

__device__ __align__(256) double g_static_x[kStaticMaxStates];
__device__ __align__(256) double g_static_y[kStaticMaxStates];

struct StaticStage {
    double* x = nullptr;
    double* y = nullptr;
    bool ready = false;
};

constexpr int kMaxDevices = 64;
std::mutex g_stage_mutex;
StaticStage g_stage[kMaxDevices];

// Device addresses of the two arrays for the current device (looked up once).
qsi_status stage_for_current_device(StaticStage& out) {
    int dev = 0;
    QSI_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(QSI_INVALID_ARG, "qsi_op_apply_static: device %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_stage_mutex);
    StaticStage& s = g_stage[dev];
    if (!s.ready) {
        void* px = nullptr;
        void* py = nullptr;
        QSI_CUDA(cudaGetSymbolAddress(&px, g_static_x));
        QSI_CUDA(cudaGetSymbolAddress(&py, g_static_y));
        s.x = static_cast<double*>(px);
        s.y = static_cast<double*>(py);
        s.ready = true;
    }
    out = s;
    return QSI_OK;
}

}  // namespace
}  // namespace qsi

using namespace qsi;

extern "C" qsi_status qsi_op_apply_static(qsi_op* op, const double* x, double* y, int32_t accumulate) {
    return guarded([&]() -> qsi_status {
        if (!op || !x || !y) return fail(QSI_INVALID_ARG, "qsi_op_apply_static: null argument");
        const int64_t n = op->basis->n;
        if (n > kStaticMaxStates)
            return fail(QSI_INVALID_ARG,
                        "qsi_op_apply_static: basis of %lld states exceeds the static staging limit of %lld states",
                        (long long)n, (long long)kStaticMaxStates);
        StaticStage stage;
        qsi_status s = stage_for_current_device(stage);
        if (s != QSI_OK) return s;
        cudaStream_t st = op->stream;
        const size_t bytes = (size_t)n * sizeof(double);
        QSI_CUDA(cudaMemcpyAsync(stage.x, x, bytes, cudaMemcpyHostToDevice, st));
        if (accumulate) QSI_CUDA(cudaMemcpyAsync(stage.y, y, bytes, cudaMemcpyHostToDevice, st));
        s = launch_apply(op, stage.x, stage.y, 1, QSI_F64, accumulate ? 1 : 0, st);
        if (s != QSI_OK) return s;
        QSI_CUDA(cudaMemcpyAsync(y, stage.y, bytes, cudaMemcpyDeviceToHost, st));
        QSI_CUDA(cudaStreamSynchronize(st));
        return QSI_OK;
    });
}
