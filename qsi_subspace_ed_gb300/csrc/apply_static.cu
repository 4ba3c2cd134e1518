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
//  * CUDA loads a library's device code and its __device__ arrays lazily, at
//    first use, so qsi_op_create reserves them: it looks the arrays' device
//    addresses up (cudaGetSymbolAddress, once per device, with that device
//    current) and loads the single-vector apply kernels.  From the first
//    operator on a device, the two arrays (4 MiB) stay reserved on it for the
//    life of the process;
//  * every call on a device uses the same two arrays, which keep the previous
//    call's contents; each call overwrites x (and y when accumulating) before
//    the kernel reads them, so nothing has to start at zero.  Calls that
//    overlap on the GPU (from several host threads, or on several streams)
//    race on the arrays; calls from one thread, one after another, do not,
//    because every call returns only after its result is copied back;
//  * a call runs on the operator's device (it makes that device current for
//    the call's duration and restores the caller's afterwards).
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

// Makes `dev` current for the lifetime of the guard, then restores the caller's device.
struct DeviceGuard {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceGuard(int dev) {
        err = cudaGetDevice(&prev);
        if (err == cudaSuccess && prev != dev) err = cudaSetDevice(dev);
        else prev = -1;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

}  // namespace

qsi_status static_stage_prepare() {
    int dev = 0;
    QSI_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(QSI_INVALID_ARG, "static staging: device %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_stage_mutex);
    StaticStage& s = g_stage[dev];
    if (s.ready) return QSI_OK;
    void* px = nullptr;
    void* py = nullptr;
    QSI_CUDA(cudaGetSymbolAddress(&px, g_static_x));
    QSI_CUDA(cudaGetSymbolAddress(&py, g_static_y));
    s.x = static_cast<double*>(px);
    s.y = static_cast<double*>(py);
    s.ready = true;
    return QSI_OK;
}

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
        if (op->device < 0 || op->device >= kMaxDevices)
            return fail(QSI_INVALID_ARG, "qsi_op_apply_static: device %d out of range", op->device);
        DeviceGuard dg(op->device);
        QSI_CUDA(dg.err);
        StaticStage stage;
        {
            std::lock_guard<std::mutex> lock(g_stage_mutex);
            stage = g_stage[op->device];
        }
        if (!stage.ready)
            return fail(QSI_CUDA_ERROR,
                        "qsi_op_apply_static: the static staging arrays could not be reserved on device %d when the "
                        "operator was created", op->device);
        cudaStream_t st = op->stream;
        const size_t bytes = (size_t)n * sizeof(double);
        QSI_CUDA(cudaMemcpyAsync(stage.x, x, bytes, cudaMemcpyHostToDevice, st));
        if (accumulate) QSI_CUDA(cudaMemcpyAsync(stage.y, y, bytes, cudaMemcpyHostToDevice, st));
        qsi_status s = launch_apply(op, stage.x, stage.y, 1, QSI_F64, accumulate ? 1 : 0, st);
        if (s != QSI_OK) return s;
        QSI_CUDA(cudaMemcpyAsync(y, stage.y, bytes, cudaMemcpyDeviceToHost, st));
        QSI_CUDA(cudaStreamSynchronize(st));
        return QSI_OK;
    });
}
