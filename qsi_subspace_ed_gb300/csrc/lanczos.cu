// Krylov solvers on the device: thick-restart Lanczos with full
// reorthogonalisation (the mfsparse path), the plain three-term Lanczos of
// projED::lanczos::eigval0 (the mfeig0 path) and batched FTLM recurrences.
//
// All dot products, norms and reorthogonalisation coefficients are FP64 and
// reduced in a fixed order (per-block partial sums, then one block), so a solve
// is deterministic for a given seed.  With precision QSI_F32 the stored Krylov
// vectors are FP32 and the operator gathers FP32, while the working vector w,
// every coefficient and the projected eigenproblem stay FP64 (sums over FP32
// vectors run in double-float on the FP32 pipe, about 2^-46 relative); the
// Ritz pairs are then polished by FP64 Rayleigh-Ritz steps with FP64 applies.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <random>
#include <string>
#include <vector>

#include "h5lite.h"
#include "qsi_device.cuh"
#include "qsi_handles.h"

namespace qsi {

constexpr int kRedBlock = 256;
constexpr int kRedGrid = 1024;  // fixed partial-sum grid: reduction order independent of the device

template <typename T>
__device__ __forceinline__ double ld(const T* p, int64_t i) {
    return (double)p[i];
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) r += sh[k];
    return r;  // valid in thread 0
}

// Double-float accumulator (two FP32 words, about 2^-46 relative): a += x * (ch + cl), x an FP32 value, with an
// error-free product and sum (TwoProd by fma, Knuth's TwoSum), all on the FP32 pipe.
struct DF {
    float hi, lo;
};
__device__ __forceinline__ void df_fma(DF& a, float ch, float cl, float x) {
    const float p = ch * x;
    const float e = fmaf(ch, x, -p) + cl * x;
    const float s = a.hi + p;
    const float bb = s - a.hi;
    const float err = (a.hi - (s - bb)) + (p - bb);
    a.hi = s;
    a.lo += err + e;
}
__device__ __forceinline__ double df_value(const DF& a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ void df_split(double v, float& h, float& l) {
    h = (float)v;
    l = (float)(v - (double)h);
}

// FP32 Krylov vectors: the dots V_i . w of eight vectors per pass over the rows (w, FP64, split into a float pair
// once per row and pass), accumulated in double-float: GB300's FP64 pipe runs at 1/64 of the FP32 rate, and the
// FP64 form of these loops is bound by it.  |w|^2 stays an FP64 sum (one FMA per row).
constexpr int kDotGroup = 8;
__global__ void __launch_bounds__(kRedBlock) k_multidot_f32(const float* __restrict__ V, int64_t ld_v, int k,
                                                            const double* __restrict__ w, int64_t n,
                                                            double* __restrict__ partial) {
    __shared__ double sh[32];
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t a = blockIdx.x * chunk, b = min(n, a + chunk);
    for (int g0 = 0; g0 < k; g0 += kDotGroup) {
        // the group's vectors (the last repeated past k, its sums unused): every load unconditional, so a
        // row's kDotGroup + 1 loads are in flight together
        const int nv = min(kDotGroup, k - g0);
        const float* vp[kDotGroup];
#pragma unroll
        for (int u = 0; u < kDotGroup; ++u) vp[u] = V + (int64_t)(g0 + min(u, nv - 1)) * ld_v;
        DF acc[kDotGroup];
#pragma unroll
        for (int u = 0; u < kDotGroup; ++u) acc[u] = DF{0.f, 0.f};
        for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) {
            const double wd = __ldg(w + r);
            float v[kDotGroup];
#pragma unroll
            for (int u = 0; u < kDotGroup; ++u) v[u] = __ldg(vp[u] + r);
            float wh, wl;
            df_split(wd, wh, wl);
#pragma unroll
            for (int u = 0; u < kDotGroup; ++u) df_fma(acc[u], wh, wl, v[u]);
        }
        for (int u = 0; u < nv; ++u) {
            const double s = block_sum(df_value(acc[u]), sh);
            if (threadIdx.x == 0) partial[(int64_t)blockIdx.x * (k + 1) + g0 + u] = s;
        }
    }
    double acc = 0.0;
    for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) acc += w[r] * w[r];
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) partial[(int64_t)blockIdx.x * (k + 1) + k] = s;
}

// partial[b*(k+1) + i] = sum over this block's rows of V_i . w  (i < k), and
// partial[b*(k+1) + k] = sum of w^2.
template <typename VT>
__global__ void __launch_bounds__(kRedBlock) k_multidot(const VT* __restrict__ V, int64_t ld_v, int k,
                                                        const double* __restrict__ w, int64_t n,
                                                        double* __restrict__ partial) {
    __shared__ double sh[32];
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t a = blockIdx.x * chunk, b = min(n, a + chunk);
    for (int i = 0; i <= k; ++i) {
        double acc = 0.0;
        if (i < k) {
            const VT* vi = V + (int64_t)i * ld_v;
            for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) acc += ld(vi, r) * w[r];
        } else {
            for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) acc += w[r] * w[r];
        }
        double s = block_sum(acc, sh);
        if (threadIdx.x == 0) partial[(int64_t)blockIdx.x * (k + 1) + i] = s;
    }
}

__global__ void k_reduce_partials(const double* __restrict__ partial, int nblocks, int k1, double* __restrict__ out) {
    __shared__ double sh[32];
    for (int i = 0; i < k1; ++i) {
        double acc = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) acc += partial[(int64_t)b * k1 + i];
        double s = block_sum(acc, sh);
        if (threadIdx.x == 0) out[i] = s;
    }
}

// w -= sum_i h_i V_i ; partial[b] = this block's sum of the new w^2.
template <typename VT>
__global__ void __launch_bounds__(kRedBlock) k_multi_axpy(const VT* __restrict__ V, int64_t ld_v, int k,
                                                          const double* __restrict__ h, double* __restrict__ w,
                                                          int64_t n, double* __restrict__ partial) {
    __shared__ double sh[32];
    __shared__ double hs[256];
    for (int i = threadIdx.x; i < k; i += blockDim.x) hs[i] = h[i];
    __syncthreads();
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t a = blockIdx.x * chunk, b = min(n, a + chunk);
    double acc = 0.0;
    for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) {
        double v = w[r];
        for (int i = 0; i < k; ++i) v -= hs[i] * ld(V + (int64_t)i * ld_v, r);
        w[r] = v;
        acc += v * v;
    }
    double s = block_sum(acc, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// The working vector of the FP32 solve as a double-float pair array: split once per Lanczos step, then the
// reorthogonalisation (dots, updates, norms) and the store of the next Krylov vector run on the FP32 pipe with no
// FP64 operation per row.
__device__ __forceinline__ float2 df_sub(float2 a, float2 b) {  // (a - b) in double-float, renormalised
    const float s = a.x - b.x;
    const float bb = s - a.x;
    const float e = ((a.x - (s - bb)) + (-b.x - bb)) + (a.y - b.y);
    const float hi = s + e;
    return make_float2(hi, e - (hi - s));
}
__global__ void k_split_f64(const double* __restrict__ w, float2* __restrict__ wf, int64_t n) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        float h, l;
        df_split(w[r], h, l);
        wf[r] = make_float2(h, l);
    }
}
// partial[b*(k+1) + i] = V_i . w (i < k) and partial[b*(k+1) + k] = |w|^2 over this block's rows, w a pair array.
__global__ void __launch_bounds__(kRedBlock) k_multidot_df(const float* __restrict__ V, int64_t ld_v, int k,
                                                           const float2* __restrict__ wf, int64_t n,
                                                           double* __restrict__ partial) {
    __shared__ double sh[32];
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t a = blockIdx.x * chunk, b = min(n, a + chunk);
    for (int g0 = 0; g0 < k; g0 += kDotGroup) {
        const int nv = min(kDotGroup, k - g0);
        const float* vp[kDotGroup];
#pragma unroll
        for (int u = 0; u < kDotGroup; ++u) vp[u] = V + (int64_t)(g0 + min(u, nv - 1)) * ld_v;
        DF acc[kDotGroup];
#pragma unroll
        for (int u = 0; u < kDotGroup; ++u) acc[u] = DF{0.f, 0.f};
        for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) {
            const float2 wv = __ldg(wf + r);
            float v[kDotGroup];
#pragma unroll
            for (int u = 0; u < kDotGroup; ++u) v[u] = __ldg(vp[u] + r);
#pragma unroll
            for (int u = 0; u < kDotGroup; ++u) df_fma(acc[u], wv.x, wv.y, v[u]);
        }
        for (int u = 0; u < nv; ++u) {
            const double t = block_sum(df_value(acc[u]), sh);
            if (threadIdx.x == 0) partial[(int64_t)blockIdx.x * (k + 1) + g0 + u] = t;
        }
    }
    DF nrm{0.f, 0.f};
    for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) {
        const float2 wv = __ldg(wf + r);
        df_fma(nrm, wv.x, 2.f * wv.y, wv.x);  // hi^2 + 2 hi lo
    }
    const double t = block_sum(df_value(nrm), sh);
    if (threadIdx.x == 0) partial[(int64_t)blockIdx.x * (k + 1) + k] = t;
}
// w -= sum_i h_i V_i on the pair array: the sum in double-float with h_i as float pairs (four interleaved partial
// sums combined in a fixed order, so four loads per row are in flight and the dependent chain is a quarter as
// long), the subtraction in double-float; partial[b] = this block's |w|^2.
__global__ void __launch_bounds__(kRedBlock) k_multi_axpy_df(const float* __restrict__ V, int64_t ld_v, int k,
                                                             const double* __restrict__ h, float2* __restrict__ wf,
                                                             int64_t n, double* __restrict__ partial) {
    __shared__ double sh[32];
    __shared__ float hh[256], hl[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        hh[i] = hl[i] = 0.f;
        if (i < k) df_split(h[i], hh[i], hl[i]);
    }
    __syncthreads();
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t a = blockIdx.x * chunk, b = min(n, a + chunk);
    const int k4 = (k + 3) & ~3;
    DF nrm{0.f, 0.f};
    for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) {
        DF s[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
        for (int i = 0; i < k4; i += 4) {
            float v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = __ldg(V + (int64_t)min(i + u, k - 1) * ld_v + r);  // h = 0 past k
#pragma unroll
            for (int u = 0; u < 4; ++u) df_fma(s[u], hh[i + u], hl[i + u], v[u]);
        }
        float2 t = df_sub(make_float2(s[0].hi, s[0].lo), make_float2(-s[1].hi, -s[1].lo));
        t = df_sub(t, make_float2(-s[2].hi, -s[2].lo));
        t = df_sub(t, make_float2(-s[3].hi, -s[3].lo));
        const float2 wv = df_sub(wf[r], t);
        wf[r] = wv;
        df_fma(nrm, wv.x, 2.f * wv.y, wv.x);
    }
    const double t = block_sum(df_value(nrm), sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}
// out = w / |w| rounded to FP32 (beta_sq: the squared norm on the device).
__global__ void k_scale_store_df(const float2* __restrict__ wf, const double* __restrict__ beta_sq,
                                 float* __restrict__ out, int64_t n) {
    const double inv = 1.0 / sqrt(*beta_sq);
    float ih, il;
    df_split(inv, ih, il);
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const float2 wv = wf[r];
        const float p = wv.x * ih;
        out[r] = p + (fmaf(wv.x, ih, -p) + (wv.x * il + wv.y * ih));
    }
}

// out = w * (1/beta), converted to the storage type.// out = w * (1/beta), converted to the storage type.
template <typename VT>
__global__ void k_scale_store(const double* __restrict__ w, const double* __restrict__ beta, VT* __restrict__ out,
                              int64_t n) {
    const double inv = 1.0 / sqrt(*beta);  // beta holds the squared norm
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        out[r] = (VT)(w[r] * inv);
}

// Deterministic N(0,1) start vector: counter-based SplitMix64 bits, Box-Muller.
__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

__global__ void k_randn(double* __restrict__ w, int64_t n, uint64_t seed, int rademacher) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        uint64_t a = splitmix64(seed * 0x632be59bd9b4e019ULL + 2 * (uint64_t)r);
        if (rademacher) {
            w[r] = (a >> 63) ? 1.0 : -1.0;
            continue;
        }
        uint64_t b = splitmix64(seed * 0x632be59bd9b4e019ULL + 2 * (uint64_t)r + 1);
        double u1 = ((a >> 11) + 1) * (1.0 / 9007199254740993.0);  // (0,1]
        double u2 = (b >> 11) * (1.0 / 9007199254740992.0);        // [0,1)
        double rad = sqrt(-2.0 * log(u1));
        w[r] = rad * cospi(2.0 * u2);
    }
}

template <typename VT>
__global__ void k_to_f64(const VT* __restrict__ v, double* __restrict__ w, int64_t n) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        w[r] = (double)v[r];
}

// V[:, 0..k) <- V[:, 0..m) * Y[0..m, 0..k) in place, row chunk by row chunk.  FP32 vectors: each sum in
// double-float with Y as float pairs (FP32 pipe); FP64 vectors: FP64.
template <typename VT>
__global__ void __launch_bounds__(128) k_rotate(VT* __restrict__ V, int64_t ld_v, int m, int k,
                                                const double* __restrict__ Y, int64_t n) {
    extern __shared__ double ys[];  // m*k
    if constexpr (sizeof(VT) == 4) {
        float2* y2 = reinterpret_cast<float2*>(ys);
        for (int i = threadIdx.x; i < m * k; i += blockDim.x) df_split(Y[i], y2[i].x, y2[i].y);
        __syncthreads();
        for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
            float row[160];
            for (int j = 0; j < m; ++j) row[j] = (float)V[(int64_t)j * ld_v + r];
            for (int i = 0; i < k; ++i) {
                DF acc{0.f, 0.f};
                for (int j = 0; j < m; ++j) df_fma(acc, y2[j * k + i].x, y2[j * k + i].y, row[j]);
                V[(int64_t)i * ld_v + r] = (VT)(acc.hi + acc.lo);
            }
        }
        return;
    }
    for (int i = threadIdx.x; i < m * k; i += blockDim.x) ys[i] = Y[i];
    __syncthreads();
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        double row[160];
        for (int j = 0; j < m; ++j) row[j] = (double)V[(int64_t)j * ld_v + r];
        for (int i = 0; i < k; ++i) {
            double acc = 0.0;
            for (int j = 0; j < m; ++j) acc += row[j] * ys[j * k + i];
            V[(int64_t)i * ld_v + r] = (VT)acc;
        }
    }
}

// X[:, i] = sum_j V[:, j] Y[j, i]  (i < k) into a separate FP64 output.
template <typename VT>
__global__ void __launch_bounds__(128) k_ritz_vectors(const VT* __restrict__ V, int64_t ld_v, int m, int k,
                                                      const double* __restrict__ Y, double* __restrict__ X,
                                                      int64_t n) {
    extern __shared__ double ys[];
    for (int i = threadIdx.x; i < m * k; i += blockDim.x) ys[i] = Y[i];
    __syncthreads();
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        for (int i = 0; i < k; ++i) {
            double acc = 0.0;
            for (int j = 0; j < m; ++j) acc += (double)V[(int64_t)j * ld_v + r] * ys[j * k + i];
            X[(int64_t)i * n + r] = acc;
        }
    }
}

// ------------------------------------------------------------------ small dense symmetric eigensolver
// Cyclic Jacobi with round-robin pair ordering, one thread block per matrix.
// A (M x M, row-major, M even, M <= 128) is read from global, diagonalised in
// shared memory; eigenvalues ascending to evals, eigenvectors as columns of
// evecs (row-major M x M).  Padding rows/columns of zeros stay decoupled.
__global__ void __launch_bounds__(256) k_jacobi(const double* __restrict__ Ain, int M, double* __restrict__ evals,
                                                double* __restrict__ evecs, int max_sweeps) {
    extern __shared__ double sm[];
    double* A = sm;                 // M*M
    double* cs = A + M * M;         // M/2 cosines
    double* sn = cs + M / 2;        // M/2 sines
    int* pp = (int*)(sn + M / 2);   // M/2 p indices
    int* qq = pp + M / 2;           // M/2 q indices
    int* perm = qq + M / 2;         // M positions
    __shared__ double red[32];
    __shared__ int stop;
    const double* Ab = Ain + (int64_t)blockIdx.x * M * M;
    double* Vb = evecs + (int64_t)blockIdx.x * M * M;
    double* eb = evals + (int64_t)blockIdx.x * M;
    for (int i = threadIdx.x; i < M * M; i += blockDim.x) {
        A[i] = Ab[i];
        Vb[i] = (i / M == i % M) ? 1.0 : 0.0;
    }
    for (int i = threadIdx.x; i < M; i += blockDim.x) perm[i] = i;
    __syncthreads();
    const int H = M / 2;
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        // convergence: off-diagonal mass relative to total
        double off = 0.0, tot = 0.0;
        for (int i = threadIdx.x; i < M * M; i += blockDim.x) {
            double a = A[i] * A[i];
            tot += a;
            if (i / M != i % M) off += a;
        }
        double offs = block_sum(off, red);
        double tots = block_sum(tot, red);
        if (threadIdx.x == 0) stop = !(offs > 1e-32 * tots) || tots == 0.0;
        __syncthreads();
        if (stop) break;
        for (int round = 0; round < M - 1; ++round) {
            for (int t = threadIdx.x; t < H; t += blockDim.x) {
                int p = perm[t], q = perm[M - 1 - t];
                if (p > q) {
                    int tmp = p;
                    p = q;
                    q = tmp;
                }
                pp[t] = p;
                qq[t] = q;
                double apq = A[p * M + q];
                double c = 1.0, s = 0.0;
                if (apq != 0.0) {
                    double theta = (A[q * M + q] - A[p * M + p]) / (2.0 * apq);
                    double tt = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                    c = 1.0 / sqrt(tt * tt + 1.0);
                    s = tt * c;
                }
                cs[t] = c;
                sn[t] = s;
            }
            __syncthreads();
            // rows: A <- J^T A
            for (int idx = threadIdx.x; idx < H * M; idx += blockDim.x) {
                int t = idx / M, col = idx % M;
                int p = pp[t], q = qq[t];
                double c = cs[t], s = sn[t];
                double ap = A[p * M + col], aq = A[q * M + col];
                A[p * M + col] = c * ap - s * aq;
                A[q * M + col] = s * ap + c * aq;
            }
            __syncthreads();
            // columns: A <- A J, V <- V J
            for (int idx = threadIdx.x; idx < H * M; idx += blockDim.x) {
                int t = idx / M, row = idx % M;
                int p = pp[t], q = qq[t];
                double c = cs[t], s = sn[t];
                double ap = A[row * M + p], aq = A[row * M + q];
                A[row * M + p] = c * ap - s * aq;
                A[row * M + q] = s * ap + c * aq;
                double vp = Vb[row * M + p], vq = Vb[row * M + q];
                Vb[row * M + p] = c * vp - s * vq;
                Vb[row * M + q] = s * vp + c * vq;
            }
            __syncthreads();
            // rotate positions 1..M-1 (position 0 fixed)
            if (threadIdx.x == 0) {
                int last = perm[M - 1];
                for (int i = M - 1; i > 1; --i) perm[i] = perm[i - 1];
                perm[1] = last;
            }
            __syncthreads();
        }
    }
    // sort ascending (selection sort by one thread; M <= 128), permute columns
    if (threadIdx.x == 0) {
        for (int i = 0; i < M; ++i) perm[i] = i;
        for (int i = 0; i < M; ++i) {
            int best = i;
            for (int j = i + 1; j < M; ++j)
                if (A[perm[j] * M + perm[j]] < A[perm[best] * M + perm[best]]) best = j;
            int tmp = perm[i];
            perm[i] = perm[best];
            perm[best] = tmp;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < M; i += blockDim.x) eb[i] = A[perm[i] * M + perm[i]];
    // permute eigenvector columns through shared memory row by row
    for (int row = 0; row < M; ++row) {
        __syncthreads();
        for (int j = threadIdx.x; j < M; j += blockDim.x) A[j] = Vb[row * M + perm[j]];
        __syncthreads();
        for (int j = threadIdx.x; j < M; j += blockDim.x) Vb[row * M + j] = A[j];
    }
}

// Host wrapper: batch of n_mat symmetric m x m matrices (row-major, host),
// returns ascending eigenvalues and eigenvector columns (host, m x m each).
qsi_status jacobi_eigh(const std::vector<double>& A, int m, int n_mat, std::vector<double>& w, std::vector<double>& V,
                       cudaStream_t st) {
    const int M = m + (m & 1);
    if (M > 128) return fail(QSI_INVALID_ARG, "projected matrix of size %d exceeds 128", m);
    std::vector<double> Ap((size_t)n_mat * M * M, 0.0);
    for (int b = 0; b < n_mat; ++b)
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < m; ++j) Ap[(size_t)b * M * M + i * M + j] = A[(size_t)b * m * m + i * m + j];
    // a padded index gets a diagonal above the spectrum so it sorts last
    if (M != m) {
        for (int b = 0; b < n_mat; ++b) {
            double big = 0.0;
            for (int i = 0; i < m; ++i) {
                double r = 0.0;
                for (int j = 0; j < m; ++j) r += fabs(A[(size_t)b * m * m + i * m + j]);
                big = std::max(big, r);
            }
            Ap[(size_t)b * M * M + (M - 1) * M + (M - 1)] = 2.0 * big + 1.0;
        }
    }
    double *dA = nullptr, *dw = nullptr, *dV = nullptr;
    QSI_CUDA(cudaMallocAsync(&dA, Ap.size() * 8, st));
    QSI_CUDA(cudaMallocAsync(&dw, (size_t)n_mat * M * 8, st));
    QSI_CUDA(cudaMallocAsync(&dV, Ap.size() * 8, st));
    QSI_CUDA(cudaMemcpyAsync(dA, Ap.data(), Ap.size() * 8, cudaMemcpyHostToDevice, st));
    size_t smem = (size_t)M * M * 8 + (size_t)M * 8 + (size_t)M * 2 * 4 + (size_t)M * 4 + 64;
    cudaFuncSetAttribute(k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_jacobi<<<n_mat, 256, smem, st>>>(dA, M, dw, dV, 60);
    std::vector<double> wp((size_t)n_mat * M), Vp(Ap.size());
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(wp.data(), dw, wp.size() * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(Vp.data(), dV, Vp.size() * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFreeAsync(dA, st);
    cudaFreeAsync(dw, st);
    cudaFreeAsync(dV, st);
    if (e != cudaSuccess) return fail(QSI_CUDA_ERROR, "jacobi: %s", cudaGetErrorString(e));
    w.assign((size_t)n_mat * m, 0.0);
    V.assign((size_t)n_mat * m * m, 0.0);
    for (int b = 0; b < n_mat; ++b) {
        for (int i = 0; i < m; ++i) w[(size_t)b * m + i] = wp[(size_t)b * M + i];
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < m; ++j) V[(size_t)b * m * m + i * m + j] = Vp[(size_t)b * M * M + i * M + j];
    }
    return QSI_OK;
}

// ------------------------------------------------------------------ vector toolkit
struct Vecs {
    int64_t n = 0;
    cudaStream_t st = nullptr;
    double* partial = nullptr;  // kRedGrid * 257
    double* red = nullptr;      // 257
    std::vector<double> hred;
    qsi_status init(int64_t n_, cudaStream_t s) {
        n = n_;
        st = s;
        QSI_CUDA(cudaMallocAsync(&partial, (size_t)kRedGrid * 257 * 8, st));
        QSI_CUDA(cudaMallocAsync(&red, 257 * 8, st));
        hred.resize(257);
        return QSI_OK;
    }
    ~Vecs() {
        cudaFreeAsync(partial, st);
        cudaFreeAsync(red, st);
    }
    // h[0..k) = V_i . w and h[k] = |w|^2, copied to host
    template <typename VT>
    qsi_status dots(const VT* V, int64_t ldv, int k, const double* w, std::vector<double>& h) {
        if constexpr (sizeof(VT) == 4) k_multidot_f32<<<kRedGrid, kRedBlock, 0, st>>>(V, ldv, k, w, n, partial);
        else k_multidot<VT><<<kRedGrid, kRedBlock, 0, st>>>(V, ldv, k, w, n, partial);
        k_reduce_partials<<<1, 256, 0, st>>>(partial, kRedGrid, k + 1, red);
        h.resize(k + 1);
        QSI_CUDA(cudaMemcpyAsync(h.data(), red, (size_t)(k + 1) * 8, cudaMemcpyDeviceToHost, st));
        QSI_CUDA(cudaStreamSynchronize(st));
        return QSI_OK;
    }
    // FP32 Krylov vectors with the working vector as a pair array: h[0..k) = V_i . w, h[k] = |w|^2
    qsi_status dots_df(const float* V, int64_t ldv, int k, const float2* wf, std::vector<double>& h) {
        k_multidot_df<<<kRedGrid, kRedBlock, 0, st>>>(V, ldv, k, wf, n, partial);
        k_reduce_partials<<<1, 256, 0, st>>>(partial, kRedGrid, k + 1, red);
        h.resize(k + 1);
        QSI_CUDA(cudaMemcpyAsync(h.data(), red, (size_t)(k + 1) * 8, cudaMemcpyDeviceToHost, st));
        QSI_CUDA(cudaStreamSynchronize(st));
        return QSI_OK;
    }
    // ... w -= V h; returns |w|^2 (device copy left in red[0])
    qsi_status axpy_df(const float* V, int64_t ldv, int k, const std::vector<double>& h, float2* wf, double& nrm2) {
        QSI_CUDA(cudaMemcpyAsync(red + 1, h.data(), (size_t)k * 8, cudaMemcpyHostToDevice, st));
        k_multi_axpy_df<<<kRedGrid, kRedBlock, 0, st>>>(V, ldv, k, red + 1, wf, n, partial);
        k_reduce_partials<<<1, 256, 0, st>>>(partial, kRedGrid, 1, red);
        QSI_CUDA(cudaMemcpyAsync(&nrm2, red, 8, cudaMemcpyDeviceToHost, st));
        QSI_CUDA(cudaStreamSynchronize(st));
        return QSI_OK;
    }
    // w -= V h ; returns |w|^2 (device copy left in red[0])
    template <typename VT>
    qsi_status axpy(const VT* V, int64_t ldv, int k, const std::vector<double>& h, double* w, double& nrm2) {
        QSI_CUDA(cudaMemcpyAsync(red + 1, h.data(), (size_t)k * 8, cudaMemcpyHostToDevice, st));
        k_multi_axpy<VT><<<kRedGrid, kRedBlock, 0, st>>>(V, ldv, k, red + 1, w, n, partial);
        k_reduce_partials<<<1, 256, 0, st>>>(partial, kRedGrid, 1, red);
        QSI_CUDA(cudaMemcpyAsync(&nrm2, red, 8, cudaMemcpyDeviceToHost, st));
        QSI_CUDA(cudaStreamSynchronize(st));
        return QSI_OK;
    }
};

// w = H v with FP64 output; FP32 storage is gathered as FP32 and accumulated in FP64.
template <typename VT>
qsi_status apply_to_w(qsi_op* op, const VT* v, double* w, cudaStream_t st) {
    return launch_apply_to_f64(op, v, w, sizeof(VT) == 4 ? QSI_F32 : QSI_F64, st);
}

}  // namespace qsi

namespace qsi {

// Device buffer from the stream-ordered allocator of one stream (no device-wide
// synchronisation on allocation or release, so solves on different streams overlap).
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t count = 0;
    cudaStream_t st = nullptr;
    cudaError_t alloc(size_t n, cudaStream_t s) {
        count = n;
        st = s;
        return cudaMallocAsync(&p, std::max<size_t>(1, n) * sizeof(T), s);
    }
    void release() {
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
    }
    ~DevBuf() { release(); }
};

// Orthonormalises the FP64 block X (k vectors of length n, vector-major) with
// two passes of classical Gram-Schmidt per vector.
static qsi_status orthonormalise(Vecs& vx, double* X, int k, int64_t n) {
    std::vector<double> h;
    for (int i = 0; i < k; ++i) {
        double* xi = X + (size_t)i * n;
        for (int pass = 0; pass < 2; ++pass) {
            qsi_status s = vx.dots<double>(X, n, i, xi, h);
            if (s) return s;
            double nrm2 = h[i];
            if (i > 0) {
                h.resize(i);
                s = vx.axpy<double>(X, n, i, h, xi, nrm2);
                if (s) return s;
            }
            if (pass == 1) {
                if (!(nrm2 > 0)) return fail(QSI_NOT_CONVERGED, "polish: Ritz vectors became linearly dependent");
                QSI_CUDA(cudaMemcpyAsync(vx.red, &nrm2, 8, cudaMemcpyHostToDevice, vx.st));
                k_scale_store<double><<<grid_for(n, 256), 256, 0, vx.st>>>(xi, vx.red, xi, n);
            }
        }
    }
    QSI_CUDA(cudaStreamSynchronize(vx.st));
    return QSI_OK;
}

// Rayleigh-Ritz of H on span(S) for an orthonormal FP64 block S (k vectors),
// with HS = H S supplied; writes the lowest `keep` Ritz vectors to X, H X to HX.
static qsi_status rayleigh_ritz(Vecs& vx, const double* S, const double* HS, int k, int keep, int64_t n, double* X,
                                double* HX, std::vector<double>& theta, cudaStream_t st) {
    std::vector<double> G((size_t)k * k), h;
    for (int j = 0; j < k; ++j) {
        qsi_status s = vx.dots<double>(S, n, k, HS + (size_t)j * n, h);
        if (s) return s;
        for (int i = 0; i < k; ++i) G[(size_t)i * k + j] = h[i];
    }
    for (int i = 0; i < k; ++i)
        for (int j = i + 1; j < k; ++j) {
            double a = 0.5 * (G[(size_t)i * k + j] + G[(size_t)j * k + i]);
            G[(size_t)i * k + j] = G[(size_t)j * k + i] = a;
        }
    std::vector<double> w, Y;
    qsi_status s = jacobi_eigh(G, k, 1, w, Y, st);
    if (s) return s;
    std::vector<double> Yk((size_t)k * keep);
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < keep; ++j) Yk[(size_t)i * keep + j] = Y[(size_t)i * k + j];
    DevBuf<double> dY;
    QSI_CUDA(dY.alloc(Yk.size(), st));
    QSI_CUDA(cudaMemcpyAsync(dY.p, Yk.data(), Yk.size() * 8, cudaMemcpyHostToDevice, st));
    size_t smem = Yk.size() * 8;
    k_ritz_vectors<double><<<grid_for(n, 128), 128, smem, st>>>(S, n, k, keep, dY.p, X, n);
    k_ritz_vectors<double><<<grid_for(n, 128), 128, smem, st>>>(HS, n, k, keep, dY.p, HX, n);
    QSI_CUDA(cudaGetLastError());
    QSI_CUDA(cudaStreamSynchronize(st));
    theta.assign(w.begin(), w.begin() + keep);
    return QSI_OK;
}

__global__ void k_residual(const double* __restrict__ HX, const double* __restrict__ X, const double* __restrict__ th,
                           int k, int64_t n, double* __restrict__ R) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        for (int i = 0; i < k; ++i) R[(size_t)i * n + r] = HX[(size_t)i * n + r] - th[i] * X[(size_t)i * n + r];
}

// Wall time per phase of a solver, printed to stderr at the end when the environment sets QSI_TRACE (each mark
// then synchronises the stream, so a traced run is slower; without QSI_TRACE a mark does nothing).
struct PhaseClock {
    cudaStream_t st;
    const char* name;
    bool on = std::getenv("QSI_TRACE") != nullptr;
    std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
    std::map<std::string, std::pair<double, int>> acc;
    void mark(const char* phase) {
        if (!on) return;
        cudaStreamSynchronize(st);
        const auto now = std::chrono::steady_clock::now();
        auto& a = acc[phase];
        a.first += std::chrono::duration<double>(now - t).count();
        a.second += 1;
        t = now;
    }
    ~PhaseClock() {
        if (!on) return;
        for (auto& kv : acc)
            std::fprintf(stderr, "[qsi trace] %s %-14s %9.3f s %6d marks\n", name, kv.first.c_str(), kv.second.first,
                         kv.second.second);
    }
};

// FP64 polish of the Ritz block X (nev FP64 vectors, vector-major, Ritz values th): Rayleigh-Ritz on X, then
// `rounds - 1` Rayleigh-Ritz steps on [X, HX - X theta]; then the residual report and the solver's outputs.
static qsi_status finish_solve(qsi_op* op, const qsi_lanczos_cfg& cfg, Vecs& vx, DevBuf<double>& X, DevBuf<double>& HX,
                               std::vector<double>& th, int nev, int rounds, int64_t applies, int nconv, int restarts,
                               bool exhausted, std::chrono::steady_clock::time_point t0, double* evals, double* evecs,
                               qsi_report* rep) {
    const int64_t n = op->basis->n;
    cudaStream_t st = op->stream;
    qsi_status s = QSI_OK;
    std::vector<double> h;
    // FP64 polish: Rayleigh-Ritz on the Ritz block, then optional residual-augmented rounds
    DevBuf<double> S, HS, dth;
    if (rounds > 0) {
        QSI_CUDA(S.alloc((size_t)2 * nev * n, st));
        QSI_CUDA(HS.alloc((size_t)2 * nev * n, st));
        QSI_CUDA(dth.alloc((size_t)nev, st));
        QSI_CUDA(cudaMemcpyAsync(S.p, X.p, (size_t)nev * n * 8, cudaMemcpyDeviceToDevice, st));
        s = orthonormalise(vx, S.p, nev, n);
        if (s) return s;
        for (int i = 0; i < nev; ++i) {
            s = launch_apply(op, S.p + (size_t)i * n, HS.p + (size_t)i * n, 1, QSI_F64, 0, st);
            if (s) return s;
            ++applies;
        }
        s = rayleigh_ritz(vx, S.p, HS.p, nev, nev, n, X.p, HX.p, th, st);
        if (s) return s;
        for (int round = 1; round < rounds; ++round) {
            // S = [X, R], R = HX - X theta
            QSI_CUDA(cudaMemcpyAsync(S.p, X.p, (size_t)nev * n * 8, cudaMemcpyDeviceToDevice, st));
            QSI_CUDA(cudaMemcpyAsync(dth.p, th.data(), (size_t)nev * 8, cudaMemcpyHostToDevice, st));
            k_residual<<<grid_for(n, 256), 256, 0, st>>>(HX.p, X.p, dth.p, nev, n, S.p + (size_t)nev * n);
            s = orthonormalise(vx, S.p, 2 * nev, n);
            if (s) return s;
            for (int i = 0; i < 2 * nev; ++i) {
                s = launch_apply(op, S.p + (size_t)i * n, HS.p + (size_t)i * n, 1, QSI_F64, 0, st);
                if (s) return s;
                ++applies;
            }
            s = rayleigh_ritz(vx, S.p, HS.p, 2 * nev, nev, n, X.p, HX.p, th, st);
            if (s) return s;
        }
    } else {
        for (int i = 0; i < nev; ++i) {
            s = launch_apply(op, X.p + (size_t)i * n, HX.p + (size_t)i * n, 1, QSI_F64, 0, st);
            if (s) return s;
            ++applies;
        }
    }
    // residual norms ||H x - theta x|| / ||x||
    if (rep) {
        DevBuf<double> R, d2;
        QSI_CUDA(R.alloc((size_t)nev * n, st));
        QSI_CUDA(d2.alloc((size_t)nev, st));
        QSI_CUDA(cudaMemcpyAsync(d2.p, th.data(), (size_t)nev * 8, cudaMemcpyHostToDevice, st));
        k_residual<<<grid_for(n, 256), 256, 0, st>>>(HX.p, X.p, d2.p, nev, n, R.p);
        for (int i = 0; i < nev && i < 64; ++i) {
            s = vx.dots<double>(X.p + (size_t)i * n, n, 1, R.p + (size_t)i * n, h);
            if (s) return s;
            std::vector<double> hx;
            s = vx.dots<double>(X.p, n, 0, X.p + (size_t)i * n, hx);
            if (s) return s;
            rep->residual[i] = std::sqrt(h[1] / std::max(hx[0], 1e-300));
        }
        rep->converged = nconv;
        rep->restarts = restarts;
        rep->applies = applies;
        rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    for (int i = 0; i < nev; ++i) evals[i] = th[i];
    if (evecs && cfg.want_vectors) {
        QSI_CUDA(cudaMemcpyAsync(evecs, X.p, (size_t)nev * n * 8, cudaMemcpyDeviceToHost, st));
        QSI_CUDA(cudaStreamSynchronize(st));
    }
    if (nconv < nev && !exhausted) return fail(QSI_NOT_CONVERGED, "lanczos: %d of %d eigenpairs converged after %d restarts", nconv, nev, restarts);
    return QSI_OK;
}


// Relative residual at which an FP32 Krylov phase hands its pairs to `rounds` FP64 polish rounds: 1e-7 (what FP32
// vectors resolve) for two rounds, ten times looser for each further round (at most 1e-4), which trades FP32
// restarts for FP64 residual-augmented Rayleigh-Ritz rounds.
static double fp32_stop(int rounds) { return std::min(1e-4, 1e-7 * std::pow(10.0, std::max(0, rounds - 2))); }

// Thick-restart Lanczos (Wu & Simon) for the nev smallest eigenpairs.
template <typename VT>
static qsi_status trlan(qsi_op* op, const qsi_lanczos_cfg& cfg, double* evals, double* evecs, qsi_report* rep) {
    auto t0 = std::chrono::steady_clock::now();
    const int64_t n = op->basis->n;
    cudaStream_t st = op->stream;
    int m = std::min<int64_t>(cfg.ncv, n);
    int nev = std::min(cfg.nev, std::max(1, m - 1));  // compute_spectrum_iterative clamps, matrix_diag_bits.hpp:64-66
    if (nev < 1 || m < 2) return fail(QSI_INVALID_ARG, "lanczos: need ncv >= 2 and nev >= 1");
    if (m > 126) return fail(QSI_INVALID_ARG, "lanczos: ncv must be <= 126");
    // FP32 Krylov vectors followed by at least two FP64 polish rounds (Rayleigh-Ritz, then residual-augmented
    // Rayleigh-Ritz): the Krylov phase stops at a residual FP32 vectors resolve (1e-7 relative) and the FP64
    // rounds take the pairs the rest of the way; otherwise it runs to tol itself.
    const double tol_req = cfg.tol > 0 ? cfg.tol : 1e-10;
    const double tol = (sizeof(VT) == 4 && cfg.polish_steps >= 2) ? std::max(tol_req, fp32_stop(cfg.polish_steps)) : tol_req;
    const double eps23 = std::pow(2.220446049250313e-16, 2.0 / 3.0);
    Vecs vx;
    qsi_status s = vx.init(n, st);
    if (s) return s;
    DevBuf<VT> V;
    DevBuf<double> w, dY;
    QSI_CUDA(V.alloc((size_t)(m + 1) * n, st));
    QSI_CUDA(w.alloc((size_t)n, st));
    QSI_CUDA(dY.alloc((size_t)m * m, st));
    constexpr bool kDF = sizeof(VT) == 4;  // FP32 vectors: reorthogonalise w as a double-float pair array
    DevBuf<float2> wf;
    if (kDF) QSI_CUDA(wf.alloc((size_t)n, st));
    // the reorthogonalisation's dots and updates, on w (FP64) or on its pair array (FP32 vectors)
    auto rdots = [&](int k, std::vector<double>& hv) -> qsi_status {
        if constexpr (kDF) return vx.dots_df(reinterpret_cast<const float*>(V.p), n, k, wf.p, hv);
        else return vx.dots<VT>(V.p, n, k, w.p, hv);
    };
    auto raxpy = [&](int k, const std::vector<double>& hv, double& nrm2) -> qsi_status {
        if constexpr (kDF) return vx.axpy_df(reinterpret_cast<const float*>(V.p), n, k, hv, wf.p, nrm2);
        else return vx.axpy<VT>(V.p, n, k, hv, w.p, nrm2);
    };
    auto vec = [&](int j) { return V.p + (size_t)j * n; };
    // start vector N(0,1), normalised (stored)
    k_randn<<<grid_for(n, 256), 256, 0, st>>>(w.p, n, cfg.seed, 0);
    std::vector<double> h;
    s = vx.dots<VT>(V.p, n, 0, w.p, h);
    if (s) return s;
    QSI_CUDA(cudaMemcpyAsync(vx.red, &h[0], 8, cudaMemcpyHostToDevice, st));
    k_scale_store<VT><<<grid_for(n, 256), 256, 0, st>>>(w.p, vx.red, vec(0), n);
    std::vector<double> alpha(m, 0.0), beta(m, 0.0), theta, coup;  // coup[i] = s_i couplings after restart
    int k = 0;
    int64_t applies = 0;
    int restarts = 0, nconv = 0;
    std::vector<double> Tw, TY;
    PhaseClock clk{st, sizeof(VT) == 4 ? "trlan-f32" : "trlan-f64"};
    for (;;) {
        for (int j = k; j < m; ++j) {
            clk.mark("setup/host");
            s = apply_to_w<VT>(op, vec(j), w.p, st);
            if (s) return s;
            ++applies;
            clk.mark("apply");
            if (kDF) k_split_f64<<<grid_for(n, 256), 256, 0, st>>>(w.p, wf.p, n);
            // full reorthogonalisation: classical Gram-Schmidt against v_0..v_j, repeated once
            // when the norm drops by more than 1/sqrt(2) (DGKS criterion)
            s = rdots(j + 1, h);
            if (s) return s;
            double before = h[j + 1];
            double a = h[j];
            std::vector<double> hh(h.begin(), h.begin() + j + 1);
            double nrm2 = 0;
            s = raxpy(j + 1, hh, nrm2);
            if (s) return s;
            if (nrm2 < 0.5 * before) {
                s = rdots(j + 1, h);
                if (s) return s;
                a += h[j];
                hh.assign(h.begin(), h.begin() + j + 1);
                s = raxpy(j + 1, hh, nrm2);
                if (s) return s;
            }
            alpha[j] = a;
            double b = std::sqrt(std::max(nrm2, 0.0));
            if (!(b > 1e-13 * std::max(1.0, std::fabs(a)))) {
                // invariant subspace: continue from a fresh random direction orthogonal to V
                b = 0.0;
                k_randn<<<grid_for(n, 256), 256, 0, st>>>(w.p, n, cfg.seed + 7919 * (uint64_t)(j + 1 + restarts * m), 0);
                if (kDF) k_split_f64<<<grid_for(n, 256), 256, 0, st>>>(w.p, wf.p, n);
                for (int pass = 0; pass < 2; ++pass) {
                    s = rdots(j + 1, h);
                    if (s) return s;
                    hh.assign(h.begin(), h.begin() + j + 1);
                    s = raxpy(j + 1, hh, nrm2);
                    if (s) return s;
                }
            }
            beta[j] = b;
            QSI_CUDA(cudaMemcpyAsync(vx.red, &nrm2, 8, cudaMemcpyHostToDevice, st));
            if constexpr (kDF)
                k_scale_store_df<<<grid_for(n, 256), 256, 0, st>>>(wf.p, vx.red, reinterpret_cast<float*>(vec(j + 1)), n);
            else
                k_scale_store<VT><<<grid_for(n, 256), 256, 0, st>>>(w.p, vx.red, vec(j + 1), n);
            clk.mark("orthogonalise");
        }
        // projected matrix: arrowhead (kept Ritz values + couplings) then tridiagonal
        std::vector<double> T((size_t)m * m, 0.0);
        for (int i = 0; i < k; ++i) {
            T[(size_t)i * m + i] = theta[i];
            T[(size_t)i * m + k] = T[(size_t)k * m + i] = coup[i];
        }
        for (int j = k; j < m; ++j) {
            T[(size_t)j * m + j] = alpha[j];
            if (j + 1 < m) T[(size_t)j * m + j + 1] = T[(size_t)(j + 1) * m + j] = beta[j];
        }
        clk.mark("setup/host");
        s = jacobi_eigh(T, m, 1, Tw, TY, st);
        if (s) return s;
        clk.mark("ritz");
        const double bl = beta[m - 1];
        nconv = 0;
        for (int i = 0; i < nev; ++i) {
            double r = std::fabs(bl * TY[(size_t)(m - 1) * m + i]);
            if (r < tol * std::max(eps23, std::fabs(Tw[i]))) ++nconv;
        }
        const bool exhausted = (m >= n);
        if (nconv >= nev || restarts >= cfg.max_iter || exhausted) break;
        ++restarts;
        int knew = std::min(m - 2, nev + std::max(nconv, (m - nev) / 2));
        knew = std::max(knew, std::min(nev, m - 2));
        if (knew < 1) knew = 1;
        std::vector<double> Yk((size_t)m * knew);
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < knew; ++j) Yk[(size_t)i * knew + j] = TY[(size_t)i * m + j];
        QSI_CUDA(cudaMemcpyAsync(dY.p, Yk.data(), Yk.size() * 8, cudaMemcpyHostToDevice, st));
        size_t smem = Yk.size() * 8;
        if (smem > 48 * 1024) cudaFuncSetAttribute(k_rotate<VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_rotate<VT><<<grid_for(n, 128), 128, smem, st>>>(V.p, n, m, knew, dY.p, n);
        QSI_CUDA(cudaMemcpyAsync(vec(knew), vec(m), (size_t)n * sizeof(VT), cudaMemcpyDeviceToDevice, st));
        theta.assign(Tw.begin(), Tw.begin() + knew);
        coup.resize(knew);
        for (int i = 0; i < knew; ++i) coup[i] = bl * TY[(size_t)(m - 1) * m + i];
        k = knew;
        QSI_CUDA(cudaGetLastError());
        clk.mark("restart");
    }
    // Ritz vectors in FP64
    DevBuf<double> X, HX;
    QSI_CUDA(X.alloc((size_t)nev * n, st));
    QSI_CUDA(HX.alloc((size_t)nev * n, st));
    {
        std::vector<double> Yk((size_t)m * nev);
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < nev; ++j) Yk[(size_t)i * nev + j] = TY[(size_t)i * m + j];
        QSI_CUDA(cudaMemcpyAsync(dY.p, Yk.data(), Yk.size() * 8, cudaMemcpyHostToDevice, st));
        size_t smem = Yk.size() * 8;
        if (smem > 48 * 1024) cudaFuncSetAttribute(k_ritz_vectors<VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_ritz_vectors<VT><<<grid_for(n, 128), 128, smem, st>>>(V.p, n, m, nev, dY.p, X.p, n);
        QSI_CUDA(cudaGetLastError());
    }
    std::vector<double> th(Tw.begin(), Tw.begin() + nev);
    // free the Krylov basis before polishing
    V.release();
    clk.mark("ritz vectors");
    s = finish_solve(op, cfg, vx, X, HX, th, nev, std::max(cfg.polish_steps, sizeof(VT) == 4 ? 1 : 0), applies, nconv,
                     restarts, m >= n, t0, evals, evecs, rep);
    clk.mark("polish");
    return s;
}

// ------------------------------------------------------------------ block thick-restart Lanczos (FP32 blocks)
// The mixed-precision solve for large bases.  A single FP32 vector costs an apply as much as an FP64 one (a random
// 4-byte gather moves the same memory sector as an 8-byte one), but the batched apply moves 16 FP32 vectors for
// little more than the price of one, so the Krylov space grows a block of kBlk vectors per apply: block Lanczos
// with full reorthogonalisation (two classical Gram-Schmidt passes per block) and thick restarts that keep whole
// blocks of Ritz vectors.  Blocks are stored [row][16] in FP32, the batched apply's layout.  Projections are
// FP32 products summed per 32-row tile and carried into double-float totals, reduced in FP64 in a fixed order
// (deterministic, and none of it on GB300's slow FP64 pipe); the block QR is Cholesky QR done twice.  The phase
// stops at the FP32 resolution (1e-7 relative residual) and the FP64 polish of finish_solve finishes the pairs.
constexpr int kBlk = 16;      // vectors per Krylov block
constexpr int kMaxBlk = 8;    // blocks per projection (128 vectors)
constexpr int kProjRows = 32; // rows per shared-memory tile
constexpr int kProjGrid = 1216;

struct BlockPtrs {
    const float* p[kMaxBlk];
};

// partial[blockIdx.x][r*16 + kq][c] = sum over this CTA's rows of Q_r[i][kq] * W[i][c], r < nq.
__global__ void __launch_bounds__(256) k_block_project(BlockPtrs qs, int nq, const float* __restrict__ W, int64_t n,
                                                       double* __restrict__ partial) {
    __shared__ __align__(16) float tq[kMaxBlk + 1][kProjRows][kBlk];
    const int t = threadIdx.x, kq = t >> 4, c = t & 15;
    float hi[kMaxBlk], lo[kMaxBlk];
#pragma unroll
    for (int r = 0; r < kMaxBlk; ++r) hi[r] = lo[r] = 0.f;
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t a = blockIdx.x * chunk, b = min(n, a + chunk);
    for (int64_t r0 = a; r0 < b; r0 += kProjRows) {
        const int rows = (int)min((int64_t)kProjRows, b - r0);
        __syncthreads();
        for (int idx = t; idx < (nq + 1) * kProjRows * 4; idx += blockDim.x) {
            const int blk = idx / (kProjRows * 4), e = idx % (kProjRows * 4), row = e >> 2, q4 = e & 3;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (row < rows) {
                const float* src = (blk < nq) ? qs.p[blk] : W;
                v = *reinterpret_cast<const float4*>(src + (r0 + row) * kBlk + q4 * 4);
            }
            *reinterpret_cast<float4*>(&tq[blk == nq ? kMaxBlk : blk][row][q4 * 4]) = v;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kMaxBlk; ++r) {
            if (r >= nq) break;
            float s = 0.f;
            for (int row = 0; row < rows; ++row) s = fmaf(tq[r][row][kq], tq[kMaxBlk][row][c], s);
            const float sum = hi[r] + s, bb = sum - hi[r];
            lo[r] += (hi[r] - (sum - bb)) + (s - bb);
            hi[r] = sum;
        }
    }
    for (int r = 0; r < nq; ++r)
        partial[((int64_t)blockIdx.x * nq * kBlk + r * kBlk + kq) * kBlk + c] = (double)hi[r] + (double)lo[r];
}

// out[e] = sum over blocks of partial[b][e] (e < count), fixed order.
__global__ void k_sum_partials(const double* __restrict__ partial, int nblocks, int count, double* __restrict__ out) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nblocks; ++b) s += partial[(int64_t)b * count + e];
        out[e] = s;
    }
}

// out_o[i][c'] = sum_k Q[i][k] Y[k][o*16 + c'] for the nout output blocks (sub: out_o[i][c'] -= that sum), with
// Y given as (hi, lo) float pairs ([16 nq][16 nout] row-major).  FP64 output: the first n64 of those vectors into
// out64 (vector-major, vector v at out64 + v * n) instead of FP32 blocks.
__global__ void __launch_bounds__(256) k_block_combine(BlockPtrs qs, int nq, const float2* __restrict__ Y, int nout,
                                                       float* const* __restrict__ outs, int sub, double* __restrict__ out64,
                                                       int n64, int64_t n) {
    extern __shared__ __align__(16) unsigned char smem[];
    float2* ys = reinterpret_cast<float2*>(smem);                                   // [16 nq][16 nout]
    float* tq = reinterpret_cast<float*>(ys + (size_t)nq * kBlk * nout * kBlk);  // [nq][16 rows][16]
    const int ncol = nout * kBlk;
    for (int e = threadIdx.x; e < nq * kBlk * ncol; e += blockDim.x) ys[e] = Y[e];
    const int rowl = threadIdx.x >> 4, c = threadIdx.x & 15;
    for (int64_t r0 = (int64_t)blockIdx.x * 16; r0 < n; r0 += (int64_t)gridDim.x * 16) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < nq * 16 * 4; idx += blockDim.x) {
            const int blk = idx >> 6, e = idx & 63, row = e >> 2, q4 = e & 3;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (r0 + row < n) v = *reinterpret_cast<const float4*>(qs.p[blk] + (r0 + row) * kBlk + q4 * 4);
            *reinterpret_cast<float4*>(tq + (blk * 16 + row) * kBlk + q4 * 4) = v;
        }
        __syncthreads();
        const int64_t i = r0 + rowl;
        if (i >= n) continue;
        for (int o = 0; o < nout; ++o) {
            float sh = 0.f, sl = 0.f;
            for (int r = 0; r < nq; ++r)
#pragma unroll
                for (int k = 0; k < kBlk; ++k) {
                    const float q = tq[(r * 16 + rowl) * kBlk + k];
                    const float2 y = ys[(size_t)(r * kBlk + k) * ncol + o * kBlk + c];
                    sh = fmaf(q, y.x, sh);
                    sl = fmaf(q, y.y, sl);
                }
            if (out64) {
                if (o * kBlk + c < n64) out64[(int64_t)(o * kBlk + c) * n + i] = (double)sh + (double)sl;
            } else {
                float* dst = outs[o] + i * kBlk + c;
                *dst = sub ? *dst - (sh + sl) : sh + sl;
            }
        }
    }
}

// Deterministic N(0,1) entries of an FP32 block (count = rows * 16).
__global__ void k_randn_f32(float* __restrict__ w, int64_t count, uint64_t seed) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < count; r += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t a = splitmix64(seed * 0x632be59bd9b4e019ULL + 2 * (uint64_t)r);
        const uint64_t b = splitmix64(seed * 0x632be59bd9b4e019ULL + 2 * (uint64_t)r + 1);
        const double u1 = ((a >> 11) + 1) * (1.0 / 9007199254740993.0), u2 = (b >> 11) * (1.0 / 9007199254740992.0);
        w[r] = (float)(sqrt(-2.0 * log(u1)) * cospi(2.0 * u2));
    }
}

struct BlockSolver {
    qsi_op* op;
    int64_t n;
    cudaStream_t st;
    DevBuf<double> partial, red;
    DevBuf<float2> ymat;
    DevBuf<float*> outp;
    qsi_status init() {
        n = op->basis->n;
        st = op->stream;
        QSI_CUDA(partial.alloc((size_t)kProjGrid * kMaxBlk * kBlk * kBlk, st));
        QSI_CUDA(red.alloc((size_t)kMaxBlk * kBlk * kBlk, st));
        QSI_CUDA(ymat.alloc((size_t)kMaxBlk * kBlk * kMaxBlk * kBlk, st));
        QSI_CUDA(outp.alloc(kMaxBlk, st));
        return QSI_OK;
    }
    // C (16 nq x 16, row-major, host) = [Q_0 .. Q_{nq-1}]^T W
    qsi_status project(float* const* Q, int nq, const float* W, std::vector<double>& C) {
        BlockPtrs bp{};
        for (int r = 0; r < nq; ++r) bp.p[r] = Q[r];
        k_block_project<<<kProjGrid, 256, 0, st>>>(bp, nq, W, n, partial.p);
        const int count = nq * kBlk * kBlk;
        k_sum_partials<<<(count + 255) / 256, 256, 0, st>>>(partial.p, kProjGrid, count, red.p);
        C.resize(count);
        QSI_CUDA(cudaMemcpyAsync(C.data(), red.p, (size_t)count * 8, cudaMemcpyDeviceToHost, st));
        QSI_CUDA(cudaStreamSynchronize(st));
        return QSI_OK;
    }
    // outs (nout blocks) = or -= Q Y, Y (16 nq x 16 nout, row-major FP64); or FP64 vector-major into out64
    qsi_status combine(float* const* Q, int nq, const std::vector<double>& Y, int nout, float* const* outs, int sub,
                       double* out64 = nullptr, int n64 = 0) {
        BlockPtrs bp{};
        for (int r = 0; r < nq; ++r) bp.p[r] = Q[r];
        std::vector<float2> yf(Y.size());
        for (size_t e = 0; e < Y.size(); ++e) {
            const float h = (float)Y[e];
            yf[e] = make_float2(h, (float)(Y[e] - (double)h));
        }
        QSI_CUDA(cudaMemcpyAsync(ymat.p, yf.data(), yf.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
        if (!out64) QSI_CUDA(cudaMemcpyAsync(outp.p, outs, (size_t)nout * sizeof(float*), cudaMemcpyHostToDevice, st));
        const size_t smem = yf.size() * sizeof(float2) + (size_t)nq * 16 * kBlk * sizeof(float);
        if (smem > 48 * 1024) cudaFuncSetAttribute(k_block_combine, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int dev = 0, sms = 148;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int grid = (int)std::min<int64_t>((n + 15) / 16, (int64_t)sms * 4);
        k_block_combine<<<grid, 256, smem, st>>>(bp, nq, ymat.p, nout, outp.p, sub, out64, n64, n);
        QSI_CUDA(cudaGetLastError());
        QSI_CUDA(cudaStreamSynchronize(st));  // the host-side Y / pointer copies are reused by the next call
        return QSI_OK;
    }
    // W <- W - Q C twice (classical Gram-Schmidt, repeated); C accumulates both passes' coefficients
    qsi_status orthogonalise(float* const* Q, int nq, float* W, std::vector<double>& C) {
        std::vector<double> C2;
        qsi_status s = project(Q, nq, W, C);
        if (s) return s;
        s = combine(Q, nq, C, 1, &W, 1);
        if (s) return s;
        s = project(Q, nq, W, C2);
        if (s) return s;
        s = combine(Q, nq, C2, 1, &W, 1);
        if (s) return s;
        for (size_t e = 0; e < C.size(); ++e) C[e] += C2[e];
        return QSI_OK;
    }
    // Cholesky QR of W (twice): Qout = W R^{-1} with R upper triangular (16 x 16, row-major, returned).  ok =
    // false when W is numerically rank deficient.
    qsi_status cholqr(float* W, float* Qout, std::vector<double>& R, bool& ok) {
        R.assign(kBlk * kBlk, 0.0);
        for (int e = 0; e < kBlk; ++e) R[e * kBlk + e] = 1.0;
        float* src = W;
        for (int pass = 0; pass < 2; ++pass) {
            std::vector<double> G;
            qsi_status s = project(&src, 1, src, G);
            if (s) return s;
            // G = L L^T (lower), R_pass = L^T; R_pass^{-1}
            std::vector<double> L(kBlk * kBlk, 0.0);
            double gmax = 0.0;
            for (int e = 0; e < kBlk; ++e) gmax = std::max(gmax, G[e * kBlk + e]);
            ok = gmax > 0.0;
            for (int j = 0; j < kBlk && ok; ++j) {
                double d = G[j * kBlk + j];
                for (int k = 0; k < j; ++k) d -= L[j * kBlk + k] * L[j * kBlk + k];
                if (!(d > 1e-24 * gmax)) {
                    ok = false;
                    break;
                }
                L[j * kBlk + j] = std::sqrt(d);
                for (int i = j + 1; i < kBlk; ++i) {
                    double v = G[i * kBlk + j];
                    for (int k = 0; k < j; ++k) v -= L[i * kBlk + k] * L[j * kBlk + k];
                    L[i * kBlk + j] = v / L[j * kBlk + j];
                }
            }
            if (!ok) return QSI_OK;
            // Rinv = (L^T)^{-1} (upper triangular): solve L^T X = I column by column
            std::vector<double> Rinv(kBlk * kBlk, 0.0), Rp(kBlk * kBlk, 0.0);
            for (int i = 0; i < kBlk; ++i)
                for (int j = 0; j < kBlk; ++j) Rp[i * kBlk + j] = L[j * kBlk + i];
            for (int c = 0; c < kBlk; ++c)
                for (int i = kBlk - 1; i >= 0; --i) {
                    double v = (i == c) ? 1.0 : 0.0;
                    for (int k = i + 1; k < kBlk; ++k) v -= Rp[i * kBlk + k] * Rinv[k * kBlk + c];
                    Rinv[i * kBlk + c] = v / Rp[i * kBlk + i];
                }
            s = combine(&src, 1, Rinv, 1, &Qout, 0);
            if (s) return s;
            // R <- Rp R
            std::vector<double> Rn(kBlk * kBlk, 0.0);
            for (int i = 0; i < kBlk; ++i)
                for (int j = 0; j < kBlk; ++j) {
                    double v = 0.0;
                    for (int k = 0; k < kBlk; ++k) v += Rp[i * kBlk + k] * R[k * kBlk + j];
                    Rn[i * kBlk + j] = v;
                }
            R = Rn;
            if (pass == 0) {  // second pass in place on Qout: copy into W's buffer first
                QSI_CUDA(cudaMemcpyAsync(W, Qout, (size_t)n * kBlk * sizeof(float), cudaMemcpyDeviceToDevice, st));
                src = W;
            }
        }
        return QSI_OK;
    }
};

// Block thick-restart Lanczos, FP32 Krylov blocks of kBlk vectors (see above), then the FP64 polish.
static qsi_status btrlan(qsi_op* op, const qsi_lanczos_cfg& cfg, double* evals, double* evecs, qsi_report* rep) {
    auto t0 = std::chrono::steady_clock::now();
    BlockSolver B{op};
    qsi_status s = B.init();
    if (s) return s;
    const int64_t n = B.n;
    cudaStream_t st = B.st;
    PhaseClock clk{st, "btrlan"};
    const int nev = std::max(1, cfg.nev);
    const int keep = ((nev + std::max(nev, 6) + kBlk - 1) / kBlk) * kBlk;  // kept Ritz vectors, whole blocks
    const int kb = keep / kBlk;
    int nblk = std::max(kb + 4, (cfg.ncv + kBlk - 1) / kBlk);  // at least four new blocks per restart cycle
    nblk = std::min(nblk, kMaxBlk - 1);
    if (kb + 2 > nblk || nev > keep || (int64_t)(nblk + 1) * kBlk > n)
        return fail(QSI_INVALID_ARG, "block lanczos: nev %d needs more Krylov blocks than fit (dim %lld)", nev, (long long)n);
    const int m = nblk * kBlk;
    const double tol = std::max(cfg.tol > 0 ? cfg.tol : 1e-10, cfg.polish_steps >= 2 ? fp32_stop(cfg.polish_steps) : 0.0);
    const double eps23 = std::pow(2.220446049250313e-16, 2.0 / 3.0);
    // nblk + 1 Krylov blocks, W and one spare block (the Cholesky QR output; also half of the restart scratch)
    std::vector<DevBuf<float>> store(nblk + 3);
    for (auto& b : store) QSI_CUDA(b.alloc((size_t)n * kBlk, st));
    std::vector<float*> Q(nblk + 1);
    for (int j = 0; j <= nblk; ++j) Q[j] = store[j].p;
    float* W = store[nblk + 1].p;
    float* spare = store[nblk + 2].p;
    // start block: N(0,1), orthonormalised
    std::vector<double> R, C;
    bool ok = false;
    for (int attempt = 0; attempt < 4 && !ok; ++attempt) {
        k_randn_f32<<<grid_for(n * kBlk, 256), 256, 0, st>>>(W, n * kBlk, cfg.seed + 1000003ULL * attempt);
        s = B.cholqr(W, Q[0], R, ok);
        if (s) return s;
    }
    if (!ok) return fail(QSI_NOT_CONVERGED, "block lanczos: no independent start block");
    std::vector<double> T((size_t)m * m, 0.0), Tw, TY, Blast(kBlk * kBlk, 0.0);
    int k0 = 0;  // blocks kept from the previous cycle
    int64_t applies = 0;
    int restarts = 0, nconv = 0;
    uint64_t breakdowns = 0;
    for (;;) {
        for (int j = k0; j < nblk; ++j) {
            clk.mark("setup/host");
            s = launch_apply(op, Q[j], W, kBlk, QSI_F32, 0, st);
            if (s) return s;
            applies += kBlk;
            clk.mark("apply");
            s = B.orthogonalise(Q.data(), j + 1, W, C);
            if (s) return s;
            clk.mark("orthogonalise");
            // projected matrix column block j: T[0 .. 16(j+1), 16j .. 16j+16) = C, mirrored; its diagonal block
            // symmetrised
            for (int r = 0; r < (j + 1) * kBlk; ++r)
                for (int c = 0; c < kBlk; ++c) {
                    const int cc = j * kBlk + c;
                    double v = C[(size_t)r * kBlk + c];
                    if (r >= j * kBlk) v = 0.5 * (v + C[(size_t)(j * kBlk + c) * kBlk + (r - j * kBlk)]);
                    T[(size_t)r * m + cc] = T[(size_t)cc * m + r] = v;
                }
            s = B.cholqr(W, Q[j + 1], R, ok);
            if (s) return s;
            clk.mark("cholqr");
            if (!ok) {  // the Krylov space became invariant: continue from random directions orthogonal to it
                ++breakdowns;
                for (int attempt = 0; attempt < 4 && !ok; ++attempt) {
                    k_randn_f32<<<grid_for(n * kBlk, 256), 256, 0, st>>>(W, n * kBlk, cfg.seed + 7919ULL * (breakdowns * 16 + attempt));
                    s = B.orthogonalise(Q.data(), j + 1, W, C);
                    if (s) return s;
                    s = B.cholqr(W, Q[j + 1], R, ok);
                    if (s) return s;
                }
                if (!ok) return fail(QSI_NOT_CONVERGED, "block lanczos: breakdown");
                std::fill(R.begin(), R.end(), 0.0);
            }
            if (j + 1 < nblk) {
                for (int a = 0; a < kBlk; ++a)
                    for (int c = 0; c < kBlk; ++c)
                        T[(size_t)((j + 1) * kBlk + a) * m + j * kBlk + c] = T[(size_t)(j * kBlk + c) * m + (j + 1) * kBlk + a] =
                            R[(size_t)a * kBlk + c];
            } else {
                Blast = R;
            }
        }
        clk.mark("setup/host");
        s = jacobi_eigh(T, m, 1, Tw, TY, st);
        if (s) return s;
        clk.mark("ritz");
        // residual of Ritz pair i: || Blast y_last,i ||, y_last,i = the last block's components
        std::vector<double> res(m, 0.0);
        for (int i = 0; i < m; ++i) {
            double acc = 0.0;
            for (int a = 0; a < kBlk; ++a) {
                double v = 0.0;
                for (int c = 0; c < kBlk; ++c) v += Blast[(size_t)a * kBlk + c] * TY[(size_t)(m - kBlk + c) * m + i];
                acc += v * v;
            }
            res[i] = std::sqrt(acc);
        }
        nconv = 0;
        for (int i = 0; i < nev; ++i)
            if (res[i] < tol * std::max(eps23, std::fabs(Tw[i]))) ++nconv;
        if (nconv >= nev || restarts >= cfg.max_iter) break;
        ++restarts;
        // thick restart: the lowest `keep` Ritz vectors Q Y[:, :keep] into W and spare (kb <= 2 blocks), then
        // the residual block continues the space
        std::vector<double> Yk((size_t)m * keep);
        for (int r = 0; r < m; ++r)
            for (int c = 0; c < keep; ++c) Yk[(size_t)r * keep + c] = TY[(size_t)r * m + c];
        if (kb > 2) return fail(QSI_INVALID_ARG, "block lanczos: more than two kept blocks");
        float* outs[2] = {W, spare};
        s = B.combine(Q.data(), nblk, Yk, kb, outs, 0);
        if (s) return s;
        clk.mark("restart");
        // new basis: the Ritz blocks, then the residual block; every other buffer returns to the pool
        float* res_blk = Q[nblk];
        std::vector<float*> pool;
        for (int j = 0; j < nblk; ++j) pool.push_back(Q[j]);
        if (kb == 1) pool.push_back(spare);
        Q[0] = W;
        if (kb > 1) Q[1] = spare;
        Q[kb] = res_blk;
        size_t f = 0;
        for (int j = kb + 1; j <= nblk; ++j) Q[j] = pool[f++];
        W = pool[f++];
        spare = pool[f++];
        std::fill(T.begin(), T.end(), 0.0);
        for (int i = 0; i < keep; ++i) T[(size_t)i * m + i] = Tw[i];
        k0 = kb;
    }
    // FP64 Ritz vectors (vector-major) for the polish
    DevBuf<double> X, HX;
    QSI_CUDA(X.alloc((size_t)nev * n, st));
    QSI_CUDA(HX.alloc((size_t)nev * n, st));
    {
        const int nout = (nev + kBlk - 1) / kBlk;
        std::vector<double> Yn((size_t)m * nout * kBlk, 0.0);
        for (int r = 0; r < m; ++r)
            for (int c = 0; c < nev; ++c) Yn[(size_t)r * nout * kBlk + c] = TY[(size_t)r * m + c];
        s = B.combine(Q.data(), nblk, Yn, nout, nullptr, 0, X.p, nev);
        if (s) return s;
    }
    std::vector<double> th(Tw.begin(), Tw.begin() + nev);
    for (auto& b : store) b.release();
    Vecs vx;
    s = vx.init(n, st);
    if (s) return s;
    clk.mark("ritz vectors");
    s = finish_solve(op, cfg, vx, X, HX, th, nev, std::max(cfg.polish_steps, 1), applies, nconv, restarts, false, t0,
                     evals, evecs, rep);
    clk.mark("polish");
    return s;
}

// ------------------------------------------------------------------ eigval0 (mfeig0)
// Lowest eigenvalue of the symmetric tridiagonal (a, b) by Sturm-count
// multisection: each of the block's threads counts eigenvalues below one
// point; the bracket shrinks by blockDim+1 per round.
__global__ void k_tridiag_lowest(const double* __restrict__ a, const double* __restrict__ b, int m, double lo, double hi,
                                 double* out) {
    __shared__ int cnt[256];
    __shared__ double bounds[2];
    if (threadIdx.x == 0) bounds[0] = lo, bounds[1] = hi;
    __syncthreads();
    for (int round = 0; round < 12; ++round) {
        double L = bounds[0], H = bounds[1];
        double x = L + (H - L) * (threadIdx.x + 1) / (blockDim.x + 1);
        int c = 0;
        double d = 1.0;
        for (int i = 0; i < m; ++i) {
            double bb = (i > 0) ? b[i - 1] * b[i - 1] : 0.0;
            d = (a[i] - x) - (i > 0 ? bb / d : 0.0);
            if (d == 0.0) d = -1e-300;
            c += (d < 0.0);
        }
        cnt[threadIdx.x] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            // first point whose count >= 1 bounds the lowest eigenvalue from above
            int t = 0;
            while (t < (int)blockDim.x && cnt[t] < 1) ++t;
            double nl = (t == 0) ? L : L + (H - L) * t / (blockDim.x + 1);
            double nh = (t == (int)blockDim.x) ? H : L + (H - L) * (t + 1) / (blockDim.x + 1);
            bounds[0] = nl;
            bounds[1] = nh;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = 0.5 * (bounds[0] + bounds[1]);
}

// Eigenvector of the tridiagonal for eigenvalue lam by inverse iteration with
// a partially pivoted LU of (T - lam I) (one thread; m is the Krylov length).
__global__ void k_tridiag_vector(const double* __restrict__ a, const double* __restrict__ b, int m, double lam,
                                 double* __restrict__ work, double* __restrict__ y) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double* u0 = work;           // diagonal of U
    double* u1 = work + m;       // first superdiagonal
    double* u2 = work + 2 * m;   // second superdiagonal (from pivoting)
    double* l = work + 3 * m;    // multipliers
    int* piv = (int*)(work + 4 * m);
    double anorm = 0.0;
    for (int i = 0; i < m; ++i) anorm = fmax(anorm, fabs(a[i]) + (i ? fabs(b[i - 1]) : 0.0) + (i + 1 < m ? fabs(b[i]) : 0.0));
    double tiny = 1e-300 + 2.2e-16 * anorm;
    // factor
    double d = a[0] - lam, e = (m > 1) ? b[0] : 0.0, f = 0.0;
    for (int i = 0; i < m; ++i) {
        if (i + 1 < m) {
            double sub = b[i];
            double nd = a[i + 1] - lam, ne = (i + 2 < m) ? b[i + 1] : 0.0;
            if (fabs(d) >= fabs(sub)) {
                piv[i] = 0;
                double mult = (d != 0.0) ? sub / d : 0.0;
                l[i] = mult;
                u0[i] = d, u1[i] = e, u2[i] = f;
                d = nd - mult * e;
                e = ne - mult * f;
                f = 0.0;
                if (fabs(u0[i]) < tiny) u0[i] = tiny;
            } else {
                piv[i] = 1;
                double mult = d / sub;
                l[i] = mult;
                u0[i] = sub, u1[i] = nd, u2[i] = ne;
                double nd2 = e - mult * nd, ne2 = f - mult * ne;
                d = nd2;
                e = ne2;
                f = 0.0;
            }
        } else {
            u0[i] = (fabs(d) < tiny) ? tiny : d;
            u1[i] = 0.0;
            u2[i] = 0.0;
            piv[i] = 0;
            l[i] = 0.0;
        }
    }
    // Start from e_0: without reorthogonalisation the long recurrence holds
    // near-degenerate copies of the lowest Ritz value; the component of e_0 in
    // that cluster is the copy built from the start of the Lanczos sequence,
    // which is the part the second pass accumulates.
    for (int i = 0; i < m; ++i) y[i] = (i == 0) ? 1.0 : 0.0;
    for (int it = 0; it < 4; ++it) {
        // forward: apply row operations
        for (int i = 0; i + 1 < m; ++i) {
            if (piv[i]) {
                double t = y[i];
                y[i] = y[i + 1];
                y[i + 1] = t;
            }
            y[i + 1] -= l[i] * y[i];
        }
        // back substitution
        for (int i = m - 1; i >= 0; --i) {
            double v = y[i];
            if (i + 1 < m) v -= u1[i] * y[i + 1];
            if (i + 2 < m) v -= u2[i] * y[i + 2];
            y[i] = v / u0[i];
        }
        double nrm = 0.0;
        for (int i = 0; i < m; ++i) nrm += y[i] * y[i];
        nrm = sqrt(nrm);
        for (int i = 0; i < m; ++i) y[i] /= nrm;
    }
}

__global__ void k_axpby(double* __restrict__ y, const double* __restrict__ x, double a, double b, int64_t n) {
    // y = b*y + a*x
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        y[r] = b * y[r] + a * x[r];
}

static qsi_status lowest_of_tridiag(const std::vector<double>& al, const std::vector<double>& be, double& e0,
                                    cudaStream_t st) {
    const int m = (int)al.size();
    double lo = 1e300, hi = -1e300;
    for (int i = 0; i < m; ++i) {
        double r = (i ? std::fabs(be[i - 1]) : 0.0) + (i + 1 < m ? std::fabs(be[i]) : 0.0);
        lo = std::min(lo, al[i] - r);
        hi = std::max(hi, al[i] + r);
    }
    DevBuf<double> d;
    QSI_CUDA(d.alloc((size_t)2 * m + 1, st));
    QSI_CUDA(cudaMemcpyAsync(d.p, al.data(), (size_t)m * 8, cudaMemcpyHostToDevice, st));
    if (m > 1) QSI_CUDA(cudaMemcpyAsync(d.p + m, be.data(), (size_t)(m - 1) * 8, cudaMemcpyHostToDevice, st));
    k_tridiag_lowest<<<1, 256, 0, st>>>(d.p, d.p + m, m, lo - 1e-12 * std::fabs(lo) - 1e-300, hi, d.p + 2 * m);
    QSI_CUDA(cudaMemcpyAsync(&e0, d.p + 2 * m, 8, cudaMemcpyDeviceToHost, st));
    QSI_CUDA(cudaStreamSynchronize(st));
    return QSI_OK;
}

}  // namespace qsi

using namespace qsi;

extern "C" qsi_status qsi_lanczos_solve(qsi_op* op, const qsi_lanczos_cfg* cfg, double* evals, double* evecs,
                                        qsi_report* report) {
    return guarded([&]() -> qsi_status {
        if (!op || !cfg || !evals) return fail(QSI_INVALID_ARG, "qsi_lanczos_solve: null argument");
        if (report) std::memset(report, 0, sizeof(*report));
        if (cfg->precision == QSI_F32) {
            // FP32 Krylov blocks through the batched apply (btrlan) when asked (block == 16); by default the
            // single-vector solver with FP32 Krylov vectors (on the 96-spin sector the block solver needs seven
            // times the vector applies of single-vector Lanczos for the same ten eigenpairs, more than the
            // batched apply saves per vector)
            const bool block = cfg->block == kBlk;
            if (block) return btrlan(op, *cfg, evals, evecs, report);
            if (cfg->block != 0 && cfg->block != 1) return fail(QSI_INVALID_ARG, "qsi_lanczos_solve: block must be 0, 1 or 16");
            return trlan<float>(op, *cfg, evals, evecs, report);
        }
        return trlan<double>(op, *cfg, evals, evecs, report);
    });
}

namespace qsi {

// Checkpoint of the first eigval0 pass, the fields of projED::checkpoint::CheckpointData
// (components/operator/include/checkpoint_utils.hpp:48-57) as HDF5 datasets of the same names: v (current
// Lanczos vector), u (previous one), alphas, betas, beta, iteration, eigval, random_seed.
struct Eigval0Checkpoint {
    const char* path;
    int every;            // write every `every` iterations (0: only when stopping early)
    int stop_after;       // stop (and write) after this many iterations of this call (0: no limit)
    double wall_limit_s;  // stop (and write) once this much wall time has passed (0: no limit)
};

static qsi_status write_eigval0_checkpoint(const char* path, const double* d_v, const double* d_u, int64_t n,
                                           const std::vector<double>& al, const std::vector<double>& be, double beta,
                                           int64_t iteration, double eigval, uint64_t seed, cudaStream_t st) {
    auto f64 = [](const char* name, const double* p, size_t count, bool scalar) {
        h5::OutDataset d;
        d.name = name;
        d.type_class = 1;
        d.type_size = 8;
        if (!scalar) d.dims = {(uint64_t)count};
        d.data.resize(count * 8);
        if (count && p) std::memcpy(d.data.data(), p, count * 8);  // p == nullptr: filled by the caller
        return d;
    };
    std::vector<h5::OutDataset> ds;
    ds.push_back(f64("v", nullptr, (size_t)n, false));
    ds.push_back(f64("u", nullptr, (size_t)n, false));
    QSI_CUDA(cudaMemcpyAsync(ds[0].data.data(), d_v, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
    QSI_CUDA(cudaMemcpyAsync(ds[1].data.data(), d_u, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
    QSI_CUDA(cudaStreamSynchronize(st));
    ds.push_back(f64("alphas", al.data(), al.size(), false));
    ds.push_back(f64("betas", be.data(), be.size(), false));
    ds.push_back(f64("beta", &beta, 1, true));
    ds.push_back(f64("eigval", &eigval, 1, true));
    h5::OutDataset it;
    it.name = "iteration";
    it.type_class = 0;
    it.type_size = 8;
    it.data.resize(8);
    std::memcpy(it.data.data(), &iteration, 8);
    ds.push_back(it);
    h5::OutDataset sd;
    sd.name = "random_seed";
    sd.type_class = 0;
    sd.type_size = 4;
    sd.is_signed = true;
    const int32_t seed32 = (int32_t)(uint32_t)seed;
    sd.data.resize(4);
    std::memcpy(sd.data.data(), &seed32, 4);
    ds.push_back(sd);
    const std::string tmp = std::string(path) + ".tmp";
    try {
        h5::write_datasets(tmp.c_str(), ds);
    } catch (const std::exception& e) {
        return fail(QSI_IO_ERROR, "eigval0 checkpoint: %s", e.what());
    }
    if (std::rename(tmp.c_str(), path) != 0) return fail(QSI_IO_ERROR, "eigval0 checkpoint: cannot rename %s", tmp.c_str());
    return QSI_OK;
}

// projED::lanczos::eigval0 (components/linalg_routines/src/lanczos.cpp:67-227):
// unit start vector from std::mt19937(seed) + std::normal_distribution
// (set_random_unit, :55-62); u = -beta*u_prev + H v, alpha = <v,u>, u -= alpha v,
// beta = |u|; stop when beta < abs_tol, or from min_iterations on when the
// lowest Ritz value changes by less than abs_tol (absolute) or rel_tol
// (relative); a second identical pass accumulates the Ritz vector.  With a
// checkpoint, the first pass resumes from it and writes it at the top of an
// iteration (the state that iteration starts from).
static qsi_status eigval0_run(qsi_op* op, const qsi_eigval0_cfg* cfg, const Eigval0Checkpoint* ck, double* e0,
                              double* eigvec, int32_t* iterations) {
    const int64_t n = op->basis->n;
    cudaStream_t st = op->stream;
    std::vector<double> v0(n);
    {
        std::mt19937 rng((unsigned)cfg->seed);
        std::normal_distribution<double> dist(0.0, 1.0);
        for (auto& x : v0) x = dist(rng);
        double nrm = 0.0;
        for (double x : v0) nrm += x * x;
        nrm = std::sqrt(nrm);
        for (auto& x : v0) x /= nrm;
    }
    Vecs vx;
    qsi_status s = vx.init(n, st);
    if (s) return s;
    DevBuf<double> v, u, ev;
    QSI_CUDA(v.alloc(n, st));
    QSI_CUDA(u.alloc(n, st));
    std::vector<double> alphas, betas, ritz, h;
    double eig = 1e308, e0_pass0 = 0.0;
    int its = 0;
    const auto t_start = std::chrono::steady_clock::now();
    for (int pass = 0; pass < (cfg->calc_eigenvector ? 2 : 1); ++pass) {
        QSI_CUDA(cudaMemcpyAsync(v.p, v0.data(), (size_t)n * 8, cudaMemcpyHostToDevice, st));
        QSI_CUDA(cudaMemsetAsync(u.p, 0, (size_t)n * 8, st));
        if (pass == 1) {
            QSI_CUDA(ev.alloc(n, st));
            QSI_CUDA(cudaMemsetAsync(ev.p, 0, (size_t)n * 8, st));
        }
        std::vector<double> al, be;
        double beta = 0.0;
        int it, it0 = 0;
        if (pass == 0 && ck) {  // resume the first pass from an existing checkpoint of this run
            h5::OutDataset dv, du, da, db, dbeta, dit, dseed;
            bool have = false;
            try {
                have = h5::read_dataset(ck->path, "v", dv);
                if (have && !(h5::read_dataset(ck->path, "u", du) && h5::read_dataset(ck->path, "alphas", da) &&
                              h5::read_dataset(ck->path, "betas", db) && h5::read_dataset(ck->path, "beta", dbeta) &&
                              h5::read_dataset(ck->path, "iteration", dit) &&
                              h5::read_dataset(ck->path, "random_seed", dseed)))
                    return fail(QSI_IO_ERROR, "eigval0 checkpoint %s: missing datasets", ck->path);
            } catch (const std::exception& e) {
                return fail(QSI_IO_ERROR, "eigval0 checkpoint %s: %s", ck->path, e.what());
            }
            if (have) {
                int64_t itv = 0;
                int32_t seed32 = 0;
                if (dit.data.size() == 8) std::memcpy(&itv, dit.data.data(), 8);
                if (dseed.data.size() == 4) std::memcpy(&seed32, dseed.data.data(), 4);
                const size_t m = da.data.size() / 8;
                if (dv.type_class != 1 || dv.data.size() != (size_t)n * 8 || du.data.size() != (size_t)n * 8 ||
                    db.data.size() != m * 8 || (int64_t)m != itv || dbeta.data.size() != 8 ||
                    seed32 != (int32_t)(uint32_t)cfg->seed || itv > cfg->max_iterations)
                    return fail(QSI_INVALID_ARG, "eigval0 checkpoint %s: not a checkpoint of this run", ck->path);
                QSI_CUDA(cudaMemcpyAsync(v.p, dv.data.data(), (size_t)n * 8, cudaMemcpyHostToDevice, st));
                QSI_CUDA(cudaMemcpyAsync(u.p, du.data.data(), (size_t)n * 8, cudaMemcpyHostToDevice, st));
                QSI_CUDA(cudaStreamSynchronize(st));
                al.resize(m);
                be.resize(m);
                std::memcpy(al.data(), da.data.data(), m * 8);
                std::memcpy(be.data(), db.data.data(), m * 8);
                std::memcpy(&beta, dbeta.data.data(), 8);
                it0 = (int)itv;
            }
        }
        if (pass == 1) eig = 1e308;
        for (it = it0; it < cfg->max_iterations; ++it) {
            if (pass == 0 && ck && it > it0) {
                const double elapsed =
                    std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
                const bool stop = (ck->stop_after > 0 && it - it0 >= ck->stop_after) ||
                                  (ck->wall_limit_s > 0 && elapsed >= ck->wall_limit_s);
                if (stop || (ck->every > 0 && it % ck->every == 0)) {
                    double est = std::nan("");
                    if (!al.empty()) {
                        std::vector<double> b2(be.begin(), be.end() - 1);
                        s = lowest_of_tridiag(al, b2, est, st);
                        if (s) return s;
                    }
                    s = write_eigval0_checkpoint(ck->path, v.p, u.p, n, al, be, beta, it, est, cfg->seed, st);
                    if (s) return s;
                }
                if (stop) {
                    if (iterations) *iterations = it;
                    return fail(QSI_TIMEOUT, "eigval0: stopped at iteration %d, checkpoint written to %s", it, ck->path);
                }
            }
            if (pass == 1 && it < (int)ritz.size())
                k_axpby<<<grid_for(n, 256), 256, 0, st>>>(ev.p, v.p, ritz[it], 1.0, n);
            if (it > 0) k_axpby<<<grid_for(n, 256), 256, 0, st>>>(u.p, v.p, 0.0, -beta, n);
            s = launch_apply(op, v.p, u.p, 1, QSI_F64, 1, st);
            if (s) return s;
            s = vx.dots<double>(v.p, n, 1, u.p, h);
            if (s) return s;
            double alpha = h[0];
            k_axpby<<<grid_for(n, 256), 256, 0, st>>>(u.p, v.p, -alpha, 1.0, n);
            s = vx.dots<double>(v.p, n, 0, u.p, h);
            if (s) return s;
            beta = std::sqrt(h[0]);
            if (beta < cfg->abs_tol) break;
            std::swap(v.p, u.p);
            k_axpby<<<grid_for(n, 256), 256, 0, st>>>(v.p, v.p, 0.0, 1.0 / beta, n);
            al.push_back(alpha);
            be.push_back(beta);
            // The first pass never stops on convergence (lanczos.cpp:163-167 breaks
            // only when a Ritz vector is being accumulated); the second pass does.
            if (pass == 1 && it >= cfg->min_iterations) {
                double old = eig;
                std::vector<double> b2(be.begin(), be.end() - 1);
                s = lowest_of_tridiag(al, b2, eig, st);
                if (s) return s;
                double err = std::fabs(eig - old);
                double rel = err / std::max(std::fabs(eig), 1e-10);
                if (err < cfg->abs_tol || rel < cfg->rel_tol) break;
            }
        }
        if (pass == 0) {
            its = it;
            alphas = al;
            betas = be;
            std::vector<double> b2(be.begin(), be.empty() ? be.end() : be.end() - 1);
            s = lowest_of_tridiag(al, b2, eig, st);
            if (s) return s;
            e0_pass0 = eig;
            if (cfg->calc_eigenvector) {
                const int m = (int)al.size();
                DevBuf<double> d, work, y;
                QSI_CUDA(d.alloc((size_t)2 * m, st));
                QSI_CUDA(work.alloc((size_t)5 * m + 8, st));
                QSI_CUDA(y.alloc((size_t)m, st));
                QSI_CUDA(cudaMemcpyAsync(d.p, al.data(), (size_t)m * 8, cudaMemcpyHostToDevice, st));
                if (m > 1) QSI_CUDA(cudaMemcpyAsync(d.p + m, b2.data(), (size_t)(m - 1) * 8, cudaMemcpyHostToDevice, st));
                k_tridiag_vector<<<1, 32, 0, st>>>(d.p, d.p + m, m, eig, work.p, y.p);
                ritz.resize(m);
                QSI_CUDA(cudaMemcpyAsync(ritz.data(), y.p, (size_t)m * 8, cudaMemcpyDeviceToHost, st));
                QSI_CUDA(cudaStreamSynchronize(st));
            }
        }
    }
    *e0 = e0_pass0;
    if (iterations) *iterations = its;
    if (cfg->calc_eigenvector && eigvec) {
        QSI_CUDA(cudaMemcpyAsync(eigvec, ev.p, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
        QSI_CUDA(cudaStreamSynchronize(st));
    }
    return QSI_OK;
}

}  // namespace qsi

extern "C" qsi_status qsi_eigval0(qsi_op* op, const qsi_eigval0_cfg* cfg, double* e0, double* eigvec,
                                  int32_t* iterations) {
    return guarded([&]() -> qsi_status {
        if (!op || !cfg || !e0) return fail(QSI_INVALID_ARG, "qsi_eigval0: null argument");
        return eigval0_run(op, cfg, nullptr, e0, eigvec, iterations);
    });
}

extern "C" qsi_status qsi_eigval0_checkpointed(qsi_op* op, const qsi_eigval0_cfg* cfg, const char* path, int32_t every,
                                               int32_t stop_after, double wall_limit_s, double* e0, double* eigvec,
                                               int32_t* iterations) {
    return guarded([&]() -> qsi_status {
        if (!op || !cfg || !e0 || !path || every < 0 || stop_after < 0 || wall_limit_s < 0)
            return fail(QSI_INVALID_ARG, "qsi_eigval0_checkpointed: bad argument");
        const Eigval0Checkpoint ck{path, every, stop_after, wall_limit_s};
        return eigval0_run(op, cfg, &ck, e0, eigvec, iterations);
    });
}

// ------------------------------------------------------------------ expectation values
// compute_all_expectations / compute_cross_correlation (src/expectation_eval.cpp:27-110) on the device:
// expect[l][i][j] = psi_j . (O_l psi_i), cross[l][m][i][j] = (O_l psi_i) . (O_m psi_j).  Each operator l
// (terms[off[l] .. off[l+1])) is bound to the basis in turn; W_{l,i} = O_l psi_i is one FP64 apply.  The
// dots are the fixed-order FP64 reductions of the Lanczos drivers.
extern "C" qsi_status qsi_expectations(qsi_basis* b, const qsi_term* terms, const int32_t* op_offsets, int32_t n_ops,
                                       const double* psi, int32_t nvec, double* expect, double* cross) {
    return guarded([&]() -> qsi_status {
        if (!b || !terms || !op_offsets || n_ops < 1 || !psi || nvec < 1 || nvec > 256 || !expect)
            return fail(QSI_INVALID_ARG, "qsi_expectations: bad argument (1 <= nvec <= 256)");
        for (int l = 0; l < n_ops; ++l)
            if (op_offsets[l + 1] < op_offsets[l] || op_offsets[l] < 0)
                return fail(QSI_INVALID_ARG, "qsi_expectations: operator offsets must not decrease");
        const int64_t n = b->n;
        const int64_t K = (int64_t)n_ops * nvec;  // vectors W_{l,i}, index l*nvec + i
        cudaStream_t st = nullptr;
        QSI_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard() {
                cudaStreamSynchronize(s);
                cudaStreamDestroy(s);
            }
        } guard{st};
        if (cross) {
            size_t free_b = 0, total_b = 0;
            QSI_CUDA(cudaMemGetInfo(&free_b, &total_b));
            const double need = ((double)K + nvec + 1) * (double)n * 8.0;
            if (need > 0.9 * (double)free_b)
                return fail(QSI_OOM, "qsi_expectations: %lld vectors of %lld states exceed device memory",
                            (long long)K, (long long)n);
        }
        Vecs vx;
        qsi_status s = vx.init(n, st);
        if (s) return s;
        DevBuf<double> P, W;
        QSI_CUDA(P.alloc((size_t)n * nvec, st));
        QSI_CUDA(cudaMemcpyAsync(P.p, psi, (size_t)n * nvec * 8, cudaMemcpyHostToDevice, st));
        QSI_CUDA(W.alloc((size_t)n * (cross ? K : 1), st));
        std::vector<double> h;
        for (int l = 0; l < n_ops; ++l) {
            qsi_op* op = nullptr;
            s = qsi_op_create(b, terms + op_offsets[l], op_offsets[l + 1] - op_offsets[l], &op);
            if (s) return s;
            for (int i = 0; i < nvec && s == QSI_OK; ++i) {
                double* w = W.p + (cross ? (size_t)(l * nvec + i) * n : 0);
                QSI_CUDA(cudaStreamSynchronize(st));
                s = launch_apply(op, P.p + (size_t)i * n, w, 1, QSI_F64, 0, op->stream);
                if (s == QSI_OK && cudaStreamSynchronize(op->stream) != cudaSuccess) s = fail(QSI_CUDA_ERROR, "apply");
                if (s == QSI_OK) s = vx.dots<double>(P.p, n, nvec, w, h);
                for (int j = 0; j < nvec && s == QSI_OK; ++j) expect[((size_t)l * nvec + i) * nvec + j] = h[j];
            }
            qsi_op_destroy(op);
            if (s) return s;
        }
        if (cross) {
            std::vector<double> col((size_t)K);
            for (int m = 0; m < n_ops; ++m)
                for (int j = 0; j < nvec; ++j) {
                    const double* wmj = W.p + (size_t)(m * nvec + j) * n;
                    for (int64_t c0 = 0; c0 < K; c0 += 256) {  // the reduction buffers hold 256 dots
                        const int kc = (int)std::min<int64_t>(256, K - c0);
                        s = vx.dots<double>(W.p + (size_t)c0 * n, n, kc, wmj, h);
                        if (s) return s;
                        std::copy(h.begin(), h.begin() + kc, col.begin() + c0);
                    }
                    for (int l = 0; l < n_ops; ++l)
                        for (int i = 0; i < nvec; ++i)
                            cross[(((size_t)l * n_ops + m) * nvec + i) * nvec + j] = col[(size_t)l * nvec + i];
                }
        }
        return QSI_OK;
    });
}

// ------------------------------------------------------------------ FTLM
namespace qsi {

// Rademacher start vectors +-1/sqrt(n), one per column r: [row][R] layout.
template <typename VT>
__global__ void k_ftlm_init(VT* __restrict__ cur, VT* __restrict__ prev, int64_t n, int R, uint64_t seed) {
    const double inv = rsqrt((double)n);
    const int64_t total = n * R;
    const int shift = __ffs(R) - 1;  // R is a power of two
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e >> shift;
        const int r = (int)(e & (R - 1));
        uint64_t h = splitmix64(seed ^ splitmix64(((uint64_t)r << 40) ^ (uint64_t)i));
        cur[e] = (VT)((h >> 63) ? inv : -inv);
        prev[e] = (VT)0;
    }
}

// Double-float helpers for the FP32 recurrences: error-free products of FP32
// values and FP64 coefficients split into (hi, lo) floats.
struct F2 {
    float hi, lo;
};
__device__ __forceinline__ void f2_fma(F2& a, float ch, float cl, float x) {
    const float p = ch * x;
    const float e = fmaf(ch, x, -p) + cl * x;
    const float s = a.hi + p;
    const float bb = s - a.hi;
    const float err = (a.hi - (s - bb)) + (p - bb);
    a.hi = s;
    a.lo += err + e;
}
__device__ __forceinline__ double f2_value(const F2& a) { return (double)a.hi + (double)a.lo; }

// VW consecutive elements of a row-major [n][R] array in registers, moved with one 16-byte access when
// VW > 1 (R is a multiple of VW and the arrays are 16-byte aligned).
template <typename VT, int VW>
__device__ __forceinline__ void load_vec(const VT* __restrict__ p, VT (&v)[VW]) {
    if constexpr (VW == 1) {
        v[0] = *p;
    } else if constexpr (sizeof(VT) == 4 && VW == 4) {
        const float4 t = *reinterpret_cast<const float4*>(p);
        v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w;
    } else {
        static_assert(sizeof(VT) == 8 && VW == 2, "16-byte vectors");
        const double2 t = *reinterpret_cast<const double2*>(p);
        v[0] = t.x, v[1] = t.y;
    }
}
template <typename VT, int VW>
__device__ __forceinline__ void store_vec(VT* __restrict__ p, const VT (&v)[VW]) {
    if constexpr (VW == 1) {
        *p = v[0];
    } else if constexpr (sizeof(VT) == 4 && VW == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
        *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
    }
}

// Layout of the column kernels: a thread owns VW consecutive columns of a row, R/VW threads cover a row,
// a block takes blockDim*VW/R rows per pass over its contiguous chunk of rows, kColUnroll passes at a
// time (their loads in flight together).  Per-column block sums are formed in a fixed order.
constexpr int kColUnroll = 4;
struct ColLayout {
    int lpr, rpp, c0, sub;
    int64_t i0, i1;
    template <int VW>
    __device__ static ColLayout make(int64_t n, int R) {
        ColLayout L;
        L.lpr = R / VW;
        L.rpp = blockDim.x / L.lpr;
        L.c0 = (threadIdx.x % L.lpr) * VW;
        L.sub = threadIdx.x / L.lpr;
        const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
        L.i0 = blockIdx.x * chunk;
        L.i1 = min(n, L.i0 + chunk);
        return L;
    }
};

// partial[block][c] = sum over the block's threads of res (VW columns per thread), in sub order.
template <int VW>
__device__ __forceinline__ void col_block_sum(const ColLayout& L, const double (&res)[VW], int R, double* sh,
                                              double* __restrict__ partial) {
#pragma unroll
    for (int k = 0; k < VW; ++k) sh[L.sub * R + L.c0 + k] = res[k];
    __syncthreads();
    for (int c = threadIdx.x; c < R; c += blockDim.x) {
        double t = 0.0;
        for (int q = 0; q < L.rpp; ++q) t += sh[q * R + c];
        partial[(int64_t)blockIdx.x * R + c] = t;
    }
}

// Per-column partial sums over one block's rows of a[i][r] * b[i][r]: FP64 for
// FP64 storage, double-float for FP32 storage.
template <typename VT, int VW>
__global__ void __launch_bounds__(256) k_col_dots(const VT* __restrict__ a, const VT* __restrict__ b, int64_t n, int R,
                                                  double* __restrict__ partial) {
    __shared__ double sh[256 * VW];
    const ColLayout L = ColLayout::make<VW>(n, R);
    double res[VW];
    if constexpr (sizeof(VT) == 4) {
        F2 acc[VW];
#pragma unroll
        for (int k = 0; k < VW; ++k) acc[k] = F2{0.f, 0.f};
        for (int64_t i = L.i0 + L.sub; i < L.i1; i += (int64_t)L.rpp * kColUnroll) {
            VT av[kColUnroll][VW], bv[kColUnroll][VW];
#pragma unroll
            for (int u = 0; u < kColUnroll; ++u) {
                const int64_t ii = i + (int64_t)u * L.rpp;
                if (ii < L.i1) {
                    load_vec<VT, VW>(a + ii * R + L.c0, av[u]);
                    load_vec<VT, VW>(b + ii * R + L.c0, bv[u]);
                } else {
#pragma unroll
                    for (int k = 0; k < VW; ++k) av[u][k] = bv[u][k] = (VT)0;
                }
            }
#pragma unroll
            for (int u = 0; u < kColUnroll; ++u)
#pragma unroll
                for (int k = 0; k < VW; ++k) f2_fma(acc[k], (float)av[u][k], 0.f, (float)bv[u][k]);
        }
#pragma unroll
        for (int k = 0; k < VW; ++k) res[k] = f2_value(acc[k]);
    } else {
#pragma unroll
        for (int k = 0; k < VW; ++k) res[k] = 0.0;
        for (int64_t i = L.i0 + L.sub; i < L.i1; i += (int64_t)L.rpp * kColUnroll) {
            VT av[kColUnroll][VW], bv[kColUnroll][VW];
#pragma unroll
            for (int u = 0; u < kColUnroll; ++u) {
                const int64_t ii = i + (int64_t)u * L.rpp;
                if (ii < L.i1) {
                    load_vec<VT, VW>(a + ii * R + L.c0, av[u]);
                    load_vec<VT, VW>(b + ii * R + L.c0, bv[u]);
                } else {
#pragma unroll
                    for (int k = 0; k < VW; ++k) av[u][k] = bv[u][k] = (VT)0;
                }
            }
#pragma unroll
            for (int u = 0; u < kColUnroll; ++u)
#pragma unroll
                for (int k = 0; k < VW; ++k) res[k] += (double)av[u][k] * (double)bv[u][k];
        }
    }
    col_block_sum<VW>(L, res, R, sh, partial);
}

// out[r] = sum over blocks of partial[b][r] (its square root with sqrt_out, and then also the column's
// scale 1/out[r] for k_col_scale: FP64 and as a (hi, lo) float pair).
__global__ void k_col_reduce(const double* __restrict__ partial, int nblocks, int R, double* __restrict__ out,
                             int sqrt_out, double* __restrict__ inv = nullptr, float2* __restrict__ inv_ff = nullptr,
                             float2* __restrict__ neg_ff = nullptr) {
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        double t = 0.0;
        for (int b = 0; b < nblocks; ++b) t += partial[(int64_t)b * R + r];
        out[r] = sqrt_out ? sqrt(t) : t;
        if (inv) {
            const double v = out[r] > 0 ? 1.0 / out[r] : 1.0;
            const float h = (float)v;
            inv[r] = v;
            inv_ff[r] = make_float2(h, (float)(v - (double)h));
        }
        if (neg_ff) {  // -out[r] as a (hi, lo) float pair
            const float h = (float)(-out[r]);
            neg_ff[r] = make_float2(h, (float)(-out[r] - (double)h));
        }
    }
}

// prev <- w - alpha cur - beta_prev prev (per column), with partial column sums of its square.  kInPlace
// (two-block recurrence): prev already holds H cur - beta_prev prev, and prev <- prev - alpha cur (w unused).
template <typename VT, int VW, bool kInPlace = false>
__global__ void __launch_bounds__(256) k_ftlm_update(VT* __restrict__ prev, const VT* __restrict__ cur,
                                                     const VT* __restrict__ w, const double* __restrict__ alpha,
                                                     const double* __restrict__ beta_prev, int64_t n, int R,
                                                     double* __restrict__ partial) {
    __shared__ double sh[256 * VW];
    const ColLayout L = ColLayout::make<VW>(n, R);
    double a[VW], b[VW], res[VW];
#pragma unroll
    for (int k = 0; k < VW; ++k) {
        a[k] = alpha[L.c0 + k];
        b[k] = (beta_prev && !kInPlace) ? beta_prev[L.c0 + k] : 0.0;
    }
    if constexpr (sizeof(VT) == 4) {
        float ah[VW], al[VW], bh[VW], bl[VW];
        F2 nrm[VW];
#pragma unroll
        for (int k = 0; k < VW; ++k) {
            ah[k] = (float)(-a[k]), al[k] = (float)(-a[k] - (double)ah[k]);
            bh[k] = (float)(-b[k]), bl[k] = (float)(-b[k] - (double)bh[k]);
            nrm[k] = F2{0.f, 0.f};
        }
        for (int64_t i = L.i0 + L.sub; i < L.i1; i += (int64_t)L.rpp * kColUnroll) {
            VT wv[kColUnroll][VW], cv[kColUnroll][VW], pv[kColUnroll][VW];
#pragma unroll
            for (int u = 0; u < kColUnroll; ++u) {
                const int64_t ii = i + (int64_t)u * L.rpp;
                if (ii < L.i1) {
                    if constexpr (!kInPlace) load_vec<VT, VW>(w + ii * R + L.c0, wv[u]);
                    load_vec<VT, VW>(cur + ii * R + L.c0, cv[u]);
                    load_vec<VT, VW>(prev + ii * R + L.c0, pv[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < kColUnroll; ++u) {
                const int64_t ii = i + (int64_t)u * L.rpp;
                if (ii >= L.i1) continue;
                VT out[VW];
#pragma unroll
                for (int k = 0; k < VW; ++k) {
                    F2 v{(float)(kInPlace ? pv[u][k] : wv[u][k]), 0.f};
                    f2_fma(v, ah[k], al[k], (float)cv[u][k]);
                    if constexpr (!kInPlace) f2_fma(v, bh[k], bl[k], (float)pv[u][k]);
                    const float vf = v.hi + v.lo;
                    out[k] = (VT)vf;
                    f2_fma(nrm[k], vf, 0.f, vf);
                }
                store_vec<VT, VW>(prev + ii * R + L.c0, out);
            }
        }
#pragma unroll
        for (int k = 0; k < VW; ++k) res[k] = f2_value(nrm[k]);
    } else {
#pragma unroll
        for (int k = 0; k < VW; ++k) res[k] = 0.0;
        for (int64_t i = L.i0 + L.sub; i < L.i1; i += (int64_t)L.rpp * kColUnroll) {
            VT wv[kColUnroll][VW], cv[kColUnroll][VW], pv[kColUnroll][VW];
#pragma unroll
            for (int u = 0; u < kColUnroll; ++u) {
                const int64_t ii = i + (int64_t)u * L.rpp;
                if (ii < L.i1) {
                    if constexpr (!kInPlace) load_vec<VT, VW>(w + ii * R + L.c0, wv[u]);
                    load_vec<VT, VW>(cur + ii * R + L.c0, cv[u]);
                    load_vec<VT, VW>(prev + ii * R + L.c0, pv[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < kColUnroll; ++u) {
                const int64_t ii = i + (int64_t)u * L.rpp;
                if (ii >= L.i1) continue;
                VT out[VW];
#pragma unroll
                for (int k = 0; k < VW; ++k) {
                    const double v = kInPlace ? (double)pv[u][k] - a[k] * (double)cv[u][k]
                                              : (double)wv[u][k] - a[k] * (double)cv[u][k] - b[k] * (double)pv[u][k];
                    out[k] = (VT)v;
                    res[k] += v * v;
                }
                store_vec<VT, VW>(prev + ii * R + L.c0, out);
            }
        }
    }
    col_block_sum<VW>(L, res, R, sh, partial);
}

// v *= inv per column (1/beta from k_col_reduce; a double-float multiply for FP32 storage).  With v2 (the
// two-block recurrence) also v2 *= -beta, the next step's accumulated term.  R is a power of two.
template <typename VT>
__device__ __forceinline__ VT col_mul(VT x, double c, float2 c_ff) {
    if constexpr (sizeof(VT) == 4) {
        const float xf = (float)x;
        const float p = c_ff.x * xf;
        return (VT)(p + (fmaf(c_ff.x, xf, -p) + c_ff.y * xf));
    } else {
        return (VT)((double)x * c);
    }
}
template <typename VT, int VW>
__global__ void k_col_scale(VT* __restrict__ v, const double* __restrict__ inv, const float2* __restrict__ inv_ff,
                            int64_t n, int R, VT* __restrict__ v2 = nullptr, const double* __restrict__ beta = nullptr,
                            const float2* __restrict__ nbeta_ff = nullptr) {
    const int64_t total = n * R / VW;
#pragma unroll 4
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int c0 = (int)(e * VW) & (R - 1);
        VT x[VW];
        load_vec<VT, VW>(v + e * VW, x);
#pragma unroll
        for (int k = 0; k < VW; ++k)
            x[k] = col_mul<VT>(x[k], inv[c0 + k], sizeof(VT) == 4 ? inv_ff[c0 + k] : make_float2(0.f, 0.f));
        store_vec<VT, VW>(v + e * VW, x);
        if (v2) {
            load_vec<VT, VW>(v2 + e * VW, x);
#pragma unroll
            for (int k = 0; k < VW; ++k)
                x[k] = col_mul<VT>(x[k], -beta[c0 + k], sizeof(VT) == 4 ? nbeta_ff[c0 + k] : make_float2(0.f, 0.f));
            store_vec<VT, VW>(v2 + e * VW, x);
        }
    }
}

// The two-block recurrence's column work in two passes instead of three (FP32 storage, sector launch).  One
// read of C and P gives <C, P>, |P|^2 and |C|^2 per column; with alpha = <C, P> the norm of P - alpha C follows
// without another pass, |P - alpha C|^2 = |P|^2 - 2 alpha <C, P> + alpha^2 |C|^2, and a second pass writes
// (P - alpha C) / beta.  The subtraction in that formula loses (alpha / beta)^2 times the sums' relative rounding
// (double-float, about 2^-46), far below the FP32 storage of the vectors.
template <int VW>
__global__ void __launch_bounds__(256) k_col_dots3(const float* __restrict__ c, const float* __restrict__ p, int64_t n,
                                                   int R, double* __restrict__ partial) {
    __shared__ double sh[256 * VW];
    const ColLayout L = ColLayout::make<VW>(n, R);
    F2 cp[VW], pp[VW], cc[VW];
#pragma unroll
    for (int k = 0; k < VW; ++k) cp[k] = pp[k] = cc[k] = F2{0.f, 0.f};
    for (int64_t i = L.i0 + L.sub; i < L.i1; i += (int64_t)L.rpp * kColUnroll) {
        float cv[kColUnroll][VW], pv[kColUnroll][VW];
#pragma unroll
        for (int u = 0; u < kColUnroll; ++u) {
            const int64_t ii = i + (int64_t)u * L.rpp;
            if (ii < L.i1) {
                load_vec<float, VW>(c + ii * R + L.c0, cv[u]);
                load_vec<float, VW>(p + ii * R + L.c0, pv[u]);
            } else {
#pragma unroll
                for (int k = 0; k < VW; ++k) cv[u][k] = pv[u][k] = 0.f;
            }
        }
#pragma unroll
        for (int u = 0; u < kColUnroll; ++u)
#pragma unroll
            for (int k = 0; k < VW; ++k) {
                f2_fma(cp[k], cv[u][k], 0.f, pv[u][k]);
                f2_fma(pp[k], pv[u][k], 0.f, pv[u][k]);
                f2_fma(cc[k], cv[u][k], 0.f, cv[u][k]);
            }
    }
    const int64_t stride = (int64_t)gridDim.x * R;
    double res[VW];
#pragma unroll
    for (int k = 0; k < VW; ++k) res[k] = f2_value(cp[k]);
    col_block_sum<VW>(L, res, R, sh, partial);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < VW; ++k) res[k] = f2_value(pp[k]);
    col_block_sum<VW>(L, res, R, sh, partial + stride);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < VW; ++k) res[k] = f2_value(cc[k]);
    col_block_sum<VW>(L, res, R, sh, partial + 2 * stride);
}

// alpha = <C, P>, beta = |P - alpha C| from k_col_dots3's partial sums (summed over blocks in block order), with
// 1/beta as FP64 and as a (hi, lo) float pair, and -beta as a float pair (the next step's accumulate coefficient).
__global__ void k_ftlm_coef3(const double* __restrict__ partial, int nblocks, int R, double* __restrict__ alpha,
                             double* __restrict__ beta, double* __restrict__ inv, float2* __restrict__ inv_ff,
                             float2* __restrict__ neg_ff) {
    const int64_t stride = (int64_t)nblocks * R;
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        double cp = 0.0, pp = 0.0, cc = 0.0;
        for (int b = 0; b < nblocks; ++b) {
            cp += partial[(int64_t)b * R + r];
            pp += partial[stride + (int64_t)b * R + r];
            cc += partial[2 * stride + (int64_t)b * R + r];
        }
        const double a = cp;
        const double b2 = pp - 2.0 * a * cp + a * a * cc;
        const double b = b2 > 0.0 ? sqrt(b2) : 0.0;
        alpha[r] = a;
        beta[r] = b;
        const double v = b > 0 ? 1.0 / b : 1.0;
        const float h = (float)v;
        inv[r] = v;
        inv_ff[r] = make_float2(h, (float)(v - (double)h));
        const float nh = (float)(-b);
        neg_ff[r] = make_float2(nh, (float)(-b - (double)nh));
    }
}

// prev <- (prev - alpha cur) / beta per column, in double-float, rounded to FP32 once.
template <int VW>
__global__ void __launch_bounds__(256) k_ftlm_update_scaled(float* __restrict__ prev, const float* __restrict__ cur,
                                                            const double* __restrict__ alpha,
                                                            const float2* __restrict__ inv_ff, int64_t n, int R) {
    const ColLayout L = ColLayout::make<VW>(n, R);
    float ah[VW], al[VW], ih[VW], il[VW];
#pragma unroll
    for (int k = 0; k < VW; ++k) {
        const double a = alpha[L.c0 + k];
        ah[k] = (float)(-a), al[k] = (float)(-a - (double)ah[k]);
        ih[k] = inv_ff[L.c0 + k].x, il[k] = inv_ff[L.c0 + k].y;
    }
    for (int64_t i = L.i0 + L.sub; i < L.i1; i += (int64_t)L.rpp * kColUnroll) {
        float cv[kColUnroll][VW], pv[kColUnroll][VW];
#pragma unroll
        for (int u = 0; u < kColUnroll; ++u) {
            const int64_t ii = i + (int64_t)u * L.rpp;
            if (ii < L.i1) {
                load_vec<float, VW>(cur + ii * R + L.c0, cv[u]);
                load_vec<float, VW>(prev + ii * R + L.c0, pv[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < kColUnroll; ++u) {
            const int64_t ii = i + (int64_t)u * L.rpp;
            if (ii >= L.i1) continue;
            float out[VW];
#pragma unroll
            for (int k = 0; k < VW; ++k) {
                F2 v{pv[u][k], 0.f};
                f2_fma(v, ah[k], al[k], cv[u][k]);  // v = prev - alpha cur
                const float w = v.hi * ih[k];
                const float e = fmaf(v.hi, ih[k], -w) + (v.hi * il[k] + v.lo * ih[k]);
                out[k] = w + e;
            }
            store_vec<float, VW>(prev + ii * R + L.c0, out);
        }
    }
}

constexpr int kColGrid = 1024;

template <typename VT>
struct FtlmSector {
    qsi_op* op;
    int R;
    int64_t n;
    DevBuf<VT> P, C, W;
    DevBuf<double> partial, ab, inv;
    DevBuf<float2> inv_ff, nbeta_ff;
};

// All sectors advance together: per step one apply launch covering every sector
// (FP32 storage with hash indexes) or one per sector, then the per-sector
// recurrence kernels.  The whole M-step run is captured into one CUDA graph.
//
// Three blocks of R vectors per sector (prev P, current C, W = H C):
//   W = H C;  alpha = <C, W>;  P <- W - alpha C - beta_prev P;  beta = |P|;  P /= beta;  swap(P, C).
// Two blocks (blocks == 2, or blocks == 0 when three do not fit in free device memory), the in-place
// recurrence with P holding q_prev at the start of a step:
//   P <- H C - beta_prev P;  alpha = <C, P>;  P <- P - alpha C;  beta = |P|;  P /= beta;  swap(P, C).
// The one-launch sector apply takes -beta_prev per column as its accumulate coefficient (double-float), and its
// column work is two passes (k_col_dots3: <C, P>, |P|^2 and |C|^2 in one read; k_ftlm_update_scaled:
// P <- (P - alpha C) / beta), so a step moves 6 blocks beyond the apply's gathers against 9 for three blocks,
// though the accumulating apply is slower on small sectors: three blocks are taken when they fit.  The
// per-sector launches instead have the column pass also scale C by -beta for the next step.
template <typename VT>
static qsi_status ftlm_run(qsi_op** ops, int ns, const int32_t* Rs, int M, uint64_t seed, double* alphas,
                           double* betas, int blocks) {
    cudaStream_t st = ops[0]->stream;
    std::vector<FtlmSector<VT>> S(ns);
    bool one_launch = (sizeof(VT) == 4);
    size_t block_bytes = 0;
    for (int s = 0; s < ns; ++s) {
        const int R = Rs[s];
        if (R <= 0 || R > 256 || (R & (R - 1))) return fail(QSI_INVALID_ARG, "ftlm: R must be a power of two in [1,256]");
        if (ops[s]->basis->n < 1) return fail(QSI_INVALID_ARG, "ftlm: empty sector");
        block_bytes += (size_t)ops[s]->basis->n * R * sizeof(VT);
        one_launch = one_launch && ops[s]->kernel == 1 && ops[s]->ff_accumulate;
    }
    if (blocks == 0) {  // three blocks when they fit with 4 GiB to spare, else two
        size_t free_b = 0, total_b = 0;
        QSI_CUDA(cudaMemGetInfo(&free_b, &total_b));
        blocks = (3 * block_bytes + ((size_t)4 << 30) <= free_b) ? 3 : 2;
    }
    if (blocks != 2 && blocks != 3) return fail(QSI_INVALID_ARG, "ftlm: blocks must be 0, 2 or 3");
    const bool two = (blocks == 2);
    for (int s = 0; s < ns; ++s) {
        const int R = Rs[s];
        S[s].op = ops[s];
        S[s].R = R;
        S[s].n = ops[s]->basis->n;
        QSI_CUDA(S[s].P.alloc((size_t)S[s].n * R, st));
        QSI_CUDA(S[s].C.alloc((size_t)S[s].n * R, st));
        if (!two) QSI_CUDA(S[s].W.alloc((size_t)S[s].n * R, st));
        QSI_CUDA(S[s].partial.alloc((size_t)3 * kColGrid * R, st));  // three dots per column (k_col_dots3)
        QSI_CUDA(S[s].ab.alloc((size_t)2 * M * R, st));
        QSI_CUDA(S[s].inv.alloc((size_t)R, st));
        QSI_CUDA(S[s].inv_ff.alloc((size_t)R, st));
        QSI_CUDA(S[s].nbeta_ff.alloc((size_t)R, st));
        QSI_CUDA(cudaMemsetAsync(S[s].nbeta_ff.p, 0, (size_t)R * sizeof(float2), st));
        k_ftlm_init<VT><<<grid_for(S[s].n * R, 256), 256, 0, st>>>(S[s].C.p, S[s].P.p, S[s].n, R, seed + (uint64_t)s);
    }
    std::vector<VT*> prev(ns), cur(ns);
    for (int s = 0; s < ns; ++s) prev[s] = S[s].P.p, cur[s] = S[s].C.p;
    // one-launch plans for even steps (input C) and odd steps (input P), uploaded before capture
    SectorPlan plan[2];
    DevBuf<unsigned char> d_plan[2];
    if (one_launch) {
        std::vector<qsi_op*> opv(ops, ops + ns);
        // Blocks are shared out in proportion to each sector's apply time alone (rows, vectors, hits and lookup
        // misses all count): one warm-up and one timed apply per sector, W = H C on the run's own buffers.
        std::vector<double> weight(ns, 1.0);
        if (ns > 1) {
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            QSI_CUDA(cudaEventCreate(&e0));
            QSI_CUDA(cudaEventCreate(&e1));
            qsi_status ts = QSI_OK;
            for (int s = 0; s < ns && ts == QSI_OK; ++s) {
                VT* out = two ? S[s].P.p : S[s].W.p;  // P is zeroed again below
                ts = launch_apply(ops[s], S[s].C.p, out, S[s].R, QSI_F32, 0, st);
                if (ts == QSI_OK && cudaEventRecord(e0, st) != cudaSuccess) ts = QSI_CUDA_ERROR;
                if (ts == QSI_OK) ts = launch_apply(ops[s], S[s].C.p, out, S[s].R, QSI_F32, 0, st);
                float ms = 0.f;
                if (ts == QSI_OK && (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                                     cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
                    ts = fail(QSI_CUDA_ERROR, "ftlm: sector timing failed");
                weight[s] = std::max(1e-3, (double)ms);
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            if (ts != QSI_OK) return ts;
            if (two)
                for (int s = 0; s < ns; ++s)
                    QSI_CUDA(cudaMemsetAsync(S[s].P.p, 0, (size_t)S[s].n * S[s].R * sizeof(VT), st));
        }
        for (int parity = 0; parity < 2; ++parity) {
            std::vector<const float*> X(ns);
            std::vector<float*> Y(ns);
            for (int s = 0; s < ns; ++s) {
                X[s] = (const float*)(parity ? S[s].P.p : S[s].C.p);
                Y[s] = (float*)(two ? (parity ? S[s].C.p : S[s].P.p) : S[s].W.p);
            }
            // two blocks: the accumulating apply scales the previous block by -beta_prev itself
            std::vector<const float2*> yc(ns);
            for (int s = 0; s < ns; ++s) yc[s] = S[s].nbeta_ff.p;
            qsi_status ps = plan_sectors(opv.data(), ns, X.data(), Y.data(), Rs, plan[parity], weight.data(),
                                         two ? yc.data() : nullptr);
            if (ps != QSI_OK) return ps;
            QSI_CUDA(d_plan[parity].alloc(plan[parity].records.size(), st));
            QSI_CUDA(cudaMemcpyAsync(d_plan[parity].p, plan[parity].records.data(), plan[parity].records.size(),
                                     cudaMemcpyHostToDevice, st));
        }
    }
    QSI_CUDA(cudaStreamSynchronize(st));
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    QSI_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    qsi_status status = QSI_OK;
    const int blk = 256;
    for (int j = 0; j < M && status == QSI_OK; ++j) {
        // two blocks: the apply accumulates into prev, which holds q_prev (zero at the first step) and is scaled
        // by -beta_prev on the way: inside the sector launch, else by the previous step's column pass
        if (one_launch) {
            status = launch_sectors(d_plan[j & 1].p, plan[j & 1], two ? 1 : 0, st);
        } else {
            for (int s = 0; s < ns && status == QSI_OK; ++s)
                status = launch_apply(ops[s], cur[s], two ? prev[s] : S[s].W.p, S[s].R,
                                      sizeof(VT) == 4 ? QSI_F32 : QSI_F64, two ? 1 : 0, st);
        }
        for (int s = 0; s < ns; ++s) {
            FtlmSector<VT>& F = S[s];
            double* dA = F.ab.p;
            double* dB = F.ab.p + (size_t)M * F.R;
            const double* bprev = j ? dB + (size_t)(j - 1) * F.R : nullptr;
            double* beta = dB + (size_t)j * F.R;
            auto col_step = [&](auto vw) {
                constexpr int VW = decltype(vw)::value;
                if constexpr (sizeof(VT) == 4) {
                    if (one_launch && two) {  // two passes: three dots, then (P - alpha C) / beta
                        const float* c = reinterpret_cast<const float*>(cur[s]);
                        float* p = reinterpret_cast<float*>(prev[s]);
                        k_col_dots3<VW><<<kColGrid, blk, 0, st>>>(c, p, F.n, F.R, F.partial.p);
                        k_ftlm_coef3<<<1, 256, 0, st>>>(F.partial.p, kColGrid, F.R, dA + (size_t)j * F.R, beta,
                                                        F.inv.p, F.inv_ff.p, F.nbeta_ff.p);
                        k_ftlm_update_scaled<VW><<<kColGrid, blk, 0, st>>>(p, c, dA + (size_t)j * F.R, F.inv_ff.p,
                                                                           F.n, F.R);
                        return;
                    }
                }
                k_col_dots<VT, VW><<<kColGrid, blk, 0, st>>>(cur[s], two ? prev[s] : F.W.p, F.n, F.R, F.partial.p);
                k_col_reduce<<<1, 256, 0, st>>>(F.partial.p, kColGrid, F.R, dA + (size_t)j * F.R, 0);
                if (two)
                    k_ftlm_update<VT, VW, true><<<kColGrid, blk, 0, st>>>(prev[s], cur[s], nullptr, dA + (size_t)j * F.R,
                                                                          nullptr, F.n, F.R, F.partial.p);
                else
                    k_ftlm_update<VT, VW><<<kColGrid, blk, 0, st>>>(prev[s], cur[s], F.W.p, dA + (size_t)j * F.R,
                                                                    bprev, F.n, F.R, F.partial.p);
                k_col_reduce<<<1, 256, 0, st>>>(F.partial.p, kColGrid, F.R, beta, 1, F.inv.p, F.inv_ff.p,
                                                two ? F.nbeta_ff.p : nullptr);
                k_col_scale<VT, VW><<<grid_for(F.n * F.R / VW, 256), 256, 0, st>>>(
                    prev[s], F.inv.p, F.inv_ff.p, F.n, F.R, (two && !one_launch) ? cur[s] : nullptr, beta,
                    F.nbeta_ff.p);
            };
            constexpr int kVW = 16 / sizeof(VT);  // 16-byte accesses when R allows
            if (F.R % kVW == 0) col_step(std::integral_constant<int, kVW>{});
            else col_step(std::integral_constant<int, 1>{});
            std::swap(prev[s], cur[s]);
        }
    }
    cudaError_t ce = cudaStreamEndCapture(st, &graph);
    if (status != QSI_OK) {
        if (graph) cudaGraphDestroy(graph);
        return status;
    }
    QSI_CUDA(ce);
    QSI_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    cudaError_t e = cudaGraphLaunch(exec, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(QSI_CUDA_ERROR, "ftlm graph: %s", cudaGetErrorString(e));
    size_t off = 0;
    for (int s = 0; s < ns; ++s) {
        const int R = S[s].R;
        std::vector<double> h((size_t)2 * M * R);
        QSI_CUDA(cudaMemcpyAsync(h.data(), S[s].ab.p, h.size() * 8, cudaMemcpyDeviceToHost, st));
        QSI_CUDA(cudaStreamSynchronize(st));
        for (int r = 0; r < R; ++r)
            for (int j = 0; j < M; ++j) {
                alphas[off + (size_t)r * M + j] = h[(size_t)j * R + r];
                betas[off + (size_t)r * M + j] = h[(size_t)M * R + (size_t)j * R + r];
            }
        off += (size_t)R * M;
    }
    return QSI_OK;
}

}  // namespace qsi

extern "C" qsi_status qsi_ftlm_run(qsi_op** ops, int32_t n_sectors, const int32_t* R, int32_t M, uint64_t seed,
                                   int32_t precision, double* alphas, double* betas) {
    return guarded([&]() -> qsi_status {
        if (!ops || n_sectors <= 0 || !R || M <= 0 || !alphas || !betas) return fail(QSI_INVALID_ARG, "qsi_ftlm_run: bad argument");
        for (int s = 0; s < n_sectors; ++s)
            if (!ops[s]) return fail(QSI_INVALID_ARG, "qsi_ftlm_run: null operator");
        // sector s uses seed + s, so a sector run alone with seed + s gets the same vectors
        return (precision == QSI_F32) ? ftlm_run<float>(ops, n_sectors, R, M, seed, alphas, betas, 0)
                                      : ftlm_run<double>(ops, n_sectors, R, M, seed, alphas, betas, 0);
    });
}

extern "C" qsi_status qsi_ftlm_run_blocks(qsi_op** ops, int32_t n_sectors, const int32_t* R, int32_t M, uint64_t seed,
                                          int32_t precision, int32_t blocks, double* alphas, double* betas) {
    return guarded([&]() -> qsi_status {
        if (!ops || n_sectors <= 0 || !R || M <= 0 || !alphas || !betas) return fail(QSI_INVALID_ARG, "qsi_ftlm_run_blocks: bad argument");
        for (int s = 0; s < n_sectors; ++s)
            if (!ops[s]) return fail(QSI_INVALID_ARG, "qsi_ftlm_run_blocks: null operator");
        return (precision == QSI_F32) ? ftlm_run<float>(ops, n_sectors, R, M, seed, alphas, betas, blocks)
                                      : ftlm_run<double>(ops, n_sectors, R, M, seed, alphas, betas, blocks);
    });
}

// Batched eigen-decomposition of symmetric tridiagonals (FTLM Ritz data).
extern "C" qsi_status qsi_tridiag_ritz(const double* a, const double* b, int32_t m, int32_t n_mat, double* evals,
                                       double* first) {
    return guarded([&]() -> qsi_status {
        if (!a || !b || m <= 0 || n_mat <= 0 || !evals || !first) return fail(QSI_INVALID_ARG, "qsi_tridiag_ritz: bad argument");
        std::vector<double> A((size_t)n_mat * m * m, 0.0), w, V;
        for (int k = 0; k < n_mat; ++k)
            for (int i = 0; i < m; ++i) {
                A[(size_t)k * m * m + i * m + i] = a[(size_t)k * m + i];
                if (i + 1 < m) {
                    A[(size_t)k * m * m + i * m + i + 1] = b[(size_t)k * m + i];
                    A[(size_t)k * m * m + (i + 1) * m + i] = b[(size_t)k * m + i];
                }
            }
        qsi_status s = jacobi_eigh(A, m, n_mat, w, V, nullptr);
        if (s) return s;
        for (int k = 0; k < n_mat; ++k)
            for (int j = 0; j < m; ++j) {
                evals[(size_t)k * m + j] = w[(size_t)k * m + j];
                first[(size_t)k * m + j] = V[(size_t)k * m * m + j];
            }
        return QSI_OK;
    });
}
