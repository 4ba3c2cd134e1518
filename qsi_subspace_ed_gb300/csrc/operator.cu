// Device-resident basis, operator handles and the matrix-free apply.
//
// The apply is a row-wise pull/gather: for every basis row i with state s,
//   y[i] = diag(s) x[i] + sum_t cs_t (-1)^popc(~s & Z_t) x[index(s ^ X_t)]
// over the off-diagonal terms t whose (transposed) masks admit s.  This is the
// same operator as the reference's push form
//   for t, for i: y[index(t s_i)] += c_t x[i] sign_t(s_i)
// (components/operator/src/operator_matrix.cpp:28-60) with every term
// replaced by its transpose, so no atomics are needed and every row is summed
// in a fixed order (deterministic).  Lookup misses contribute nothing
// (projected ED, operator_matrix.cpp:17,49), and sources with |x| <= 1e-15 are
// skipped as APPLY_TOL does (operator_matrix.hpp:113).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "qsi_device.cuh"
#include "qsi_handles.h"

namespace qsi {

// ------------------------------------------------------------------ basis build
__global__ void k_check_sorted(const state2* s, int64_t n, int* bad) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x + 1;
    for (; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        state2 a = s[i - 1], b = s[i];
        if (!less128(a.x, a.y, b.x, b.y)) atomicOr(bad, 1);
    }
}

// bstart[v] = first index whose bucket >= v, for v in [0, nb].
__global__ void k_fill_buckets(BasisView B, uint32_t* bstart) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; i <= B.n; i += (int64_t)gridDim.x * blockDim.x) {
        bool ok;
        int64_t cur = (i < B.n) ? (int64_t)bucket_of(B, B.states[i].x, B.states[i].y, ok) : (int64_t)B.n_buckets;
        int64_t prev = (i > 0) ? (int64_t)bucket_of(B, B.states[i - 1].x, B.states[i - 1].y, ok) : -1;
        for (int64_t v = prev + 1; v <= cur; ++v) bstart[v] = (uint32_t)i;
    }
}

__global__ void k_fill_u32(uint32_t* p, int64_t n, uint32_t v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

// Entries of a bucket table of nb buckets: bstart[0 .. nb] rounded up to whole groups of four, plus one group, so
// that bucket_bounds' 16-byte reads stay inside the allocation.
size_t bucket_table_entries(uint32_t nb) { return ((size_t)nb + 1 + 3) / 4 * 4 + 4; }

qsi_status build_buckets(qsi_basis* b) {
    k_fill_buckets<<<grid_for(b->n + 1, 256), 256>>>(b->view(), b->d_bstart);
    const int64_t pad = (int64_t)bucket_table_entries(b->n_buckets) - ((int64_t)b->n_buckets + 1);
    k_fill_u32<<<1, 32>>>(b->d_bstart + b->n_buckets + 1, pad, (uint32_t)b->n);
    QSI_CUDA(cudaGetLastError());
    return QSI_OK;
}

__global__ void k_search(BasisView B, const state2* q, int64_t n, int64_t* idx) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; i < n; i += (int64_t)gridDim.x * blockDim.x) idx[i] = basis_find(B, q[i].x, q[i].y);
}

// ------------------------------------------------------------------ apply kernels
// One thread per row, FP64 (or FP32-stored) single vector.
template <typename XT, typename YT>
__global__ void __launch_bounds__(256) k_apply_rowthread(BasisView B, const PullTerm* __restrict__ gterms, int n_off,
                                                         DiagSpec D, const PushTerm* __restrict__ gdiag,
                                                         const XT* __restrict__ x, YT* __restrict__ y,
                                                         int accumulate) {
    extern __shared__ unsigned char smem_raw[];
    PullTerm* terms = reinterpret_cast<PullTerm*>(smem_raw);
    PushTerm* dgen = reinterpret_cast<PushTerm*>(terms + n_off);
    for (int k = threadIdx.x; k < n_off; k += blockDim.x) terms[k] = gterms[k];
    for (int k = threadIdx.x; k < D.n_generic; k += blockDim.x) dgen[k] = gdiag[k];
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < B.n; i += (int64_t)gridDim.x * blockDim.x) {
        const state2 s = B.states[i];
        double acc = diag_value(D, dgen, s.x, s.y) * (double)x[i];
        for (int t = 0; t < n_off; ++t) {
            const PullTerm& T = terms[t];
            if (((s.x & T.dn0) | (s.y & T.dn1)) != 0) continue;
            if ((((s.x & T.up0) ^ T.up0) | ((s.y & T.up1) ^ T.up1)) != 0) continue;
            const int64_t J = basis_find(B, s.x ^ T.x0, s.y ^ T.x1);
            if (J < 0) continue;
            const double xj = (double)x[J];
            if (!(fabs(xj) > 1e-15)) continue;
            double cs = T.cs;
            if (T.has_z && ((__popcll(~s.x & T.z0) + __popcll(~s.y & T.z1)) & 1)) cs = -cs;
            acc += cs * xj;
        }
        if (accumulate) acc += (double)y[i];
        y[i] = (YT)acc;
    }
}

// One warp per row over R vectors stored [row][R]: lanes test terms 32 at a
// time, each admitted lane looks its column up, then the whole warp gathers
// that column's R values in term order.
template <typename XT>
__global__ void __launch_bounds__(256) k_apply_warprow(BasisView B, const PullTerm* __restrict__ gterms, int n_off,
                                                       DiagSpec D, const PushTerm* __restrict__ gdiag,
                                                       const XT* __restrict__ x, XT* __restrict__ y, int R,
                                                       int accumulate) {
    extern __shared__ unsigned char smem_raw[];
    PullTerm* terms = reinterpret_cast<PullTerm*>(smem_raw);
    PushTerm* dgen = reinterpret_cast<PushTerm*>(terms + n_off);
    for (int k = threadIdx.x; k < n_off; k += blockDim.x) terms[k] = gterms[k];
    for (int k = threadIdx.x; k < D.n_generic; k += blockDim.x) dgen[k] = gdiag[k];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    constexpr int kMaxR = 4;  // up to 128 vectors per warp pass
    for (int64_t i = warp; i < B.n; i += nwarps) {
        const state2 s = B.states[i];
        const double d = diag_value(D, dgen, s.x, s.y);
        for (int r0 = 0; r0 < R; r0 += 32 * kMaxR) {
            double acc[kMaxR];
#pragma unroll
            for (int m = 0; m < kMaxR; ++m) {
                int r = r0 + lane + 32 * m;
                acc[m] = (r < R) ? d * (double)x[i * R + r] : 0.0;
            }
            for (int t0 = 0; t0 < n_off; t0 += 32) {
                const int t = t0 + lane;
                int64_t J = -1;
                double cs = 0.0;
                if (t < n_off) {
                    const PullTerm& T = terms[t];
                    if (((s.x & T.dn0) | (s.y & T.dn1)) == 0 && (((s.x & T.up0) ^ T.up0) | ((s.y & T.up1) ^ T.up1)) == 0) {
                        J = basis_find(B, s.x ^ T.x0, s.y ^ T.x1);
                        cs = T.cs;
                        if (T.has_z && ((__popcll(~s.x & T.z0) + __popcll(~s.y & T.z1)) & 1)) cs = -cs;
                    }
                }
                unsigned hits = __ballot_sync(0xffffffffu, J >= 0);
                while (hits) {
                    const int k = __ffs(hits) - 1;
                    hits &= hits - 1;
                    const int64_t Jk = __shfl_sync(0xffffffffu, J, k);
                    const double ck = __shfl_sync(0xffffffffu, cs, k);
#pragma unroll
                    for (int m = 0; m < kMaxR; ++m) {
                        int r = r0 + lane + 32 * m;
                        if (r < R) {
                            double xj = (double)x[Jk * R + r];
                            if (fabs(xj) > 1e-15) acc[m] += ck * xj;
                        }
                    }
                }
            }
#pragma unroll
            for (int m = 0; m < kMaxR; ++m) {
                int r = r0 + lane + 32 * m;
                if (r < R) {
                    double v = acc[m];
                    if (accumulate) v += (double)y[i * R + r];
                    y[i * R + r] = (XT)v;
                }
            }
        }
    }
}

// ------------------------------------------------------------------ connectivity
// Per basis index j (the reference's column), in term order: count (pass 0)
// or write (pass 1) the triplets of LazyOpSum::toSparseMatrix.
__global__ void k_triplets(BasisView B, const PushTerm* __restrict__ off, int n_off, const PushTerm* __restrict__ dg,
                           int n_diag, double tol, const int64_t* __restrict__ offsets, int64_t* counts,
                           int64_t* rows, int64_t* cols, double* vals) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < B.n; j += (int64_t)gridDim.x * blockDim.x) {
        const state2 s = B.states[j];
        int64_t w = offsets ? offsets[j] : 0;
        int64_t c = 0;
        for (int t = 0; t < n_off; ++t) {
            const PushTerm& T = off[t];
            bool ok = ((s.x & T.dn0) | (s.y & T.dn1)) == 0 && (s.x & T.up0) == T.up0 && (s.y & T.up1) == T.up1;
            if (!ok) continue;
            uint64_t f0 = s.x ^ T.x0, f1 = s.y ^ T.x1;
            int par = (__popcll(~f0 & T.z0) + __popcll(~f1 & T.z1)) & 1;
            int sign = T.sign * (1 - 2 * par);
            if (sign == 0) continue;
            int64_t J = basis_find(B, f0, f1);
            if (J < 0) continue;
            double res = T.c * (double)sign;
            if (!(fabs(res) > tol)) continue;
            if (rows) {
                rows[w] = J;
                cols[w] = j;
                vals[w] = res;
                ++w;
            }
            ++c;
        }
        double acc = 0.0;
        for (int t = 0; t < n_diag; ++t) {
            const PushTerm& T = dg[t];
            bool ok = ((s.x & T.dn0) | (s.y & T.dn1)) == 0 && (s.x & T.up0) == T.up0 && (s.y & T.up1) == T.up1;
            int par = (__popcll(~s.x & T.z0) + __popcll(~s.y & T.z1)) & 1;
            int sign = ok ? T.sign * (1 - 2 * par) : 0;
            acc += T.c * (double)sign;
        }
        if (rows) {
            rows[w] = j;
            cols[w] = j;
            vals[w] = acc;
        }
        if (counts) counts[j] = c + 1;
    }
}

// counts[0] += off-diagonal terms that land in the basis, counts[1] += those that miss
__global__ void k_count_connectivity(BasisView B, const PushTerm* __restrict__ off, int n_off,
                                     unsigned long long* counts) {
    unsigned long long hit = 0, miss = 0;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < B.n; j += (int64_t)gridDim.x * blockDim.x) {
        const state2 s = B.states[j];
        for (int t = 0; t < n_off; ++t) {
            const PushTerm& T = off[t];
            bool ok = ((s.x & T.dn0) | (s.y & T.dn1)) == 0 && (s.x & T.up0) == T.up0 && (s.y & T.up1) == T.up1;
            if (!ok || T.sign == 0) continue;
            if (basis_find(B, s.x ^ T.x0, s.y ^ T.x1) < 0) ++miss;
            else ++hit;
        }
    }
    for (int o = 16; o; o >>= 1) {
        hit += __shfl_down_sync(0xffffffffu, hit, o);
        miss += __shfl_down_sync(0xffffffffu, miss, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (hit) atomicAdd(counts, hit);
        if (miss) atomicAdd(counts + 1, miss);
    }
}

// hit[t] = 1 when transposed term t maps some row's state onto a basis state.  A block stops once every term
// is known to hit (terms that hit usually do so within the first rows); terms that never hit are tested on
// every row they admit.
template <class LK>
__global__ void k_pull_term_hits(BasisView B, LK lk, const PullTerm* __restrict__ terms, int n, int* __restrict__ hit) {
    extern __shared__ int known[];
    __shared__ int n_known;
    if (threadIdx.x == 0) n_known = 0;
    __syncthreads();
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        known[t] = hit[t];
        if (known[t]) atomicAdd(&n_known, 1);
    }
    __syncthreads();
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < B.n; j += (int64_t)gridDim.x * blockDim.x) {
        if (*(volatile int*)&n_known == n) break;
        const state2 s = B.states[j];
        for (int t = 0; t < n; ++t) {
            if (((volatile int*)known)[t]) continue;
            const PullTerm& T = terms[t];
            const bool ok = ((s.x & T.dn0) | (s.y & T.dn1)) == 0 && (s.x & T.up0) == T.up0 && (s.y & T.up1) == T.up1;
            if (ok && lk.find(s.x ^ T.x0, s.y ^ T.x1) >= 0 && atomicExch(known + t, 1) == 0) {
                atomicAdd(&n_known, 1);
                hit[t] = 1;
            }
        }
    }
}

// Removes the transposed terms that map no row into the basis (their contributions are all dropped misses), keeping
// the order of the others: an exact reduction of the lookups the apply issues.
static qsi_status prune_pull_terms(qsi_basis* b, std::vector<PullTerm>& pull) {
    const int n = (int)pull.size();
    if (n == 0 || b->n == 0) return QSI_OK;
    PullTerm* d_terms = nullptr;
    int* d_hit = nullptr;
    cudaError_t e = cudaMalloc(&d_terms, n * sizeof(PullTerm));
    if (e == cudaSuccess) e = cudaMalloc(&d_hit, n * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(d_terms, pull.data(), n * sizeof(PullTerm), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_hit, 0, n * sizeof(int));
    if (e == cudaSuccess) {
        const size_t smem = (size_t)n * sizeof(int);
        const int grid = grid_for(b->n, 256);
        if (b->d_hash) {
            auto k = k_pull_term_hits<LookupHash>;
            if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k<<<grid, 256, smem>>>(b->view(), LookupHash{b->hview()}, d_terms, n, d_hit);
        } else {
            auto k = k_pull_term_hits<LookupTable>;
            if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k<<<grid, 256, smem>>>(b->view(), LookupTable{b->view()}, d_terms, n, d_hit);
        }
        e = cudaGetLastError();
    }
    std::vector<int> hit(n, 1);
    if (e == cudaSuccess) e = cudaMemcpy(hit.data(), d_hit, n * sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d_terms);
    cudaFree(d_hit);
    if (e != cudaSuccess)
        return fail(e == cudaErrorMemoryAllocation ? QSI_OOM : QSI_CUDA_ERROR, "qsi_op_create (term pruning): %s",
                    cudaGetErrorString(e));
    std::vector<PullTerm> kept;
    kept.reserve(n);
    for (int t = 0; t < n; ++t)
        if (hit[t]) kept.push_back(pull[t]);
    pull.swap(kept);
    return QSI_OK;
}

// ------------------------------------------------------------------ host helpers
int grid_for(int64_t n, int block) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t g = (n + block - 1) / block;
    int64_t cap = (int64_t)sms * 16;
    return (int)std::max<int64_t>(1, std::min(g, cap));
}

static bool is_single_site_z(const qsi_term& t) {
    if (t.x[0] | t.x[1] | t.up[0] | t.up[1] | t.down[0] | t.down[1]) return false;
    return __builtin_popcountll(t.z[0]) + __builtin_popcountll(t.z[1]) == 1;
}

}  // namespace qsi

using namespace qsi;

// ------------------------------------------------------------------ C-ABI: basis
extern "C" qsi_status qsi_basis_create(const uint64_t* lohi, int64_t n, int32_t bucket_bits, qsi_basis** out) {
    return guarded([&]() -> qsi_status {
        if (!out || n <= 0 || !lohi) return fail(QSI_INVALID_ARG, "qsi_basis_create: empty basis or null pointer");
        if (n >= (int64_t)UINT32_MAX) return fail(QSI_INVALID_ARG, "qsi_basis_create: basis larger than 2^32-1 states");
        auto* b = new qsi_basis();
        b->n = n;
        // highest bit used by any state (the last state is the largest)
        uint64_t lo = lohi[2 * (n - 1)], hi = lohi[2 * (n - 1) + 1];
        int hb = hi ? 64 + 63 - __builtin_clzll(hi) : (lo ? 63 - __builtin_clzll(lo) : 0);
        int bits = bucket_bits;
        if (bits <= 0) {
            int lg = 0;
            while ((1LL << lg) < n) ++lg;
            bits = std::min(28, std::max(8, lg + 2));
        }
        bits = std::min(bits, std::min(31, hb + 1));
        b->bits = bits;
        b->hb = hb;
        b->shift = hb + 1 - bits;
        b->n_buckets = 1u << bits;
        cudaError_t e = cudaMalloc(&b->d_states, (size_t)n * sizeof(state2));
        if (e == cudaSuccess) e = cudaMalloc(&b->d_bstart, bucket_table_entries(b->n_buckets) * sizeof(uint32_t));
        if (e != cudaSuccess) {
            qsi_basis_destroy(b);
            return fail(e == cudaErrorMemoryAllocation ? QSI_OOM : QSI_CUDA_ERROR, "qsi_basis_create: %s", cudaGetErrorString(e));
        }
        int* d_bad = nullptr;
        cudaStream_t st = nullptr;
        auto cleanup = [&](qsi_status s) {
            if (d_bad) cudaFree(d_bad);
            if (s != QSI_OK) qsi_basis_destroy(b);
            return s;
        };
        if (cudaMemcpy(b->d_states, lohi, (size_t)n * 16, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMalloc(&d_bad, sizeof(int)) != cudaSuccess || cudaMemset(d_bad, 0, sizeof(int)) != cudaSuccess)
            return cleanup(fail(QSI_CUDA_ERROR, "qsi_basis_create: copy failed"));
        k_check_sorted<<<grid_for(n, 256), 256, 0, st>>>(b->d_states, n, d_bad);
        const qsi_status bs = build_buckets(b);
        if (bs != QSI_OK) return cleanup(bs);
        int bad = 0;
        if (cudaMemcpy(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
            return cleanup(fail(QSI_CUDA_ERROR, "qsi_basis_create: %s", cudaGetErrorString(cudaGetLastError())));
        if (bad) return cleanup(fail(QSI_INVALID_ARG, "qsi_basis_create: basis states are not strictly increasing"));
        // hash index for states of at most 96 bits (skipped, not fatal, when it does not fit in memory)
        if (hb < 96) {
            if (build_hash(b) != QSI_OK) {
                if (b->d_hash) cudaFree(b->d_hash);
                b->d_hash = nullptr;
                b->hash_slots = 0;
                cudaGetLastError();
            }
        }
        *out = b;
        return cleanup(QSI_OK);
    });
}

extern "C" qsi_status qsi_basis_destroy(qsi_basis* b) {
    if (!b) return QSI_OK;
    if (b->d_states) cudaFree(b->d_states);
    if (b->d_bstart) cudaFree(b->d_bstart);
    if (b->d_hash) cudaFree(b->d_hash);
    delete b;
    return QSI_OK;
}

extern "C" qsi_status qsi_basis_dim(const qsi_basis* b, int64_t* dim) {
    if (!b || !dim) return fail(QSI_INVALID_ARG, "qsi_basis_dim: null argument");
    *dim = b->n;
    return QSI_OK;
}

extern "C" qsi_status qsi_basis_search(qsi_basis* b, const uint64_t* states_lohi, int64_t n, int64_t* idx, int32_t flags,
                                       void* stream) {
    return guarded([&]() -> qsi_status {
        if (!b || n < 0 || (n > 0 && (!states_lohi || !idx))) return fail(QSI_INVALID_ARG, "qsi_basis_search: bad argument");
        if (n == 0) return QSI_OK;
        cudaStream_t st = (cudaStream_t)stream;
        if (flags == QSI_PTR_DEVICE) {
            k_search<<<grid_for(n, 256), 256, 0, st>>>(b->view(), (const state2*)states_lohi, n, idx);
            QSI_CUDA(cudaGetLastError());
            return QSI_OK;
        }
        state2* dq = nullptr;
        int64_t* di = nullptr;
        QSI_CUDA(cudaMalloc(&dq, (size_t)n * 16));
        if (cudaMalloc(&di, (size_t)n * 8) != cudaSuccess) {
            cudaFree(dq);
            return fail(QSI_OOM, "qsi_basis_search: allocation failed");
        }
        cudaMemcpy(dq, states_lohi, (size_t)n * 16, cudaMemcpyHostToDevice);
        k_search<<<grid_for(n, 256), 256>>>(b->view(), dq, n, di);
        cudaError_t e = cudaMemcpy(idx, di, (size_t)n * 8, cudaMemcpyDeviceToHost);
        cudaFree(dq);
        cudaFree(di);
        if (e != cudaSuccess) return fail(QSI_CUDA_ERROR, "qsi_basis_search: %s", cudaGetErrorString(e));
        return QSI_OK;
    });
}

// ------------------------------------------------------------------ C-ABI: operator
extern "C" qsi_status qsi_op_create(qsi_basis* b, const qsi_term* terms, int32_t n_terms, qsi_op** out) {
    return guarded([&]() -> qsi_status {
        if (!b || !out || n_terms < 0 || (n_terms > 0 && !terms)) return fail(QSI_INVALID_ARG, "qsi_op_create: bad argument");
        auto* op = new qsi_op();
        op->basis = b;
        std::vector<PullTerm> pull;
        std::vector<PushTerm> push_off, push_diag, diag_generic;
        std::map<double, std::pair<uint64_t, uint64_t>> zcls;  // weight -> mask
        for (int k = 0; k < n_terms; ++k) {
            const qsi_term& t = terms[k];
            PushTerm p{};
            p.x0 = t.x[0], p.x1 = t.x[1], p.z0 = t.z[0], p.z1 = t.z[1];
            p.up0 = t.up[0], p.up1 = t.up[1], p.dn0 = t.down[0], p.dn1 = t.down[1];
            p.c = t.c;
            p.sign = t.sign;
            const bool diagonal = (t.x[0] | t.x[1]) == 0;  // SymbolicOpSum::add_term split, operator.hpp:489-495
            if (diagonal) {
                push_diag.push_back(p);
                if (t.sign != 0 && is_single_site_z(t)) {
                    double w = t.c * (double)t.sign;
                    auto& m = zcls[w];
                    m.first |= t.z[0];
                    m.second |= t.z[1];
                } else if (t.sign != 0) {
                    diag_generic.push_back(p);
                }
                continue;
            }
            push_off.push_back(p);
            if (t.sign == 0) continue;
            PullTerm q{};
            q.x0 = t.x[0], q.x1 = t.x[1], q.z0 = t.z[0], q.z1 = t.z[1];
            // transpose: bits flipped by X swap their up/down requirement
            q.up0 = (t.up[0] & ~t.x[0]) | (t.down[0] & t.x[0]);
            q.up1 = (t.up[1] & ~t.x[1]) | (t.down[1] & t.x[1]);
            q.dn0 = (t.down[0] & ~t.x[0]) | (t.up[0] & t.x[0]);
            q.dn1 = (t.down[1] & ~t.x[1]) | (t.up[1] & t.x[1]);
            // the element is evaluated on the row (pre-image) state: same sign as the
            // reference's evaluation on the image state, see operator.hpp:246-253
            q.cs = t.c * (double)t.sign;
            q.has_z = (t.z[0] | t.z[1]) != 0;
            q.cs_hi = (float)q.cs;
            q.cs_lo = (float)(q.cs - (double)q.cs_hi);
            pull.push_back(q);
        }
        const int n_pull_given = (int)pull.size();
        {
            qsi_status ps = prune_pull_terms(b, pull);
            if (ps != QSI_OK) {
                qsi_op_destroy(op);
                return ps;
            }
        }
        op->n_pull_pruned = n_pull_given - (int)pull.size();
        // A single-site z class whose bits overlap another class with a
        // different weight would double count; the map above merges equal
        // weights only, and each bit can carry several terms.  Handle repeated
        // bits by falling back to the generic list.
        DiagSpec D{};
        {
            uint64_t seen0 = 0, seen1 = 0;
            bool overlap = false;
            for (auto& kv : zcls) {
                if ((kv.second.first & seen0) | (kv.second.second & seen1)) overlap = true;
                seen0 |= kv.second.first, seen1 |= kv.second.second;
            }
            // a bit set twice within one class (two terms on the same site with the
            // same weight) is also merged away by |=: detect by counting terms
            size_t z_terms = 0, z_bits = 0;
            for (int k = 0; k < n_terms; ++k)
                if ((terms[k].x[0] | terms[k].x[1]) == 0 && terms[k].sign != 0 && is_single_site_z(terms[k])) ++z_terms;
            z_bits = (size_t)__builtin_popcountll(seen0) + (size_t)__builtin_popcountll(seen1);
            if (overlap || z_terms != z_bits || (int)zcls.size() > kMaxZClasses) {
                for (int k = 0; k < n_terms; ++k) {
                    const qsi_term& t = terms[k];
                    if ((t.x[0] | t.x[1]) == 0 && t.sign != 0 && is_single_site_z(t)) {
                        PushTerm p{};
                        p.z0 = t.z[0], p.z1 = t.z[1], p.c = t.c, p.sign = t.sign;
                        diag_generic.push_back(p);
                    }
                }
                zcls.clear();
            }
        }
        D.n_cls = 0;
        D.constant = 0.0;
        for (auto& kv : zcls) {
            D.w2[D.n_cls] = 2.0 * kv.first;
            D.m0[D.n_cls] = kv.second.first;
            D.m1[D.n_cls] = kv.second.second;
            D.constant -= kv.first * (double)(__builtin_popcountll(kv.second.first) + __builtin_popcountll(kv.second.second));
            ++D.n_cls;
        }
        D.n_generic = (int)diag_generic.size();
        op->diag = D;
        op->n_pull = (int)pull.size();
        op->n_push_off = (int)push_off.size();
        op->n_push_diag = (int)push_diag.size();
        op->n_diag_generic = (int)diag_generic.size();
        auto upload = [&](void** dst, const void* src, size_t bytes) -> cudaError_t {
            if (!bytes) return cudaSuccess;
            cudaError_t e = cudaMalloc(dst, bytes);
            if (e != cudaSuccess) return e;
            return cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
        };
        cudaError_t e = upload((void**)&op->d_pull, pull.data(), pull.size() * sizeof(PullTerm));
        if (e == cudaSuccess) e = upload((void**)&op->d_push_off, push_off.data(), push_off.size() * sizeof(PushTerm));
        if (e == cudaSuccess) e = upload((void**)&op->d_push_diag, push_diag.data(), push_diag.size() * sizeof(PushTerm));
        if (e == cudaSuccess) e = upload((void**)&op->d_diag_generic, diag_generic.data(), diag_generic.size() * sizeof(PushTerm));
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&op->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            qsi_op_destroy(op);
            return fail(e == cudaErrorMemoryAllocation ? QSI_OOM : QSI_CUDA_ERROR, "qsi_op_create: %s", cudaGetErrorString(e));
        }
        size_t smem = pull.size() * sizeof(PullTerm) + diag_generic.size() * sizeof(PushTerm);
        if (smem > 200 * 1024) {
            qsi_op_destroy(op);
            return fail(QSI_INVALID_ARG, "qsi_op_create: %zu terms exceed the shared-memory term table", pull.size());
        }
        op->smem_bytes = smem;
        // literal lists for the bit-sliced admission test
        std::vector<uint16_t> lit_off{0};
        std::vector<uint8_t> lits;
        int maxbit = b->hb;
        for (const PullTerm& t : pull) {
            const uint64_t um[2] = {t.up0, t.up1}, dm[2] = {t.dn0, t.dn1}, xm[2] = {t.x0, t.x1};
            for (int w = 0; w < 2; ++w) {
                for (int bit = 0; bit < 64; ++bit) {
                    if ((um[w] >> bit) & 1) lits.push_back((uint8_t)(64 * w + bit));
                    if ((dm[w] >> bit) & 1) lits.push_back((uint8_t)(0x80 | (64 * w + bit)));
                    if (((um[w] | dm[w] | xm[w]) >> bit) & 1) maxbit = std::max(maxbit, 64 * w + bit);
                }
            }
            if (lits.size() > 65535) {
                qsi_op_destroy(op);
                return fail(QSI_INVALID_ARG, "qsi_op_create: more than 65535 literals in the term list");
            }
            lit_off.push_back((uint16_t)lits.size());
        }
        op->n_lits = (int)lits.size();
        op->nwords = maxbit / 32 + 1;
        if (lits.empty()) lits.push_back(0);
        e = upload((void**)&op->d_lit_off, lit_off.data(), lit_off.size() * 2);
        if (e == cudaSuccess) e = upload((void**)&op->d_lits, lits.data(), lits.size());
        if (e != cudaSuccess) {
            qsi_op_destroy(op);
            return fail(e == cudaErrorMemoryAllocation ? QSI_OOM : QSI_CUDA_ERROR, "qsi_op_create: %s", cudaGetErrorString(e));
        }
        qsi_status ds = build_diag(op);
        if (ds != QSI_OK) {
            qsi_op_destroy(op);
            return ds;
        }
        cudaGetDevice(&op->device);
        // Device memory that qsi_op_apply_static relies on is reserved here, while allocation is allowed: its
        // staging arrays and the code of the kernels it launches (both are loaded lazily otherwise, at first use).
        // A failure leaves that entry point unavailable on this device and the operator usable.
        if (preload_apply_f64() != QSI_OK || static_stage_prepare() != QSI_OK) cudaGetLastError();
        *out = op;
        return QSI_OK;
    });
}

extern "C" qsi_status qsi_op_destroy(qsi_op* op) {
    if (!op) return QSI_OK;
    if (op->stream) cudaStreamSynchronize(op->stream);
    if (op->family) family_release_member(op);
    if (op->d_fcoef) cudaFree(op->d_fcoef);
    cudaFree(op->d_pull);
    cudaFree(op->d_push_off);
    cudaFree(op->d_push_diag);
    cudaFree(op->d_diag_generic);
    cudaFree(op->d_lit_off);
    if (op->d_diag) cudaFreeAsync(op->d_diag, op->stream);
    if (op->d_diag_ff) cudaFreeAsync(op->d_diag_ff, op->stream);
    if (op->stream) cudaStreamSynchronize(op->stream);
    cudaFree(op->d_lits);
    cudaFree(op->d_x);
    cudaFree(op->d_y);
    cudaFree(op->d_cache_cols);
    cudaFree(op->d_cache_off);
    cudaFree(op->d_cache_tid);
    if (op->stream) cudaStreamDestroy(op->stream);
    delete op;
    return QSI_OK;
}

extern "C" qsi_status qsi_op_materialise(qsi_op* op, int32_t enable, int64_t* bytes) {
    return guarded([&]() -> qsi_status {
        if (!op || (enable != 0 && enable != 1)) return fail(QSI_INVALID_ARG, "qsi_op_materialise: bad argument");
        if (op->stream) QSI_CUDA(cudaStreamSynchronize(op->stream));
        return materialise(op, enable != 0, bytes);
    });
}

namespace qsi {

qsi_status preload_apply_f64_rows() {
    cudaFuncAttributes a;
    QSI_CUDA(cudaFuncGetAttributes(&a, k_apply_rowthread<double, double>));
    return QSI_OK;
}

// Enqueues y (+)= H x on `st` for device pointers.
qsi_status launch_apply(qsi_op* op, const void* x, void* y, int R, int dtype, int accumulate, cudaStream_t st) {
    if (op->family && R == 1 && dtype == QSI_F64)
        return family_apply(op, (const double*)x, (double*)y, accumulate, st);
    if (op->kernel == 1) return launch_apply_tiles(op, x, y, R, dtype, dtype, accumulate, st);
    BasisView V = op->basis->view();
    const int block = 256;
    const size_t smem = op->smem_bytes;
    if (R == 1) {
        int grid = grid_for(V.n, block);
        if (dtype == QSI_F64) {
            auto k = k_apply_rowthread<double, double>;
            if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k<<<grid, block, smem, st>>>(V, op->d_pull, op->n_pull, op->diag, op->d_diag_generic, (const double*)x,
                                         (double*)y, accumulate);
        } else {
            auto k = k_apply_rowthread<float, float>;
            if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k<<<grid, block, smem, st>>>(V, op->d_pull, op->n_pull, op->diag, op->d_diag_generic, (const float*)x,
                                         (float*)y, accumulate);
        }
    } else {
        int grid = grid_for(V.n * 32, block);
        if (dtype == QSI_F64) {
            auto k = k_apply_warprow<double>;
            if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k<<<grid, block, smem, st>>>(V, op->d_pull, op->n_pull, op->diag, op->d_diag_generic, (const double*)x,
                                         (double*)y, R, accumulate);
        } else {
            auto k = k_apply_warprow<float>;
            if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k<<<grid, block, smem, st>>>(V, op->d_pull, op->n_pull, op->diag, op->d_diag_generic, (const float*)x,
                                         (float*)y, R, accumulate);
        }
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(QSI_CUDA_ERROR, "apply launch: %s", cudaGetErrorString(e));
    return QSI_OK;
}

qsi_status launch_apply_to_f64(qsi_op* op, const void* x, double* y, int xdtype, cudaStream_t st) {
    if (xdtype == QSI_F64) return launch_apply(op, x, y, 1, QSI_F64, 0, st);
    if (op->kernel == 1) return launch_apply_tiles(op, x, y, 1, xdtype, QSI_F64, 0, st);
    BasisView V = op->basis->view();
    const size_t smem = op->smem_bytes;
    auto k = k_apply_rowthread<float, double>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k<<<grid_for(V.n, 256), 256, smem, st>>>(V, op->d_pull, op->n_pull, op->diag, op->d_diag_generic, (const float*)x, y, 0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(QSI_CUDA_ERROR, "apply launch: %s", cudaGetErrorString(e));
    return QSI_OK;
}

static qsi_status ensure_host_staging(qsi_op* op, size_t bytes) {
    if (op->staging_bytes >= bytes) return QSI_OK;
    cudaFree(op->d_x);
    cudaFree(op->d_y);
    op->d_x = op->d_y = nullptr;
    op->staging_bytes = 0;
    QSI_CUDA(cudaMalloc(&op->d_x, bytes));
    QSI_CUDA(cudaMalloc(&op->d_y, bytes));
    op->staging_bytes = bytes;
    return QSI_OK;
}

// Device address of page-locked host memory mapped into the device's address space (nullptr otherwise).
static void* mapped_host(void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (a.type == cudaMemoryTypeHost && a.devicePointer) ? a.devicePointer : nullptr;
}

qsi_status apply_any(qsi_op* op, const void* x, void* y, int R, int dtype, int accumulate, int flags, void* stream) {
    if (!op || !x || !y || R <= 0 || (dtype != QSI_F64 && dtype != QSI_F32))
        return fail(QSI_INVALID_ARG, "apply: bad argument");
    cudaStream_t st = stream ? (cudaStream_t)stream : op->stream;
    if (flags == QSI_PTR_DEVICE) return launch_apply(op, x, y, R, dtype, accumulate, st);
    const size_t bytes = (size_t)op->basis->n * R * (dtype == QSI_F64 ? 8 : 4);
    qsi_status s = ensure_host_staging(op, bytes);
    if (s != QSI_OK) return s;
    QSI_CUDA(cudaMemcpyAsync(op->d_x, x, bytes, cudaMemcpyHostToDevice, st));
    // A pinned, mapped result buffer (y = H x, no accumulation) takes the kernel's row stores directly over the
    // host link (every kernel writes each y element once and reads y only when accumulating), so no device-to-host
    // copy follows the apply.  Pageable buffers go through the staging copy.
    void* y_mapped = accumulate ? nullptr : mapped_host(y);
    if (accumulate) QSI_CUDA(cudaMemcpyAsync(op->d_y, y, bytes, cudaMemcpyHostToDevice, st));
    s = launch_apply(op, op->d_x, y_mapped ? y_mapped : op->d_y, R, dtype, accumulate, st);
    if (s != QSI_OK) return s;
    if (!y_mapped) QSI_CUDA(cudaMemcpyAsync(y, op->d_y, bytes, cudaMemcpyDeviceToHost, st));
    QSI_CUDA(cudaStreamSynchronize(st));
    return QSI_OK;
}

}  // namespace qsi

extern "C" qsi_status qsi_op_apply(qsi_op* op, const double* x, double* y, int32_t accumulate, int32_t flags,
                                   void* stream) {
    return guarded([&]() { return apply_any(op, x, y, 1, QSI_F64, accumulate, flags, stream); });
}

extern "C" qsi_status qsi_op_apply_batched(qsi_op* op, const void* X, void* Y, int32_t R, int32_t dtype,
                                           int32_t accumulate, int32_t flags, void* stream) {
    return guarded([&]() { return apply_any(op, X, Y, R, dtype, accumulate, flags, stream); });
}

extern "C" qsi_status qsi_op_triplets(qsi_op* op, double tol, int64_t* rows, int64_t* cols, double* vals, int64_t cap,
                                      int64_t* n_out) {
    return guarded([&]() -> qsi_status {
        if (!op || !n_out) return fail(QSI_INVALID_ARG, "qsi_op_triplets: null argument");
        BasisView V = op->basis->view();
        const int64_t n = V.n;
        int64_t *d_counts = nullptr, *d_offs = nullptr;
        QSI_CUDA(cudaMalloc(&d_counts, (size_t)n * 8));
        QSI_CUDA(cudaMalloc(&d_offs, (size_t)(n + 1) * 8));
        k_triplets<<<grid_for(n, 128), 128>>>(V, op->d_push_off, op->n_push_off, op->d_push_diag, op->n_push_diag, tol,
                                               nullptr, d_counts, nullptr, nullptr, nullptr);
        // prefix sum on the host (export path, not performance critical)
        std::vector<int64_t> cnt(n), offs(n + 1);
        QSI_CUDA(cudaMemcpy(cnt.data(), d_counts, (size_t)n * 8, cudaMemcpyDeviceToHost));
        offs[0] = 0;
        for (int64_t i = 0; i < n; ++i) offs[i + 1] = offs[i] + cnt[i];
        const int64_t total = offs[n];
        *n_out = total;
        if (!rows) {
            cudaFree(d_counts);
            cudaFree(d_offs);
            return QSI_OK;
        }
        if (!cols || !vals || cap < total) {
            cudaFree(d_counts);
            cudaFree(d_offs);
            return fail(QSI_INVALID_ARG, "qsi_op_triplets: output capacity %lld < %lld", (long long)cap, (long long)total);
        }
        QSI_CUDA(cudaMemcpy(d_offs, offs.data(), (size_t)(n + 1) * 8, cudaMemcpyHostToDevice));
        int64_t *dr = nullptr, *dc = nullptr;
        double* dv = nullptr;
        QSI_CUDA(cudaMalloc(&dr, (size_t)total * 8));
        QSI_CUDA(cudaMalloc(&dc, (size_t)total * 8));
        QSI_CUDA(cudaMalloc(&dv, (size_t)total * 8));
        k_triplets<<<grid_for(n, 128), 128>>>(V, op->d_push_off, op->n_push_off, op->d_push_diag, op->n_push_diag, tol,
                                               d_offs, nullptr, dr, dc, dv);
        cudaError_t e = cudaMemcpy(rows, dr, (size_t)total * 8, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(cols, dc, (size_t)total * 8, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(vals, dv, (size_t)total * 8, cudaMemcpyDeviceToHost);
        cudaFree(dr);
        cudaFree(dc);
        cudaFree(dv);
        cudaFree(d_counts);
        cudaFree(d_offs);
        if (e != cudaSuccess) return fail(QSI_CUDA_ERROR, "qsi_op_triplets: %s", cudaGetErrorString(e));
        return QSI_OK;
    });
}

extern "C" qsi_status qsi_op_connectivity(qsi_op* op, int64_t* hits, int64_t* misses) {
    return guarded([&]() -> qsi_status {
        if (!op) return fail(QSI_INVALID_ARG, "qsi_op_connectivity: null argument");
        unsigned long long* d = nullptr;
        QSI_CUDA(cudaMalloc(&d, 16));
        QSI_CUDA(cudaMemset(d, 0, 16));
        BasisView V = op->basis->view();
        k_count_connectivity<<<grid_for(V.n, 256), 256>>>(V, op->d_push_off, op->n_push_off, d);
        unsigned long long h[2] = {0, 0};
        cudaError_t e = cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost);
        cudaFree(d);
        if (e != cudaSuccess) return fail(QSI_CUDA_ERROR, "qsi_op_connectivity: %s", cudaGetErrorString(e));
        if (hits) *hits = (int64_t)h[0];
        if (misses) *misses = (int64_t)h[1];
        return QSI_OK;
    });
}

extern "C" qsi_status qsi_op_count_misses(qsi_op* op, int64_t* misses) {
    if (!misses) return fail(QSI_INVALID_ARG, "qsi_op_count_misses: null argument");
    return qsi_op_connectivity(op, nullptr, misses);
}

extern "C" qsi_status qsi_basis_index(qsi_basis* b, int32_t use_hash, int32_t bucket_bits) {
    return guarded([&]() -> qsi_status {
        if (!b) return fail(QSI_INVALID_ARG, "qsi_basis_index: null basis");
        if (bucket_bits > 0 && bucket_bits != b->bits) {
            int bits = std::min<int>(bucket_bits, std::min(31, b->hb + 1));
            uint32_t* nb = nullptr;
            QSI_CUDA(cudaMalloc(&nb, bucket_table_entries(1u << bits) * sizeof(uint32_t)));
            cudaFree(b->d_bstart);
            b->d_bstart = nb;
            b->bits = bits;
            b->shift = b->hb + 1 - bits;
            b->n_buckets = 1u << bits;
            qsi_status bs = build_buckets(b);
            if (bs != QSI_OK) return bs;
            QSI_CUDA(cudaDeviceSynchronize());
            if (b->d_hash) {  // the hash's regions are the table's buckets
                if (!use_hash) {
                    cudaFree(b->d_hash);
                    b->d_hash = nullptr;
                    b->hash_slots = 0;
                    return QSI_OK;
                }
                return build_hash(b);
            }
        }
        if (use_hash && !b->d_hash) return build_hash(b);
        if (!use_hash && b->d_hash) {
            cudaFree(b->d_hash);
            b->d_hash = nullptr;
            b->hash_slots = 0;
        }
        return QSI_OK;
    });
}

extern "C" qsi_status qsi_basis_info(const qsi_basis* b, int32_t* bucket_bits, int32_t* has_hash, int64_t* index_bytes) {
    if (!b) return fail(QSI_INVALID_ARG, "qsi_basis_info: null basis");
    if (bucket_bits) *bucket_bits = b->bits;
    if (has_hash) *has_hash = b->d_hash != nullptr;
    if (index_bytes)
        *index_bytes = (int64_t)(bucket_table_entries(b->n_buckets) * 4 +
                                 (b->d_hash ? b->hash_slots * sizeof(HashSlot) : 0));
    return QSI_OK;
}

extern "C" qsi_status qsi_op_info(const qsi_op* op, int32_t* n_offdiag, int32_t* n_pruned, int32_t* n_diag_classes,
                                   int32_t* n_diag_generic) {
    if (!op) return fail(QSI_INVALID_ARG, "qsi_op_info: null operator");
    if (n_offdiag) *n_offdiag = op->n_pull;
    if (n_pruned) *n_pruned = op->n_pull_pruned;
    if (n_diag_classes) *n_diag_classes = op->diag.n_cls;
    if (n_diag_generic) *n_diag_generic = op->n_diag_generic;
    return QSI_OK;
}

extern "C" qsi_status qsi_op_set_kernel(qsi_op* op, int32_t kernel, int32_t use_hash, int32_t list_cap) {
    if (!op || kernel < 0 || kernel > 1 || list_cap < 0) return fail(QSI_INVALID_ARG, "qsi_op_set_kernel: bad argument");
    op->kernel = kernel;
    for (qsi_tuning& T : op->tune) {
        T.use_hash = use_hash & 1;
        if (list_cap > 0) T.list_cap = list_cap;
    }
    op->ff_accumulate = (use_hash & 2) ? 0 : 1;
    return QSI_OK;
}
