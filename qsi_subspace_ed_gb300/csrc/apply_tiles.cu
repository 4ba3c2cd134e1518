// Bit-sliced tile kernels of the pull-gather apply, and the hash index.
//
// A warp owns a tile of 32 consecutive basis rows.  The tile's 32 states are
// transposed with warp shuffles into one 32-bit word per spin (bit l = spin
// of row l), so one lane evaluates one off-diagonal term for all 32 rows with
// a few AND/XOR operations over that term's literals (the spins its
// transposed up/down masks constrain).  A second transpose hands each row its
// admitted terms as a bit set, visited in term order, so every row is summed
// in the same fixed order as the one-row-per-thread kernel (deterministic,
// bit-identical results).
//
// Single vector: each lane finds its own row's columns and gathers x.
// Batched (R vectors, [row][R] layout): lanes first look up all columns of
// the tile into a shared-memory hit list; then the warp walks the list row
// by row and gathers each column's R values with coalesced loads.
#include <algorithm>
#include <cmath>
#include <vector>
#include <type_traits>

#include <cub/device/device_scan.cuh>

#include "qsi_device.cuh"
#include "qsi_handles.h"

namespace qsi {

struct TileParams {
    BasisView B;
    const PullTerm* terms;
    const uint16_t* lit_off;
    const uint8_t* lits;
    const PushTerm* dgen;
    DiagSpec D;
    const double* diag;  // per-row diagonal, precomputed with diag_value
    const float2* diag_ff;  // the same as (hi, lo) float pairs
    int n_off, n_lits, nwords;
    int vchunk;             // vectors per pass of the 16-byte batched kernel (16, 32, 64 or 128; 0 = 128)
    // operator families (family mode kernels only): the terms' coefficients encode their class as +-(class + 1)
    // and fcoef[class * fR + column] is the coefficient of that class in each column's operator
    const double* fcoef = nullptr;
    int fR = 1;
};

// Family mode: the coefficient of a hit whose term's coefficient encodes +-(class + 1), for column col.
__device__ __forceinline__ double fam_coef(const TileParams& P, double enc, int col) {
    const double c = P.fcoef[((int)(fabs(enc) + 0.5) - 1) * P.fR + col];
    return enc < 0 ? -c : c;
}
// Family mode: the diagonal of state s for column col, sum over the single-site z groups of the template's
// diagonal (weight +-(class + 1) each) of coefficient(class) * sign * (2 popcount(s & M) - |M|), in group order.
__device__ __forceinline__ double fam_diag(const TileParams& P, uint64_t s0, uint64_t s1, int col) {
    double d = 0.0;
    for (int k = 0; k < P.D.n_cls; ++k) {
        const double w = 0.5 * P.D.w2[k];
        const int cls = (int)(fabs(w) + 0.5) - 1;
        const int cnt = __popcll(P.D.m0[k]) + __popcll(P.D.m1[k]);
        const int v = 2 * (__popcll(s0 & P.D.m0[k]) + __popcll(s1 & P.D.m1[k])) - cnt;
        const double c = P.fcoef[cls * P.fR + col];
        d += (w < 0 ? -c : c) * (double)v;
    }
    return d;
}

// |x| > 1e-15 (APPLY_TOL, operator_matrix.hpp:113) as integer compares on the
// bit pattern: magnitude above the threshold and not a NaN.  For FP32 x the
// threshold is the largest float whose value is <= 1e-15, so the test equals
// fabs((double)x) > 1e-15 exactly.
constexpr uint64_t kTolBitsF64 = 0x3CD203AF9EE75616ULL;  // 1e-15
constexpr uint32_t kTolBitsF32 = 0x26901D7CU;            // largest float <= 1e-15
__device__ __forceinline__ bool above_tol(double v) {
    const uint64_t m = (uint64_t)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFULL;
    return m > kTolBitsF64 && m <= 0x7FF0000000000000ULL;
}
__device__ __forceinline__ bool above_tol(float v) {
    const uint32_t m = __float_as_uint(v) & 0x7FFFFFFFu;
    return m - (kTolBitsF32 + 1) <= 0x7F800000u - (kTolBitsF32 + 1);  // kTolBitsF32 < m <= inf, one compare
}
// v where the tolerance test admits it (or keep is set), else 0: selected, not branched, so the
// double-float update that follows runs unconditionally (adding 0 leaves the sum unchanged).  The float
// compare |v| > largest-float-below-1e-15 is the same test as above_tol (false for NaN, true for inf).
__device__ __forceinline__ float tol_select(float v, bool keep) {
    return (keep || fabsf(v) > __uint_as_float(kTolBitsF32)) ? v : 0.0f;
}

// Double-float accumulator (hi + lo, two FP32 words, ~2^-48 relative):
// error-free product c*x with c = ch + cl and error-free sum into hi.
struct FF {
    float hi, lo;
};
__device__ __forceinline__ void ff_fma(FF& a, float ch, float cl, float x) {
    const float p = ch * x;
    const float e = fmaf(ch, x, -p) + cl * x;
    const float s = a.hi + p;
    const float bb = s - a.hi;
    const float err = (a.hi - (s - bb)) + (p - bb);
    a.hi = s;
    a.lo += err + e;
}
// Two double-float accumulators held as packed FP32 pairs and updated with the f32x2 instructions of
// sm_100-family GPUs (one instruction per operation for both): the same operations, in the same order,
// as ff_fma on each lane of the pair.
struct FF2 {
    uint64_t hi, lo;
};
__device__ __forceinline__ uint64_t pk2(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float2 unpk2(uint64_t v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
// a += (ch + cl) * x on both lanes; cn = -ch.  q = cn*x = -(ch*x) exactly, so hi - q is hi + p and
// fma(ch, x, q) is the exact error of the product p = ch*x, as in ff_fma.
__device__ __forceinline__ void ff2_fma(FF2& a, uint64_t ch, uint64_t cn, uint64_t cl, uint64_t x) {
    const uint64_t q = mul2(cn, x);
    const uint64_t e = fma2(cl, x, fma2(ch, x, q));
    const uint64_t s = sub2(a.hi, q);
    const uint64_t bb = sub2(s, a.hi);
    const uint64_t err = sub2(sub2(a.hi, sub2(s, bb)), add2(q, bb));
    a.hi = s;
    a.lo = add2(a.lo, add2(err, e));
}

// Shared-memory layout common to both tile kernels.
struct TileSmem {
    PullTerm* terms;
    PushTerm* dgen;
    uint16_t* off;
    uint8_t* lit;
    unsigned char* tail;  // per-warp scratch follows
};

__device__ __forceinline__ TileSmem stage_terms(const TileParams& P, unsigned char* smem) {
    TileSmem S;
    S.terms = reinterpret_cast<PullTerm*>(smem);
    S.dgen = reinterpret_cast<PushTerm*>(S.terms + P.n_off);
    S.off = reinterpret_cast<uint16_t*>(S.dgen + P.D.n_generic);
    S.lit = reinterpret_cast<uint8_t*>(S.off + P.n_off + 1);
    size_t used = (size_t)P.n_off * sizeof(PullTerm) + (size_t)P.D.n_generic * sizeof(PushTerm) +
                  (size_t)(P.n_off + 1) * 2 + (size_t)P.n_lits;
    S.tail = smem + ((used + 15) & ~(size_t)15);
    for (int k = threadIdx.x; k < P.n_off; k += blockDim.x) S.terms[k] = P.terms[k];
    for (int k = threadIdx.x; k < P.D.n_generic; k += blockDim.x) S.dgen[k] = P.dgen[k];
    for (int k = threadIdx.x; k <= P.n_off; k += blockDim.x) S.off[k] = P.lit_off[k];
    for (int k = threadIdx.x; k < P.n_lits; k += blockDim.x) S.lit[k] = P.lits[k];
    __syncthreads();
    return S;
}

// Transposes the tile's states into per-spin words spinw[0 .. 32*nwords).
__device__ __forceinline__ void tile_spin_words(const state2 s, int nwords, int lane, uint32_t* spinw) {
    const uint32_t w[4] = {(uint32_t)s.x, (uint32_t)(s.x >> 32), (uint32_t)s.y, (uint32_t)(s.y >> 32)};
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (k < nwords) spinw[32 * k + lane] = warp_transpose32(w[k], lane);
    __syncwarp();
}

// Admission bits of terms t0..t0+31 for this lane's row (bit j = term t0+j).
__device__ __forceinline__ uint32_t tile_admitted(const TileSmem& S, int n_off, int t0, int lane, uint32_t vmask,
                                                  const uint32_t* spinw) {
    const int t = t0 + lane;
    uint32_t A = 0;
    if (t < n_off) {
        A = vmask;
        const int e = S.off[t + 1];
        for (int k = S.off[t]; k < e; ++k) {
            const uint8_t L = S.lit[k];
            A &= spinw[L & 127] ^ ((L & 128) ? 0xFFFFFFFFu : 0u);
        }
    }
    return warp_transpose32(A, lane);
}

__device__ __forceinline__ double term_coeff(const PullTerm& T, const state2 s) {
    double cs = T.cs;
    if (T.has_z && ((__popcll(~s.x & T.z0) + __popcll(~s.y & T.z1)) & 1)) cs = -cs;
    return cs;
}

template <typename XT, typename YT, class LK, bool kFam = false>
__global__ void __launch_bounds__(256, LK::kMinBlocks) k_apply_tile(TileParams P, LK lk, const XT* __restrict__ x,
                                                                 YT* __restrict__ y, int accumulate) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const TileSmem S = stage_terms(P, smem_raw);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int n_rounds = (P.n_off + 31) >> 5;
    uint32_t* spinw = reinterpret_cast<uint32_t*>(S.tail) + wid * (128 + 32 * n_rounds);
    uint32_t* adm = spinw + 128;  // admission words of the tile, one per lane and 32-term round
    const int64_t ntiles = (P.B.n + 31) >> 5;
    for (int64_t tile = (int64_t)blockIdx.x * nw + wid; tile < ntiles; tile += (int64_t)gridDim.x * nw) {
        const int64_t row = tile * 32 + lane;
        const bool valid = row < P.B.n;
        const state2 s = valid ? P.B.states[row] : make_ulonglong2(0, 0);
        const uint32_t vmask = __ballot_sync(0xffffffffu, valid);
        tile_spin_words(s, P.nwords, lane, spinw);
        for (int r = 0; r < n_rounds; ++r) adm[r * 32 + lane] = tile_admitted(S, P.n_off, r * 32, lane, vmask, spinw);
        double acc = valid ? (kFam ? fam_diag(P, s.x, s.y, 0) : P.diag[row]) * (double)x[row] : 0.0;
        const uint64_t cur = lk.cursor(tile, lane);
        int kk = 0;  // admitted terms of this row looked up so far
        int r = 0;
        uint32_t a = adm[lane];
        while (true) {
            // up to kNB admitted terms at a time (across rounds): lookups and gathers in flight together,
            // contributions added in term order
            constexpr int kNB = LK::kNB;
            int tt[kNB];
            uint64_t tl[kNB], th[kNB];
            int64_t J[kNB];
            int nh = 0;
#pragma unroll
            for (int u = 0; u < kNB; ++u) {
                tt[u] = 0;
                tl[u] = th[u] = 0;
                while (!a && r + 1 < n_rounds) a = adm[++r * 32 + lane];
                if (a) {
                    tt[u] = r * 32 + __ffs(a) - 1;
                    a &= a - 1;
                    const PullTerm& T = S.terms[tt[u]];
                    tl[u] = s.x ^ T.x0;
                    th[u] = s.y ^ T.x1;
                    ++nh;
                }
            }
            if (!nh) break;
            lk.template find_batch<kNB>(tl, th, J, nh, cur, kk);
            kk += nh;
            XT xv[kNB];
#pragma unroll
            for (int u = 0; u < kNB; ++u) xv[u] = (u < nh && J[u] >= 0) ? x[J[u]] : (XT)0;
#pragma unroll
            for (int u = 0; u < kNB; ++u)
                if (u < nh && J[u] >= 0 && above_tol(xv[u])) {
                    const double cs = term_coeff(S.terms[tt[u]], s);
                    acc += (kFam ? fam_coef(P, cs, 0) : cs) * (double)xv[u];
                }
        }
        if (valid) {
            if (accumulate) acc += (double)y[row];
            y[row] = (YT)acc;
        }
        __syncwarp();
    }
}

// Family mode with a few columns (FP64 [row][R], 2 <= R <= RC): the single-vector tile kernel with each lane
// summing all R columns of its row, the R values of a hit gathered from one place.  Each column's sum is the one
// k_apply_tile forms for that column alone (same terms in the same order, same coefficients and tests), so a
// member's result does not depend on the batch it ran in.
template <class LK, int RC>
__global__ void __launch_bounds__(256, RC <= 4 ? 4 : 2) k_apply_tile_cols(TileParams P, LK lk, const double* __restrict__ x,
                                                            double* __restrict__ y, int accumulate) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const TileSmem S = stage_terms(P, smem_raw);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int n_rounds = (P.n_off + 31) >> 5;
    const int R = P.fR;
    uint32_t* spinw = reinterpret_cast<uint32_t*>(S.tail) + wid * (128 + 32 * n_rounds);
    uint32_t* adm = spinw + 128;
    const int64_t ntiles = (P.B.n + 31) >> 5;
    for (int64_t tile = (int64_t)blockIdx.x * nw + wid; tile < ntiles; tile += (int64_t)gridDim.x * nw) {
        const int64_t row = tile * 32 + lane;
        const bool valid = row < P.B.n;
        const state2 s = valid ? P.B.states[row] : make_ulonglong2(0, 0);
        const uint32_t vmask = __ballot_sync(0xffffffffu, valid);
        tile_spin_words(s, P.nwords, lane, spinw);
        for (int r = 0; r < n_rounds; ++r) adm[r * 32 + lane] = tile_admitted(S, P.n_off, r * 32, lane, vmask, spinw);
        double acc[RC];
#pragma unroll
        for (int c = 0; c < RC; ++c) acc[c] = (valid && c < R) ? fam_diag(P, s.x, s.y, c) * x[row * R + c] : 0.0;
        const uint64_t cur = lk.cursor(tile, lane);
        int kk = 0, r = 0;
        uint32_t a = adm[lane];
        while (true) {
            constexpr int kNB = 4;
            int tt[kNB];
            uint64_t tl[kNB], th[kNB];
            int64_t J[kNB];
            int nh = 0;
#pragma unroll
            for (int u = 0; u < kNB; ++u) {
                tt[u] = 0;
                tl[u] = th[u] = 0;
                while (!a && r + 1 < n_rounds) a = adm[++r * 32 + lane];
                if (a) {
                    tt[u] = r * 32 + __ffs(a) - 1;
                    a &= a - 1;
                    const PullTerm& T = S.terms[tt[u]];
                    tl[u] = s.x ^ T.x0;
                    th[u] = s.y ^ T.x1;
                    ++nh;
                }
            }
            if (!nh) break;
            lk.template find_batch<kNB>(tl, th, J, nh, cur, kk);
            kk += nh;
#pragma unroll
            for (int u = 0; u < kNB; ++u) {
                if (u >= nh || J[u] < 0) continue;
                const double cs = term_coeff(S.terms[tt[u]], s);
                const double* xj = x + J[u] * R;
                double xv[RC];
#pragma unroll
                for (int c = 0; c < RC; ++c) xv[c] = (c < R) ? xj[c] : 0.0;
#pragma unroll
                for (int c = 0; c < RC; ++c)
                    if (c < R && above_tol(xv[c])) acc[c] += fam_coef(P, cs, c) * xv[c];
            }
        }
        if (valid) {
#pragma unroll
            for (int c = 0; c < RC; ++c) {
                if (c >= R) break;
                double v = acc[c];
                if (accumulate) v += y[row * R + c];
                y[row * R + c] = v;
            }
        }
        __syncwarp();
    }
}

// KM values selecting 16-byte FP32 gathers of 4 (kVec4) or 8 (kVec8) vectors per lane (see batched_body), and
// the bases, vector counts and pointers each takes.  Their hit lists mark the diagonal slot with the top bit of
// the row index.
constexpr int kVec4 = 0;
constexpr int kVec8 = -1;
constexpr int kVec16 = -2;
constexpr uint32_t kDiagSlot = 0x80000000u;
inline bool vec4_ok(int64_t n, int R, const void* x, const void* y) {
    return n < (int64_t)kDiagSlot - 1 && R >= 16 && (R & 3) == 0 &&
           (R <= 128 ? (R & (R - 1)) == 0 : (R & 127) == 0) &&
           ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15) == 0;
}
inline bool vec8_ok(int64_t n, int R, const void* x, const void* y) {
    return vec4_ok(n, R, x, y) && R >= 32 && (R <= 256 ? (R & (R - 1)) == 0 : (R & 255) == 0);
}
inline bool vec16_ok(int64_t n, int R, const void* x, const void* y) {
    return vec4_ok(n, R, x, y) && R >= 64 && (R <= 512 ? (R & (R - 1)) == 0 : (R & 511) == 0);
}

// Body of the batched tile kernel for one block (block_id of n_blocks working on this operator).
template <typename XT, class LK, bool kFF, int KM, bool kFam = false>
__device__ __forceinline__ void batched_body(const TileParams& P, const LK& lk, const XT* __restrict__ x,
                                             XT* __restrict__ y, int R, int accumulate, int cap, int64_t block_id,
                                             int64_t n_blocks, unsigned char* smem_raw,
                                             const float2* __restrict__ ycoef = nullptr) {
    // accumulate: y <- H x + c y per column, c = 1, or the (hi, lo) float pair ycoef[column] (double-float paths)
    const TileSmem S = stage_terms(P, smem_raw);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int n_rounds = (P.n_off + 31) >> 5;
    // per-warp scratch: spin words (128 u32), admission words (n_rounds*32 u32), hit list
    unsigned char* mine = S.tail + (size_t)wid * (512 + (size_t)n_rounds * 128 + (size_t)cap * 12);
    uint32_t* spinw = reinterpret_cast<uint32_t*>(mine);
    uint32_t* adm = spinw + 128;
    double* hc = reinterpret_cast<double*>(adm + n_rounds * 32);  // coefficients (8-byte aligned)
    float2* hcf = reinterpret_cast<float2*>(hc);                   // the same slots as (hi, lo) floats
    uint32_t* hJ = reinterpret_cast<uint32_t*>(hc + cap);
    // KM == kVec4 / kVec8 (FP32, R accepted by vec4_ok / vec8_ok): 16-byte gathers.  A lane owns VPL = 4 or 8
    // consecutive vectors, lpc lanes cover one column's vectors (up to 32*VPL per pass), and the warp's
    // cpw = 32/lpc lane groups sum cpw rows at once.  Otherwise a lane owns KM vectors and the warp sums one
    // row at a time.
    constexpr bool v4 = (KM == kVec4 || KM == kVec8 || KM == kVec16);
    constexpr int VPL = (KM == kVec16) ? 16 : (KM == kVec8) ? 8 : 4;
    static_assert(!v4 || kFF, "16-byte gathers are for FP32 vectors with double-float accumulation");
    int lpc = 32, cpw = 1;
    if constexpr (v4) {
        const int vc = P.vchunk > 0 ? P.vchunk : 32 * VPL;
        lpc = (R >= vc ? vc : R) / VPL;
        cpw = 32 / lpc;
    }
    const int64_t ntiles = (P.B.n + 31) >> 5;
    for (int64_t tile = block_id * nw + wid; tile < ntiles; tile += n_blocks * nw) {
        const int64_t row = tile * 32 + lane;
        const bool valid = row < P.B.n;
        const state2 s = valid ? P.B.states[row] : make_ulonglong2(0, 0);
        const uint32_t vmask = __ballot_sync(0xffffffffu, valid);
        tile_spin_words(s, P.nwords, lane, spinw);
        int cnt = 0;
        for (int r = 0; r < n_rounds; ++r) {
            const uint32_t a = tile_admitted(S, P.n_off, r * 32, lane, vmask, spinw);
            adm[r * 32 + lane] = a;
            cnt += __popc(a);
        }
        const int pc = v4 ? cnt + 1 : cnt;  // list slots of this row: (the diagonal,) the hits
        const double d = valid ? P.diag[row] : 0.0;
        int row_start = 0;
        while (row_start < 32) {
            // rows [row_start, row_end) whose slots fit the list (at least one row; cap >= a row's slots)
            int c = (lane >= row_start) ? pc : 0;
            int incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            const bool in_chunk = lane >= row_start && (incl <= cap || lane == row_start);
            const uint32_t cm = __ballot_sync(0xffffffffu, in_chunk);
            const int row_end = 32 - __clz(cm);
            int base = incl - c;
            if (in_chunk) {
                int k = base;
                if constexpr (v4) {  // the diagonal leads the row's list (gathered like a hit, no tolerance test)
                    hJ[k] = valid ? (uint32_t)row | kDiagSlot : kEmpty;
                    hcf[k] = valid ? P.diag_ff[row] : make_float2(0.f, 0.f);
                    ++k;
                }
                // this row's admitted terms in term order, kNB lookups at a time across the 32-term rounds
                const uint64_t cur = lk.cursor(tile, lane);
                int kk = 0;
                int r = 0;
                uint32_t a = adm[lane];
                while (true) {
                    {
                        constexpr int kNB = v4 ? 6 : 4;
                        int tt[kNB];
                        uint64_t tl[kNB], th[kNB];
                        int64_t J[kNB];
                        int nh = 0;
#pragma unroll
                        for (int u = 0; u < kNB; ++u) {
                            tt[u] = 0;
                            tl[u] = th[u] = 0;
                            while (!a && r + 1 < n_rounds) a = adm[++r * 32 + lane];
                            if (a) {
                                tt[u] = r * 32 + __ffs(a) - 1;
                                a &= a - 1;
                                tl[u] = s.x ^ S.terms[tt[u]].x0;
                                th[u] = s.y ^ S.terms[tt[u]].x1;
                                ++nh;
                            }
                        }
                        if (!nh) break;
                        lk.template find_batch<kNB>(tl, th, J, nh, cur, kk);
                        kk += nh;
#pragma unroll
                        for (int u = 0; u < kNB; ++u) {
                            if (u >= nh) continue;
                            hJ[k] = (J[u] < 0) ? kEmpty : (uint32_t)J[u];
                            const PullTerm& T = S.terms[tt[u]];
                            if constexpr (kFF) {
                                const bool neg = T.has_z && ((__popcll(~s.x & T.z0) + __popcll(~s.y & T.z1)) & 1);
                                hcf[k] = neg ? make_float2(-T.cs_hi, -T.cs_lo) : make_float2(T.cs_hi, T.cs_lo);
                            } else {
                                hc[k] = term_coeff(T, s);
                            }
                            ++k;
                        }
                    }
                }
            }
            __syncwarp();
            if constexpr (kFF) {
                // FP32 storage, double-float accumulation, no FP64 instruction.  The chunk's hit list
                // is walked in order across row boundaries with kU column gathers in flight.
                static_assert(std::is_same<XT, float>::value, "double-float accumulation is for FP32 vectors");
                constexpr int kU = 32 / VPL;  // column gathers in flight per lane (kU * VPL = 32 floats)
                const int kbeg = __shfl_sync(0xffffffffu, base, row_start);
                const int last = row_end - 1;
                const int kend = __shfl_sync(0xffffffffu, base + pc, last);
                if constexpr (v4) {
                    // Lane group g (lpc lanes, VPL vectors each) sums rows row_start + g, + g + cpw, ...: each
                    // group walks its own row's slots, kU column gathers in flight per lane, and the warp
                    // steps as long as its longest row of the set.
                    constexpr int NQ = VPL / 4;  // float4 loads per lane and column
                    const int g = lane / lpc, rr = VPL * (lane % lpc);
                    for (int r0 = 0; r0 < R; r0 += VPL * lpc) {
                        for (int l0 = row_start; l0 < row_end; l0 += cpw) {
                            const int l = l0 + g;
                            const bool mine = l < row_end;
                            const int lsrc = mine ? l : row_end - 1;
                            const int kb = __shfl_sync(0xffffffffu, base, lsrc);
                            int nl = __shfl_sync(0xffffffffu, pc, lsrc);
                            if (!mine) nl = 0;
                            int steps = nl;
#pragma unroll
                            for (int o = 16; o; o >>= 1) steps = max(steps, __shfl_xor_sync(0xffffffffu, steps, o));
                            FF2 acc[2 * NQ];  // vector pairs (0, 1), (2, 3), ... of this lane
#pragma unroll
                            for (int i = 0; i < 2 * NQ; ++i) acc[i] = FF2{0, 0};
                            auto run_batch = [&](int s0, auto width) {
                                constexpr int W = decltype(width)::value;
                                float4 xv[W][NQ];
                                float2 ck[W];
                                uint32_t dg = 0;  // bit u: slot u holds the diagonal
#pragma unroll
                                for (int u = 0; u < W; ++u) {
                                    const int k = kb + s0 + u;
                                    const uint32_t J = (s0 + u < nl) ? hJ[k] : kEmpty;
                                    if (J != kEmpty && (J & kDiagSlot)) dg |= 1u << u;
                                    ck[u] = (J == kEmpty) ? make_float2(0.f, 0.f) : hcf[k];
                                    const float4* src =
                                        reinterpret_cast<const float4*>(x + (int64_t)(J & ~kDiagSlot) * R + r0 + rr);
#pragma unroll
                                    for (int q = 0; q < NQ; ++q)
                                        xv[u][q] = (J == kEmpty) ? make_float4(0.f, 0.f, 0.f, 0.f) : src[q];
                                }
#pragma unroll
                                for (int u = 0; u < W; ++u) {
                                    const bool all = (dg >> u) & 1;
                                    const uint64_t ch = pk2(ck[u].x, ck[u].x), cn = pk2(-ck[u].x, -ck[u].x),
                                                   cl = pk2(ck[u].y, ck[u].y);
#pragma unroll
                                    for (int q = 0; q < NQ; ++q) {
                                        ff2_fma(acc[2 * q], ch, cn, cl,
                                                pk2(tol_select(xv[u][q].x, all), tol_select(xv[u][q].y, all)));
                                        ff2_fma(acc[2 * q + 1], ch, cn, cl,
                                                pk2(tol_select(xv[u][q].z, all), tol_select(xv[u][q].w, all)));
                                    }
                                }
                            };
                            for (int s0 = 0; s0 < steps;) {  // full batches, and a half batch for a short tail
                                if (steps - s0 > kU / 2) {
                                    run_batch(s0, std::integral_constant<int, kU>{});
                                    s0 += kU;
                                } else {
                                    constexpr int kH = kU / 2 > 0 ? kU / 2 : 1;
                                    run_batch(s0, std::integral_constant<int, kH>{});
                                    s0 += kH;
                                }
                            }
                            const int64_t rl = tile * 32 + l;
                            if (mine && rl < P.B.n) {
                                float4* yp = reinterpret_cast<float4*>(y + rl * R + r0 + rr);
#pragma unroll
                                for (int q = 0; q < NQ; ++q) {
                                    if (accumulate) {
                                        const float4 yv = yp[q];
                                        if (ycoef) {
                                            const float4 ca = *reinterpret_cast<const float4*>(ycoef + r0 + rr + 4 * q);
                                            const float4 cb =
                                                *reinterpret_cast<const float4*>(ycoef + r0 + rr + 4 * q + 2);
                                            ff2_fma(acc[2 * q], pk2(ca.x, ca.z), pk2(-ca.x, -ca.z), pk2(ca.y, ca.w),
                                                    pk2(yv.x, yv.y));
                                            ff2_fma(acc[2 * q + 1], pk2(cb.x, cb.z), pk2(-cb.x, -cb.z),
                                                    pk2(cb.y, cb.w), pk2(yv.z, yv.w));
                                        } else {
                                            const uint64_t one = pk2(1.0f, 1.0f), mone = pk2(-1.0f, -1.0f),
                                                           zero = pk2(0.f, 0.f);
                                            ff2_fma(acc[2 * q], one, mone, zero, pk2(yv.x, yv.y));
                                            ff2_fma(acc[2 * q + 1], one, mone, zero, pk2(yv.z, yv.w));
                                        }
                                    }
                                    const float2 a = unpk2(add2(acc[2 * q].hi, acc[2 * q].lo)),
                                                 b = unpk2(add2(acc[2 * q + 1].hi, acc[2 * q + 1].lo));
                                    yp[q] = make_float4(a.x, a.y, b.x, b.y);
                                }
                            }
                        }
                    }
                } else {
                for (int r0 = 0; r0 < R; r0 += 32 * KM) {
                    int l = row_start;
                    int lend = __shfl_sync(0xffffffffu, base + pc, l);
                    FF acc[KM];
                    auto start_row = [&](int rr_l) {
                        const int64_t rl = tile * 32 + rr_l;
                        const float2 dd = (rl < P.B.n) ? P.diag_ff[rl] : make_float2(0.f, 0.f);
#pragma unroll
                        for (int m = 0; m < KM; ++m) {
                            const int rr = r0 + lane + 32 * m;
                            acc[m] = FF{0.f, 0.f};
                            if (rr < R && rl < P.B.n) ff_fma(acc[m], dd.x, dd.y, (float)x[rl * R + rr]);
                        }
                    };
                    auto finish_row = [&](int rr_l) {
                        const int64_t rl = tile * 32 + rr_l;
                        if (rl >= P.B.n) return;
#pragma unroll
                        for (int m = 0; m < KM; ++m) {
                            const int rr = r0 + lane + 32 * m;
                            if (rr < R) {
                                if (accumulate) {
                                    const float2 c = ycoef ? ycoef[rr] : make_float2(1.0f, 0.0f);
                                    ff_fma(acc[m], c.x, c.y, (float)y[rl * R + rr]);
                                }
                                y[rl * R + rr] = (XT)(acc[m].hi + acc[m].lo);
                            }
                        }
                    };
                    start_row(l);
                    for (int k0 = kbeg; k0 < kend; k0 += kU) {
                        float xv[kU][KM];
                        float2 ck[kU];
#pragma unroll
                        for (int u = 0; u < kU; ++u) {
                            const uint32_t J = (k0 + u < kend) ? hJ[k0 + u] : kEmpty;
                            ck[u] = (J == kEmpty) ? make_float2(0.f, 0.f) : hcf[k0 + u];
#pragma unroll
                            for (int m = 0; m < KM; ++m) {
                                const int rr = r0 + lane + 32 * m;
                                xv[u][m] = (J != kEmpty && rr < R) ? (float)x[(int64_t)J * R + rr] : 0.f;
                            }
                        }
#pragma unroll
                        for (int u = 0; u < kU; ++u) {
                            const int k = k0 + u;
                            if (k >= kend) break;
                            while (k >= lend) {  // rows whose hits are complete
                                finish_row(l);
                                ++l;
                                lend = __shfl_sync(0xffffffffu, base + pc, l);
                                start_row(l);
                            }
#pragma unroll
                            for (int m = 0; m < KM; ++m) ff_fma(acc[m], ck[u].x, ck[u].y, tol_select(xv[u][m], false));
                        }
                    }
                    finish_row(l);
                    for (++l; l <= last; ++l) {  // trailing rows without hits
                        start_row(l);
                        finish_row(l);
                    }
                }
                }
            } else {
            for (int l = row_start; l < row_end; ++l) {
                const int b0 = __shfl_sync(0xffffffffu, base, l);
                const int nl = __shfl_sync(0xffffffffu, cnt, l);
                const double dl = __shfl_sync(0xffffffffu, d, l);
                const uint64_t sl0 = __shfl_sync(0xffffffffu, s.x, l), sl1 = __shfl_sync(0xffffffffu, s.y, l);
                const int64_t rl = tile * 32 + l;
                if (rl >= P.B.n) break;
                for (int r0 = 0; r0 < R; r0 += 32 * KM) {
                    {
                        double acc[KM];
#pragma unroll
                        for (int m = 0; m < KM; ++m) {
                            const int rr = r0 + lane + 32 * m;
                            acc[m] = (rr < R) ? (kFam ? fam_diag(P, sl0, sl1, rr) : dl) * (double)x[rl * R + rr] : 0.0;
                        }
                        for (int k = b0; k < b0 + nl; k += 4) {
                            XT xv[4][KM];
                            double ck[4];
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                const uint32_t J = (k + u < b0 + nl) ? hJ[k + u] : kEmpty;
                                ck[u] = (J == kEmpty) ? 0.0 : hc[k + u];
#pragma unroll
                                for (int m = 0; m < KM; ++m) {
                                    const int rr = r0 + lane + 32 * m;
                                    xv[u][m] = (J != kEmpty && rr < R) ? x[(int64_t)J * R + rr] : (XT)0;
                                }
                            }
#pragma unroll
                            for (int u = 0; u < 4; ++u)
#pragma unroll
                                for (int m = 0; m < KM; ++m)
                                    if (above_tol(xv[u][m]))
                                        acc[m] += (kFam ? fam_coef(P, ck[u], r0 + lane + 32 * m) : ck[u]) * (double)xv[u][m];
                        }
#pragma unroll
                        for (int m = 0; m < KM; ++m) {
                            const int rr = r0 + lane + 32 * m;
                            if (rr < R) {
                                double v = acc[m];
                                if (accumulate) v += (double)y[rl * R + rr];
                                y[rl * R + rr] = (XT)v;
                            }
                        }
                    }
                }
            }
            }
            __syncwarp();
            row_start = row_end;
        }
    }
}

template <typename XT, class LK, bool kFF, int KM, bool kFam = false>
__global__ void __launch_bounds__(256, KM <= kVec4 ? 2 : 3) k_apply_tile_batched(TileParams P, LK lk, const XT* __restrict__ x,
                                                            XT* __restrict__ y, int R, int accumulate, int cap) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    batched_body<XT, LK, kFF, KM, kFam>(P, lk, x, y, R, accumulate, cap, blockIdx.x, gridDim.x, smem_raw);
}

// Several operators (sectors) in one launch: the grid is partitioned into
// per-sector block ranges in proportion to each sector's rows x vectors;
// each block stages its own sector's terms and works through that sector's
// tiles.  FP32 storage, double-float accumulation; the lookup caches when every
// sector is materialised, else hash lookups when every sector's batched applies
// use them, else bucket-table lookups.
struct SectorLaunch {
    TileParams P;
    HashView H;
    CacheView C;
    const float* x;
    float* y;
    const float2* ycoef;  // accumulating launches: y <- H x + ycoef[c] y per column (nullptr: coefficient 1)
    int R;
    int cap;
    int block_begin;
    int n_blocks;
};

template <int KM, class LK>
__global__ void __launch_bounds__(256, KM <= kVec4 ? 2 : 3) k_apply_sectors(const SectorLaunch* __restrict__ secs, int n_secs,
                                                          int accumulate) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ SectorLaunch L;
    if (threadIdx.x == 0) {
        int s = 0;
        while (s + 1 < n_secs && (int)blockIdx.x >= secs[s + 1].block_begin) ++s;
        L = secs[s];
    }
    __syncthreads();
    LK lk;
    if constexpr (std::is_same<LK, LookupHash>::value) lk = LookupHash{L.H};
    else if constexpr (std::is_same<LK, LookupCache>::value) lk = LookupCache{L.C};
    else lk = LookupTable{L.P.B};
    batched_body<float, LK, true, KM>(L.P, lk, L.x, L.y, L.R, accumulate, L.cap, (int64_t)blockIdx.x - L.block_begin,
                                      L.n_blocks, smem_raw, L.ycoef);
}

// Per-row diagonal, evaluated once per operator with the same arithmetic as
// diag_value in the row kernels.
__global__ void k_diag_precompute(BasisView B, DiagSpec D, const PushTerm* __restrict__ dgen, double* __restrict__ out,
                                  float2* __restrict__ out_ff) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < B.n; i += (int64_t)gridDim.x * blockDim.x) {
        const state2 s = B.states[i];
        const double d = diag_value(D, dgen, s.x, s.y);
        out[i] = d;
        const float h = (float)d;
        out_ff[i] = make_float2(h, (float)(d - (double)h));
    }
}

qsi_status build_diag(qsi_op* op) {
    cudaStream_t st = op->stream;
    QSI_CUDA(cudaMallocAsync(&op->d_diag, (size_t)op->basis->n * sizeof(double), st));
    QSI_CUDA(cudaMallocAsync(&op->d_diag_ff, (size_t)op->basis->n * sizeof(float2), st));
    k_diag_precompute<<<grid_for(op->basis->n, 256), 256, 0, st>>>(op->basis->view(), op->diag, op->d_diag_generic,
                                                                    op->d_diag, op->d_diag_ff);
    QSI_CUDA(cudaGetLastError());
    QSI_CUDA(cudaStreamSynchronize(st));
    return QSI_OK;
}

// ------------------------------------------------------------------ hash index build
__global__ void k_hash_clear(HashSlot* slots, uint64_t n_slots) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_slots; i += (uint64_t)gridDim.x * blockDim.x) {
        slots[i].lo = 0;
        slots[i].hi = 0;
        slots[i].idx = kEmpty;
    }
}

__global__ void k_hash_insert(const state2* __restrict__ states, int64_t n, HashView H, HashSlot* slots,
                              int* overflow) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const state2 s = states[i];
        const HashSlot* creg;
        const uint64_t cap = hash_region(H, s.x, s.y, creg);
        HashSlot* reg = slots + (creg - H.slots);
        uint64_t off = cap ? region_first(s.x, s.y, cap) : 0;
        bool done = false;
        for (uint64_t probe = 0; probe < cap; ++probe) {
            if (atomicCAS(&reg[off].idx, kEmpty, (uint32_t)i) == kEmpty) {
                reg[off].lo = s.x;
                reg[off].hi = (uint32_t)s.y;
                done = true;
                break;
            }
            off = (off + 1 == cap) ? 0 : off + 1;
        }
        if (!done) atomicOr(overflow, 1);
    }
}

// The regional hash index over the basis's current bucket table (built again whenever the table is): 2n slots.
qsi_status build_hash(qsi_basis* b) {
    if (b->hb >= 96) return fail(QSI_INVALID_ARG, "hash index needs states of at most 96 bits");
    if (b->n >= ((int64_t)1 << 31)) return fail(QSI_INVALID_ARG, "hash index needs fewer than 2^31 states");
    const uint64_t n_slots = 2 * (uint64_t)b->n;
    if (!b->d_hash || b->hash_slots != n_slots) {
        if (b->d_hash) cudaFree(b->d_hash);
        b->d_hash = nullptr;
        b->hash_slots = 0;
        QSI_CUDA(cudaMalloc(&b->d_hash, n_slots * sizeof(HashSlot)));
        b->hash_slots = n_slots;
    }
    int* d_over = nullptr;
    QSI_CUDA(cudaMalloc(&d_over, sizeof(int)));
    QSI_CUDA(cudaMemset(d_over, 0, sizeof(int)));
    k_hash_clear<<<grid_for((int64_t)n_slots, 256), 256>>>(b->d_hash, n_slots);
    k_hash_insert<<<grid_for(b->n, 256), 256>>>(b->d_states, b->n, b->hview(), b->d_hash, d_over);
    int over = 0;
    cudaError_t e = cudaMemcpy(&over, d_over, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d_over);
    if (e != cudaSuccess) return fail(QSI_CUDA_ERROR, "hash build: %s", cudaGetErrorString(e));
    if (over) return fail(QSI_CUDA_ERROR, "hash build: a state found no slot in its region");
    return QSI_OK;
}

// ------------------------------------------------------------------ lookup cache (materialised operator)
// Single-vector apply of a materialised operator: a sliced-ELL product over the cache alone (no states, no
// admission test): lane l of tile t sums row 32 t + l as the diagonal, then its entries in cache order (the
// admission order of the tile kernels) with coefficient +-cs of the entry's term and the entry's sign, the same
// sums in the same order as k_apply_tile, so the result is bitwise the matrix-free one.
template <typename XT, typename YT, typename TT>
__global__ void __launch_bounds__(256) k_apply_cached(const PullTerm* __restrict__ terms, int n_off,
                                                      const double* __restrict__ diag, CacheView C,
                                                      const TT* __restrict__ tids, int64_t n, const XT* __restrict__ x,
                                                      YT* __restrict__ y, int accumulate) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* cs = reinterpret_cast<double*>(smem_raw);
    for (int k = threadIdx.x; k < n_off; k += blockDim.x) cs[k] = terms[k].cs;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int64_t ntiles = (n + 31) >> 5;
    for (int64_t tile = (int64_t)blockIdx.x * nw + wid; tile < ntiles; tile += (int64_t)gridDim.x * nw) {
        const int64_t row = tile * 32 + lane;
        const bool valid = row < n;
        const uint64_t o0 = C.off[tile];
        const int width = (int)(C.off[tile + 1] - o0);
        double acc = valid ? diag[row] * (double)x[row] : 0.0;
        const uint32_t* cp = C.cols + o0 * 32 + lane;
        const TT* tp = tids + o0 * 32 + lane;
        constexpr int kU = 8;  // entries in flight per lane
        for (int k0 = 0; k0 < width; k0 += kU) {
            uint32_t c[kU];
            TT t[kU];
            XT xv[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const bool in = k0 + u < width;
                c[u] = in ? __ldg(cp + (uint64_t)(k0 + u) * 32) : kEmpty;
                t[u] = in ? __ldg(tp + (uint64_t)(k0 + u) * 32) : (TT)0;
            }
#pragma unroll
            for (int u = 0; u < kU; ++u) xv[u] = (c[u] != kEmpty) ? x[c[u] & ~kCacheNeg] : (XT)0;
#pragma unroll
            for (int u = 0; u < kU; ++u)
                if (c[u] != kEmpty && above_tol(xv[u])) {
                    // -cs for a negative entry as a flip of the sign bit (integer work, exactly the negation), so
                    // the FP64 pipe, GB300's bottleneck here, sees one multiply-add per hit
                    const double v = __longlong_as_double(__double_as_longlong(cs[t[u]]) ^
                                                          ((unsigned long long)(c[u] & kCacheNeg) << 32));
                    acc += v * (double)xv[u];
                }
        }
        if (valid) {
            if (accumulate) acc += (double)y[row];
            y[row] = (YT)acc;
        }
    }
}

static qsi_status launch_cached(qsi_op* op, const void* x, void* y, int xdtype, int ydtype, int accumulate,
                                cudaStream_t st) {
    const int64_t n = op->basis->n;
    const int block = 256, nw = block / 32;
    const int64_t ntiles = (n + 31) / 32;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int bps = op->tune[0].grid_bps > 0 ? op->tune[0].grid_bps : 8;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((ntiles + nw - 1) / nw, (int64_t)sms * bps));
    const size_t smem = (size_t)std::max(op->n_pull, 1) * 8;
    const CacheView C{op->d_cache_cols, op->d_cache_off};
    auto go = [&](auto xt, auto yt, auto tt) {
        using XT = decltype(xt);
        using YT = decltype(yt);
        using TT = decltype(tt);
        auto k = k_apply_cached<XT, YT, TT>;
        if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<grid, block, smem, st>>>(op->d_pull, op->n_pull, op->d_diag, C, (const TT*)op->d_cache_tid, n,
                                     (const XT*)x, (YT*)y, accumulate);
    };
    auto by_tid = [&](auto xt, auto yt) {
        if (op->cache_tid_bytes == 1) go(xt, yt, uint8_t{});
        else go(xt, yt, uint16_t{});
    };
    if (xdtype == QSI_F64) by_tid(double{}, double{});
    else if (ydtype == QSI_F64) by_tid(float{}, double{});
    else by_tid(float{}, float{});
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(QSI_CUDA_ERROR, "cached apply launch: %s", cudaGetErrorString(e));
    return QSI_OK;
}


// Admitted terms of the tile's widest row: the tile's number of cache lines.
__global__ void __launch_bounds__(256) k_cache_widths(TileParams P, uint64_t* __restrict__ width) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const TileSmem S = stage_terms(P, smem_raw);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int n_rounds = (P.n_off + 31) >> 5;
    uint32_t* spinw = reinterpret_cast<uint32_t*>(S.tail) + wid * 128;
    const int64_t ntiles = (P.B.n + 31) >> 5;
    for (int64_t tile = (int64_t)blockIdx.x * nw + wid; tile < ntiles; tile += (int64_t)gridDim.x * nw) {
        const int64_t row = tile * 32 + lane;
        const bool valid = row < P.B.n;
        const state2 s = valid ? P.B.states[row] : make_ulonglong2(0, 0);
        const uint32_t vmask = __ballot_sync(0xffffffffu, valid);
        tile_spin_words(s, P.nwords, lane, spinw);
        int cnt = 0;
        for (int r = 0; r < n_rounds; ++r) cnt += __popc(tile_admitted(S, P.n_off, r * 32, lane, vmask, spinw));
#pragma unroll
        for (int o = 16; o; o >>= 1) cnt = max(cnt, __shfl_xor_sync(0xffffffffu, cnt, o));
        if (lane == 0) width[tile] = (uint64_t)cnt;
        __syncwarp();
    }
}

// The column of every admitted term of every row (kEmpty outside the basis), looked up with lk, at the positions
// LookupCache reads them from.
template <class LK, typename TT>
__global__ void __launch_bounds__(256) k_cache_fill(TileParams P, LK lk, const uint64_t* __restrict__ off,
                                                    uint32_t* __restrict__ cols, TT* __restrict__ tids) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const TileSmem S = stage_terms(P, smem_raw);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int n_rounds = (P.n_off + 31) >> 5;
    uint32_t* spinw = reinterpret_cast<uint32_t*>(S.tail) + wid * (128 + 32 * n_rounds);
    uint32_t* adm = spinw + 128;
    const int64_t ntiles = (P.B.n + 31) >> 5;
    for (int64_t tile = (int64_t)blockIdx.x * nw + wid; tile < ntiles; tile += (int64_t)gridDim.x * nw) {
        const int64_t row = tile * 32 + lane;
        const bool valid = row < P.B.n;
        const state2 s = valid ? P.B.states[row] : make_ulonglong2(0, 0);
        const uint32_t vmask = __ballot_sync(0xffffffffu, valid);
        tile_spin_words(s, P.nwords, lane, spinw);
        for (int r = 0; r < n_rounds; ++r) adm[r * 32 + lane] = tile_admitted(S, P.n_off, r * 32, lane, vmask, spinw);
        uint32_t* out = cols + off[tile] * 32 + lane;
        TT* tout = tids + off[tile] * 32 + lane;
        int kk = 0, r = 0;
        uint32_t a = adm[lane];
        while (true) {
            constexpr int kNB = 4;
            int tt[kNB];
            uint64_t tl[kNB], th[kNB];
            int64_t J[kNB];
            int nh = 0;
#pragma unroll
            for (int u = 0; u < kNB; ++u) {
                tt[u] = 0;
                tl[u] = th[u] = 0;
                while (!a && r + 1 < n_rounds) a = adm[++r * 32 + lane];
                if (a) {
                    tt[u] = r * 32 + __ffs(a) - 1;
                    const PullTerm& T = S.terms[tt[u]];
                    a &= a - 1;
                    tl[u] = s.x ^ T.x0;
                    th[u] = s.y ^ T.x1;
                    ++nh;
                }
            }
            if (!nh) break;
            lk.template find_batch<kNB>(tl, th, J, nh);
#pragma unroll
            for (int u = 0; u < kNB; ++u)
                if (u < nh) {
                    // the column, with the sign of the term's matrix element on this row in the top bit
                    const PullTerm& T = S.terms[tt[u]];
                    const bool neg = T.has_z && ((__popcll(~s.x & T.z0) + __popcll(~s.y & T.z1)) & 1);
                    out[(uint64_t)(kk + u) * 32] = (J[u] < 0) ? kEmpty : ((uint32_t)J[u] | (neg ? kCacheNeg : 0u));
                    tout[(uint64_t)(kk + u) * 32] = (TT)tt[u];
                }
            kk += nh;
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ launchers
static size_t term_smem(const qsi_op* op) {
    size_t used = (size_t)op->n_pull * sizeof(PullTerm) + (size_t)op->n_diag_generic * sizeof(PushTerm) +
                  (size_t)(op->n_pull + 1) * 2 + (size_t)op->n_lits;
    return (used + 15) & ~(size_t)15;
}

template <class K>
static void set_smem(K kernel, size_t smem) {
    if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// Grid of one wave (the blocks that fit on the GPU at once, each working through tiles with a grid
// stride) or of bps blocks per SM when bps > 0; at most one block per 8 tiles.
template <class K>
static int one_wave(K kernel, int block, size_t smem, int64_t ntiles, int bps = 0) {
    int dev = 0, sms = 148, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (bps > 0) per_sm = bps;
    else if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return (int)std::max<int64_t>(1, std::min<int64_t>((ntiles + block / 32 - 1) / (block / 32), (int64_t)sms * per_sm));
}

template <class LK>
static qsi_status launch_tiles_lk(qsi_op* op, LK lk, const void* x, void* y, int R, int xdtype, int ydtype,
                                  int accumulate, cudaStream_t st) {
    const qsi_tuning& T = op->tune[R > 1];
    TileParams P{op->basis->view(), op->d_pull, op->d_lit_off, op->d_lits, op->d_diag_generic, op->diag,
                 op->d_diag, op->d_diag_ff, op->n_pull, op->n_lits, op->nwords, T.vec_chunk};
    const int block = 256, nw = block / 32;
    const int64_t ntiles = (P.B.n + 31) / 32;
    if (R == 1) {
        // several waves of blocks: measured faster than one wave for the single-vector kernel
        const size_t smem = term_smem(op) + (size_t)nw * (512 + (size_t)(op->n_pull + 31) / 32 * 128);
        int dev = 0, sms = 148;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int grid = (int)std::max<int64_t>(
            1, std::min<int64_t>((ntiles + nw - 1) / nw, (int64_t)sms * (T.grid_bps > 0 ? T.grid_bps : 8)));
        if (xdtype == QSI_F64) {
            auto k = k_apply_tile<double, double, LK>;
            set_smem(k, smem);
            k<<<grid, block, smem, st>>>(P, lk, (const double*)x, (double*)y, accumulate);
        } else if (ydtype == QSI_F64) {
            auto k = k_apply_tile<float, double, LK>;
            set_smem(k, smem);
            k<<<grid, block, smem, st>>>(P, lk, (const float*)x, (double*)y, accumulate);
        } else {
            auto k = k_apply_tile<float, float, LK>;
            set_smem(k, smem);
            k<<<grid, block, smem, st>>>(P, lk, (const float*)x, (float*)y, accumulate);
        }
    } else {
        const int cap = (std::max(T.list_cap, op->n_pull + 1) + 7) & ~7;  // a row: diagonal + terms, padded to 8
        const int n_rounds = (op->n_pull + 31) / 32;
        const size_t per_warp = 512 + (size_t)n_rounds * 128 + (size_t)cap * 12;
        const size_t smem = term_smem(op) + (size_t)nw * per_warp;
        if (smem > 227 * 1024) return fail(QSI_INVALID_ARG, "batched apply: %zu bytes of shared memory needed", smem);
        auto go = [&](auto km) -> void {
            constexpr int KM = decltype(km)::value;
            if (xdtype == QSI_F64) {
                auto k = k_apply_tile_batched<double, LK, false, KM>;
                set_smem(k, smem);
                k<<<one_wave(k, block, smem, ntiles, T.grid_bps), block, smem, st>>>(P, lk, (const double*)x, (double*)y, R,
                                                                         accumulate, cap);
            } else if (op->ff_accumulate) {
                auto k = (T.vec_width == 16 && vec16_ok(P.B.n, R, x, y)) ? k_apply_tile_batched<float, LK, true, kVec16>
                         : (T.vec_width == 8 && vec8_ok(P.B.n, R, x, y))  ? k_apply_tile_batched<float, LK, true, kVec8>
                         : vec4_ok(P.B.n, R, x, y)                        ? k_apply_tile_batched<float, LK, true, kVec4>
                                                                          : k_apply_tile_batched<float, LK, true, KM>;
                set_smem(k, smem);
                k<<<one_wave(k, block, smem, ntiles, T.grid_bps), block, smem, st>>>(P, lk, (const float*)x, (float*)y, R,
                                                                         accumulate, cap);
            } else {
                auto k = k_apply_tile_batched<float, LK, false, KM>;
                set_smem(k, smem);
                k<<<one_wave(k, block, smem, ntiles, T.grid_bps), block, smem, st>>>(P, lk, (const float*)x, (float*)y, R,
                                                                         accumulate, cap);
            }
        };
        if (R <= 32) go(std::integral_constant<int, 1>{});
        else if (R <= 64) go(std::integral_constant<int, 2>{});
        else go(std::integral_constant<int, 4>{});
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(QSI_CUDA_ERROR, "tile apply launch: %s", cudaGetErrorString(e));
    return QSI_OK;
}

// Several sectors in one launch (FP32 batched, double-float), in two steps: plan_sectors builds the per-sector
// launch records on the host (block ranges in proportion to weights, e.g. each sector's measured apply time, or
// else to rows x vectors; shared memory for the largest sector); the caller copies plan.records to device memory once, and launch_sectors enqueues the
// kernel (capturable into a CUDA graph: it does no host-to-device copy).
qsi_status plan_sectors(qsi_op* const* ops, int n, const float* const* X, float* const* Y, const int* R,
                        SectorPlan& plan, const double* weights, const float2* const* ycoef) {
    std::vector<SectorLaunch> L(n);
    plan.vec4 = true;
    plan.vec8 = true;
    plan.vec16 = true;
    plan.hash = true;
    plan.cache = true;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int nw = 8;
    size_t smem = 0;
    int maxR = 1;
    double work_total = 0;
    for (int s = 0; s < n; ++s) {
        qsi_op* op = ops[s];
        if (op->kernel != 1) return fail(QSI_INVALID_ARG, "sector launch needs the tile kernels");
        plan.hash = plan.hash && op->basis->d_hash && op->tune[1].use_hash;
        plan.cache = plan.cache && op->d_cache_cols;
        const int cap = (std::max(op->tune[1].list_cap, op->n_pull + 1) + 7) & ~7;  // a row: diagonal + terms
        const int n_rounds = (op->n_pull + 31) / 32;
        smem = std::max(smem, term_smem(op) + (size_t)nw * (512 + (size_t)n_rounds * 128 + (size_t)cap * 12));
        L[s].P = TileParams{op->basis->view(), op->d_pull, op->d_lit_off, op->d_lits, op->d_diag_generic, op->diag,
                            op->d_diag, op->d_diag_ff, op->n_pull, op->n_lits, op->nwords, op->tune[1].vec_chunk};
        L[s].H = op->basis->hview();
        L[s].C = CacheView{op->d_cache_cols, op->d_cache_off};
        L[s].x = X[s];
        L[s].y = Y[s];
        L[s].ycoef = ycoef ? ycoef[s] : nullptr;
        L[s].R = R[s];
        L[s].cap = cap;
        maxR = std::max(maxR, R[s]);
        plan.vec4 = plan.vec4 && vec4_ok(op->basis->n, R[s], X[s], Y[s]);
        plan.vec8 = plan.vec8 && op->tune[1].vec_width == 8 && vec8_ok(op->basis->n, R[s], X[s], Y[s]);
        plan.vec16 = plan.vec16 && op->tune[1].vec_width == 16 && vec16_ok(op->basis->n, R[s], X[s], Y[s]);
        work_total += weights ? weights[s] : (double)op->basis->n * R[s];
    }
    if (smem > 227 * 1024) return fail(QSI_INVALID_ARG, "sector launch: %zu bytes of shared memory needed", smem);
    // one wave of the kernel's resident blocks per SM, or the first sector's tuned blocks per SM
    const int bps = ops[0]->tune[1].grid_bps;
    const int total = sms * (bps > 0 ? bps : plan.vec4 ? 2 : 3);
    int begin = 0;
    for (int s = 0; s < n; ++s) {
        const int64_t tiles = (ops[s]->basis->n + 31) / 32;
        const double work = weights ? weights[s] : (double)ops[s]->basis->n * R[s];
        int b = (int)std::llround(total * work / std::max(work_total, 1e-30));
        b = (int)std::max<int64_t>(1, std::min<int64_t>(b, (tiles + nw - 1) / nw));
        L[s].block_begin = begin;
        L[s].n_blocks = b;
        begin += b;
    }
    plan.records.assign((const unsigned char*)L.data(), (const unsigned char*)(L.data() + n));
    plan.smem = smem;
    plan.maxR = maxR;
    plan.grid = begin;
    plan.n = n;
    return QSI_OK;
}

qsi_status launch_sectors(const void* d_records, const SectorPlan& plan, int accumulate, cudaStream_t st) {
    auto go = [&](auto km) {
        constexpr int KM = decltype(km)::value;
        auto k = plan.cache ? k_apply_sectors<KM, LookupCache>
                 : plan.hash ? k_apply_sectors<KM, LookupHash>
                             : k_apply_sectors<KM, LookupTable>;
        set_smem(k, plan.smem);
        k<<<plan.grid, 256, plan.smem, st>>>((const SectorLaunch*)d_records, plan.n, accumulate);
    };
    if (plan.vec16) go(std::integral_constant<int, kVec16>{});
    else if (plan.vec8) go(std::integral_constant<int, kVec8>{});
    else if (plan.vec4) go(std::integral_constant<int, kVec4>{});
    else if (plan.maxR <= 32) go(std::integral_constant<int, 1>{});
    else if (plan.maxR <= 64) go(std::integral_constant<int, 2>{});
    else go(std::integral_constant<int, 4>{});
    QSI_CUDA(cudaGetLastError());
    return QSI_OK;
}

size_t sector_launch_bytes() { return sizeof(SectorLaunch); }

qsi_status preload_apply_f64_rows();  // operator.cu: the row-per-thread kernel

qsi_status preload_apply_f64() {
    cudaFuncAttributes a;
    QSI_CUDA(cudaFuncGetAttributes(&a, k_apply_tile<double, double, LookupHash>));
    QSI_CUDA(cudaFuncGetAttributes(&a, k_apply_tile<double, double, LookupTable>));
    return preload_apply_f64_rows();
}

// Family mode applies of the template operator tmpl: y = H(p_c) x per column c (FP64, [row][R]), fcoef
// [classes][R] on the device.  One column runs the single-vector tile kernel, several the batched one; both sum a
// row in the same order, so a column's result does not depend on R.
template <class LK>
static qsi_status launch_family_lk(qsi_op* tmpl, LK lk, const double* x, double* y, int R, const double* fcoef,
                                   int accumulate, cudaStream_t st) {
    const qsi_tuning& T = tmpl->tune[0];
    TileParams P{tmpl->basis->view(), tmpl->d_pull, tmpl->d_lit_off, tmpl->d_lits, tmpl->d_diag_generic, tmpl->diag,
                 tmpl->d_diag, tmpl->d_diag_ff, tmpl->n_pull, tmpl->n_lits, tmpl->nwords, 0, fcoef, R};
    const int block = 256, nw = block / 32;
    const int64_t ntiles = (P.B.n + 31) / 32;
    if (R == 1) {
        const size_t smem = term_smem(tmpl) + (size_t)nw * (512 + (size_t)(tmpl->n_pull + 31) / 32 * 128);
        int dev = 0, sms = 148;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int grid = (int)std::max<int64_t>(
            1, std::min<int64_t>((ntiles + nw - 1) / nw, (int64_t)sms * (T.grid_bps > 0 ? T.grid_bps : 8)));
        auto k = k_apply_tile<double, double, LK, true>;
        set_smem(k, smem);
        k<<<grid, block, smem, st>>>(P, lk, x, y, accumulate);
    } else if (R <= 8) {  // a few columns: every lane sums all columns of its row
        const size_t smem = term_smem(tmpl) + (size_t)nw * (512 + (size_t)(tmpl->n_pull + 31) / 32 * 128);
        int dev = 0, sms = 148;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((ntiles + nw - 1) / nw, (int64_t)sms * 8));
        auto k = (R <= 2) ? k_apply_tile_cols<LK, 2> : (R <= 4) ? k_apply_tile_cols<LK, 4> : k_apply_tile_cols<LK, 8>;
        set_smem(k, smem);
        k<<<grid, block, smem, st>>>(P, lk, x, y, accumulate);
    } else {
        const int cap = (std::max(tmpl->tune[1].list_cap, tmpl->n_pull + 1) + 7) & ~7;
        const int n_rounds = (tmpl->n_pull + 31) / 32;
        const size_t smem = term_smem(tmpl) + (size_t)nw * (512 + (size_t)n_rounds * 128 + (size_t)cap * 12);
        if (smem > 227 * 1024) return fail(QSI_INVALID_ARG, "family apply: %zu bytes of shared memory needed", smem);
        auto go = [&](auto km) {
            constexpr int KM = decltype(km)::value;
            auto k = k_apply_tile_batched<double, LK, false, KM, true>;
            set_smem(k, smem);
            k<<<one_wave(k, block, smem, ntiles, tmpl->tune[1].grid_bps), block, smem, st>>>(P, lk, x, y, R, accumulate,
                                                                                             cap);
        };
        if (R <= 32) go(std::integral_constant<int, 1>{});
        else if (R <= 64) go(std::integral_constant<int, 2>{});
        else go(std::integral_constant<int, 4>{});
    }
    QSI_CUDA(cudaGetLastError());
    return QSI_OK;
}

qsi_status launch_family(qsi_op* tmpl, const double* x, double* y, int R, const double* fcoef, int accumulate,
                         cudaStream_t st) {
    if (R < 1 || R > 128) return fail(QSI_INVALID_ARG, "family apply: %d columns (1..128)", R);
    if (tmpl->basis->d_hash && tmpl->tune[R > 1].use_hash)
        return launch_family_lk(tmpl, LookupHash{tmpl->basis->hview()}, x, y, R, fcoef, accumulate, st);
    return launch_family_lk(tmpl, LookupTable{tmpl->basis->view()}, x, y, R, fcoef, accumulate, st);
}

qsi_status launch_apply_tiles(qsi_op* op, const void* x, void* y, int R, int xdtype, int ydtype, int accumulate,
                              cudaStream_t st) {
    if (op->d_cache_cols) {
        if (R == 1) return launch_cached(op, x, y, xdtype, ydtype, accumulate, st);
        return launch_tiles_lk(op, LookupCache{CacheView{op->d_cache_cols, op->d_cache_off}}, x, y, R, xdtype, ydtype,
                               accumulate, st);
    }
    if (op->basis->d_hash && op->tune[R > 1].use_hash) return launch_tiles_lk(op, LookupHash{op->basis->hview()}, x, y, R, xdtype, ydtype, accumulate, st);
    return launch_tiles_lk(op, LookupTable{op->basis->view()}, x, y, R, xdtype, ydtype, accumulate, st);
}

// Builds (enable) or frees the operator's lookup cache; *bytes: its size.
qsi_status materialise(qsi_op* op, bool enable, int64_t* bytes) {
    cudaFree(op->d_cache_cols);
    cudaFree(op->d_cache_off);
    cudaFree(op->d_cache_tid);
    op->d_cache_cols = nullptr;
    op->d_cache_off = nullptr;
    op->d_cache_tid = nullptr;
    op->cache_entries = 0;
    if (enable) {
        if (op->kernel != 1) return fail(QSI_INVALID_ARG, "qsi_op_materialise: the cache serves the tile kernels (kernel 1)");
        cudaStream_t st = op->stream;
        const int64_t ntiles = (op->basis->n + 31) / 32;
        TileParams P{op->basis->view(), op->d_pull, op->d_lit_off, op->d_lits, op->d_diag_generic, op->diag,
                     op->d_diag, op->d_diag_ff, op->n_pull, op->n_lits, op->nwords, 0};
        const int block = 256, nw = block / 32;
        const int n_rounds = (op->n_pull + 31) / 32;
        int dev = 0, sms = 148;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((ntiles + nw - 1) / nw, (int64_t)sms * 8));
        // widths, their exclusive scan (tile offsets in cache lines), then the columns
        // the scratch arrays are freed, and a failure leaves no partial cache behind, on every path out
        uint64_t* width = nullptr;
        void* tmp = nullptr;
        auto scratch_free = [&]() {
            cudaFreeAsync(tmp, st);
            cudaFreeAsync(width, st);
            tmp = nullptr;
            width = nullptr;
        };
        auto fail_partial = [&](cudaError_t e, const char* what) {
            scratch_free();
            cudaFree(op->d_cache_off);
            op->d_cache_off = nullptr;
            return fail(e == cudaErrorMemoryAllocation ? QSI_OOM : QSI_CUDA_ERROR, "qsi_op_materialise: %s: %s", what,
                        cudaGetErrorString(e));
        };
        cudaError_t e = cudaMallocAsync(&width, (size_t)(ntiles + 1) * 8, st);
        if (e == cudaSuccess) e = cudaMallocAsync(&op->d_cache_off, (size_t)(ntiles + 1) * 8, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(width + ntiles, 0, 8, st);
        if (e != cudaSuccess) return fail_partial(e, "tile offsets");
        const size_t smem_w = term_smem(op) + (size_t)nw * 512;
        set_smem(k_cache_widths, smem_w);
        k_cache_widths<<<grid, block, smem_w, st>>>(P, width);
        size_t tmp_bytes = 0;
        e = cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, width, op->d_cache_off, ntiles + 1, st);
        if (e == cudaSuccess) e = cudaMallocAsync(&tmp, tmp_bytes, st);
        if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, width, op->d_cache_off, ntiles + 1, st);
        uint64_t lines = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&lines, op->d_cache_off + ntiles, 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return fail_partial(e, "tile widths");
        scratch_free();
        const size_t n_entries = (size_t)lines * 32;
        op->cache_tid_bytes = op->n_pull <= 256 ? 1 : 2;
        e = cudaMalloc(&op->d_cache_cols, std::max<size_t>(n_entries, 1) * 4);
        if (e == cudaSuccess) e = cudaMalloc(&op->d_cache_tid, std::max<size_t>(n_entries, 1) * op->cache_tid_bytes);
        if (e != cudaSuccess) {
            cudaFree(op->d_cache_off);
            cudaFree(op->d_cache_cols);
            op->d_cache_off = nullptr;
            op->d_cache_cols = nullptr;
            op->d_cache_tid = nullptr;
            return fail(e == cudaErrorMemoryAllocation ? QSI_OOM : QSI_CUDA_ERROR,
                        "qsi_op_materialise: %zu bytes for the cache: %s", n_entries * (4 + op->cache_tid_bytes),
                        cudaGetErrorString(e));
        }
        auto drop_cache = [&](cudaError_t err) {  // a cache that was not filled completely is never used
            cudaFree(op->d_cache_cols);
            cudaFree(op->d_cache_tid);
            cudaFree(op->d_cache_off);
            op->d_cache_cols = nullptr;
            op->d_cache_tid = nullptr;
            op->d_cache_off = nullptr;
            return fail(QSI_CUDA_ERROR, "qsi_op_materialise: %s", cudaGetErrorString(err));
        };
        e = cudaMemsetAsync(op->d_cache_cols, 0xFF, n_entries * 4, st);  // the lanes below their tile's width
        if (e == cudaSuccess) e = cudaMemsetAsync(op->d_cache_tid, 0, n_entries * op->cache_tid_bytes, st);
        if (e != cudaSuccess) return drop_cache(e);
        const size_t smem_f = term_smem(op) + (size_t)nw * (512 + (size_t)n_rounds * 128);
        auto fill = [&](auto lk, auto* tids) {
            auto k = k_cache_fill<decltype(lk), std::remove_pointer_t<decltype(tids)>>;
            set_smem(k, smem_f);
            k<<<grid, block, smem_f, st>>>(P, lk, op->d_cache_off, op->d_cache_cols, tids);
        };
        if (op->basis->d_hash) {
            if (op->cache_tid_bytes == 1) fill(LookupHash{op->basis->hview()}, (uint8_t*)op->d_cache_tid);
            else fill(LookupHash{op->basis->hview()}, (uint16_t*)op->d_cache_tid);
        } else {
            if (op->cache_tid_bytes == 1) fill(LookupTable{op->basis->view()}, (uint8_t*)op->d_cache_tid);
            else fill(LookupTable{op->basis->view()}, (uint16_t*)op->d_cache_tid);
        }
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return drop_cache(e);
        op->cache_entries = n_entries;
    }
    if (bytes)
        *bytes = op->d_cache_cols ? (int64_t)(op->cache_entries * (4 + op->cache_tid_bytes) +
                                              ((op->basis->n + 31) / 32 + 1) * 8)
                                  : 0;
    return QSI_OK;
}

}  // namespace qsi
