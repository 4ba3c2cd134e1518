// Device-side data structures shared by the CUDA translation units.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "qsi_internal.h"

namespace qsi {

// A 128-bit basis state as stored in HBM: x = low word, y = high word.
using state2 = ulonglong2;

// Pull-form off-diagonal term: applicability masks are those of the
// transposed operator, so a row state s is admitted when
// (s & down) == 0 && (s & up) == up, and its column is s ^ X.
// The matrix element is cs * (-1)^popcount(~s & Z).
struct PullTerm {
    uint64_t x0, x1, z0, z1, up0, up1, dn0, dn1;
    double cs;       // coefficient times construction sign
    int32_t has_z;
    float cs_hi;     // cs as a double-float pair (cs_hi + cs_lo), for FP32 accumulation
    float cs_lo;
    int32_t pad;
};

// Push-form term (the reference's own orientation; used for connectivity
// export and for generic diagonal terms).
struct PushTerm {
    uint64_t x0, x1, z0, z1, up0, up1, dn0, dn1;
    double c;
    int32_t sign;
    int32_t pad;
};

// Diagonal part: single-site pure-z terms grouped by weight w into masks,
// contributing w * (2 * popcount(s & M) - popcount(M)); remaining diagonal
// terms are evaluated one by one.
constexpr int kMaxZClasses = 32;
struct DiagSpec {
    int n_cls;
    int n_generic;
    double w2[kMaxZClasses];  // 2*w
    uint64_t m0[kMaxZClasses], m1[kMaxZClasses];
    double constant;  // -sum_k w_k * popcount(M_k)
};

// Sorted basis with a direct bucket table over the top `bits` bits below
// `shift`: bucket(s) = s >> shift; bstart[v] .. bstart[v+1] is the index
// range of states in bucket v.
struct BasisView {
    const state2* states;
    const uint32_t* bstart;
    int64_t n;
    int shift;
    uint32_t n_buckets;
};

// Slot of the basis hash index (states of at most 96 bits): {low word, high 32 bits, position in the sorted
// basis}; idx == kEmpty marks a free slot.
struct HashSlot {
    uint64_t lo;
    uint32_t hi;
    uint32_t idx;
};
constexpr uint32_t kEmpty = 0xFFFFFFFFu;

__host__ __device__ __forceinline__ uint64_t state_mix(uint64_t lo, uint64_t hi) {
    uint64_t h = lo * 0x9E3779B97F4A7C15ULL ^ (hi + 0x632BE59BD9B4E019ULL) * 0xC2B2AE3D27D4EB4FULL;
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ULL;
    h ^= h >> 29;
    return h;
}


__device__ __forceinline__ bool less128(uint64_t alo, uint64_t ahi, uint64_t blo, uint64_t bhi) {
    return ahi < bhi || (ahi == bhi && alo < blo);
}

__device__ __forceinline__ uint64_t bucket_of(const BasisView& B, uint64_t lo, uint64_t hi, bool& in_range) {
    uint64_t v;
    if (B.shift >= 64) {
        v = hi >> (B.shift - 64);
    } else if (B.shift == 0) {
        v = lo;
        if (hi) v = ~0ULL;
    } else {
        if (hi >> B.shift) v = ~0ULL;
        else v = (hi << (64 - B.shift)) | (lo >> B.shift);
    }
    in_range = v < B.n_buckets;
    return v;
}

// Bounds [a, b) of bucket v: one 16-byte load of the aligned group of four table entries holding bstart[v]
// (the table is 16-byte aligned and padded to a multiple of four entries plus four), a second load only when v is
// the last of its group.  The apply kernels are bound by the throughput of their uncoalesced loads, so every load
// saved per lookup counts.
__device__ __forceinline__ void bucket_bounds(const BasisView& B, uint64_t v, uint32_t& a, uint32_t& b) {
    const uint4 q = __ldg(reinterpret_cast<const uint4*>(B.bstart + (v & ~3ULL)));
    switch ((int)(v & 3)) {
        case 0: a = q.x, b = q.y; break;
        case 1: a = q.y, b = q.z; break;
        case 2: a = q.z, b = q.w; break;
        default: a = q.w, b = __ldg(B.bstart + v + 1); break;
    }
}

// Exact index of state (lo, hi) in the basis, or -1.  Lower-bound bisection over the state's bucket; the state at
// the final position was loaded by the bisection itself whenever that position lies inside the bucket (the last
// probe that moved the upper end there), and a search that never moved the upper end ends past the bucket, where
// the state cannot be: no reload either way.
__device__ __forceinline__ int64_t basis_find(const BasisView& B, uint64_t lo, uint64_t hi) {
    bool ok;
    const uint64_t v = bucket_of(B, lo, hi, ok);
    if (!ok) return -1;
    uint32_t a, b;
    bucket_bounds(B, v, a, b);
    state2 e = make_ulonglong2(0, 0);
    bool seen = false;  // e holds states[b]
    while (a < b) {
        const uint32_t m = (a + b) >> 1;
        const state2 t = __ldg(B.states + m);
        if (less128(t.x, t.y, lo, hi)) {
            a = m + 1;
        } else {
            b = m;
            e = t;
            seen = true;
        }
    }
    return (seen && e.x == lo && e.y == hi) ? (int64_t)a : -1;
}

// Regional hash index of the basis: bucket v of the top-bits table owns the slots [2 bstart[v], 2 bstart[v+1])
// of a table of 2n slots.  A state's probe starts at a hash of the state scaled to its bucket's slots and
// continues linearly, wrapping inside them.  The regions keep the locality of the sorted basis (the columns of
// neighbouring rows fall in the same few regions, whose slots stay in L2), and at the fixed load factor of 1/2 a
// lookup takes about 1.5 probes whatever its bucket's size, where a bisection takes log2 of it (the buckets of
// spin-ice bases are very uneven: on the 96-spin 12.12.12.12 sector a state's 30-bit bucket holds 18.7 states on
// average).  One 16-byte load of the table gives the region, as for the bisection.
struct HashView {
    const HashSlot* slots;
    BasisView B;
};

// First probe of (lo, hi) in a region of cap slots.
__device__ __forceinline__ uint32_t region_first(uint64_t lo, uint64_t hi, uint64_t cap) {
    return (uint32_t)(((state_mix(lo, hi) >> 32) * cap) >> 32);
}

// Region of (lo, hi): its first slot and size (0: the state's bucket is empty or out of range, or the state has
// more than 96 bits, so it is not in the basis).
__device__ __forceinline__ uint64_t hash_region(const HashView& Hv, uint64_t lo, uint64_t hi, const HashSlot*& reg) {
    reg = Hv.slots;
    if (hi >> 32) return 0;
    bool ok;
    const uint64_t v = bucket_of(Hv.B, lo, hi, ok);
    if (!ok) return 0;
    uint32_t a, b;
    bucket_bounds(Hv.B, v, a, b);
    reg = Hv.slots + 2 * (uint64_t)a;
    return 2 * (uint64_t)(b - a);
}

__device__ __forceinline__ bool slot_holds(const uint4& e, uint64_t lo, uint64_t hi) {
    return e.x == (uint32_t)lo && e.y == (uint32_t)(lo >> 32) && e.z == (uint32_t)hi;
}

// Exact position of (lo, hi) through the hash index, or -1.  A region is never full (load 1/2), so the probes
// end at a free slot at the latest.
__device__ __forceinline__ int64_t hash_find(const HashView& Hv, uint64_t lo, uint64_t hi) {
    const HashSlot* reg;
    const uint64_t cap = hash_region(Hv, lo, hi, reg);
    if (!cap) return -1;
    uint64_t off = region_first(lo, hi, cap);
    for (uint64_t probe = 0; probe < cap; ++probe) {
        const uint4 e = __ldg(reinterpret_cast<const uint4*>(reg + off));
        if (e.w == kEmpty) return -1;
        if (slot_holds(e, lo, hi)) return (int64_t)e.w;
        off = (off + 1 == cap) ? 0 : off + 1;
    }
    return -1;
}

// Lookups of up to NB states at once.  The hash variant issues the first
// probe of every state before resolving any (independent loads in flight);
// further probes, needed after a collision, follow one by one.
// Every lookup class takes the states to look up and, for the materialised operator's cache, where the row's
// entries start (cursor(tile, lane), once per tile) and the admission ordinal of the batch's first term.
struct LookupTable {
    BasisView B;
    static constexpr int kNB = 4, kMinBlocks = 3;  // lookups per batch per lane, resident 256-thread blocks
    __device__ __forceinline__ int64_t find(uint64_t lo, uint64_t hi) const { return basis_find(B, lo, hi); }
    __device__ __forceinline__ uint64_t cursor(int64_t, int) const { return 0; }
    template <int NB>
    __device__ __forceinline__ void find_batch(const uint64_t* lo, const uint64_t* hi, int64_t* J, int n,
                                               uint64_t = 0, int = 0) const {
#pragma unroll
        for (int u = 0; u < NB; ++u)
            if (u < n) J[u] = basis_find(B, lo[u], hi[u]);
    }
};

struct LookupHash {
    HashView H;
    // 4 resident blocks (64 registers, a 64-byte spill): 66.9 ms against 74-75 ms at 3 (80 registers) on the
    // 96-spin sector, whose single-vector apply is bound by the latency of its dependent lookups
    static constexpr int kNB = 4, kMinBlocks = 4;
    __device__ __forceinline__ int64_t find(uint64_t lo, uint64_t hi) const { return hash_find(H, lo, hi); }
    __device__ __forceinline__ uint64_t cursor(int64_t, int) const { return 0; }
    // every state's region (one table load each), then every first probe, before resolving any
    template <int NB>
    __device__ __forceinline__ void find_batch(const uint64_t* lo, const uint64_t* hi, int64_t* J, int n,
                                               uint64_t = 0, int = 0) const {
        const HashSlot* reg[NB];
        uint32_t cap[NB], off[NB];
        uint4 e[NB];
#pragma unroll
        for (int u = 0; u < NB; ++u) {
            cap[u] = 0;
            reg[u] = H.slots;
            if (u < n) cap[u] = (uint32_t)hash_region(H, lo[u], hi[u], reg[u]);
        }
#pragma unroll
        for (int u = 0; u < NB; ++u) {
            off[u] = 0;
            e[u] = make_uint4(0, 0, 0, kEmpty);
            if (cap[u]) {
                off[u] = region_first(lo[u], hi[u], cap[u]);
                e[u] = __ldg(reinterpret_cast<const uint4*>(reg[u] + off[u]));
            }
        }
#pragma unroll
        for (int u = 0; u < NB; ++u) {
            if (u >= n) continue;
            int64_t r = -1;
            uint32_t o = off[u];
            uint4 v = e[u];
            for (uint32_t probe = 0; probe < cap[u]; ++probe) {
                if (v.w == kEmpty) break;
                if (slot_holds(v, lo[u], hi[u])) {
                    r = (int64_t)v.w;
                    break;
                }
                o = (o + 1 == cap[u]) ? 0 : o + 1;
                v = __ldg(reinterpret_cast<const uint4*>(reg[u] + o));
            }
            J[u] = r;
        }
    }
};

// The materialised operator's lookup cache (qsi_op_materialise): the column of every admitted term of every row,
// kEmpty for a column outside the basis, in the order the tile kernels visit them (with the term's index and the
// sign of its matrix element on the row beside it, for the single-vector kernel that reads only the cache).  Tile t's entries start at
// 32 * off[t]; the row in lane l has its k-th admitted term at 32 * (off[t] + k) + l, so a warp reads one
// coalesced 128-byte line per admission ordinal.  Results are those of the lookups it replaces, bit for bit.
// Bit 31 of a cached column holds the sign of the term's matrix element on that row (columns are below 2^31).
constexpr uint32_t kCacheNeg = 0x80000000u;
struct CacheView {
    const uint32_t* cols;
    const uint64_t* off;
};
struct LookupCache {
    CacheView C;
    static constexpr int kNB = 8, kMinBlocks = 3;
    __device__ __forceinline__ uint64_t cursor(int64_t tile, int lane) const { return C.off[tile] * 32 + lane; }
    template <int NB>
    __device__ __forceinline__ void find_batch(const uint64_t*, const uint64_t*, int64_t* J, int n, uint64_t cur,
                                               int k0) const {
#pragma unroll
        for (int u = 0; u < NB; ++u)
            if (u < n) {
                const uint32_t c = __ldg(C.cols + cur + (uint64_t)(k0 + u) * 32);
                J[u] = (c == kEmpty) ? -1 : (int64_t)(c & ~kCacheNeg);
            }
    }
};

// 32x32 bit-matrix transpose across a warp: lane r holds row r (bit c = [r][c]);
// on return lane r holds column r (bit c = [c][r]).  Five shuffle stages,
// each swapping the off-diagonal j x j blocks.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t w, int lane) {
    const uint32_t m0[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const int j = 16 >> k;
        const uint32_t m = m0[k];
        const uint32_t x = __shfl_xor_sync(0xffffffffu, w, j);
        w = (lane & j) ? ((w & ~m) | ((x & ~m) >> j)) : ((w & m) | ((x & m) << j));
    }
    return w;
}

__device__ __forceinline__ double diag_value(const DiagSpec& D, const PushTerm* gen, uint64_t s0, uint64_t s1) {
    double d = D.constant;
    for (int k = 0; k < D.n_cls; ++k) d += D.w2[k] * (double)(__popcll(s0 & D.m0[k]) + __popcll(s1 & D.m1[k]));
    for (int k = 0; k < D.n_generic; ++k) {
        const PushTerm& T = gen[k];
        bool ok = ((s0 & T.dn0) | (s1 & T.dn1)) == 0 && (s0 & T.up0) == T.up0 && (s1 & T.up1) == T.up1;
        if (!ok) continue;
        int par = (__popcll(~s0 & T.z0) + __popcll(~s1 & T.z1)) & 1;
        d += T.c * (double)(T.sign * (1 - 2 * par));
    }
    return d;
}

}  // namespace qsi

#define QSI_CUDA(call)                                                                            \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            return ::qsi::fail(e_ == cudaErrorMemoryAllocation ? QSI_OOM : QSI_CUDA_ERROR,        \
                               "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
        }                                                                                         \
    } while (0)
