// Spin-ice basis enumeration on the GPU, with or without spinon pairs.
//
// The host walks the search tree (same visiting order and admission tests as
// enumerate.cpp's fast search) down to a prefix depth with enough subtree
// roots to fill the GPU; then every root is searched to the leaves by one
// GPU thread with an iterative DFS that keeps the tetrahedron and sublattice
// up-counts incrementally.  Pass 1 counts the leaves of every root, an
// exclusive scan gives each root its output offset, pass 2 writes the leaves.
// The device walk keeps only the partial state in registers: tetrahedron and
// sublattice up-counts are popcounts against per-step masks in shared memory.
// Leaves are mapped back to the original spin numbering with byte tables and
// sorted as 128-bit keys by two stable LSD radix sorts (low word, then high
// word) with CUB's device radix sort.
//
// Bases with spinon pairs follow the reference's forking rule
// (components/build_basis/src/pyro_tree.cpp:168-189): a value that fails the
// admission test is still taken while pairs are left, spending one.  The set
// then depends on exactly which values the test rejects, so that walk uses the
// reference's own test (pyro_tree.cpp:87-162: every sublattice checked against
// all N - i unknown spins) rather than the tighter per-sublattice capacity
// test of the pair-free walk.  The walk keeps no per-level record of pairs
// spent: coming back to a level, it re-evaluates the test for the value that
// level took (the state below the level is unchanged), which says whether a
// pair was spent there.
#include <algorithm>
#include <array>
#include <cstring>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "qsi_device.cuh"
#include "qsi_handles.h"

namespace qsi {
namespace {

constexpr int kMaxSpins = 128;
constexpr int kMaxTets = 128;

struct EnumStep {
    int8_t tet[4];
    int8_t unk[4];
    int8_t tmin[4];
    int8_t tmax[4];
    int8_t sl;
    int8_t rem;
    int8_t n_tet;
    int8_t pad;
};

struct EnumProblem {
    EnumStep step[kMaxSpins];
    int8_t target[8];
    int N;
    int n_tets;
    int has_sector;
    int d0;
    int n_pairs;  // spinon pairs allowed (0: the pair-free walk)
};

// Mask form of one search step for the device walk: the (permuted-space)
// masks of the spin's tetrahedra and of its sublattice, so that up-counts are
// popcounts of the partial state and no per-node arrays are needed.
struct MaskStep {
    uint64_t tm[4][2];   // tetrahedron masks
    uint64_t sm[2];      // sublattice mask (spins of this step's sublattice)
    int8_t n_tet, target, rem, sl;  // sl: this step's sublattice
    int8_t unk[4], tmin[4], tmax[4];
};

struct MaskProblem {
    MaskStep step[kMaxSpins];
    int N, has_sector, d0, n_pairs;
    int n_sl, pad2;
    uint64_t slm[8][2];  // sublattice masks (permuted space) and targets, for the spinon-pair walk's sector test
    int8_t target[8];
};

__device__ __forceinline__ int popc2(uint64_t a0, uint64_t a1, const uint64_t* m) {
    return __popcll(a0 & m[0]) + __popcll(a1 & m[1]);
}

__device__ __forceinline__ bool admit_step(const MaskProblem& P, const MaskStep& st, int v, uint64_t s0, uint64_t s1) {
    for (int k = 0; k < st.n_tet; ++k) {
        const int q = popc2(s0, s1, st.tm[k]) + v;
        if (q > st.tmax[k] || q + st.unk[k] < st.tmin[k]) return false;
    }
    if (P.has_sector) {
        const int c = popc2(s0, s1, st.sm) + v;
        if (c > st.target || c + st.rem < st.target) return false;
    }
    return true;
}

// The reference's admission test of value v for the spin at step i (spinon-pair walk).
__device__ __forceinline__ bool admit_ref(const MaskProblem& P, const MaskStep& st, int v, uint64_t s0, uint64_t s1,
                                          int i, int sl_i) {
    for (int k = 0; k < st.n_tet; ++k) {
        const int q = popc2(s0, s1, st.tm[k]) + v;
        if (q > st.tmax[k] || q + st.unk[k] < st.tmin[k]) return false;
    }
    if (P.has_sector)
        for (int a = 0; a < P.n_sl; ++a) {
            const int c = popc2(s0, s1, P.slm[a]) + (a == sl_i ? v : 0);
            if (c + (P.N - i) < P.target[a] || c > P.target[a]) return false;
        }
    return true;
}

// Walk of one subtree with spinon pairs (see the file comment): pass 0 counts leaves, pass 1 writes them.
__global__ void __launch_bounds__(128) k_enum_pairs(const MaskProblem* __restrict__ gP, const state2* __restrict__ roots,
                                                    const int8_t* __restrict__ root_pairs, int64_t n_roots,
                                                    unsigned long long* __restrict__ counts,
                                                    const unsigned long long* __restrict__ offsets,
                                                    state2* __restrict__ out, unsigned long long* cursor) {
    __shared__ MaskProblem P;
    for (int k = threadIdx.x; k < (int)(sizeof(MaskProblem) / 8); k += blockDim.x)
        reinterpret_cast<uint64_t*>(&P)[k] = reinterpret_cast<const uint64_t*>(gP)[k];
    __syncthreads();
    for (;;) {
        const unsigned long long r = atomicAdd(cursor, 1ULL);
        if (r >= (unsigned long long)n_roots) break;
        const state2 root = roots[r];
        uint64_t s0 = root.x, s1 = root.y;
        int pairs = root_pairs[r];
        unsigned long long found = 0, steps = 0;
        const unsigned long long w = offsets ? offsets[r] : 0;
        int i = P.d0;
        bool down = true;
        auto set_bit = [&](int b) {
            if (b < 64) s0 |= 1ULL << b;
            else s1 |= 1ULL << (b - 64);
        };
        for (;;) {
            if (++steps > (1ULL << 38)) {
                atomicOr(cursor + 1, 1ULL);
                break;
            }
            if (down) {
                if (i == P.N) {
                    if (out) out[w + found] = make_ulonglong2(s0, s1);
                    ++found;
                    down = false;
                    --i;
                    if (i < P.d0) break;
                    continue;
                }
                const MaskStep& st = P.step[i];
                const bool a0 = admit_ref(P, st, 0, s0, s1, i, st.sl);
                if (a0 || pairs < P.n_pairs) {  // value 0 (bit stays clear)
                    pairs += !a0;
                    ++i;
                    continue;
                }
                const bool a1 = admit_ref(P, st, 1, s0, s1, i, st.sl);
                if (a1 || pairs < P.n_pairs) {
                    pairs += !a1;
                    set_bit(i);
                    ++i;
                    continue;
                }
                down = false;
                --i;
                if (i < P.d0) break;
                continue;
            }
            // returning to level i: its bit tells which value was taken; the test for that value says whether
            // it spent a pair
            const MaskStep& st = P.step[i];
            const bool set = (i < 64) ? ((s0 >> i) & 1) : ((s1 >> (i - 64)) & 1);
            if (set) {
                if (i < 64) s0 &= ~(1ULL << i);
                else s1 &= ~(1ULL << (i - 64));
                pairs -= !admit_ref(P, st, 1, s0, s1, i, st.sl);
                --i;
                if (i < P.d0) break;
                continue;
            }
            pairs -= !admit_ref(P, st, 0, s0, s1, i, st.sl);
            const bool a1 = admit_ref(P, st, 1, s0, s1, i, st.sl);
            if (a1 || pairs < P.n_pairs) {
                pairs += !a1;
                set_bit(i);
                ++i;
                down = true;
                continue;
            }
            --i;
            if (i < P.d0) break;
        }
        if (counts) counts[r] = found;
    }
}

// Register-only walk of one subtree: descending tries 0 then 1 at each level;
// on the way back the level's bit tells whether 1 is still to be tried.
// Pass 0 counts leaves, pass 1 writes them at the root's offset.
__global__ void __launch_bounds__(128) k_enum_mask(const MaskProblem* __restrict__ gP, const state2* __restrict__ roots,
                                                   int64_t n_roots, unsigned long long* __restrict__ counts,
                                                   const unsigned long long* __restrict__ offsets,
                                                   state2* __restrict__ out, unsigned long long* cursor) {
    __shared__ MaskProblem P;
    for (int k = threadIdx.x; k < (int)(sizeof(MaskProblem) / 8); k += blockDim.x)
        reinterpret_cast<uint64_t*>(&P)[k] = reinterpret_cast<const uint64_t*>(gP)[k];
    __syncthreads();
    for (;;) {
        const unsigned long long r = atomicAdd(cursor, 1ULL);
        if (r >= (unsigned long long)n_roots) break;
        const state2 root = roots[r];
        uint64_t s0 = root.x, s1 = root.y;
        unsigned long long found = 0, steps = 0;
        const unsigned long long w = offsets ? offsets[r] : 0;
        int i = P.d0;
        bool down = true;
        for (;;) {
            if (++steps > (1ULL << 36)) {
                atomicOr(cursor + 1, 1ULL);
                break;
            }
            if (down) {
                if (i == P.N) {
                    if (out) out[w + found] = make_ulonglong2(s0, s1);
                    ++found;
                    down = false;
                    --i;
                    if (i < P.d0) break;
                    continue;
                }
                const MaskStep& st = P.step[i];
                if (admit_step(P, st, 0, s0, s1)) {
                    ++i;
                    continue;
                }
                if (admit_step(P, st, 1, s0, s1)) {
                    if (i < 64) s0 |= 1ULL << i;
                    else s1 |= 1ULL << (i - 64);
                    ++i;
                    continue;
                }
                down = false;
                --i;
                if (i < P.d0) break;
                continue;
            }
            // returning to level i: its bit tells which value was taken
            const bool set = (i < 64) ? ((s0 >> i) & 1) : ((s1 >> (i - 64)) & 1);
            if (set) {
                if (i < 64) s0 &= ~(1ULL << i);
                else s1 &= ~(1ULL << (i - 64));
                --i;
                if (i < P.d0) break;
                continue;
            }
            const MaskStep& st = P.step[i];
            if (admit_step(P, st, 1, s0, s1)) {
                if (i < 64) s0 |= 1ULL << i;
                else s1 |= 1ULL << (i - 64);
                ++i;
                down = true;
                continue;
            }
            --i;
            if (i < P.d0) break;
        }
        if (counts) counts[r] = found;
    }
}

// Maps a permuted-space state back: bit i -> spin order[i], eight bits at a time.
__global__ void k_unpermute(state2* __restrict__ v, int64_t n, const state2* __restrict__ table, int nbytes,
                            uint64_t* __restrict__ lo, uint64_t* __restrict__ hi) {
    __shared__ state2 T[16 * 256];
    for (int k = threadIdx.x; k < nbytes * 256; k += blockDim.x) T[k] = table[k];
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const state2 s = v[i];
        uint64_t a = 0, b = 0;
        for (int byte = 0; byte < nbytes; ++byte) {
            const int val = (int)(((byte < 8) ? (s.x >> (8 * byte)) : (s.y >> (8 * (byte - 8)))) & 0xff);
            const state2 e = T[byte * 256 + val];
            a |= e.x;
            b |= e.y;
        }
        lo[i] = a;
        hi[i] = b;
    }
}

__global__ void k_interleave(const uint64_t* __restrict__ lo, const uint64_t* __restrict__ hi, state2* __restrict__ out,
                             int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = make_ulonglong2(lo[i], hi[i]);
}

std::vector<int> greedy(int N, const std::vector<std::vector<int>>& spin_tets, int n_tets) {
    std::vector<int> order{0};
    std::vector<char> sel(N, 0), cov(n_tets, 0);
    sel[0] = 1;
    for (int t : spin_tets[0]) cov[t] = 1;
    for (int it = 1; it < N; ++it) {
        int best = -1, bo = -1;
        for (int i = 0; i < N; ++i) {
            if (sel[i]) continue;
            int ov = 0;
            for (int t : spin_tets[i]) ov += cov[t];
            if (ov > bo) bo = ov, best = i;
        }
        sel[best] = 1;
        order.push_back(best);
        for (int t : spin_tets[best]) cov[t] = 1;
    }
    return order;
}

// Host DFS to depth d (same tests as the device), collecting prefixes.
void host_prefixes(const EnumProblem& P, int d, int i, u128 state, std::vector<int>& Q, std::vector<int>& cnt,
                   std::vector<u128>& out) {
    if (i == d) {
        out.push_back(state);
        return;
    }
    const EnumStep& st = P.step[i];
    for (int v = 0; v < 2; ++v) {
        bool ok = true;
        for (int k = 0; k < st.n_tet; ++k) {
            int q = Q[st.tet[k]] + v;
            if (q > st.tmax[k] || q + st.unk[k] < st.tmin[k]) ok = false;
        }
        if (P.has_sector) {
            int c = cnt[st.sl] + v;
            if (c > P.target[st.sl] || c + st.rem < P.target[st.sl]) ok = false;
        }
        if (!ok) continue;
        if (v) {
            for (int k = 0; k < st.n_tet; ++k) Q[st.tet[k]]++;
            cnt[st.sl]++;
        }
        host_prefixes(P, d, i + 1, v ? (state | ((u128)1 << i)) : state, Q, cnt, out);
        if (v) {
            for (int k = 0; k < st.n_tet; ++k) Q[st.tet[k]]--;
            cnt[st.sl]--;
        }
    }
}

// Host walk to depth d with spinon pairs (the reference's test and forking rule), collecting (prefix, pairs spent).
void host_prefixes_pairs(const EnumProblem& P, const std::vector<u128>& slm, int d, int i, u128 state, int pairs,
                         std::vector<int>& Q, std::vector<int>& cnt, std::vector<u128>& out, std::vector<int8_t>& outp) {
    if (i == d) {
        out.push_back(state);
        outp.push_back((int8_t)pairs);
        return;
    }
    const EnumStep& st = P.step[i];
    for (int v = 0; v < 2; ++v) {
        bool ok = true;
        for (int k = 0; k < st.n_tet; ++k) {
            int q = Q[st.tet[k]] + v;
            if (q > st.tmax[k] || q + st.unk[k] < st.tmin[k]) ok = false;
        }
        if (P.has_sector)
            for (size_t a = 0; a < slm.size(); ++a) {
                int c = cnt[a] + ((int)a == st.sl ? v : 0);
                if (c + (P.N - i) < P.target[a] || c > P.target[a]) ok = false;
            }
        if (!ok && pairs >= P.n_pairs) continue;
        if (v) {
            for (int k = 0; k < st.n_tet; ++k) Q[st.tet[k]]++;
            cnt[st.sl]++;
        }
        host_prefixes_pairs(P, slm, d, i + 1, v ? (state | ((u128)1 << i)) : state, pairs + (ok ? 0 : 1), Q, cnt, out,
                            outp);
        if (v) {
            for (int k = 0; k < st.n_tet; ++k) Q[st.tet[k]]--;
            cnt[st.sl]--;
        }
    }
}

template <typename T>
struct DBuf {
    T* p = nullptr;
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T)); }
    ~DBuf() { cudaFree(p); }
};

}  // namespace
}  // namespace qsi

using namespace qsi;

extern "C" qsi_status qsi_enumerate_basis_gpu(int32_t n_spins, const int32_t* tetra_spins, int32_t n_tetra,
                                              int32_t tetra_size, const int32_t* sublattice, int32_t n_sublattices,
                                              const int32_t* sector, int32_t n_spinon_pairs, uint64_t** out_lohi,
                                              int64_t* n_out) {
    return guarded([&]() -> qsi_status {
        if (n_spins <= 0 || n_spins > kMaxSpins || !tetra_spins || n_tetra <= 0 || n_tetra > kMaxTets ||
            tetra_size <= 0 || tetra_size > 127 || !out_lohi || !n_out || n_spinon_pairs < 0 || n_spinon_pairs > 64)
            return fail(QSI_INVALID_ARG, "qsi_enumerate_basis_gpu: bad argument");
        if (sector && (!sublattice || n_sublattices <= 0 || n_sublattices > 8))
            return fail(QSI_INVALID_ARG, "qsi_enumerate_basis_gpu: sector needs 1..8 sublattices");
        const int N = n_spins;
        std::vector<std::vector<int>> spin_tets(N), tets(n_tetra);
        for (int t = 0; t < n_tetra; ++t)
            for (int k = 0; k < tetra_size; ++k) {
                int s = tetra_spins[t * tetra_size + k];
                if (s < 0 || s >= N) return fail(QSI_INVALID_ARG, "tetrahedron %d names spin %d", t, s);
                spin_tets[s].push_back(t);
                tets[t].push_back(s);
            }
        for (int s = 0; s < N; ++s)
            if (spin_tets[s].empty() || spin_tets[s].size() > 4)
                return fail(QSI_INVALID_ARG, "spin %d belongs to %zu tetrahedra (1..4 supported)", s, spin_tets[s].size());
        std::vector<int> order = greedy(N, spin_tets, n_tetra);
        std::vector<int> pos(N);
        for (int i = 0; i < N; ++i) pos[order[i]] = i;
        EnumProblem P;
        std::memset(&P, 0, sizeof(P));
        P.N = N;
        P.n_tets = n_tetra;
        P.has_sector = sector != nullptr;
        P.n_pairs = n_spinon_pairs;
        for (int i = 0; i < N; ++i) {
            EnumStep& st = P.step[i];
            const int s = order[i];
            st.n_tet = (int8_t)spin_tets[s].size();
            for (int k = 0; k < st.n_tet; ++k) {
                const int t = spin_tets[s][k];
                int unk = 0;
                for (int m : tets[t]) unk += (pos[m] > i);
                st.tet[k] = (int8_t)t;
                st.unk[k] = (int8_t)unk;
                st.tmin[k] = (int8_t)(tets[t].size() / 2);
                st.tmax[k] = (int8_t)((tets[t].size() + 1) / 2);
            }
            st.sl = (int8_t)(sublattice ? sublattice[s] : 0);
            if (st.sl < 0 || st.sl >= 8) return fail(QSI_INVALID_ARG, "bad sublattice of spin %d", s);
            int rem = 0;
            for (int j = i + 1; j < N; ++j) rem += ((sublattice ? sublattice[order[j]] : 0) == st.sl);
            st.rem = (int8_t)rem;
        }
        if (sector)
            for (int a = 0; a < n_sublattices; ++a) P.target[a] = (int8_t)sector[a];
        // sublattice masks in the permuted space (the spinon-pair walk tests every sublattice)
        const int n_sl = sector ? n_sublattices : 0;
        std::vector<u128> slm(n_sl, 0);
        for (int j = 0; j < N; ++j)
            if (sector) slm[sublattice[order[j]]] |= (u128)1 << j;
        // prefix depth: deepen until there are enough roots to fill the GPU
        std::vector<u128> roots;
        std::vector<int8_t> root_pairs;
        int d0 = std::min(N, 16);
        for (;;) {
            roots.clear();
            root_pairs.clear();
            std::vector<int> Q(n_tetra, 0), cnt(8, 0);
            if (n_spinon_pairs) host_prefixes_pairs(P, slm, d0, 0, 0, 0, Q, cnt, roots, root_pairs);
            else host_prefixes(P, d0, 0, 0, Q, cnt, roots);
            if (roots.size() >= 2000000 || d0 >= N || d0 >= N - 8) break;
            d0 = std::min(N, d0 + 4);
        }
        P.d0 = d0;
        MaskProblem M;
        std::memset(&M, 0, sizeof(M));
        M.N = N;
        M.has_sector = sector != nullptr;
        M.d0 = d0;
        M.n_pairs = n_spinon_pairs;
        M.n_sl = n_sl;
        for (int a = 0; a < n_sl; ++a) {
            M.slm[a][0] = lo64(slm[a]);
            M.slm[a][1] = hi64(slm[a]);
            M.target[a] = (int8_t)sector[a];
        }
        for (int i = 0; i < N; ++i) {
            const int s = order[i];
            MaskStep& ms = M.step[i];
            ms.n_tet = P.step[i].n_tet;
            for (int k = 0; k < ms.n_tet; ++k) {
                u128 tm = 0;
                for (int m : tets[spin_tets[s][k]]) tm |= (u128)1 << pos[m];
                ms.tm[k][0] = lo64(tm);
                ms.tm[k][1] = hi64(tm);
                ms.unk[k] = P.step[i].unk[k];
                ms.tmin[k] = P.step[i].tmin[k];
                ms.tmax[k] = P.step[i].tmax[k];
            }
            u128 sm = 0;
            for (int j = 0; j < N; ++j)
                if ((sublattice ? sublattice[order[j]] : 0) == P.step[i].sl) sm |= (u128)1 << j;
            ms.sm[0] = lo64(sm);
            ms.sm[1] = hi64(sm);
            ms.target = sector ? (int8_t)sector[P.step[i].sl] : 0;
            ms.rem = P.step[i].rem;
            ms.sl = P.step[i].sl;
        }
        const int64_t n_roots = (int64_t)roots.size();
        std::vector<state2> hroots(n_roots);
        for (int64_t k = 0; k < n_roots; ++k) hroots[k] = make_ulonglong2(lo64(roots[k]), hi64(roots[k]));
        DBuf<MaskProblem> dP;
        DBuf<state2> dRoots;
        DBuf<int8_t> dRootPairs;
        DBuf<unsigned long long> dCounts, dOffs, dCur;
        QSI_CUDA(dP.alloc(1));
        QSI_CUDA(dRoots.alloc(n_roots));
        if (n_spinon_pairs) {
            QSI_CUDA(dRootPairs.alloc(n_roots));
            QSI_CUDA(cudaMemcpy(dRootPairs.p, root_pairs.data(), (size_t)n_roots, cudaMemcpyHostToDevice));
        }
        QSI_CUDA(dCounts.alloc(n_roots));
        QSI_CUDA(dOffs.alloc(n_roots + 1));
        QSI_CUDA(dCur.alloc(2));
        QSI_CUDA(cudaMemcpy(dP.p, &M, sizeof(M), cudaMemcpyHostToDevice));
        QSI_CUDA(cudaMemcpy(dRoots.p, hroots.data(), (size_t)n_roots * sizeof(state2), cudaMemcpyHostToDevice));
        int dev = 0, sms = 148;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int grid = sms * 16;
        auto walk = [&](unsigned long long* counts, const unsigned long long* offs, state2* leaves) {
            if (n_spinon_pairs)
                k_enum_pairs<<<grid, 128>>>(dP.p, dRoots.p, dRootPairs.p, n_roots, counts, offs, leaves, dCur.p);
            else
                k_enum_mask<<<grid, 128>>>(dP.p, dRoots.p, n_roots, counts, offs, leaves, dCur.p);
        };
        QSI_CUDA(cudaMemset(dCur.p, 0, 16));
        walk(dCounts.p, nullptr, nullptr);
        QSI_CUDA(cudaGetLastError());
        unsigned long long flags[2] = {0, 0};
        QSI_CUDA(cudaMemcpy(flags, dCur.p, 16, cudaMemcpyDeviceToHost));
        if (flags[1]) return fail(QSI_INVALID_ARG, "enumeration: a subtree exceeded the step bound");
        // exclusive scan of the counts
        size_t tmp_bytes = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, dCounts.p, dOffs.p, (int)n_roots + 0);
        DBuf<unsigned char> tmp;
        QSI_CUDA(tmp.alloc(tmp_bytes));
        QSI_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tmp_bytes, dCounts.p, dOffs.p, (int)n_roots));
        unsigned long long last_off = 0, last_cnt = 0;
        QSI_CUDA(cudaMemcpy(&last_off, dOffs.p + n_roots - 1, 8, cudaMemcpyDeviceToHost));
        QSI_CUDA(cudaMemcpy(&last_cnt, dCounts.p + n_roots - 1, 8, cudaMemcpyDeviceToHost));
        const int64_t total = (int64_t)(last_off + last_cnt);
        if (total >= (int64_t)UINT32_MAX) return fail(QSI_INVALID_ARG, "enumeration: %lld states exceed 2^32-1", (long long)total);
        DBuf<state2> dLeaves;
        QSI_CUDA(dLeaves.alloc(total));
        QSI_CUDA(cudaMemset(dCur.p, 0, 16));
        walk(nullptr, dOffs.p, dLeaves.p);
        QSI_CUDA(cudaGetLastError());
        // byte tables and un-permutation into separate key arrays
        const int nbytes = (N + 7) / 8;
        std::vector<state2> table(16 * 256, make_ulonglong2(0, 0));
        for (int byte = 0; byte < nbytes; ++byte)
            for (int v = 0; v < 256; ++v) {
                u128 acc = 0;
                for (int b = 0; b < 8; ++b) {
                    int i = byte * 8 + b;
                    if (i < N && ((v >> b) & 1)) acc |= (u128)1 << order[i];
                }
                table[byte * 256 + v] = make_ulonglong2(lo64(acc), hi64(acc));
            }
        DBuf<state2> dTable;
        DBuf<uint64_t> klo, khi, klo2, khi2;
        QSI_CUDA(dTable.alloc(16 * 256));
        QSI_CUDA(cudaMemcpy(dTable.p, table.data(), table.size() * sizeof(state2), cudaMemcpyHostToDevice));
        QSI_CUDA(klo.alloc(total));
        QSI_CUDA(khi.alloc(total));
        QSI_CUDA(klo2.alloc(total));
        QSI_CUDA(khi2.alloc(total));
        k_unpermute<<<grid_for(total, 256), 256>>>(dLeaves.p, total, dTable.p, nbytes, klo.p, khi.p);
        QSI_CUDA(cudaGetLastError());
        // stable LSD: sort by low word, then by high word
        size_t sb = 0, sb2 = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, sb, klo.p, klo2.p, khi.p, khi2.p, total);
        const int hi_bits = std::max(1, N - 64);
        cub::DeviceRadixSort::SortPairs(nullptr, sb2, khi2.p, khi.p, klo2.p, klo.p, total, 0, hi_bits);
        DBuf<unsigned char> stmp;
        QSI_CUDA(stmp.alloc(std::max(sb, sb2)));
        QSI_CUDA(cub::DeviceRadixSort::SortPairs(stmp.p, sb, klo.p, klo2.p, khi.p, khi2.p, total, 0, std::min(64, N)));
        if (N > 64) {
            QSI_CUDA(cub::DeviceRadixSort::SortPairs(stmp.p, sb2, khi2.p, khi.p, klo2.p, klo.p, total, 0, hi_bits));
        } else {
            QSI_CUDA(cudaMemcpy(klo.p, klo2.p, (size_t)total * 8, cudaMemcpyDeviceToDevice));
            QSI_CUDA(cudaMemcpy(khi.p, khi2.p, (size_t)total * 8, cudaMemcpyDeviceToDevice));
        }
        k_interleave<<<grid_for(total, 256), 256>>>(klo.p, khi.p, dLeaves.p, total);
        QSI_CUDA(cudaGetLastError());
        uint64_t* host = (uint64_t*)std::malloc(std::max<size_t>(1, (size_t)total) * 16);
        if (!host) return fail(QSI_OOM, "qsi_enumerate_basis_gpu: host allocation of %lld states", (long long)total);
        cudaError_t e = cudaMemcpy(host, dLeaves.p, (size_t)total * 16, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            std::free(host);
            return fail(QSI_CUDA_ERROR, "qsi_enumerate_basis_gpu: %s", cudaGetErrorString(e));
        }
        *out_lohi = host;
        *n_out = total;
        return QSI_OK;
    });
}
