// Spin-ice basis enumerator (host, multi-threaded).
//
// Depth-first search over spins in a fixed visiting order.  Setting spin i to
// a value is admitted when every tetrahedron containing it can still reach
// the ice rule (count of up spins in [min_up, max_up]) and, with a sector,
// when the sublattice up-counts can still reach their targets.  A value that
// fails these tests may still be taken by spending one spinon pair, up to
// n_spinon_pairs (the forking rule of
// components/build_basis/src/pyro_tree.cpp:20-189).  The admission tests and
// the greedy visiting order (components/common/src/tetra_graph_io.cpp:105-150)
// follow the reference, so the produced set is the reference's set, also with
// spinon pairs where that set depends on the visiting order.
//
// Parallelism: a breadth-first expansion produces a few thousand subtree
// roots; worker threads pull roots from an atomic counter and run iterative
// DFS.  Leaves are mapped back to the original bit order with byte tables and
// the result is sorted by a parallel most-significant-bits bucket pass plus
// per-bucket std::sort.
//
// Bases without spinon pairs use a tighter search (fast_dfs below) with
// incremental counts and an exact per-sublattice capacity test; it yields the
// same set, since without spinon pairs the set is exactly the states that
// satisfy every tetrahedron and sector constraint.
#include <algorithm>
#include <array>
#include <atomic>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <thread>
#include <vector>

#include "qsi_internal.h"

namespace qsi {
namespace {

struct Step {
    // tetrahedra containing the spin visited at this step (permuted bit space)
    int n_tet = 0;
    u128 tmask[4];
    int known[4];   // spins of that tetrahedron known after this step (incl. this one)
    int size[4];
    int min_up[4], max_up[4];
    int sl = 0;             // sublattice of this spin
    int total_unknown = 0;  // N - i, the count the reference's sector test uses
};

struct Problem {
    int N = 0;
    std::vector<Step> steps;
    int n_pairs = 0;
    bool has_sector = false;
    int n_sl = 0;
    std::vector<u128> sl_mask;  // permuted bit space
    std::vector<int> sl_target;
    // per-step remaining spins of the visited spin's sublattice (strong prune, only used with n_pairs==0)
    std::vector<int> sl_remaining_after;
};

// Returns bit mask of admissible values {0b01: down ok, 0b10: up ok}.
inline int admissible(const Problem& P, int i, u128 state) {
    const Step& st = P.steps[i];
    int res = 3;
    for (int v = 0; v < 2; ++v) {
        u128 s = v ? (state | ((u128)1 << i)) : state;
        bool ok = true;
        if (P.has_sector) {
            for (int a = 0; a < P.n_sl && ok; ++a) {
                int n_up = popc128(s & P.sl_mask[a]);
                if (n_up + st.total_unknown < P.sl_target[a] || n_up > P.sl_target[a]) ok = false;
            }
            if (ok && P.n_pairs == 0) {
                // necessary condition with the exact remaining count of this sublattice
                int a = st.sl;
                int n_up = popc128(s & P.sl_mask[a]);
                if (n_up + P.sl_remaining_after[i] < P.sl_target[a]) ok = false;
            }
        }
        for (int k = 0; k < st.n_tet && ok; ++k) {
            int Q = popc128(s & st.tmask[k]);
            int unknown = st.size[k] - st.known[k];
            if (Q + unknown < st.min_up[k] || Q > st.max_up[k]) ok = false;
        }
        if (!ok) res &= ~(1 << v);
    }
    return res;
}

struct Node {
    u128 state;
    int depth;
    int pairs;
};

// Expands one node into its children (push order: 0 then 1), as fork_state_impl.
template <class Push>
inline void fork(const Problem& P, const Node& n, Push&& push) {
    int poss = admissible(P, n.depth, n.state);
    bool may_pair = n.pairs < P.n_pairs;
    u128 b = (u128)1 << n.depth;
    if (poss & 1) push(Node{n.state, n.depth + 1, n.pairs});
    else if (may_pair) push(Node{n.state, n.depth + 1, n.pairs + 1});
    if (poss & 2) push(Node{n.state | b, n.depth + 1, n.pairs});
    else if (may_pair) push(Node{n.state | b, n.depth + 1, n.pairs + 1});
}

void dfs(const Problem& P, Node root, std::vector<u128>& out) {
    std::vector<Node> stack;
    stack.reserve(4 * (P.N + 2));
    stack.push_back(root);
    while (!stack.empty()) {
        Node n = stack.back();
        stack.pop_back();
        if (n.depth == P.N) {
            out.push_back(n.state);
            continue;
        }
        fork(P, n, [&](const Node& c) { stack.push_back(c); });
    }
}

// lattice::greedy_spin_ordering: next spin = most tetrahedra already touched,
// ties to the lowest index.
std::vector<int> greedy_order(int N, const std::vector<std::vector<int>>& spin_tets) {
    std::vector<int> order{0};
    std::vector<char> selected(N, 0), covered;
    int n_tets = 0;
    for (auto& v : spin_tets)
        for (int t : v) n_tets = std::max(n_tets, t + 1);
    covered.assign(n_tets, 0);
    selected[0] = 1;
    for (int t : spin_tets[0]) covered[t] = 1;
    for (int it = 1; it < N; ++it) {
        int best = -1, best_overlap = -1;
        for (int i = 0; i < N; ++i) {
            if (selected[i]) continue;
            int ov = 0;
            for (int t : spin_tets[i]) ov += covered[t];
            if (ov > best_overlap) best_overlap = ov, best = i;
        }
        selected[best] = 1;
        order.push_back(best);
        for (int t : spin_tets[best]) covered[t] = 1;
    }
    return order;
}

void parallel_for(int n_threads, int64_t n, const std::function<void(int64_t, int64_t)>& body) {
    if (n_threads <= 1 || n < 1024) {
        body(0, n);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < n_threads; ++t) {
        int64_t a = n * t / n_threads, b = n * (t + 1) / n_threads;
        th.emplace_back([&, a, b] { body(a, b); });
    }
    for (auto& x : th) x.join();
}


// Lattice description shared by the DFS and the split join.
struct Lattice {
    int N = 0;
    int tsize = 0;
    std::vector<std::vector<int>> tets;       // spin ids per tetrahedron
    std::vector<std::vector<int>> spin_tets;  // tetrahedra per spin
    std::vector<int> sl;                      // sublattice per spin (0 when absent)
    int n_sl = 0;
};

// Builds the search over `visit` (a subset of spins, in visiting order).
// Spins outside `visit` count as never known, so all tests stay necessary
// conditions for the subset; with visit = all spins this is the reference's
// full search.
Problem build_problem(const Lattice& L, const std::vector<int>& visit, int n_pairs, const int32_t* sector) {
    Problem P;
    const int M = (int)visit.size();
    P.N = M;
    P.n_pairs = n_pairs;
    std::vector<int> pos(L.N, -1);
    for (int i = 0; i < M; ++i) pos[visit[i]] = i;
    std::vector<u128> tmask(L.tets.size(), 0);
    for (size_t t = 0; t < L.tets.size(); ++t)
        for (int s : L.tets[t])
            if (pos[s] >= 0) tmask[t] |= (u128)1 << pos[s];
    P.steps.resize(M);
    for (int i = 0; i < M; ++i) {
        Step& st = P.steps[i];
        int s = visit[i];
        st.n_tet = (int)L.spin_tets[s].size();
        u128 known_mask = (i + 1 >= 128) ? ~(u128)0 : (((u128)1 << (i + 1)) - 1);
        for (int k = 0; k < st.n_tet; ++k) {
            int t = L.spin_tets[s][k];
            st.tmask[k] = tmask[t];
            st.known[k] = popc128(tmask[t] & known_mask);
            st.size[k] = (int)L.tets[t].size();
            st.min_up[k] = st.size[k] / 2;
            st.max_up[k] = (st.size[k] + 1) / 2;
        }
        st.sl = L.sl[s];
        st.total_unknown = L.N - i;
    }
    if (sector) {
        P.has_sector = true;
        P.n_sl = L.n_sl;
        P.sl_mask.assign(L.n_sl, 0);
        P.sl_target.assign(sector, sector + L.n_sl);
        for (int i = 0; i < M; ++i) P.sl_mask[L.sl[visit[i]]] |= (u128)1 << i;
        std::vector<int> outside(L.n_sl, 0);
        for (int s = 0; s < L.N; ++s)
            if (pos[s] < 0) outside[L.sl[s]]++;
        P.sl_remaining_after.assign(M, 0);
        for (int i = 0; i < M; ++i) {
            int a = P.steps[i].sl, rem = outside[a];
            for (int j = i + 1; j < M; ++j) rem += (L.sl[visit[j]] == a);
            P.sl_remaining_after[i] = rem;
        }
    }
    return P;
}

// Parallel search; returns leaves in the permuted bit space of P.
std::vector<u128> search(const Problem& P, int threads) {
    std::vector<Node> frontier{Node{0, 0, 0}}, next;
    std::vector<u128> leaves;
    const size_t target = (size_t)threads * 512;
    while (!frontier.empty() && frontier.size() < target) {
        next.clear();
        bool any = false;
        for (auto& n : frontier) {
            if (n.depth == P.N) {
                leaves.push_back(n.state);
                continue;
            }
            any = true;
            fork(P, n, [&](const Node& c) { next.push_back(c); });
        }
        frontier.swap(next);
        if (!any) break;
    }
    std::vector<std::vector<u128>> parts(frontier.size());
    std::atomic<size_t> cursor{0};
    auto worker = [&] {
        for (;;) {
            size_t k = cursor.fetch_add(1);
            if (k >= frontier.size()) break;
            dfs(P, frontier[k], parts[k]);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    size_t total = leaves.size();
    for (auto& p : parts) total += p.size();
    leaves.reserve(total);
    for (auto& p : parts) leaves.insert(leaves.end(), p.begin(), p.end());
    return leaves;
}

// Byte tables mapping a permuted-space state back to original bit positions.
struct Unpermuter {
    std::vector<u128> table;
    int nbytes;
    explicit Unpermuter(const std::vector<int>& visit) : table(16 * 256, 0) {
        const int M = (int)visit.size();
        nbytes = (M + 7) / 8;
        for (int byte = 0; byte < 16; ++byte)
            for (int v = 0; v < 256; ++v) {
                u128 acc = 0;
                for (int b = 0; b < 8; ++b) {
                    int i = byte * 8 + b;
                    if (i < M && ((v >> b) & 1)) acc |= (u128)1 << visit[i];
                }
                table[byte * 256 + v] = acc;
            }
    }
    u128 operator()(u128 s) const {
        u128 r = 0;
        for (int byte = 0; byte < nbytes; ++byte) r |= table[byte * 256 + (int)((s >> (8 * byte)) & 0xff)];
        return r;
    }
};

// Parallel sort of 128-bit keys: bucket by the top 16 bits below bit N, then sort buckets.
void parallel_sort(std::vector<u128>& all, int N, int threads) {
    const size_t total = all.size();
    const int B = 16;
    int shift = std::max(0, N - B);
    std::vector<u128> sorted(total);
    std::vector<std::vector<int64_t>> hist(threads, std::vector<int64_t>(1 << B, 0));
    std::vector<int64_t> ca(threads + 1);
    for (int t = 0; t <= threads; ++t) ca[t] = (int64_t)total * t / threads;
    auto run = [&](const std::function<void(int)>& f) {
        std::vector<std::thread> th;
        for (int t = 0; t < threads; ++t) th.emplace_back(f, t);
        for (auto& x : th) x.join();
    };
    run([&](int t) {
        for (int64_t k = ca[t]; k < ca[t + 1]; ++k) hist[t][(size_t)(all[k] >> shift) & ((1u << B) - 1)]++;
    });
    std::vector<int64_t> bucket_start((1 << B) + 1, 0);
    int64_t acc = 0;
    for (int v = 0; v < (1 << B); ++v) {
        bucket_start[v] = acc;
        for (int t = 0; t < threads; ++t) {
            int64_t c = hist[t][v];
            hist[t][v] = acc;
            acc += c;
        }
    }
    bucket_start[1 << B] = acc;
    run([&](int t) {
        for (int64_t k = ca[t]; k < ca[t + 1]; ++k) {
            size_t v = (size_t)(all[k] >> shift) & ((1u << B) - 1);
            sorted[hist[t][v]++] = all[k];
        }
    });
    std::atomic<int> next_bucket{0};
    run([&](int) {
        for (;;) {
            int v = next_bucket.fetch_add(64);
            if (v >= (1 << B)) break;
            for (int w = v; w < std::min(v + 64, 1 << B); ++w)
                std::sort(sorted.begin() + bucket_start[w], sorted.begin() + bucket_start[w + 1]);
        }
    });
    all.swap(sorted);
}

// Fast search for ice bases without spinon pairs: recursive DFS with the
// per-tetrahedron and per-sublattice up-counts kept incrementally.  Setting a
// spin is admitted iff each of its tetrahedra can still end with an up-count
// in [min_up, max_up] and its sublattice can still end exactly on the sector
// target.  At the last spin of every tetrahedron / sublattice these tests are
// the constraints themselves, so the leaves are exactly the admissible states.
struct FastProblem {
    int N = 0;
    std::vector<int> spin;               // spin visited at step i
    std::vector<std::array<int, 4>> tet;  // its tetrahedra (-1 = none)
    std::vector<std::array<int, 4>> unk_after, tmin, tmax;
    std::vector<int> sl, rem_after;       // sublattice and remaining spins of it after step i
    std::vector<int> target;              // per sublattice, or empty
    int n_tets = 0, n_sl = 1;
};

struct FastState {
    std::vector<int8_t> Q;
    std::vector<int> cnt;
};

void fast_dfs(const FastProblem& F, int i, u128 state, FastState& S, std::vector<u128>& out) {
    if (i == F.N) {
        out.push_back(state);
        return;
    }
    const auto& tt = F.tet[i];
    const int a = F.sl[i];
    for (int v = 0; v < 2; ++v) {
        bool ok = true;
        for (int k = 0; k < 4 && tt[k] >= 0; ++k) {
            int q = S.Q[tt[k]] + v;
            if (q > F.tmax[i][k] || q + F.unk_after[i][k] < F.tmin[i][k]) ok = false;
        }
        if (!F.target.empty()) {
            int c = S.cnt[a] + v;
            if (c > F.target[a] || c + F.rem_after[i] < F.target[a]) ok = false;
        }
        if (!ok) continue;
        if (v) {
            for (int k = 0; k < 4 && tt[k] >= 0; ++k) S.Q[tt[k]]++;
            S.cnt[a]++;
        }
        fast_dfs(F, i + 1, v ? (state | ((u128)1 << i)) : state, S, out);
        if (v) {
            for (int k = 0; k < 4 && tt[k] >= 0; ++k) S.Q[tt[k]]--;
            S.cnt[a]--;
        }
    }
}

FastProblem build_fast(const Lattice& L, const std::vector<int>& order, const int32_t* sector) {
    FastProblem F;
    F.N = L.N;
    F.n_tets = (int)L.tets.size();
    F.n_sl = L.n_sl;
    std::vector<int> pos(L.N);
    for (int i = 0; i < L.N; ++i) pos[order[i]] = i;
    F.spin = order;
    F.tet.assign(L.N, {-1, -1, -1, -1});
    F.unk_after.assign(L.N, {0, 0, 0, 0});
    F.tmin = F.unk_after;
    F.tmax = F.unk_after;
    F.sl.assign(L.N, 0);
    F.rem_after.assign(L.N, 0);
    for (int i = 0; i < L.N; ++i) {
        int s = order[i];
        for (size_t k = 0; k < L.spin_tets[s].size(); ++k) {
            int t = L.spin_tets[s][k];
            int unk = 0;
            for (int m : L.tets[t]) unk += (pos[m] > i);
            F.tet[i][k] = t;
            F.unk_after[i][k] = unk;
            F.tmin[i][k] = (int)L.tets[t].size() / 2;
            F.tmax[i][k] = ((int)L.tets[t].size() + 1) / 2;
        }
        F.sl[i] = L.sl[s];
        int rem = 0;
        for (int j = i + 1; j < L.N; ++j) rem += (L.sl[order[j]] == L.sl[s]);
        F.rem_after[i] = rem;
    }
    if (sector) F.target.assign(sector, sector + L.n_sl);
    return F;
}

// Parallel driver: enumerate all admissible prefixes of depth d0 (in order),
// then run fast_dfs from each prefix on a worker pool.
std::vector<u128> fast_search(const FastProblem& F, int threads) {
    int d0 = std::min(F.N, 22);
    std::vector<u128> prefixes;
    {
        FastProblem G = F;
        G.N = d0;
        FastState S{std::vector<int8_t>(F.n_tets, 0), std::vector<int>(F.n_sl, 0)};
        fast_dfs(G, 0, 0, S, prefixes);
    }
    std::vector<std::vector<u128>> parts(prefixes.size());
    std::atomic<size_t> cursor{0};
    auto worker = [&] {
        FastState S{std::vector<int8_t>(F.n_tets, 0), std::vector<int>(F.n_sl, 0)};
        for (;;) {
            size_t k = cursor.fetch_add(1);
            if (k >= prefixes.size()) break;
            std::fill(S.Q.begin(), S.Q.end(), 0);
            std::fill(S.cnt.begin(), S.cnt.end(), 0);
            u128 p = prefixes[k];
            for (int i = 0; i < d0; ++i)
                if ((p >> i) & 1) {
                    for (int m = 0; m < 4 && F.tet[i][m] >= 0; ++m) S.Q[F.tet[i][m]]++;
                    S.cnt[F.sl[i]]++;
                }
            fast_dfs(F, d0, p, S, parts[k]);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    size_t total = 0;
    for (auto& p : parts) total += p.size();
    std::vector<u128> leaves;
    leaves.reserve(total);
    for (auto& p : parts) {
        leaves.insert(leaves.end(), p.begin(), p.end());
        std::vector<u128>().swap(p);
    }
    return leaves;
}

}  // namespace
}  // namespace qsi

using namespace qsi;

extern "C" void qsi_free_host(void* p) { std::free(p); }

extern "C" qsi_status qsi_enumerate_basis(int32_t n_spins, const int32_t* tetra_spins, int32_t n_tetra,
                                          int32_t tetra_size, const int32_t* sublattice, int32_t n_sublattices,
                                          int32_t n_spinon_pairs, const int32_t* sector, int32_t ordering,
                                          int32_t n_threads, uint64_t** out_lohi, int64_t* n_out) {
    return guarded([&]() -> qsi_status {
        if (n_spins <= 0 || n_spins > 128 || !tetra_spins || n_tetra <= 0 || tetra_size <= 0 || !out_lohi || !n_out)
            return fail(QSI_INVALID_ARG, "qsi_enumerate_basis: bad argument");
        if (sector && (!sublattice || n_sublattices <= 0)) return fail(QSI_INVALID_ARG, "qsi_enumerate_basis: sector needs sublattices");
        if (n_spinon_pairs < 0) return fail(QSI_INVALID_ARG, "qsi_enumerate_basis: negative n_spinon_pairs");
        Lattice L;
        L.N = n_spins;
        L.tsize = tetra_size;
        L.spin_tets.resize(L.N);
        L.sl.assign(L.N, 0);
        L.n_sl = sublattice ? n_sublattices : 1;
        for (int t = 0; t < n_tetra; ++t) {
            std::vector<int> mem;
            for (int k = 0; k < tetra_size; ++k) {
                int s = tetra_spins[t * tetra_size + k];
                if (s < 0 || s >= L.N) return fail(QSI_INVALID_ARG, "tetrahedron %d names spin %d outside [0,%d)", t, s, L.N);
                mem.push_back(s);
                L.spin_tets[s].push_back(t);
            }
            L.tets.push_back(mem);
        }
        for (int s = 0; s < L.N; ++s) {
            if (L.spin_tets[s].empty() || L.spin_tets[s].size() > 4)
                return fail(QSI_INVALID_ARG, "spin %d belongs to %zu tetrahedra (1..4 supported)", s, L.spin_tets[s].size());
            if (sublattice) {
                if (sublattice[s] < 0 || sublattice[s] >= n_sublattices) return fail(QSI_INVALID_ARG, "bad sublattice of spin %d", s);
                L.sl[s] = sublattice[s];
            }
        }
        std::vector<int> order(L.N);
        if (ordering == 1) order = greedy_order(L.N, L.spin_tets);
        else for (int i = 0; i < L.N; ++i) order[i] = i;
        unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        int threads = n_threads > 0 ? n_threads : (int)hw;

        std::vector<u128> leaves;
        if (n_spinon_pairs == 0) {
            leaves = fast_search(build_fast(L, order, sector), threads);
        } else {
            leaves = search(build_problem(L, order, n_spinon_pairs, sector), threads);
        }
        Unpermuter up(order);
        std::vector<u128> all(leaves.size());
        parallel_for(threads, (int64_t)leaves.size(), [&](int64_t a, int64_t b) {
            for (int64_t k = a; k < b; ++k) all[k] = up(leaves[k]);
        });
        std::vector<u128>().swap(leaves);
        parallel_sort(all, L.N, threads);
        const size_t total = all.size();
        uint64_t* out = (uint64_t*)std::malloc(std::max<size_t>(1, total) * 16);
        if (!out) return fail(QSI_OOM, "qsi_enumerate_basis: cannot allocate %zu states", total);
        parallel_for(threads, (int64_t)total, [&](int64_t a, int64_t b) {
            for (int64_t k = a; k < b; ++k) {
                out[2 * k] = lo64(all[k]);
                out[2 * k + 1] = hi64(all[k]);
            }
        });
        *out_lohi = out;
        *n_out = (int64_t)total;
        return QSI_OK;
    });
}
