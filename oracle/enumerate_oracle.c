/*
 * ORACLE — test infrastructure, not product code.
 *
 * Plain-C restatement of the reference's spin-ice basis enumerator, used by
 * tests/ (against the reference's stored bases and the engine's enumerators)
 * and by bench.py's reference arm, which must build its basis without the
 * engine's library:
 *
 *   visiting order   lattice::greedy_spin_ordering(0)
 *                    (components/common/src/tetra_graph_io.cpp:105-150): start at spin 0, then repeatedly the
 *                    unvisited spin with the most tetrahedra already touched (ties: the lowest index)
 *   admission        lat_container(_with_sector)::possible_spin_states
 *                    (components/build_basis/src/pyro_tree.cpp:20-162): a value of the next spin is admitted
 *                    when each of its tetrahedra can still reach [min_up, max_up] = [size/2, (size+1)/2]
 *                    (tetra_graph_io.hpp:45-46) and, with a sector, every sublattice count can still reach
 *                    its target with the unknown spins
 *   forking          fork_state_impl (pyro_tree.cpp:168-189): an inadmissible value is still taken while
 *                    spinon pairs are left, spending one
 *   output           every leaf (all spins set), sorted (pyro_vtree::sort, pyro_tree.cpp:244-249)
 *
 * Without spinon pairs the produced set is exactly the states that satisfy every tetrahedron bound and the
 * sector, whatever the visiting order and however strong the pruning, so that case adds an exact per-sublattice
 * capacity test (remaining spins of the sublattice instead of all unknown spins), which removes dead subtrees
 * early and leaves the set unchanged.  With spinon pairs the set depends on which values the test rejects, so
 * the reference's own test is used as it stands: all sublattices checked against N - k unknown spins
 * (pyro_tree.cpp:94-125).
 *
 * Leaves are written directly in the original bit order (spin perm[k] is bit perm[k]), subtrees below a
 * breadth-first frontier run on OpenMP threads, and the result is sorted by a parallel most-significant-bits
 * partition followed by per-bucket sorts.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

#define MAX_SPINS 128
#define MAX_TET_PER_SPIN 4

typedef struct {
    int n_tet;
    int tet[MAX_TET_PER_SPIN];
    int unknown_after[MAX_TET_PER_SPIN]; /* members of that tetrahedron visited after this step */
    int min_up[MAX_TET_PER_SPIN], max_up[MAX_TET_PER_SPIN];
    int sl;
    int bit; /* original spin index */
} ostep;

typedef struct {
    int N, n_tet, n_sl, n_pairs, has_sector;
    ostep st[MAX_SPINS];
    int target[8];
    int sl_remaining_after[MAX_SPINS]; /* spins of step k's sublattice visited after step k */
} oproblem;

typedef struct {
    u128 state;
    int k, pairs;
    uint8_t tet_up[256];
    uint8_t sl_up[8];
} onode;

typedef struct {
    u128* v;
    size_t n, cap;
} obuf;

static int push_state(obuf* b, u128 s) {
    if (b->n == b->cap) {
        size_t cap = b->cap ? 2 * b->cap : 1 << 16;
        u128* nv = (u128*)realloc(b->v, cap * sizeof(u128));
        if (!nv) return -1;
        b->v = nv;
        b->cap = cap;
    }
    b->v[b->n++] = s;
    return 0;
}

/* bit 0: value 0 admitted, bit 1: value 1 admitted */
static int admissible(const oproblem* P, const onode* nd) {
    const ostep* s = &P->st[nd->k];
    int res = 3;
    for (int v = 0; v < 2; ++v) {
        int ok = 1;
        if (P->has_sector) {
            if (P->n_pairs == 0) {
                int n = nd->sl_up[s->sl] + v;
                if (n > P->target[s->sl] || n + P->sl_remaining_after[nd->k] < P->target[s->sl]) ok = 0;
            } else {
                for (int a = 0; a < P->n_sl && ok; ++a) {
                    int n = nd->sl_up[a] + (a == s->sl ? v : 0);
                    if (n + (P->N - nd->k) < P->target[a] || n > P->target[a]) ok = 0;
                }
            }
        }
        for (int j = 0; j < s->n_tet && ok; ++j) {
            int q = nd->tet_up[s->tet[j]] + v;
            if (q + s->unknown_after[j] < s->min_up[j] || q > s->max_up[j]) ok = 0;
        }
        if (!ok) res &= ~(1 << v);
    }
    return res;
}

static void child(const oproblem* P, const onode* nd, int v, int spend, onode* out) {
    const ostep* s = &P->st[nd->k];
    *out = *nd;
    out->k = nd->k + 1;
    out->pairs = nd->pairs + spend;
    if (v) {
        out->state |= (u128)1 << s->bit;
        for (int j = 0; j < s->n_tet; ++j) out->tet_up[s->tet[j]]++;
        out->sl_up[s->sl]++;
    }
}

/* children of nd in fork_state_impl's rule; returns their count (0..2) */
static int fork_node(const oproblem* P, const onode* nd, onode* kids) {
    const int poss = admissible(P, nd);
    const int may_pair = nd->pairs < P->n_pairs;
    int c = 0;
    for (int v = 0; v < 2; ++v) {
        if (poss & (1 << v)) child(P, nd, v, 0, &kids[c++]);
        else if (may_pair) child(P, nd, v, 1, &kids[c++]);
    }
    return c;
}

/* Depth-first walk below `nd`, counts updated in place and undone on the way back. */
static int walk(const oproblem* P, onode* nd, obuf* out) {
    if (nd->k == P->N) return push_state(out, nd->state);
    const ostep* s = &P->st[nd->k];
    const int poss = admissible(P, nd);
    const int may_pair = nd->pairs < P->n_pairs;
    const u128 state0 = nd->state;
    const int k0 = nd->k, pairs0 = nd->pairs;
    for (int v = 0; v < 2; ++v) {
        const int spend = !(poss & (1 << v));
        if (spend && !may_pair) continue;
        nd->k = k0 + 1;
        nd->pairs = pairs0 + spend;
        if (v) {
            nd->state = state0 | ((u128)1 << s->bit);
            for (int j = 0; j < s->n_tet; ++j) nd->tet_up[s->tet[j]]++;
            nd->sl_up[s->sl]++;
        }
        const int rc = walk(P, nd, out);
        if (v) {
            for (int j = 0; j < s->n_tet; ++j) nd->tet_up[s->tet[j]]--;
            nd->sl_up[s->sl]--;
            nd->state = state0;
        }
        nd->k = k0;
        nd->pairs = pairs0;
        if (rc) return rc;
    }
    return 0;
}

static int dfs(const oproblem* P, const onode* root, obuf* out) {
    onode nd = *root;
    return walk(P, &nd, out);
}

static int u128_cmp(const void* a, const void* b) {
    u128 x = *(const u128*)a, y = *(const u128*)b;
    return x < y ? -1 : (x > y);
}

/* Greedy visiting order of tetra_graph_io.cpp:105-150 (ties to the lowest index). */
static void greedy_order(int N, int n_tet, const int32_t* tet_off, const int32_t* tet_mem, int* perm) {
    int* covered = (int*)calloc((size_t)n_tet, sizeof(int));
    int* selected = (int*)calloc((size_t)N, sizeof(int));
    /* spin -> its tetrahedra */
    int* cnt = (int*)calloc((size_t)N, sizeof(int));
    int* nbr = (int*)malloc(sizeof(int) * (size_t)N * MAX_TET_PER_SPIN);
    for (int t = 0; t < n_tet; ++t)
        for (int m = tet_off[t]; m < tet_off[t + 1]; ++m) {
            int s = tet_mem[m];
            if (cnt[s] < MAX_TET_PER_SPIN) nbr[s * MAX_TET_PER_SPIN + cnt[s]++] = t;
        }
    perm[0] = 0;
    selected[0] = 1;
    for (int j = 0; j < cnt[0]; ++j) covered[nbr[j]] = 1;
    for (int it = 1; it < N; ++it) {
        int best = -1, best_ov = -1;
        for (int i = 0; i < N; ++i) {
            if (selected[i]) continue;
            int ov = 0;
            for (int j = 0; j < cnt[i]; ++j) ov += covered[nbr[i * MAX_TET_PER_SPIN + j]];
            if (ov > best_ov) best_ov = ov, best = i;
        }
        selected[best] = 1;
        perm[it] = best;
        for (int j = 0; j < cnt[best]; ++j) covered[nbr[best * MAX_TET_PER_SPIN + j]] = 1;
    }
    free(covered);
    free(selected);
    free(cnt);
    free(nbr);
}

/*
 * n_spins spins with sublattice sl[i]; n_tet tetrahedra whose members are tet_mem[tet_off[t] .. tet_off[t+1]);
 * sector: n_sl targets (NULL: no sector).  Returns the number of states and a malloc'd array of (lo, hi) pairs in
 * *out (free with oracle_free), or -1 on bad input / no memory.
 */
int64_t oracle_enumerate(int n_spins, const int32_t* sl, int n_tet, const int32_t* tet_off, const int32_t* tet_mem,
                         const int32_t* sector, int n_sl, int n_pairs, int threads, uint64_t** out) {
    if (n_spins < 1 || n_spins > MAX_SPINS || n_tet < 0 || n_tet > 256 || n_sl > 8 || n_pairs < 0 || !out) return -1;
    oproblem* P = (oproblem*)calloc(1, sizeof(oproblem));
    if (!P) return -1;
    P->N = n_spins;
    P->n_tet = n_tet;
    P->n_pairs = n_pairs;
    P->has_sector = sector != NULL && n_sl > 0;
    P->n_sl = P->has_sector ? n_sl : 0;
    for (int a = 0; a < P->n_sl; ++a) P->target[a] = sector[a];
    int perm[MAX_SPINS], pos[MAX_SPINS];
    greedy_order(n_spins, n_tet, tet_off, tet_mem, perm);
    for (int k = 0; k < n_spins; ++k) pos[perm[k]] = k;
    for (int k = 0; k < n_spins; ++k) {
        ostep* s = &P->st[k];
        const int sp = perm[k];
        s->bit = sp;
        s->sl = sl[sp];
        if (P->has_sector && (s->sl < 0 || s->sl >= n_sl)) {
            free(P);
            return -1;
        }
        for (int t = 0; t < n_tet; ++t) {
            int member = 0, after = 0;
            const int size = tet_off[t + 1] - tet_off[t];
            for (int m = tet_off[t]; m < tet_off[t + 1]; ++m) {
                if (tet_mem[m] == sp) member = 1;
                if (pos[tet_mem[m]] > k) ++after;
            }
            if (!member) continue;
            if (s->n_tet == MAX_TET_PER_SPIN) {
                free(P);
                return -1;
            }
            s->tet[s->n_tet] = t;
            s->unknown_after[s->n_tet] = after;
            s->min_up[s->n_tet] = size / 2;
            s->max_up[s->n_tet] = (size + 1) / 2;
            s->n_tet++;
        }
        int rem = 0;
        for (int j = k + 1; j < n_spins; ++j)
            if (sl[perm[j]] == s->sl) ++rem;
        P->sl_remaining_after[k] = rem;
    }
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#else
    threads = 1;
#endif
    /* breadth-first frontier of subtree roots */
    size_t fcap = 1 << 12, fn = 1;
    onode* front = (onode*)calloc(fcap, sizeof(onode));
    if (!front) {
        free(P);
        return -1;
    }
    const size_t want = (size_t)threads * 256;
    while (fn < want) {
        int all_leaves = 1;
        for (size_t i = 0; i < fn; ++i)
            if (front[i].k < n_spins) all_leaves = 0;
        if (all_leaves) break;
        onode* next = (onode*)malloc(sizeof(onode) * (2 * fn + 1));
        if (!next) {
            free(front);
            free(P);
            return -1;
        }
        size_t nn = 0;
        for (size_t i = 0; i < fn; ++i) {
            if (front[i].k == n_spins) {
                next[nn++] = front[i];
                continue;
            }
            nn += (size_t)fork_node(P, &front[i], next + nn);
        }
        free(front);
        front = next;
        fn = nn;
        if (!fn) break;
    }
    obuf* bufs = (obuf*)calloc(fn ? fn : 1, sizeof(obuf));
    int err = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) reduction(| : err)
    for (long long i = 0; i < (long long)fn; ++i) err |= dfs(P, &front[i], &bufs[i]) != 0;
    free(front);
    size_t total = 0;
    for (size_t i = 0; i < fn; ++i) total += bufs[i].n;
    u128* all = err ? NULL : (u128*)malloc(sizeof(u128) * (total ? total : 1));
    u128* sorted = err ? NULL : (u128*)malloc(sizeof(u128) * (total ? total : 1));
    if (!all || !sorted) err = 1;
    if (!err) {
        size_t off = 0;
        for (size_t i = 0; i < fn; ++i) {
            memcpy(all + off, bufs[i].v, bufs[i].n * sizeof(u128));
            off += bufs[i].n;
        }
    }
    for (size_t i = 0; i < fn; ++i) free(bufs[i].v);
    free(bufs);
    if (err) {
        free(all);
        free(sorted);
        free(P);
        return -1;
    }
    /* parallel sort: partition by the top 16 bits below the highest bit in use, then sort each bucket */
    u128 top = 0;
    for (size_t i = 0; i < total; ++i) top |= all[i];
    int hb = 0;
    for (int b = 127; b >= 0; --b)
        if ((top >> b) & 1) {
            hb = b;
            break;
        }
    const int shift = hb + 1 > 16 ? hb + 1 - 16 : 0;
    const int NB = 1 << 16;
    size_t* counts = (size_t*)calloc((size_t)threads * NB, sizeof(size_t));
    size_t* starts = (size_t*)malloc(sizeof(size_t) * (NB + 1));
    if (!counts || !starts) {
        free(all);
        free(sorted);
        free(counts);
        free(starts);
        free(P);
        return -1;
    }
#pragma omp parallel num_threads(threads)
    {
#ifdef _OPENMP
        const int t = omp_get_thread_num(), nt = omp_get_num_threads();
#else
        const int t = 0, nt = 1;
#endif
        const size_t lo = total * t / nt, hi = total * (t + 1) / nt;
        size_t* c = counts + (size_t)t * NB;
        for (size_t i = lo; i < hi; ++i) c[(int)(all[i] >> shift) & (NB - 1)]++;
#pragma omp barrier
#pragma omp single
        {
            size_t acc = 0;
            for (int b = 0; b < NB; ++b) {
                starts[b] = acc;
                for (int u = 0; u < nt; ++u) {
                    size_t v = counts[(size_t)u * NB + b];
                    counts[(size_t)u * NB + b] = acc;
                    acc += v;
                }
            }
            starts[NB] = acc;
        }
        for (size_t i = lo; i < hi; ++i) sorted[c[(int)(all[i] >> shift) & (NB - 1)]++] = all[i];
    }
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
    for (int b = 0; b < NB; ++b) qsort(sorted + starts[b], starts[b + 1] - starts[b], sizeof(u128), u128_cmp);
    free(counts);
    free(starts);
    free(all);
    uint64_t* res = (uint64_t*)malloc(sizeof(uint64_t) * 2 * (total ? total : 1));
    if (!res) {
        free(sorted);
        free(P);
        return -1;
    }
#pragma omp parallel for num_threads(threads)
    for (long long i = 0; i < (long long)total; ++i) {
        res[2 * i] = (uint64_t)sorted[i];
        res[2 * i + 1] = (uint64_t)(sorted[i] >> 64);
    }
    free(sorted);
    free(P);
    *out = res;
    return (int64_t)total;
}

void oracle_free(void* p) { free(p); }
