/*
 * ORACLE — test infrastructure, not product code.
 *
 * Plain-C restatement of qsi_subspace_ED's CPU hot path, used only by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
 * checker.  It follows the reference's loops one to one:
 *
 *   oracle_term_compile   SymbolicPMROperator::_construct
 *                         (components/operator/include/operator.hpp:383-466)
 *   oracle_apply_state    SymbolicPMROperator::applyState (operator.hpp:232-254)
 *   oracle_search         ZBasisBST::search (components/operator/src/operator.cpp:4-34)
 *   oracle_interp_*       ZBasisInterp::find_bounds + search (operator.cpp:38-86), the basis class of
 *                         diag_DOQSI_ham and bench_apply (src/diag_DOQSI_ham.cpp:97, bench/bench_apply.cpp:44)
 *   oracle_evaluate_add   LazyOpSum::evaluate_add_off_diag_omp + evaluate_add_diagonal
 *                         (components/operator/src/operator_matrix.cpp:28-82,108-112):
 *                         per term, an OpenMP loop over rows, push y[J] += c x[i] sign
 *                         with an atomic update, |x[i]| <= 1e-15 skipped
 *   oracle_triplets       LazyOpSum::toSparseMatrix (operator_matrix.hpp:79-105)
 *
 * Terms use the qsi_term layout of include/qsi_ed.h; they are split into
 * off-diagonal (X != 0) and diagonal lists in the given order, as
 * SymbolicOpSum::add_term does (operator.hpp:489-495).
 *
 * Its pin: tests/golden holds checksums of the same quantities computed by
 * the reference's own operator.cpp (oracle/build_ref.sh -> oracle/_ref).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

typedef struct {
    double c;
    uint64_t x[2], z[2], up[2], down[2];
    int32_t sign, reserved;
} oterm;

static inline u128 mk(const uint64_t w[2]) { return ((u128)w[1] << 64) | w[0]; }
static inline int popc128(u128 v) { return __builtin_popcountll((uint64_t)v) + __builtin_popcountll((uint64_t)(v >> 64)); }

/* applyState: ok = (s & down)==0 && (s & up)==up ; s ^= X if ok ;
 * returns sign * (-1)^popcount(~s & Z) * ok */
int oracle_apply_state(const oterm* t, uint64_t st[2]) {
    u128 s = mk(st), d = mk(t->down), u = mk(t->up), X = mk(t->x), Z = mk(t->z);
    int ok = ((s & d) == 0) && ((s & u) == u);
    u128 m = (u128)0 - (u128)ok;
    s = s ^ (X & m);
    st[0] = (uint64_t)s;
    st[1] = (uint64_t)(s >> 64);
    return t->sign * (1 - 2 * (popc128(~s & Z) % 2)) * ok;
}

/* ZBasisBST::search: lower-bound bisection while the window exceeds 32
 * entries, then a linear scan of [left, right]. */
int oracle_search(const uint64_t* basis, int64_t n, const uint64_t st[2], int64_t* J) {
    const u128 s = mk(st);
    int64_t left = 0, right = n - 1;
    while (right - left > 32) {
        int64_t mid = (left + right) / 2;
        if (mk(basis + 2 * mid) < s) left = mid + 1;
        else right = mid;
    }
    for (int64_t j = left; j <= right; ++j) {
        if (j >= 0 && mk(basis + 2 * j) == s) {
            *J = j;
            return 1;
        }
    }
    *J = right + 1;
    return 0;
}

/* ZBasisInterp: find_bounds keeps, per high 64-bit word, the first and last index of the states that carry it
 * (an std::unordered_map there, open addressing here); search takes those bounds (an unseen high word makes
 * bounds.at throw there: here the lookup is a miss, counted), bisects on the LOW word only while the window
 * exceeds 32 entries, then compares whole states four at a time and one at a time. */
typedef struct {
    uint64_t key;
    uint32_t first, count; /* count 0: an empty slot */
} ibucket;
typedef struct {
    ibucket* t;
    uint64_t mask;
} interp_t;

static inline uint64_t mix64(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

static const ibucket* interp_find(const interp_t* ip, uint64_t key) {
    for (uint64_t s = mix64(key) & ip->mask;; s = (s + 1) & ip->mask) {
        const ibucket* b = &ip->t[s];
        if (!b->count) return NULL;
        if (b->key == key) return b;
    }
}

void* oracle_interp_build(const uint64_t* basis, int64_t n) {
    if (n < 1 || n >= ((int64_t)1 << 32)) return NULL;
    int64_t distinct = 0;
    for (int64_t j = 0; j < n; ++j)
        if (j == 0 || basis[2 * j + 1] != basis[2 * j - 1]) ++distinct;
    uint64_t cap = 16;
    while (cap < (uint64_t)distinct + (uint64_t)distinct / 2) cap <<= 1; /* load factor <= 2/3 */
    interp_t* ip = (interp_t*)malloc(sizeof(interp_t));
    if (!ip) return NULL;
    ip->t = (ibucket*)calloc(cap, sizeof(ibucket));
    ip->mask = cap - 1;
    if (!ip->t) {
        free(ip);
        return NULL;
    }
    /* the basis is sorted by (hi, lo): each high word's states are one run [first, last] */
    for (int64_t j = 0; j < n;) {
        const uint64_t key = basis[2 * j + 1];
        int64_t e = j;
        while (e + 1 < n && basis[2 * (e + 1) + 1] == key) ++e;
        uint64_t s = mix64(key) & ip->mask;
        while (ip->t[s].count) s = (s + 1) & ip->mask;
        ip->t[s].key = key;
        ip->t[s].first = (uint32_t)j;
        ip->t[s].count = (uint32_t)(e - j + 1);
        j = e + 1;
    }
    return ip;
}

void oracle_interp_free(void* h) {
    interp_t* ip = (interp_t*)h;
    if (ip) free(ip->t);
    free(ip);
}

/* 1 = found (J), 0 = absent, -1 = absent with an unseen high word (where the reference throws) */
int oracle_interp_search(const void* h, const uint64_t* basis, const uint64_t st[2], int64_t* J) {
    const ibucket* b = interp_find((const interp_t*)h, st[1]);
    if (!b) return -1;
    const u128 s = mk(st);
    int64_t left = b->first, right = (int64_t)b->first + b->count - 1;
    while (right - left > 32) {
        int64_t mid = (left + right) / 2;
        if (basis[2 * mid] < st[0]) left = mid + 1;
        else right = mid;
    }
    int64_t j = left;
    for (; j + 3 <= right; j += 4) {
        if (mk(basis + 2 * j) == s) { *J = j; return 1; }
        if (mk(basis + 2 * (j + 1)) == s) { *J = j + 1; return 1; }
        if (mk(basis + 2 * (j + 2)) == s) { *J = j + 2; return 1; }
        if (mk(basis + 2 * (j + 3)) == s) { *J = j + 3; return 1; }
    }
    for (; j <= right; ++j)
        if (j >= 0 && mk(basis + 2 * j) == s) { *J = j; return 1; }
    return 0;
}

/* ZBasisInterp::search over nq queries: index, -1 absent, -2 unseen high word */
void oracle_interp_search_many(const void* h, const uint64_t* basis, const uint64_t* q, int64_t nq, int64_t* idx) {
    for (int64_t k = 0; k < nq; ++k) {
        int64_t J = -1;
        const int f = oracle_interp_search(h, basis, q + 2 * k, &J);
        idx[k] = f == 1 ? J : (f == 0 ? -1 : -2);
    }
}

static void split_terms(const oterm* terms, int n, const oterm** off, int* n_off, const oterm** dg, int* n_dg) {
    int a = 0, b = 0;
    for (int k = 0; k < n; ++k) {
        if ((terms[k].x[0] | terms[k].x[1]) != 0) off[a++] = &terms[k];
        else dg[b++] = &terms[k];
    }
    *n_off = a;
    *n_dg = b;
}

/* y += H x, push form with atomics, one parallel pass per term. */
int oracle_evaluate_add(const uint64_t* basis, int64_t n, const oterm* terms, int n_terms, const double* x, double* y,
                        int n_threads) {
    const oterm** off = (const oterm**)malloc(sizeof(oterm*) * (size_t)(n_terms + 1));
    const oterm** dg = (const oterm**)malloc(sizeof(oterm*) * (size_t)(n_terms + 1));
    if (!off || !dg) return -1;
    int n_off, n_dg;
    split_terms(terms, n_terms, off, &n_off, dg, &n_dg);
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
    for (int t = 0; t < n_off; ++t) {
        const oterm* T = off[t];
        const double c = T->c;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            uint64_t st[2] = {basis[2 * i], basis[2 * i + 1]};
            int sign = oracle_apply_state(T, st);
            if (sign != 0 && fabs(x[i]) > 1e-15) {
                int64_t J;
                sign *= oracle_search(basis, n, st, &J);
                /* the reference writes y[J] += 0 on a miss, with J possibly == n;
                 * the restatement skips that write */
                if (sign != 0) {
                    double dy = c * x[i] * sign;
#pragma omp atomic
                    y[J] += dy;
                }
            }
        }
    }
    for (int t = 0; t < n_dg; ++t) {
        const oterm* T = dg[t];
        const double c = T->c;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            uint64_t st[2] = {basis[2 * i], basis[2 * i + 1]};
            double dy = c * x[i] * (double)oracle_apply_state(T, st);
            y[i] += dy;
        }
    }
    free(off);
    free(dg);
    return 0;
}

/* The push loop over source rows [row_begin, row_end) with ZBasisInterp lookups (interp from
 * oracle_interp_build), as diag_DOQSI_ham and bench_apply run it; *unseen counts the lookups whose high word the
 * basis lacks (the reference throws on the first).  A bounded sample of one apply for the CPU baseline. */
int oracle_evaluate_add_rows_interp(const uint64_t* basis, int64_t n, int64_t row_begin, int64_t row_end,
                                    const oterm* terms, int n_terms, const double* x, double* y, int n_threads,
                                    const void* interp, int64_t* unseen) {
    const oterm** off = (const oterm**)malloc(sizeof(oterm*) * (size_t)(n_terms + 1));
    const oterm** dg = (const oterm**)malloc(sizeof(oterm*) * (size_t)(n_terms + 1));
    if (!off || !dg || !interp) return -1;
    (void)n;
    int n_off, n_dg;
    split_terms(terms, n_terms, off, &n_off, dg, &n_dg);
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
    int64_t bad = 0;
    for (int t = 0; t < n_off; ++t) {
        const oterm* T = off[t];
        const double c = T->c;
#pragma omp parallel for schedule(static) reduction(+ : bad)
        for (int64_t i = row_begin; i < row_end; ++i) {
            uint64_t st[2] = {basis[2 * i], basis[2 * i + 1]};
            int sign = oracle_apply_state(T, st);
            if (sign != 0 && fabs(x[i]) > 1e-15) {
                int64_t J = 0;
                const int f = oracle_interp_search(interp, basis, st, &J);
                if (f < 0) ++bad;
                if (f == 1) {
                    double dy = c * x[i] * sign;
#pragma omp atomic
                    y[J] += dy;
                }
            }
        }
    }
    for (int t = 0; t < n_dg; ++t) {
        const oterm* T = dg[t];
        const double c = T->c;
#pragma omp parallel for schedule(static)
        for (int64_t i = row_begin; i < row_end; ++i) {
            uint64_t st[2] = {basis[2 * i], basis[2 * i + 1]};
            y[i] += c * x[i] * (double)oracle_apply_state(T, st);
        }
    }
    if (unseen) *unseen = bad;
    free(off);
    free(dg);
    return 0;
}

/* The same push loop restricted to source rows [row_begin, row_end): a
 * bounded sample of one apply for timing the CPU path on large bases. */
int oracle_evaluate_add_rows(const uint64_t* basis, int64_t n, int64_t row_begin, int64_t row_end, const oterm* terms,
                             int n_terms, const double* x, double* y, int n_threads) {
    const oterm** off = (const oterm**)malloc(sizeof(oterm*) * (size_t)(n_terms + 1));
    const oterm** dg = (const oterm**)malloc(sizeof(oterm*) * (size_t)(n_terms + 1));
    if (!off || !dg) return -1;
    int n_off, n_dg;
    split_terms(terms, n_terms, off, &n_off, dg, &n_dg);
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
    for (int t = 0; t < n_off; ++t) {
        const oterm* T = off[t];
        const double c = T->c;
#pragma omp parallel for schedule(static)
        for (int64_t i = row_begin; i < row_end; ++i) {
            uint64_t st[2] = {basis[2 * i], basis[2 * i + 1]};
            int sign = oracle_apply_state(T, st);
            if (sign != 0 && fabs(x[i]) > 1e-15) {
                int64_t J;
                sign *= oracle_search(basis, n, st, &J);
                if (sign != 0) {
                    double dy = c * x[i] * sign;
#pragma omp atomic
                    y[J] += dy;
                }
            }
        }
    }
    for (int t = 0; t < n_dg; ++t) {
        const oterm* T = dg[t];
        const double c = T->c;
#pragma omp parallel for schedule(static)
        for (int64_t i = row_begin; i < row_end; ++i) {
            uint64_t st[2] = {basis[2 * i], basis[2 * i + 1]};
            y[i] += c * x[i] * (double)oracle_apply_state(T, st);
        }
    }
    free(off);
    free(dg);
    return 0;
}

/* toSparseMatrix triplets in the reference's order; rows==NULL counts only. */
int64_t oracle_triplets(const uint64_t* basis, int64_t n, const oterm* terms, int n_terms, double tol, int64_t* rows,
                        int64_t* cols, double* vals) {
    const oterm** off = (const oterm**)malloc(sizeof(oterm*) * (size_t)(n_terms + 1));
    const oterm** dg = (const oterm**)malloc(sizeof(oterm*) * (size_t)(n_terms + 1));
    if (!off || !dg) return -1;
    int n_off, n_dg;
    split_terms(terms, n_terms, off, &n_off, dg, &n_dg);
    int64_t w = 0;
    for (int64_t j = 0; j < n; ++j) {
        for (int t = 0; t < n_off; ++t) {
            uint64_t st[2] = {basis[2 * j], basis[2 * j + 1]};
            int sign = oracle_apply_state(off[t], st);
            int64_t J = j;
            if (sign != 0) sign *= oracle_search(basis, n, st, &J);
            double res = off[t]->c * sign;
            if (fabs(res) > tol) {
                if (rows) {
                    rows[w] = J;
                    cols[w] = j;
                    vals[w] = res;
                }
                ++w;
            }
        }
        double acc = 0;
        for (int t = 0; t < n_dg; ++t) {
            uint64_t st[2] = {basis[2 * j], basis[2 * j + 1]};
            int sign = oracle_apply_state(dg[t], st);
            int64_t J = j;
            if (sign != 0) sign *= oracle_search(basis, n, st, &J);
            acc += dg[t]->c * sign;
        }
        if (rows) {
            rows[w] = j;
            cols[w] = j;
            vals[w] = acc;
        }
        ++w;
    }
    free(off);
    free(dg);
    return w;
}

/* _construct: right-to-left walk over (op, spin) pairs.  Returns 0, or -1 on
 * an unknown op character (bad_operator_spec). */
/* a *= b: SymbolicPMROperator::operator*= (operator.hpp:312-330).  The sign picks up (-1)^popcount(a.X & b.Z)
 * (moving b's Z through a's X), the Z and X masks combine by XOR, a's projector requirements are carried
 * through b's flips, and an up/down conflict kills the operator (sign 0).  Coefficients multiply. */
void oracle_term_mul(oterm* a, const oterm* b) {
    u128 aX = mk(a->x), aU = mk(a->up), aD = mk(a->down), bX = mk(b->x), bZ = mk(b->z);
    a->sign *= 1 - 2 * (popc128(aX & bZ) % 2);
    u128 Z = mk(a->z) ^ bZ, X = aX ^ bX;
    u128 req_up = (aD & bX) | (aU & ~bX);
    u128 req_dn = (aU & bX) | (aD & ~bX);
    u128 U = mk(b->up) | req_up, D = mk(b->down) | req_dn;
    if ((U & D) != 0) a->sign = 0;
    a->x[0] = (uint64_t)X, a->x[1] = (uint64_t)(X >> 64);
    a->z[0] = (uint64_t)Z, a->z[1] = (uint64_t)(Z >> 64);
    a->up[0] = (uint64_t)U, a->up[1] = (uint64_t)(U >> 64);
    a->down[0] = (uint64_t)D, a->down[1] = (uint64_t)(D >> 64);
    a->c *= b->c;
}

int oracle_term_compile(const char* ops, const int32_t* ids, int n, double c, oterm* out) {
    u128 X = 0, Z = 0, up = 0, down = 0;
    int sign = 1;
    for (int i = n - 1; i >= 0; --i) {
        const int J = ids[i];
        const u128 b = (u128)1 << J;
        switch (ops[i]) {
            case 'x': case 'X':
                X ^= b;
                if (Z & b) sign = -sign;
                break;
            case 'z': case 'Z':
                Z ^= b;
                break;
            case '+': case 'q': case 'Q':
                if (down & X & b) { sign = 0; break; }
                if (Z & b) sign = -sign;
                X ^= b;
                if (!(X & b)) up |= b;
                else down |= b;
                break;
            case '-':
                if (up & X & b) { sign = 0; break; }
                if (Z & b) sign = -sign;
                X ^= b;
                if (!(X & b)) down |= b;
                else up |= b;
                break;
            case 'p': case 'P':
                if (up & X & b) { sign = 0; break; }
                if (!(X & b)) down |= b;
                else up |= b;
                break;
            default:
                return -1;
        }
    }
    out->c = c;
    out->x[0] = (uint64_t)X, out->x[1] = (uint64_t)(X >> 64);
    out->z[0] = (uint64_t)Z, out->z[1] = (uint64_t)(Z >> 64);
    out->up[0] = (uint64_t)up, out->up[1] = (uint64_t)(up >> 64);
    out->down[0] = (uint64_t)down, out->down[1] = (uint64_t)(down >> 64);
    out->sign = sign;
    out->reserved = 0;
    return 0;
}

/* Plain three-term Lanczos step helpers for the CPU baseline of the Krylov
 * loop (lanczos.cpp:117-146 with OpenMP dot/axpy in place of BLAS). */
double oracle_dot(const double* a, const double* b, int64_t n) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

void oracle_axpby(double* y, const double* x, double a, double b, int64_t n) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) y[i] = b * y[i] + a * x[i];
}
