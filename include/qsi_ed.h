/*
 * qsi_ed.h — C-ABI of the GB300 matrix-free Hamiltonian engine for
 * projected exact diagonalisation of quantum-spin-ice ring-exchange models.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and
 * returns a qsi_status.  No C++ exception crosses this boundary; the text of
 * the last error on the calling thread is available from qsi_last_error().
 *
 * Conventions (shared with qsi_subspace_ED):
 *   - spin i is bit i of a 128-bit state; 1 = up, 0 = down
 *     (components/common/include/bittools.hpp:69-81, README.md:146);
 *   - a 128-bit state is stored as two uint64 words, LOW word first
 *     (Uint128::uint64[0] is the low word; the HDF5 basis row is [lo, hi],
 *     components/common/include/basis_io_h5.hpp:34,55);
 *   - a basis is a strictly increasing array of such states.
 *
 * Pointer kinds: entry points that take vectors accept either host or device
 * memory, selected by QSI_PTR_HOST / QSI_PTR_DEVICE in `flags`.  With host
 * pointers the call copies in, computes on the GPU and copies out, and is
 * synchronous; a page-locked (pinned) result buffer of an apply without
 * accumulation is written by the kernel directly, without a staging copy.  With device pointers the work is enqueued on `stream`
 * (a cudaStream_t, or NULL for the handle's own stream).
 */
#ifndef QSI_ED_H
#define QSI_ED_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum qsi_status {
    QSI_OK = 0,
    QSI_INVALID_ARG = 1,   /* bad spec / size / pointer (bad_operator_spec, std::logic_error) */
    QSI_OOM = 2,           /* device or host allocation failed */
    QSI_CUDA_ERROR = 3,    /* a CUDA runtime call failed */
    QSI_NOT_CONVERGED = 4, /* solver hit its iteration limit (Spectra CompInfo != Successful) */
    QSI_TIMEOUT = 5,       /* a bounded wait ran out */
    QSI_IO_ERROR = 6,      /* file missing / malformed (std::runtime_error in basis IO) */
    QSI_NOT_FOUND = 7      /* dataset or state not present */
} qsi_status;

enum { QSI_PTR_HOST = 0, QSI_PTR_DEVICE = 1 };
enum { QSI_F64 = 0, QSI_F32 = 1 };

/* One compiled operator term: coefficient times SymbolicPMROperator.
 * The mask fields are exactly SymbolicPMROperator's protected members
 * (components/operator/include/operator.hpp:343-347), each as [lo, hi]. */
typedef struct qsi_term {
    double c;
    uint64_t x[2];     /* X_mask: bits flipped */
    uint64_t z[2];     /* Z_mask: sign (-1)^popcount(~state' & Z) */
    uint64_t up[2];    /* state & up must equal up */
    uint64_t down[2];  /* state & down must be 0 */
    int32_t sign;      /* overall sign, 0 when the operator vanished at construction */
    int32_t reserved;
} qsi_term;

typedef struct qsi_basis qsi_basis; /* device-resident sorted basis + bucket table */
typedef struct qsi_op qsi_op;       /* operator bound to a basis */
typedef struct qsi_family qsi_family; /* operators H(p) = sum_t p[class(t)] term_t over one basis */

/* ---------------------------------------------------------------- errors */
const char* qsi_version(void);
/* Copies the calling thread's last error message into buf (NUL-terminated). */
qsi_status qsi_last_error(char* buf, size_t len);

/* ---------------------------------------------------------------- terms */
/* SymbolicPMROperator(opstring, spin_ids) (operator.hpp:223-227, _construct
 * :383-466).  ops is a string of n characters from "xXzZ+-pPqQ". */
qsi_status qsi_term_compile(const char* ops, const int32_t* spin_ids, int32_t n,
                            double c, qsi_term* out);
/* SymbolicPMROperator(const std::string& spec), e.g. "0+ 1- 12z"
 * (operator.hpp:229-232, parseSpec :349-381). */
qsi_status qsi_term_parse(const char* spec, double c, qsi_term* out);
/* a *= b (SymbolicPMROperator::operator*=, operator.hpp:312-330); coefficients multiply. */
qsi_status qsi_term_mul(qsi_term* a, const qsi_term* b);
/* Applies one term to one state, as SymbolicPMROperator::applyState
 * (operator.hpp:232-254): state is updated in place, the sign is returned in *sign. */
qsi_status qsi_term_apply_state(const qsi_term* t, uint64_t state[2], int32_t* sign);

/* ---------------------------------------------------------------- basis files */
/* Reads dataset `dataset` (uint64[N][2]) of an HDF5 basis file
 * (basis_io::read_basis_hdf5, basis_io_h5.hpp:90-141).  Call with out=NULL to
 * learn n; then call again with cap >= n. */
qsi_status qsi_h5_read_basis(const char* path, const char* dataset,
                             uint64_t* out_lohi, int64_t cap, int64_t* n_out);
/* Reads a float64 dataset of any rank; dims_out receives up to 4 dims. */
qsi_status qsi_h5_read_f64(const char* path, const char* dataset, double* out,
                           int64_t cap, int64_t* n_out, int64_t* dims_out, int32_t* rank_out);
/* Writes a basis file with one uint64[N][2] dataset per call (creates or
 * truncates the file when `append` is 0) (basis_io_h5.hpp:30-70). */
qsi_status qsi_h5_write_basis(const char* path, const char* dataset,
                              const uint64_t* lohi, int64_t n, int32_t append);
/* Writes the .eigs.h5 layout of diag_DOQSI_ham (src/diag_DOQSI_ham.cpp:143-173):
 * eigenvalues (nev), eigenvectors (dim x nvec, the Eigen column-major bytes
 * under a row-major (dim, nvec) shape), latfile_json and dset_name strings. */
qsi_status qsi_h5_write_eigs(const char* path, const double* evals, int64_t nev,
                             const double* evecs, int64_t dim, int64_t nvec,
                             const char* latfile_json, const char* dset_name);
/* One float64 dataset of any rank (dims[rank]) / one fixed-length string
 * dataset, in a new file (append = 0) or added to a file this library wrote
 * (append = 1): the datasets of eval_observables' .out.h5 file
 * (src/expectation_eval.cpp:127-230, src/eval_observables.cpp:119-130). */
qsi_status qsi_h5_write_f64(const char* path, const char* dataset, const double* data,
                            const int64_t* dims, int32_t rank, int32_t append);
qsi_status qsi_h5_write_string(const char* path, const char* dataset, const char* text, int32_t append);
/* Reads a string dataset (fixed-length, or the variable-length strings the
 * reference writes for latfile_json / dset_name) into buf (NUL-terminated). */
qsi_status qsi_h5_read_string(const char* path, const char* dataset, char* buf, size_t len);
/* CSV basis "0x%016hi%016lo" per line (basis_io.hpp:16-53). */
qsi_status qsi_csv_read_basis(const char* path, uint64_t* out_lohi, int64_t cap, int64_t* n_out);

/* ---------------------------------------------------------------- enumeration */
/* Enumerates the spin-ice basis: every state whose tetrahedra satisfy the
 * ice rule (member count up in [n/2, (n+1)/2]), with up to n_spinon_pairs
 * rule violations admitted by the gen_spinon_basis rule
 * (components/build_basis/src/pyro_tree.cpp:20-189), optionally restricted to
 * a sublattice polarisation sector.  tetra_spins holds n_tetra rows of
 * tetra_size spin ids.  ordering: 0 = spins in index order, 1 = the greedy
 * tetrahedron-overlap order of lattice::greedy_spin_ordering
 * (components/common/src/tetra_graph_io.cpp:105-150).  sector may be NULL.
 * The result is sorted and written to *out_lohi (release with qsi_free_host). */
qsi_status qsi_enumerate_basis(int32_t n_spins, const int32_t* tetra_spins,
                               int32_t n_tetra, int32_t tetra_size,
                               const int32_t* sublattice, int32_t n_sublattices,
                               int32_t n_spinon_pairs, const int32_t* sector,
                               int32_t ordering, int32_t n_threads,
                               uint64_t** out_lohi, int64_t* n_out);
void qsi_free_host(void* p);
/* The same enumeration on the GPU (ordering is the greedy order; states of at
 * most 128 spins, at most 128 tetrahedra and 8 sublattices), with up to 64
 * spinon pairs: the forking rule of fork_state_impl
 * (components/build_basis/src/pyro_tree.cpp:168-189) with the reference's own
 * admission test, so the set equals qsi_enumerate_basis's.  The sorted result
 * is returned in host memory (release with qsi_free_host). */
qsi_status qsi_enumerate_basis_gpu(int32_t n_spins, const int32_t* tetra_spins,
                                   int32_t n_tetra, int32_t tetra_size,
                                   const int32_t* sublattice, int32_t n_sublattices,
                                   const int32_t* sector, int32_t n_spinon_pairs,
                                   uint64_t** out_lohi, int64_t* n_out);
/* Sublattice-polarisation sectors of a basis, on the GPU (replaces
 * partition_basis_hdf5, components/build_basis/partition_basis.cpp:13-231):
 * the sector of a state is its up count on each of the n_sl (1..8) sublattice
 * masks (sl_masks: n_sl (lo, hi) pairs).  out_lohi (n x 2) receives the states
 * grouped by sector, sectors in ascending order of their counts (first
 * sublattice most significant), basis order kept inside each sector;
 * sector_counts (n_sectors x n_sl) and sector_start (n_sectors + 1 entries,
 * the last = n) describe the groups.  With out_lohi NULL only *n_sectors is
 * set; more sectors than max_sectors is QSI_INVALID_ARG. */
qsi_status qsi_partition_basis(const uint64_t* lohi, int64_t n, const uint64_t* sl_masks,
                               int32_t n_sl, uint64_t* out_lohi, int32_t* sector_counts,
                               int64_t* sector_start, int32_t max_sectors, int32_t* n_sectors);
/* The partition_basis tool (partition_basis.cpp:231-269): reads the basis
 * dataset (NULL: "basis") of in_path and writes out_path with one dataset per
 * sector, named as make_sector_string names it (basis_io_h5.hpp:77-87):
 * basis_s<n0>.<n1>...  (the datasets diag_DOQSI_ham --sector reads). */
qsi_status qsi_partition_basis_h5(const char* in_path, const char* dataset, const char* out_path,
                                  const uint64_t* sl_masks, int32_t n_sl);

/* ---------------------------------------------------------------- device basis */
/* Copies a sorted basis to the device and builds its top-bits bucket table.
 * bucket_bits <= 0 picks a size automatically.  The caller keeps its buffer
 * (LazyOpSum holds a non-owning basis reference, operator_matrix.hpp:116). */
qsi_status qsi_basis_create(const uint64_t* lohi, int64_t n, int32_t bucket_bits,
                            qsi_basis** out);
qsi_status qsi_basis_destroy(qsi_basis* b);
qsi_status qsi_basis_dim(const qsi_basis* b, int64_t* dim);
/* Rebuilds the lookup index: a top-bits bucket table with bucket_bits bits
 * (<= 0 keeps the current table) and, with use_hash, an open-addressing
 * hash index of the states (states of at most 96 bits).  Column lookups use
 * the hash index when present and enabled on the operator, else the bucket
 * table plus a binary search of the bucket. */
qsi_status qsi_basis_index(qsi_basis* b, int32_t use_hash, int32_t bucket_bits);
qsi_status qsi_basis_info(const qsi_basis* b, int32_t* bucket_bits, int32_t* has_hash,
                          int64_t* index_bytes);
/* Exact index lookup of n states (ZBasisBST::search, operator.cpp:4-34):
 * idx[k] = position of states[k] in the basis, or -1 on a miss. */
qsi_status qsi_basis_search(qsi_basis* b, const uint64_t* states_lohi, int64_t n,
                            int64_t* idx, int32_t flags, void* stream);

/* ---------------------------------------------------------------- operator */
/* LazyOpSum(basis, ops) (operator_matrix.hpp:13-17): copies the term list. */
qsi_status qsi_op_create(qsi_basis* b, const qsi_term* terms, int32_t n_terms,
                         qsi_op** out);
qsi_status qsi_op_destroy(qsi_op* op);
/* Materialises the operator, as the reference does with LazyOpSum::toSparseMatrix before its sparse solvers
 * (diag_DOQSI_ham --algorithm sparse, include/matrix_diag_bits.hpp:181-189; ftlm_DOQSI_ham,
 * src/ftlm_DOQSI_ham.cpp:150-153): enable = 1 stores the column of every admitted term of every row in device
 * memory (4 bytes per term, in 32-row tiles), so later applies of any kind read columns instead of looking them
 * up; enable = 0 frees it.  Applies give bitwise the results of the matrix-free apply either way.  *bytes (may
 * be NULL): the cache's size. */
qsi_status qsi_op_materialise(qsi_op* op, int32_t enable, int64_t* bytes);
/* Operator families for serving many parameter points of one sector at once (the request loop that replaces
 * the reference's static phase-diagram plans, driver/ed_phasedia_plan.sh:21-25 with
 * driver/execute_asynchronous.sh:1-38; no counterpart in the operator code): the terms of qsi_op_create with a
 * class per term (term_class[t] < n_classes <= 16; diagonal terms must be single-site z), H(p) has coefficient
 * p[class(t)] on term t (the terms' own coefficients are ignored).  qsi_family_member returns H(p) as an
 * ordinary operator (every entry point takes it; release with qsi_op_destroy); its FP64 single-vector applies
 * are queued with the family and the applies of all members waiting at the same time run as one batched apply,
 * one column per member (at most max_cols <= 32), so concurrent solves share every lookup.  A member's results
 * are bitwise the same whether its applies ran alone or batched.  Members may be used from several host
 * threads at once (one thread per member). */
qsi_status qsi_family_create(qsi_basis* b, const qsi_term* terms, int32_t n_terms,
                             const int32_t* term_class, int32_t n_classes, int32_t max_cols,
                             qsi_family** out);
qsi_status qsi_family_destroy(qsi_family* f);
qsi_status qsi_family_member(qsi_family* f, const double* p, qsi_op** out);
/* Batches run and member applies they served (applies / batches = mean columns per batch). */
qsi_status qsi_family_stats(const qsi_family* f, int64_t* batches, int64_t* applies);
/* Bases with fewer than min_rows states are not batched (default 131072): their applies take about a kernel
 * launch, less than queueing for partners costs, so each member's apply runs at once on its own stream (same
 * kernel and sums; a batch of one).  0 batches every basis. */
qsi_status qsi_family_set_min_rows(qsi_family* f, int64_t min_rows);
/* accumulate = 0: y = H x   (LazyOpSumProd::perform_op / LazyOpSum::evaluate,
 *                            operator_matrix.hpp:32-36,129-131)
 * accumulate = 1: y += H x  (LazyOpSum::evaluate_add, operator_matrix.cpp:108-112;
 *                            the RealApplyFn contract, common_bits.hpp:18-23) */
qsi_status qsi_op_apply(qsi_op* op, const double* x, double* y, int32_t accumulate,
                        int32_t flags, void* stream);
/* y = H x (accumulate = 0) or y += H x (accumulate = 1) for HOST x and y,
 * without allocating device memory: the vectors are staged through two
 * fixed arrays compiled into the library, for callers whose process cannot
 * make new device allocations (GPU memory owned by another allocator or an
 * exhausted quota).  The arrays (4 MiB) and the apply kernels' code are
 * reserved on a device by the first qsi_op_create there (CUDA loads device
 * code lazily), not at library load; the call itself then reserves nothing.
 * At most 262,144 basis states (QSI_INVALID_ARG beyond).  Calls share the
 * arrays: calls that overlap on the GPU race; consecutive calls from one
 * thread do not.  A call runs on the operator's device whatever the current
 * device is.  No counterpart in the reference. */
qsi_status qsi_op_apply_static(qsi_op* op, const double* x, double* y, int32_t accumulate);
/* Batched apply over R vectors stored row-major [dim][R] (element type dtype:
 * QSI_F64, or QSI_F32 storage with FP64 per-row accumulation). */
qsi_status qsi_op_apply_batched(qsi_op* op, const void* X, void* Y, int32_t R,
                                int32_t dtype, int32_t accumulate, int32_t flags,
                                void* stream);
/* Shape of the operator as the apply runs it: off-diagonal terms applied (in
 * transposed form), off-diagonal terms removed at creation because their
 * flipped state lies in the basis for no row (every contribution of such a
 * term is a dropped miss, so removing it changes no result), single-site
 * Z classes folded into the per-row diagonal, and other diagonal terms.
 * No counterpart in the reference. */
qsi_status qsi_op_info(const qsi_op* op, int32_t* n_offdiag, int32_t* n_pruned,
                       int32_t* n_diag_classes, int32_t* n_diag_generic);
/* Kernel selection (autotuning): kernel 0 = one row per thread (single
 * vector) / one warp per row (batched); kernel 1 = bit-sliced 32-row tiles
 * (default).  use_hash bit 0 selects the hash index for column lookups; bit 1
 * makes FP32 batched applies accumulate rows in FP64 instead of double-float
 * (two FP32 words, about 2^-48 relative; the default, since FP64 issue is
 * slow on this GPU);
 * list_cap (> 0) sets the per-warp hit-list size of the batched tile kernel. */
qsi_status qsi_op_set_kernel(qsi_op* op, int32_t kernel, int32_t use_hash, int32_t list_cap);
/* Launch settings of the tile kernels, kept separately for single-vector
 * applies (which = 0) and batched applies (which = 1; -1 sets both):
 * grid_bps = blocks per SM (0 = built-in choice), vec_width = FP32 vectors
 * per lane of the batched kernel (0 or 4, 8, 16), vec_chunk = vectors per pass
 * (0, 16, 32, 64, 128, 256 or 512; 0 = 32 lanes' worth).  qsi_op_get_tuning also
 * reports the kernel, use_hash (as qsi_op_set_kernel takes it) and list_cap
 * of that class.  No counterpart in the reference (its apply is an OpenMP
 * loop with nothing to tune); results do not depend on these settings. */
qsi_status qsi_op_set_tuning(qsi_op* op, int32_t which, int32_t grid_bps, int32_t vec_chunk,
                             int32_t vec_width);
qsi_status qsi_op_get_tuning(const qsi_op* op, int32_t which, int32_t* kernel, int32_t* use_hash,
                             int32_t* list_cap, int32_t* grid_bps, int32_t* vec_chunk,
                             int32_t* vec_width);
/* Autotuner: times applies of R vectors of type dtype (x, y device buffers
 * of dim*R elements, or NULL for scratch the call allocates and frees) and
 * keeps, for the class of R (single vector or batched), the fastest lookup
 * structure (with QSI_TUNE_INDEX: the hash index or the bucket table at
 * several widths, and the basis keeps the width chosen; with QSI_TUNE_LOOKUP:
 * the hash index or the table at its current width), vectors per pass, blocks
 * per SM and hit-list size, one parameter at a time, best of reps timed
 * applies each.
 * report (optional) receives one line per trial.  Results of later applies
 * are the same for every setting; only their speed changes.  No counterpart
 * in the reference. */
enum { QSI_TUNE_INDEX = 1, QSI_TUNE_LOOKUP = 2 };
qsi_status qsi_op_autotune(qsi_op* op, const void* x, void* y, int32_t R, int32_t dtype,
                           int32_t flags, int32_t reps, char* report, size_t report_len);
/* Connectivity export in the order of LazyOpSum::toSparseMatrix
 * (operator_matrix.hpp:79-105): for each basis index j, each off-diagonal
 * term with |c*sign| > tol gives (J, j, c*sign); then (j, j, sum of diagonal
 * terms).  Call with rows=NULL to get the count. */
qsi_status qsi_op_triplets(qsi_op* op, double tol, int64_t* rows, int64_t* cols,
                           double* vals, int64_t cap, int64_t* n_out);
/* MatrixMarket file of the matrix toSparseMatrix assembles, as build_hamiltonian
 * writes it with Eigen::saveMarket (src/build_hamiltonian.cpp:104-111):
 * duplicates summed, column-major order, explicit zeros kept, 1-based
 * indices, values "%.17e".  *nnz_out (optional) receives the entry count. */
qsi_status qsi_op_write_mtx(qsi_op* op, const char* path, double tol, int64_t* nnz_out);
/* Number of off-diagonal terms whose flipped state is not in the basis,
 * summed over all rows (projected-ED drops them). */
qsi_status qsi_op_count_misses(qsi_op* op, int64_t* misses);
/* Off-diagonal terms over all rows that land in the basis (hits: the
 * off-diagonal non-zeros of H) and that leave it (misses). */
qsi_status qsi_op_connectivity(qsi_op* op, int64_t* hits, int64_t* misses);

/* ---------------------------------------------------------------- solvers */
typedef struct qsi_lanczos_cfg {
    int32_t nev;          /* eigenpairs wanted (smallest algebraic) */
    int32_t ncv;          /* Krylov subspace dimension (-k/--ncv) */
    int32_t max_iter;     /* restart limit (--max_iters) */
    int32_t precision;    /* QSI_F64, or QSI_F32 = FP32 vectors + FP64 recurrences */
    double tol;           /* relative residual tolerance (10^--atol) */
    uint64_t seed;        /* start vector seed (N(0,1)) */
    int32_t polish_steps; /* FP64 Rayleigh-Ritz polish rounds after convergence; with QSI_F32 and
                             >= 2 rounds the FP32 Krylov phase stops at max(tol, 1e-7), ten times
                             looser per round beyond two (at most 1e-4), and the FP64 rounds (the
                             2nd and later on [X, HX - X theta]) refine the pairs */
    int32_t want_vectors; /* write eigenvectors */
    int32_t block;        /* QSI_F32 only: 16 = block Lanczos on FP32 blocks of 16 vectors through the
                             batched apply (nev <= 13); 0 or 1 = single-vector Lanczos on FP32 vectors */
    int32_t reserved;
} qsi_lanczos_cfg;

typedef struct qsi_report {
    int32_t converged;      /* eigenpairs converged */
    int32_t restarts;
    int64_t applies;        /* operator applications */
    double residual[64];    /* ||H v - lambda v|| per eigenpair (FP64) */
    double seconds;
} qsi_report;

/* Thick-restart Lanczos for the nev smallest eigenpairs with full
 * reorthogonalisation (the mfsparse path: compute_spectrum_iterative,
 * include/matrix_diag_bits.hpp:51-95).  evecs is dim x nev, vector-major. */
qsi_status qsi_lanczos_solve(qsi_op* op, const qsi_lanczos_cfg* cfg, double* evals,
                             double* evecs, qsi_report* report);

/* Plain 3-term Lanczos ground state without reorthogonalisation and the
 * two-pass eigenvector of projED::lanczos::eigval0 (mfeig0 path,
 * components/linalg_routines/src/lanczos.cpp:67-227). */
typedef struct qsi_eigval0_cfg {
    int32_t max_iterations;
    int32_t min_iterations;
    double abs_tol;
    double rel_tol;
    uint64_t seed;
    int32_t calc_eigenvector;
    int32_t reserved;
} qsi_eigval0_cfg;
qsi_status qsi_eigval0(qsi_op* op, const qsi_eigval0_cfg* cfg, double* e0,
                       double* eigvec, int32_t* iterations);
/* qsi_eigval0 with checkpoint/resume of its first (Lanczos) pass, the
 * checkpoint of the reference's long-run drivers
 * (components/operator/include/checkpoint_utils.hpp:48-313): an HDF5 file at
 * `path` with datasets v and u (the current and previous Lanczos vectors,
 * FP64[dim]), alphas, betas, beta, iteration (uint64), eigval (the current
 * lowest Ritz value) and random_seed (int32).  If `path` holds a checkpoint
 * of this run (same dimension and seed) the first pass resumes from it, and
 * the results are bitwise those of an uninterrupted run.  A checkpoint is
 * written every `every` iterations (0: only on stopping) and when the call
 * stops early: after `stop_after` iterations of this call (> 0) or after
 * `wall_limit_s` seconds (> 0; the role of the reference's SLURM end-time
 * check, checkpoint_utils.hpp:18-46), returning QSI_TIMEOUT.  Files are
 * written to path.tmp and renamed over path. */
qsi_status qsi_eigval0_checkpointed(qsi_op* op, const qsi_eigval0_cfg* cfg, const char* path,
                                    int32_t every, int32_t stop_after, double wall_limit_s,
                                    double* e0, double* eigvec, int32_t* iterations);

/* Finite-temperature Lanczos over several sectors at once.  Each sector s has
 * an operator ops[s] and R[s] random vectors; all run M Lanczos steps in one
 * batched apply per step.  Outputs per sector: alphas/betas of every vector
 * (R[s] x M each, concatenated over sectors). */
qsi_status qsi_ftlm_run(qsi_op** ops, int32_t n_sectors, const int32_t* R,
                        int32_t M, uint64_t seed, int32_t precision,
                        double* alphas, double* betas);

/* qsi_ftlm_run with the number of R-vector blocks kept per sector: 3 (H q in
 * its own block), 2 (in-place recurrence: H q accumulated into the previous
 * vector block, so R can double at the same device-memory footprint), or 0 =
 * three when they fit in free device memory, else two (what qsi_ftlm_run
 * does).  Both layouts give the same recurrences up to rounding. */
qsi_status qsi_ftlm_run_blocks(qsi_op** ops, int32_t n_sectors, const int32_t* R,
                               int32_t M, uint64_t seed, int32_t precision,
                               int32_t blocks, double* alphas, double* betas);

/* Expectation values of n_ops operators between nvec vectors, as eval_observables
 * computes them (src/expectation_eval.cpp:27-110, src/eval_observables.cpp:134-208):
 * operator l is the term list terms[op_offsets[l] .. op_offsets[l+1]) (a
 * SymbolicOpSum) bound to basis b; psi holds the vectors column by column
 * (dim x nvec, Eigen's column-major layout, 1 <= nvec <= 256).
 *   expect[(l*nvec + i)*nvec + j]            = psi_j . (O_l psi_i)
 *   cross[((l*n_ops + m)*nvec + i)*nvec + j] = (O_l psi_i) . (O_m psi_j)   (optional)
 * FP64 on the device; cross keeps all n_ops*nvec vectors O_l psi_i resident. */
qsi_status qsi_expectations(qsi_basis* b, const qsi_term* terms, const int32_t* op_offsets,
                            int32_t n_ops, const double* psi, int32_t nvec, double* expect,
                            double* cross);

/* Batched eigen-decomposition of n_mat symmetric tridiagonal m x m matrices
 * (diagonals a[k*m..], off-diagonals b[k*m..], the first m-1 used), m <= 128:
 * ascending eigenvalues and the first component of each eigenvector — the
 * Ritz values and weights of FTLM (the dense tridiagonal solve of
 * components/linalg_routines/include/lapack_adapter.hpp:37-91, batched). */
qsi_status qsi_tridiag_ritz(const double* a, const double* b, int32_t m, int32_t n_mat,
                            double* evals, double* first);

#ifdef __cplusplus
}
#endif
#endif /* QSI_ED_H */
