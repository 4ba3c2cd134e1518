// Handle layouts behind the opaque qsi_basis / qsi_op pointers of the C-ABI.
#pragma once
#include <cuda_runtime.h>
#include <vector>

#include "qsi_device.cuh"

struct qsi_basis {
    int64_t n = 0;
    int bits = 0, shift = 0;
    uint32_t n_buckets = 0;
    qsi::state2* d_states = nullptr;
    uint32_t* d_bstart = nullptr;
    int hb = 0;                        // highest bit used by any state
    qsi::HashSlot* d_hash = nullptr;   // optional regional hash index over the bucket table (states <= 96 bits)
    uint64_t hash_slots = 0;           // 2n
    qsi::BasisView view() const { return qsi::BasisView{d_states, d_bstart, n, shift, n_buckets}; }
    qsi::HashView hview() const { return qsi::HashView{d_hash, view()}; }
};

// Launch settings of one class of applies (single vector, batched).  None of them changes results.
struct qsi_tuning {
    int use_hash = 1;    // look columns up through the basis hash index when it exists (else bucket table)
    int list_cap = 256;  // hit-list entries per warp in the batched tile kernel
    int grid_bps = 0;    // tile-kernel blocks per SM (0: built-in choice)
    int vec_chunk = 0;   // vectors per pass of the 16-byte batched kernel (0: up to 32 lanes' worth)
    int vec_width = 0;   // FP32 vectors per lane of the 16-byte batched kernel: 4 (0), 8 or 16
};

struct qsi_family;

struct qsi_op {
    qsi_basis* basis = nullptr;
    qsi_family* family = nullptr;  // member of an operator family: FP64 single-vector applies join its batches
    double* d_fcoef = nullptr;     // the member's class coefficients on the device (family mode, one column)
    std::vector<double> fcoef;     // ... and on the host
    qsi::PullTerm* d_pull = nullptr;        // transposed off-diagonal terms (apply)
    qsi::PushTerm* d_push_off = nullptr;    // off-diagonal terms as given (export)
    qsi::PushTerm* d_push_diag = nullptr;   // diagonal terms as given (export)
    qsi::PushTerm* d_diag_generic = nullptr;
    int n_pull = 0, n_push_off = 0, n_push_diag = 0, n_diag_generic = 0;
    int n_pull_pruned = 0;                  // transposed terms removed because they map no row into the basis
    qsi::DiagSpec diag{};
    size_t smem_bytes = 0;
    // bit-sliced admission tests: per pull term, literals (spin | 0x80 when the spin must be down)
    uint16_t* d_lit_off = nullptr;  // n_pull + 1 offsets
    uint8_t* d_lits = nullptr;
    int n_lits = 0;
    int nwords = 4;                 // 32-bit words that hold any basis or term bit
    int kernel = 1;                 // 0 = row-per-thread / warp-per-row, 1 = bit-sliced tiles
    int ff_accumulate = 1;          // FP32 batched applies accumulate rows in double-float (else FP64)
    qsi_tuning tune[2];             // [0] single-vector applies, [1] batched applies (R > 1)
    double* d_diag = nullptr;       // per-row diagonal (tile kernels)
    float2* d_diag_ff = nullptr;    // the same as double-float pairs (FP32 batched kernel)
    uint32_t* d_cache_cols = nullptr;  // lookup cache of the materialised operator (qsi_op_materialise), or null
    uint64_t* d_cache_off = nullptr;   // its tile offsets in 32-entry lines
    void* d_cache_tid = nullptr;       // the term index of every entry (uint8, or uint16 beyond 256 terms)
    int cache_tid_bytes = 1;
    size_t cache_entries = 0;
    cudaStream_t stream = nullptr;
    int device = 0;        // the device current at qsi_op_create (owner of every buffer and of the stream)
    void* d_x = nullptr;   // staging for host-pointer applies
    void* d_y = nullptr;
    size_t staging_bytes = 0;
};

namespace qsi {
int grid_for(int64_t n, int block);
qsi_status launch_apply(qsi_op* op, const void* x, void* y, int R, int dtype, int accumulate, cudaStream_t st);
// y = H x with x stored as xdtype and y always FP64 (single vector).
qsi_status launch_apply_to_f64(qsi_op* op, const void* x, double* y, int xdtype, cudaStream_t st);
qsi_status launch_apply_tiles(qsi_op* op, const void* x, void* y, int R, int xdtype, int ydtype, int accumulate,
                              cudaStream_t st);
// Family mode apply of a family's template operator: y = H(p_c) x per column c of [row][R] FP64 blocks.
qsi_status launch_family(qsi_op* tmpl, const double* x, double* y, int R, const double* fcoef, int accumulate,
                         cudaStream_t st);
// A member's single-vector FP64 apply, run in a batch with the family's other waiting members.
qsi_status family_apply(qsi_op* op, const double* x, double* y, int accumulate, cudaStream_t st);
// Called by qsi_op_destroy for a family member.
void family_release_member(qsi_op* op);
qsi_status build_hash(qsi_basis* b);
// Builds (enable) or frees an operator's lookup cache (qsi_op_materialise); *bytes: its size in device memory.
qsi_status materialise(qsi_op* op, bool enable, int64_t* bytes);
// Bucket table of a basis at its current width (b->bits, b->shift, b->n_buckets), allocated with padding for the
// 16-byte reads of bucket_bounds.
qsi_status build_buckets(qsi_basis* b);
// Loads the single-vector FP64 apply kernels on the current device (CUDA loads device code lazily, on first use).
qsi_status preload_apply_f64();
// Looks the static staging arrays of qsi_op_apply_static up on the current device (once per device).
qsi_status static_stage_prepare();
qsi_status build_diag(qsi_op* op);
struct SectorPlan {
    std::vector<unsigned char> records;  // one launch record per sector, to be copied to device memory
    size_t smem = 0;
    int maxR = 1, grid = 0, n = 0;
    bool vec4 = true;  // every sector's R and vectors take 16-byte gathers
    bool vec8 = true;  // ... of 8 vectors per lane, and every sector's batched applies are set to them
    bool vec16 = true; // ... of 16 vectors per lane, likewise
    bool hash = true;  // every sector's batched applies look columns up through the hash index
    bool cache = true; // every sector is materialised (qsi_op_materialise): columns come from the lookup caches
};
qsi_status plan_sectors(qsi_op* const* ops, int n, const float* const* X, float* const* Y, const int* R,
                        SectorPlan& plan, const double* weights = nullptr, const float2* const* ycoef = nullptr);
qsi_status launch_sectors(const void* d_records, const SectorPlan& plan, int accumulate, cudaStream_t st);
qsi_status jacobi_eigh(const std::vector<double>& A, int m, int n_mat, std::vector<double>& w, std::vector<double>& V, cudaStream_t st);
}  // namespace qsi
