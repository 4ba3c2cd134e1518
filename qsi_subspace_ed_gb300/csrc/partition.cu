// Sublattice-polarisation sectors of a basis, on the GPU: the job of the reference's partition_basis tool
// (components/build_basis/partition_basis.cpp:13-231), which streams a basis file and appends every state to the
// dataset of its sector, named by make_sector_string (components/common/include/basis_io_h5.hpp:77-87) as
// basis_s<n0>.<n1>.<n2>.<n3> with n_a the state's up count on sublattice a.
//
// Here every state gets a sort key of its counts (8 bits per sublattice, the first sublattice most significant),
// a stable radix sort groups the states by sector while keeping the basis order inside each sector (so every
// sector's list stays sorted, as the reference's appends in basis order leave it), and runs of equal keys give
// the sectors.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include <cub/device/device_radix_sort.cuh>

#include "h5lite.h"
#include "qsi_device.cuh"
#include "qsi_handles.h"

namespace qsi {
namespace {

constexpr int kMaxSl = 8;

struct SlMasks {
    uint64_t m[kMaxSl][2];
    int n;
};

__global__ void k_sector_keys(const state2* __restrict__ s, int64_t n, SlMasks M, uint64_t* __restrict__ keys,
                              uint32_t* __restrict__ idx) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const state2 v = s[i];
        uint64_t k = 0;
        for (int a = 0; a < M.n; ++a)
            k = (k << 8) | (uint64_t)(__popcll(v.x & M.m[a][0]) + __popcll(v.y & M.m[a][1]));
        keys[i] = k;
        idx[i] = (uint32_t)i;
    }
}

__global__ void k_gather_states(const state2* __restrict__ s, const uint32_t* __restrict__ idx, int64_t n,
                                state2* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = s[idx[i]];
}

template <typename T>
struct Buf {
    T* p = nullptr;
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T)); }
    ~Buf() { cudaFree(p); }
};

struct Sector {
    std::vector<int> counts;
    int64_t start, end;
};

// Groups lohi by sector on the device; grouped (n x 2) and the sectors (key order) on the host.
qsi_status partition(const uint64_t* lohi, int64_t n, const uint64_t* sl_masks, int n_sl, std::vector<uint64_t>* grouped,
                     std::vector<Sector>& sectors) {
    if (n <= 0 || n >= (int64_t)UINT32_MAX) return fail(QSI_INVALID_ARG, "partition: basis of %lld states", (long long)n);
    SlMasks M{};
    M.n = n_sl;
    for (int a = 0; a < n_sl; ++a) M.m[a][0] = sl_masks[2 * a], M.m[a][1] = sl_masks[2 * a + 1];
    Buf<state2> d_s, d_out;
    Buf<uint64_t> keys, keys2;
    Buf<uint32_t> idx, idx2;
    QSI_CUDA(d_s.alloc(n));
    QSI_CUDA(keys.alloc(n));
    QSI_CUDA(keys2.alloc(n));
    QSI_CUDA(idx.alloc(n));
    QSI_CUDA(idx2.alloc(n));
    QSI_CUDA(cudaMemcpy(d_s.p, lohi, (size_t)n * 16, cudaMemcpyHostToDevice));
    k_sector_keys<<<grid_for(n, 256), 256>>>(d_s.p, n, M, keys.p, idx.p);
    QSI_CUDA(cudaGetLastError());
    size_t tmp_bytes = 0;
    QSI_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.p, keys2.p, idx.p, idx2.p, n, 0, 8 * n_sl));
    Buf<unsigned char> tmp;
    QSI_CUDA(tmp.alloc(tmp_bytes));
    QSI_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, keys.p, keys2.p, idx.p, idx2.p, n, 0, 8 * n_sl));
    std::vector<uint64_t> hk((size_t)n);
    QSI_CUDA(cudaMemcpy(hk.data(), keys2.p, (size_t)n * 8, cudaMemcpyDeviceToHost));
    if (grouped) {
        QSI_CUDA(d_out.alloc(n));
        k_gather_states<<<grid_for(n, 256), 256>>>(d_s.p, idx2.p, n, d_out.p);
        QSI_CUDA(cudaGetLastError());
        grouped->resize((size_t)n * 2);
        QSI_CUDA(cudaMemcpy(grouped->data(), d_out.p, (size_t)n * 16, cudaMemcpyDeviceToHost));
    }
    sectors.clear();
    for (int64_t i = 0; i < n;) {
        int64_t j = i + 1;
        while (j < n && hk[j] == hk[i]) ++j;
        Sector S;
        for (int a = 0; a < n_sl; ++a) S.counts.push_back((int)((hk[i] >> (8 * (n_sl - 1 - a))) & 0xff));
        S.start = i;
        S.end = j;
        sectors.push_back(std::move(S));
        i = j;
    }
    return QSI_OK;
}

std::string sector_name(const std::vector<int>& c) {
    std::string s = "basis_s";
    for (size_t a = 0; a < c.size(); ++a) s += (a ? "." : "") + std::to_string(c[a]);
    return s;
}

}  // namespace
}  // namespace qsi

using namespace qsi;

extern "C" qsi_status qsi_partition_basis(const uint64_t* lohi, int64_t n, const uint64_t* sl_masks, int32_t n_sl,
                                          uint64_t* out_lohi, int32_t* sector_counts, int64_t* sector_start,
                                          int32_t max_sectors, int32_t* n_sectors) {
    return guarded([&]() -> qsi_status {
        if (!lohi || !sl_masks || n_sl < 1 || n_sl > kMaxSl || !n_sectors || max_sectors < 0)
            return fail(QSI_INVALID_ARG, "qsi_partition_basis: bad argument");
        std::vector<uint64_t> grouped;
        std::vector<Sector> sectors;
        qsi_status s = partition(lohi, n, sl_masks, n_sl, out_lohi ? &grouped : nullptr, sectors);
        if (s != QSI_OK) return s;
        *n_sectors = (int32_t)sectors.size();
        if (!out_lohi) return QSI_OK;  // query: the number of sectors only
        if ((int64_t)sectors.size() > max_sectors)
            return fail(QSI_INVALID_ARG, "qsi_partition_basis: %zu sectors exceed max_sectors %d", sectors.size(),
                        max_sectors);
        std::memcpy(out_lohi, grouped.data(), (size_t)n * 16);
        for (size_t k = 0; k < sectors.size(); ++k) {
            if (sector_counts)
                for (int a = 0; a < n_sl; ++a) sector_counts[k * n_sl + a] = sectors[k].counts[a];
            if (sector_start) sector_start[k] = sectors[k].start;
        }
        if (sector_start) sector_start[sectors.size()] = n;
        return QSI_OK;
    });
}

extern "C" qsi_status qsi_partition_basis_h5(const char* in_path, const char* dataset, const char* out_path,
                                             const uint64_t* sl_masks, int32_t n_sl) {
    return guarded([&]() -> qsi_status {
        if (!in_path || !out_path || !sl_masks || n_sl < 1 || n_sl > kMaxSl)
            return fail(QSI_INVALID_ARG, "qsi_partition_basis_h5: bad argument");
        h5::OutDataset in;
        try {
            if (!h5::read_dataset(in_path, dataset ? dataset : "basis", in))
                return fail(QSI_NOT_FOUND, "%s: no dataset %s", in_path, dataset ? dataset : "basis");
        } catch (const std::exception& e) {
            return fail(QSI_IO_ERROR, "%s: %s", in_path, e.what());
        }
        if (in.type_class != 0 || in.type_size != 8 || in.dims.size() != 2 || in.dims[1] != 2)
            return fail(QSI_IO_ERROR, "%s: the basis must be a (N, 2) 64-bit integer dataset", in_path);
        const int64_t n = (int64_t)in.dims[0];
        std::vector<uint64_t> grouped;
        std::vector<Sector> sectors;
        qsi_status s = partition(reinterpret_cast<const uint64_t*>(in.data.data()), n, sl_masks, n_sl, &grouped, sectors);
        if (s != QSI_OK) return s;
        std::vector<h5::OutDataset> out;
        for (const Sector& S : sectors) {
            h5::OutDataset o;
            o.name = sector_name(S.counts);
            o.type_class = 0;
            o.type_size = 8;
            o.dims = {(uint64_t)(S.end - S.start), 2};
            o.data.resize((size_t)(S.end - S.start) * 16);
            std::memcpy(o.data.data(), grouped.data() + 2 * S.start, o.data.size());
            out.push_back(std::move(o));
        }
        try {
            h5::write_datasets(out_path, out);
        } catch (const std::exception& e) {
            return fail(QSI_IO_ERROR, "%s: %s", out_path, e.what());
        }
        return QSI_OK;
    });
}
