// Whole-file HDF5 datasets for other translation units of the library (checkpoint files), written and
// read by the minimal HDF5 implementation in h5lite.cpp.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace qsi {
namespace h5 {

struct OutDataset {
    std::string name;
    int type_class;  // 0 integer, 1 float, 3 string
    int type_size;
    std::vector<uint64_t> dims;  // empty = scalar
    std::vector<uint8_t> data;
    bool is_signed = false;      // integers only
};

// Writes a file holding exactly these datasets (throws std::runtime_error on failure).
void write_datasets(const char* path, const std::vector<OutDataset>& ds);
// Reads one dataset (any supported type) into out; false when the file or dataset is absent, throws on a
// malformed file.
bool read_dataset(const char* path, const char* name, OutDataset& out);

}  // namespace h5
}  // namespace qsi
