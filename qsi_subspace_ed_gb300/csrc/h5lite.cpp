// Minimal HDF5 reader/writer for the files of qsi_subspace_ED's basis and
// eigen-output layout: superblock version 0/1, version-1 object headers,
// symbol-table groups (v1 B-tree + local heap), contiguous or compact
// datasets.  That is what libhdf5 writes with default properties, which is
// how the reference creates every file on this path
// (components/common/include/basis_io_h5.hpp:30-141,
//  src/expectation_eval.cpp:127, src/diag_DOQSI_ham.cpp:143-173).
//
// The writer emits the same structures with fixed-length strings (the
// reference writes variable-length strings for latfile_json / dset_name).
#include <algorithm>
#include <cassert>
#include <cerrno>
#include <cstring>
#include <fstream>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "h5lite.h"
#include "qsi_internal.h"

namespace qsi {
namespace h5 {

struct Reader {
    std::vector<uint8_t> buf;
    uint64_t base = 0;
    int so = 8, sl = 8;  // sizes of offsets and lengths

    uint64_t rd(uint64_t pos, int n) const {
        if (pos > buf.size() || n > buf.size() - pos) throw std::runtime_error("HDF5: read past end of file");
        uint64_t v = 0;
        for (int i = 0; i < n; ++i) v |= (uint64_t)buf[pos + i] << (8 * i);
        return v;
    }
    const uint8_t* at(uint64_t pos, uint64_t n) const {
        if (pos > buf.size() || n > buf.size() - pos) throw std::runtime_error("HDF5: read past end of file");
        return buf.data() + pos;
    }
};

struct Dataset {
    int rank = 0;
    uint64_t dims[8] = {0};
    int type_class = -1;  // 0 fixed point, 1 float, 3 string
    int type_size = 0;
    bool type_signed = false;
    bool big_endian = false;
    int layout = -1;  // 0 compact, 1 contiguous
    uint64_t addr = 0, size = 0;
    std::vector<uint8_t> compact;
    uint64_t symtab_btree = 0, symtab_heap = 0;
    bool is_group = false;
    uint64_t n_elems() const {
        uint64_t n = 1;
        for (int i = 0; i < rank; ++i) n *= dims[i];
        return n;
    }
};

static void parse_message(const Reader& R, int type, uint64_t p, uint64_t size, Dataset& d,
                          std::vector<std::pair<uint64_t, uint64_t>>& cont) {
    switch (type) {
        case 0x0001: {  // dataspace
            int ver = (int)R.rd(p, 1);
            d.rank = (int)R.rd(p + 1, 1);
            if (d.rank > 8) throw std::runtime_error("HDF5: rank > 8");
            uint64_t q = (ver == 1) ? p + 8 : p + 4;
            for (int i = 0; i < d.rank; ++i) d.dims[i] = R.rd(q + (uint64_t)i * R.sl, R.sl);
            break;
        }
        case 0x0003: {  // datatype
            int cv = (int)R.rd(p, 1);
            d.type_class = cv & 0x0f;
            int bf = (int)R.rd(p + 1, 1);
            d.big_endian = (d.type_class == 0 || d.type_class == 1) && (bf & 1);
            d.type_signed = (d.type_class == 0) && (bf & 0x08);
            d.type_size = (int)R.rd(p + 4, 4);
            break;
        }
        case 0x0008: {  // data layout
            int ver = (int)R.rd(p, 1);
            if (ver == 3) {
                d.layout = (int)R.rd(p + 1, 1);
                if (d.layout == 1) {
                    d.addr = R.rd(p + 2, R.so);
                    d.size = R.rd(p + 2 + R.so, R.sl);
                } else if (d.layout == 0) {
                    uint64_t n = R.rd(p + 2, 2);
                    const uint8_t* src = R.at(p + 4, n);
                    d.compact.assign(src, src + n);
                    d.size = n;
                } else {
                    throw std::runtime_error("HDF5: chunked datasets are not supported");
                }
            } else if (ver == 1 || ver == 2) {
                int nd = (int)R.rd(p + 1, 1);
                d.layout = (int)R.rd(p + 2, 1);
                uint64_t q = p + 8;
                if (d.layout != 0) {
                    d.addr = R.rd(q, R.so);
                    q += R.so;
                }
                uint64_t elems = 1;
                for (int i = 0; i < nd; ++i) elems *= R.rd(q + 4 * i, 4);
                q += 4 * nd;
                if (d.layout == 0) {
                    uint64_t n = R.rd(q, 4);
                    const uint8_t* src = R.at(q + 4, n);
                    d.compact.assign(src, src + n);
                    d.size = n;
                } else if (d.layout == 1) {
                    d.size = elems;  // element size folded in by the last dimension
                } else {
                    throw std::runtime_error("HDF5: chunked datasets are not supported");
                }
            } else {
                throw std::runtime_error("HDF5: unsupported layout message version");
            }
            break;
        }
        case 0x0010:  // continuation
            cont.emplace_back(R.rd(p, R.so), R.rd(p + R.so, R.sl));
            break;
        case 0x0011:  // symbol table
            d.is_group = true;
            d.symtab_btree = R.rd(p, R.so);
            d.symtab_heap = R.rd(p + R.so, R.so);
            break;
        default:
            break;
    }
    (void)size;
}

static Dataset read_object_header(const Reader& R, uint64_t addr) {
    Dataset d;
    uint64_t a = addr + R.base;
    if (R.rd(a, 4) == 0x5244484fULL) throw std::runtime_error("HDF5: version-2 object headers are not supported");
    int ver = (int)R.rd(a, 1);
    if (ver != 1) throw std::runtime_error("HDF5: unexpected object header version");
    int nmsg = (int)R.rd(a + 2, 2);
    uint64_t hsize = R.rd(a + 8, 4);
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{a + 16, hsize}};
    std::vector<std::pair<uint64_t, uint64_t>> cont;
    int seen = 0;
    for (size_t b = 0; b < blocks.size() && seen < nmsg; ++b) {
        uint64_t p = blocks[b].first, end = blocks[b].first + blocks[b].second;
        while (p + 8 <= end && seen < nmsg) {
            int type = (int)R.rd(p, 2);
            uint64_t size = R.rd(p + 2, 2);
            parse_message(R, type, p + 8, size, d, cont);
            p += 8 + size;
            ++seen;
        }
        for (auto& c : cont) blocks.emplace_back(c.first + R.base, c.second);
        cont.clear();
    }
    return d;
}

static void open_file(Reader& R, const char* path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    R.buf.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

// Returns the root group's object-header address.
static uint64_t superblock(Reader& R) {
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    uint64_t off = 0;
    for (;;) {
        if (off + 8 > R.buf.size()) throw std::runtime_error("HDF5: no superblock signature");
        if (std::memcmp(R.buf.data() + off, sig, 8) == 0) break;
        off = off ? off * 2 : 512;
    }
    int ver = (int)R.rd(off + 8, 1);
    if (ver > 1) throw std::runtime_error("HDF5: superblock version >1 is not supported");
    R.so = (int)R.rd(off + 13, 1);
    R.sl = (int)R.rd(off + 14, 1);
    if (R.so < 1 || R.so > 8 || R.sl < 1 || R.sl > 8) throw std::runtime_error("HDF5: unsupported offset/length size");
    uint64_t p = off + 24 + (ver == 1 ? 4 : 0);
    R.base = R.rd(p, R.so);
    p += 4 * R.so;  // base, free-space, eof, driver
    // root symbol table entry: link name offset, object header address
    return R.rd(p + R.so, R.so);
}

static void collect_symbols(const Reader& R, uint64_t btree, uint64_t heap_data,
                            std::map<std::string, uint64_t>& out, int depth = 0) {
    if (depth > 16) throw std::runtime_error("HDF5: B-tree too deep");
    uint64_t a = btree + R.base;
    if (std::memcmp(R.at(a, 4), "TREE", 4) != 0) throw std::runtime_error("HDF5: bad B-tree signature");
    int level = (int)R.rd(a + 5, 1);
    int used = (int)R.rd(a + 6, 2);
    uint64_t p = a + 8 + 2 * R.so;
    for (int i = 0; i < used; ++i) {
        uint64_t child = R.rd(p + R.sl + (uint64_t)i * (R.sl + R.so), R.so);
        if (level > 0) {
            collect_symbols(R, child, heap_data, out, depth + 1);
            continue;
        }
        uint64_t s = child + R.base;
        if (std::memcmp(R.at(s, 4), "SNOD", 4) != 0) throw std::runtime_error("HDF5: bad symbol node signature");
        int nsym = (int)R.rd(s + 6, 2);
        uint64_t e = s + 8;
        for (int k = 0; k < nsym; ++k, e += 2 * R.so + 24) {
            uint64_t name_off = R.rd(e, R.so);
            uint64_t oh = R.rd(e + R.so, R.so);
            const char* nm = (const char*)R.at(heap_data + name_off, 1);
            size_t maxlen = R.buf.size() - (heap_data + name_off);
            out[std::string(nm, strnlen(nm, maxlen))] = oh;
        }
    }
}

// Finds a dataset by path ("a" or "group/a") below the root group.
static Dataset find_dataset(Reader& R, const std::string& path) {
    uint64_t oh = superblock(R);
    size_t start = 0;
    while (start < path.size() && path[start] == '/') ++start;
    std::string rest = path.substr(start);
    for (;;) {
        Dataset g = read_object_header(R, oh);
        if (!g.is_group) throw std::runtime_error("HDF5: path component is not a group");
        uint64_t h = g.symtab_heap + R.base;
        if (std::memcmp(R.at(h, 4), "HEAP", 4) != 0) throw std::runtime_error("HDF5: bad local heap signature");
        uint64_t heap_data = R.rd(h + 8 + 2 * R.sl, R.so) + R.base;
        std::map<std::string, uint64_t> syms;
        collect_symbols(R, g.symtab_btree, heap_data, syms);
        size_t slash = rest.find('/');
        std::string name = rest.substr(0, slash);
        auto it = syms.find(name);
        if (it == syms.end()) throw std::out_of_range("dataset not found: " + path);
        if (slash == std::string::npos) return read_object_header(R, it->second);
        oh = it->second;
        rest = rest.substr(slash + 1);
    }
}

static const uint8_t* dataset_bytes(const Reader& R, const Dataset& d, uint64_t need) {
    if (d.layout == 0) {
        if (d.compact.size() < need) throw std::runtime_error("HDF5: compact dataset too small");
        return d.compact.data();
    }
    if (d.addr == ~0ULL) throw std::runtime_error("HDF5: dataset storage not allocated");
    return R.at(d.addr + R.base, need);
}

// ------------------------------------------------------------------ writer
struct Writer {
    std::vector<uint8_t> out;
    void put(uint64_t v, int n) {  // n <= 8: a shift by 64 bits or more is undefined
        assert(n <= 8);
        for (int i = 0; i < n; ++i) out.push_back((uint8_t)(v >> (8 * i)));
    }
    void put_at(uint64_t pos, uint64_t v, int n) {
        assert(n <= 8);
        for (int i = 0; i < n; ++i) out[pos + i] = (uint8_t)(v >> (8 * i));
    }
    void align8() {
        while (out.size() % 8) out.push_back(0);
    }
    void bytes(const void* p, size_t n) {
        const uint8_t* b = (const uint8_t*)p;
        out.insert(out.end(), b, b + n);
    }
};


static void write_message(Writer& W, int type, const std::vector<uint8_t>& body) {
    size_t n = (body.size() + 7) / 8 * 8;
    W.put(type, 2);
    W.put(n, 2);
    W.put(0, 4);  // flags + reserved
    W.bytes(body.data(), body.size());
    for (size_t i = body.size(); i < n; ++i) W.out.push_back(0);
}

static std::vector<uint8_t> le(uint64_t v, int n) {
    std::vector<uint8_t> b(n);
    for (int i = 0; i < n; ++i) b[i] = (uint8_t)(v >> (8 * i));
    return b;
}
static void append(std::vector<uint8_t>& a, const std::vector<uint8_t>& b) { a.insert(a.end(), b.begin(), b.end()); }

// Writes the whole file image for the given datasets.
static void write_file(const char* path, std::vector<OutDataset> ds) {
    std::sort(ds.begin(), ds.end(), [](const OutDataset& a, const OutDataset& b) { return a.name < b.name; });
    if (ds.size() > 256) throw std::runtime_error("HDF5 writer: at most 256 datasets");
    Writer W;
    W.out.assign(96, 0);  // superblock, filled in at the end
    // local heap data: "" at 0, then names
    std::vector<uint8_t> heap(8, 0);
    std::vector<uint64_t> name_off;
    for (auto& d : ds) {
        name_off.push_back(heap.size());
        heap.insert(heap.end(), d.name.begin(), d.name.end());
        heap.push_back(0);
        while (heap.size() % 8) heap.push_back(0);
    }
    heap.resize(std::max<size_t>(heap.size() + 8, 88), 0);
    // dataset object headers and raw data
    std::vector<uint64_t> oh_addr;
    for (auto& d : ds) {
        W.align8();
        uint64_t raw = W.out.size();
        W.bytes(d.data.data(), d.data.size());
        W.align8();
        oh_addr.push_back(W.out.size());
        std::vector<uint8_t> space{1, (uint8_t)d.dims.size(), 0, 0, 0, 0, 0, 0};
        for (auto x : d.dims) append(space, le(x, 8));
        std::vector<uint8_t> dtype;
        if (d.type_class == 0) {
            dtype = {0x10, (uint8_t)(d.is_signed ? 0x08 : 0x00), 0x00, 0x00};
            append(dtype, le(d.type_size, 4));
            append(dtype, le(0, 2));                   // bit offset
            append(dtype, le(8 * d.type_size, 2));     // precision
        } else if (d.type_class == 1) {
            // IEEE little-endian double: sign at 63, exponent 52..62, mantissa 0..51
            dtype = {0x11, 0x20, 0x3f, 0x00};
            append(dtype, le(8, 4));
            append(dtype, le(0, 2));
            append(dtype, le(64, 2));
            dtype.push_back(52);
            dtype.push_back(11);
            dtype.push_back(0);
            dtype.push_back(52);
            append(dtype, le(1023, 4));
        } else {
            dtype = {0x13, 0x00, 0x00, 0x00};
            append(dtype, le(d.type_size, 4));
        }
        std::vector<uint8_t> fill{2, 2, 0, 0};
        std::vector<uint8_t> layout{3, 1};
        append(layout, le(raw, 8));
        append(layout, le(d.data.size(), 8));
        size_t h0 = W.out.size();
        W.put(1, 1);
        W.put(0, 1);
        W.put(4, 2);
        W.put(1, 4);
        W.put(0, 4);  // header size, patched below
        W.put(0, 4);
        write_message(W, 0x0001, space);
        write_message(W, 0x0003, dtype);
        write_message(W, 0x0005, fill);
        write_message(W, 0x0008, layout);
        W.put_at(h0 + 8, W.out.size() - (h0 + 16), 4);
    }
    // local heap
    W.align8();
    uint64_t heap_hdr = W.out.size();
    W.bytes("HEAP", 4);
    W.put(0, 4);
    W.put(heap.size(), 8);
    W.put(1, 8);  // H5HL_FREE_NULL: no free block
    W.put(heap_hdr + 32, 8);
    W.bytes(heap.data(), heap.size());
    // symbol nodes (2K = 8 entries each), then one level-0 B-tree node (2K = 32 children)
    const int leafK = 4, internK = 16;
    std::vector<uint64_t> snod_addr;
    for (size_t first = 0; first < ds.size() || (first == 0 && ds.empty()); first += 2 * leafK) {
        W.align8();
        snod_addr.push_back(W.out.size());
        size_t cnt = std::min<size_t>(2 * leafK, ds.size() - first);
        W.bytes("SNOD", 4);
        W.put(1, 1);
        W.put(0, 1);
        W.put(cnt, 2);
        for (int k = 0; k < 2 * leafK; ++k) {
            if ((size_t)k < cnt) {
                W.put(name_off[first + k], 8);
                W.put(oh_addr[first + k], 8);
            } else {
                W.put(0, 8);
                W.put(0, 8);
            }
            W.put(0, 4);
            W.put(0, 4);
            W.put(0, 8);  // 16-byte scratch pad, written as two 8-byte words (put takes at most 8)
            W.put(0, 8);
        }
        if (ds.empty()) break;
    }
    W.align8();
    uint64_t btree = W.out.size();
    W.bytes("TREE", 4);
    W.put(0, 1);
    W.put(0, 1);
    W.put(ds.empty() ? 0 : snod_addr.size(), 2);
    W.put(~0ULL, 8);
    W.put(~0ULL, 8);
    for (int i = 0; i <= 2 * internK; ++i) {
        uint64_t key = 0;
        if (i > 0 && (size_t)i <= snod_addr.size() && !ds.empty()) {
            size_t last = std::min(ds.size(), (size_t)i * 2 * leafK) - 1;
            key = name_off[last];
        }
        W.put(key, 8);
        if (i < 2 * internK) W.put(((size_t)i < snod_addr.size() && !ds.empty()) ? snod_addr[i] : 0, 8);
    }
    // root group object header with a symbol-table message
    W.align8();
    uint64_t root = W.out.size();
    W.put(1, 1);
    W.put(0, 1);
    W.put(1, 2);
    W.put(1, 4);
    W.put(24, 4);
    W.put(0, 4);
    std::vector<uint8_t> st = le(btree, 8);
    append(st, le(heap_hdr, 8));
    write_message(W, 0x0011, st);
    // superblock v0
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    std::memcpy(W.out.data(), sig, 8);
    W.out[8] = 0; W.out[9] = 0; W.out[10] = 0; W.out[11] = 0; W.out[12] = 0;
    W.out[13] = 8; W.out[14] = 8; W.out[15] = 0;
    W.put_at(16, leafK, 2);
    W.put_at(18, internK, 2);
    W.put_at(20, 0, 4);
    W.put_at(24, 0, 8);
    W.put_at(32, ~0ULL, 8);
    W.put_at(40, W.out.size(), 8);
    W.put_at(48, ~0ULL, 8);
    W.put_at(56, 0, 8);
    W.put_at(64, root, 8);
    W.put_at(72, 1, 4);
    W.put_at(80, btree, 8);
    W.put_at(88, heap_hdr, 8);
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f) throw std::runtime_error(std::string("cannot create ") + path);
    f.write((const char*)W.out.data(), W.out.size());
    if (!f) throw std::runtime_error(std::string("write failed: ") + path);
}

// Reads back every dataset of a file written by write_file (used for append).
static std::vector<OutDataset> read_all_for_append(const char* path) {
    Reader R;
    open_file(R, path);
    uint64_t oh = superblock(R);
    Dataset g = read_object_header(R, oh);
    uint64_t h = g.symtab_heap + R.base;
    uint64_t heap_data = R.rd(h + 8 + 2 * R.sl, R.so) + R.base;
    std::map<std::string, uint64_t> syms;
    collect_symbols(R, g.symtab_btree, heap_data, syms);
    std::vector<OutDataset> all;
    for (auto& kv : syms) {
        Dataset d = read_object_header(R, kv.second);
        if (d.is_group) continue;
        OutDataset o;
        o.name = kv.first;
        o.type_class = d.type_class == 1 ? 1 : (d.type_class == 3 ? 3 : 0);
        o.type_size = d.type_size;
        o.is_signed = d.type_signed;
        for (int i = 0; i < d.rank; ++i) o.dims.push_back(d.dims[i]);
        uint64_t nbytes = d.n_elems() * (uint64_t)d.type_size;
        const uint8_t* src = dataset_bytes(R, d, nbytes);
        o.data.assign(src, src + nbytes);
        all.push_back(std::move(o));
    }
    return all;
}

void write_datasets(const char* path, const std::vector<OutDataset>& ds) { write_file(path, ds); }

bool read_dataset(const char* path, const char* name, OutDataset& out) {
    {
        std::ifstream probe(path, std::ios::binary);
        if (!probe) return false;
    }
    Reader R;
    open_file(R, path);
    Dataset d;
    try {
        d = find_dataset(R, name);
    } catch (const std::out_of_range&) {
        return false;
    }
    if (d.is_group || d.big_endian) throw std::runtime_error(std::string(path) + ": unsupported dataset " + name);
    out.name = name;
    out.type_class = d.type_class == 1 ? 1 : (d.type_class == 3 ? 3 : 0);
    out.type_size = d.type_size;
    out.is_signed = d.type_signed;
    out.dims.assign(d.dims, d.dims + d.rank);
    const uint64_t nbytes = d.n_elems() * (uint64_t)d.type_size;
    const uint8_t* src = dataset_bytes(R, d, nbytes);
    out.data.assign(src, src + nbytes);
    return true;
}

}  // namespace h5
}  // namespace qsi

using namespace qsi;

extern "C" qsi_status qsi_h5_read_basis(const char* path, const char* dataset, uint64_t* out_lohi,
                                        int64_t cap, int64_t* n_out) {
    return guarded([&]() -> qsi_status {
        if (!path || !n_out) return fail(QSI_INVALID_ARG, "qsi_h5_read_basis: null argument");
        h5::Reader R;
        h5::Dataset d;
        try {
            h5::open_file(R, path);
            d = h5::find_dataset(R, dataset ? dataset : "basis");
        } catch (const std::out_of_range& e) {
            return fail(QSI_NOT_FOUND, "%s", e.what());
        } catch (const std::exception& e) {
            return fail(QSI_IO_ERROR, "%s: %s", path, e.what());
        }
        if (d.type_class != 0 || d.type_size != 8 || d.big_endian)
            return fail(QSI_IO_ERROR, "%s: dataset is not little-endian 64-bit integer", path);
        if (!(d.rank == 2 && d.dims[1] == 2))
            return fail(QSI_IO_ERROR, "%s: basis dataset must have shape (N, 2)", path);
        const int64_t n = (int64_t)d.dims[0];
        *n_out = n;
        if (!out_lohi) return QSI_OK;
        if (cap < n) return fail(QSI_INVALID_ARG, "qsi_h5_read_basis: cap %lld < n %lld", (long long)cap, (long long)n);
        try {
            const uint8_t* src = h5::dataset_bytes(R, d, (uint64_t)n * 16);
            std::memcpy(out_lohi, src, (size_t)n * 16);
        } catch (const std::exception& e) {
            return fail(QSI_IO_ERROR, "%s: %s", path, e.what());
        }
        return QSI_OK;
    });
}

extern "C" qsi_status qsi_h5_read_f64(const char* path, const char* dataset, double* out, int64_t cap,
                                      int64_t* n_out, int64_t* dims_out, int32_t* rank_out) {
    return guarded([&]() -> qsi_status {
        if (!path || !dataset || !n_out) return fail(QSI_INVALID_ARG, "qsi_h5_read_f64: null argument");
        h5::Reader R;
        h5::Dataset d;
        try {
            h5::open_file(R, path);
            d = h5::find_dataset(R, dataset);
        } catch (const std::out_of_range& e) {
            return fail(QSI_NOT_FOUND, "%s", e.what());
        } catch (const std::exception& e) {
            return fail(QSI_IO_ERROR, "%s: %s", path, e.what());
        }
        if (d.type_class != 1 || d.type_size != 8 || d.big_endian)
            return fail(QSI_IO_ERROR, "%s/%s: not a little-endian float64 dataset", path, dataset);
        int64_t n = (int64_t)d.n_elems();
        *n_out = n;
        if (rank_out) *rank_out = d.rank;
        if (dims_out)
            for (int i = 0; i < d.rank && i < 4; ++i) dims_out[i] = (int64_t)d.dims[i];
        if (!out) return QSI_OK;
        if (cap < n) return fail(QSI_INVALID_ARG, "qsi_h5_read_f64: cap too small");
        try {
            std::memcpy(out, h5::dataset_bytes(R, d, (uint64_t)n * 8), (size_t)n * 8);
        } catch (const std::exception& e) {
            return fail(QSI_IO_ERROR, "%s: %s", path, e.what());
        }
        return QSI_OK;
    });
}

extern "C" qsi_status qsi_h5_write_basis(const char* path, const char* dataset, const uint64_t* lohi,
                                         int64_t n, int32_t append) {
    return guarded([&]() -> qsi_status {
        if (!path || !dataset || n < 0 || (n > 0 && !lohi)) return fail(QSI_INVALID_ARG, "qsi_h5_write_basis: bad argument");
        std::vector<h5::OutDataset> all;
        if (append) {
            try {
                all = h5::read_all_for_append(path);
            } catch (const std::exception& e) {
                return fail(QSI_IO_ERROR, "%s: %s", path, e.what());
            }
            all.erase(std::remove_if(all.begin(), all.end(), [&](const h5::OutDataset& o) { return o.name == dataset; }), all.end());
        }
        h5::OutDataset o;
        o.name = dataset;
        o.type_class = 0;
        o.type_size = 8;
        o.dims = {(uint64_t)n, 2};
        o.data.resize((size_t)n * 16);
        if (n) std::memcpy(o.data.data(), lohi, (size_t)n * 16);
        all.push_back(std::move(o));
        try {
            h5::write_file(path, std::move(all));
        } catch (const std::exception& e) {
            return fail(QSI_IO_ERROR, "%s", e.what());
        }
        return QSI_OK;
    });
}

extern "C" qsi_status qsi_h5_write_eigs(const char* path, const double* evals, int64_t nev, const double* evecs,
                                        int64_t dim, int64_t nvec, const char* latfile_json, const char* dset_name) {
    return guarded([&]() -> qsi_status {
        if (!path || nev < 0 || dim < 0 || nvec < 0 || (nev && !evals) || ((dim * nvec) != 0 && !evecs))
            return fail(QSI_INVALID_ARG, "qsi_h5_write_eigs: bad argument");
        std::vector<h5::OutDataset> all;
        h5::OutDataset e;
        e.name = "eigenvalues";
        e.type_class = 1;
        e.type_size = 8;
        e.dims = {(uint64_t)nev};
        e.data.resize((size_t)nev * 8);
        if (nev) std::memcpy(e.data.data(), evals, (size_t)nev * 8);
        all.push_back(e);
        h5::OutDataset v;
        v.name = "eigenvectors";
        v.type_class = 1;
        v.type_size = 8;
        v.dims = {(uint64_t)dim, (uint64_t)nvec};
        v.data.resize((size_t)(dim * nvec) * 8);
        if ((dim * nvec) != 0) std::memcpy(v.data.data(), evecs, (size_t)(dim * nvec) * 8);
        all.push_back(v);
        auto add_str = [&](const char* name, const char* s) {
            h5::OutDataset o;
            o.name = name;
            o.type_class = 3;
            std::string str = s ? s : "";
            o.type_size = (int)str.size() + 1;
            o.data.assign(str.begin(), str.end());
            o.data.push_back(0);
            all.push_back(o);
        };
        add_str("latfile_json", latfile_json);
        add_str("dset_name", dset_name);
        try {
            h5::write_file(path, std::move(all));
        } catch (const std::exception& ex) {
            return fail(QSI_IO_ERROR, "%s", ex.what());
        }
        return QSI_OK;
    });
}

extern "C" qsi_status qsi_h5_write_f64(const char* path, const char* dataset, const double* data, const int64_t* dims,
                                       int32_t rank, int32_t append) {
    return guarded([&]() -> qsi_status {
        if (!path || !dataset || rank < 0 || rank > 8 || (rank > 0 && !dims))
            return fail(QSI_INVALID_ARG, "qsi_h5_write_f64: bad argument");
        uint64_t count = 1;
        h5::OutDataset o;
        o.name = dataset;
        o.type_class = 1;
        o.type_size = 8;
        for (int i = 0; i < rank; ++i) {
            if (dims[i] < 0) return fail(QSI_INVALID_ARG, "qsi_h5_write_f64: negative dimension");
            o.dims.push_back((uint64_t)dims[i]);
            count *= (uint64_t)dims[i];
        }
        if (count && !data) return fail(QSI_INVALID_ARG, "qsi_h5_write_f64: null data");
        o.data.resize(count * 8);
        if (count) std::memcpy(o.data.data(), data, count * 8);
        std::vector<h5::OutDataset> all;
        try {
            if (append) {
                all = h5::read_all_for_append(path);
                all.erase(std::remove_if(all.begin(), all.end(), [&](const h5::OutDataset& d) { return d.name == dataset; }),
                          all.end());
            }
            all.push_back(std::move(o));
            h5::write_file(path, std::move(all));
        } catch (const std::exception& e) {
            return fail(QSI_IO_ERROR, "%s: %s", path, e.what());
        }
        return QSI_OK;
    });
}

extern "C" qsi_status qsi_h5_write_string(const char* path, const char* dataset, const char* text, int32_t append) {
    return guarded([&]() -> qsi_status {
        if (!path || !dataset || !text) return fail(QSI_INVALID_ARG, "qsi_h5_write_string: bad argument");
        h5::OutDataset o;
        o.name = dataset;
        o.type_class = 3;
        const size_t len = std::strlen(text) + 1;
        o.type_size = (int)len;
        o.data.assign(text, text + len);
        std::vector<h5::OutDataset> all;
        try {
            if (append) {
                all = h5::read_all_for_append(path);
                all.erase(std::remove_if(all.begin(), all.end(), [&](const h5::OutDataset& d) { return d.name == dataset; }),
                          all.end());
            }
            all.push_back(std::move(o));
            h5::write_file(path, std::move(all));
        } catch (const std::exception& e) {
            return fail(QSI_IO_ERROR, "%s: %s", path, e.what());
        }
        return QSI_OK;
    });
}

// The first element of a string dataset: fixed-length (class 3), or variable-length (class 9) with the text in a
// global heap collection, which is how libhdf5 stores std::string attributes written by the reference
// (write_string_to_hdf5, src/expectation_eval.cpp).
extern "C" qsi_status qsi_h5_read_string(const char* path, const char* dataset, char* buf, size_t len) {
    return guarded([&]() -> qsi_status {
        if (!path || !dataset || !buf || len == 0) return fail(QSI_INVALID_ARG, "qsi_h5_read_string: bad argument");
        h5::Reader R;
        h5::Dataset d;
        std::string text;
        try {
            h5::open_file(R, path);
            d = h5::find_dataset(R, dataset);
            if (d.type_class == 3) {
                const uint8_t* src = h5::dataset_bytes(R, d, (uint64_t)d.type_size);
                text.assign((const char*)src, strnlen((const char*)src, (size_t)d.type_size));
            } else if (d.type_class == 9) {
                const uint8_t* e = h5::dataset_bytes(R, d, 4 + (uint64_t)R.so + 4);
                uint64_t L = 0, heap = 0, index = 0;
                for (int i = 0; i < 4; ++i) L |= (uint64_t)e[i] << (8 * i);
                for (int i = 0; i < R.so; ++i) heap |= (uint64_t)e[4 + i] << (8 * i);
                for (int i = 0; i < 4; ++i) index |= (uint64_t)e[4 + R.so + i] << (8 * i);
                const uint64_t g = heap + R.base;
                if (std::memcmp(R.at(g, 4), "GCOL", 4) != 0) throw std::runtime_error("bad global heap signature");
                const uint64_t end = g + R.rd(g + 8, R.sl);
                uint64_t q = g + 8 + R.sl;
                bool found = false;
                while (q + 8 + R.sl <= end) {
                    const uint64_t idx = R.rd(q, 2), size = R.rd(q + 8, R.sl);
                    if (idx == 0) break;  // free space
                    if (idx == index) {
                        const uint8_t* src = R.at(q + 8 + R.sl, size);
                        text.assign((const char*)src, (size_t)std::min<uint64_t>(L, size));
                        found = true;
                        break;
                    }
                    q += 8 + R.sl + ((size + 7) & ~(uint64_t)7);
                }
                if (!found) throw std::runtime_error("string not found in the global heap");
            } else {
                throw std::runtime_error("not a string dataset");
            }
        } catch (const std::out_of_range& e) {
            return fail(QSI_NOT_FOUND, "%s", e.what());
        } catch (const std::exception& e) {
            return fail(QSI_IO_ERROR, "%s/%s: %s", path, dataset, e.what());
        }
        const size_t n = std::min(len - 1, text.size());
        std::memcpy(buf, text.data(), n);
        buf[n] = 0;
        return QSI_OK;
    });
}

extern "C" qsi_status qsi_csv_read_basis(const char* path, uint64_t* out_lohi, int64_t cap, int64_t* n_out) {
    return guarded([&]() -> qsi_status {
        if (!path || !n_out) return fail(QSI_INVALID_ARG, "qsi_csv_read_basis: null argument");
        FILE* f = std::fopen(path, "r");
        if (!f) return fail(QSI_IO_ERROR, "Failed to open file: %s", path);
        char line[64];
        int64_t n = 0;
        while (std::fgets(line, sizeof(line), f)) {
            unsigned long long hi = 0, lo = 0;
            if (std::sscanf(line, "0x%016llx%016llx", &hi, &lo) != 2) break;
            if (out_lohi) {
                if (n >= cap) {
                    std::fclose(f);
                    return fail(QSI_INVALID_ARG, "qsi_csv_read_basis: cap too small");
                }
                out_lohi[2 * n] = lo;
                out_lohi[2 * n + 1] = hi;
            }
            ++n;
        }
        std::fclose(f);
        *n_out = n;
        return QSI_OK;
    });
}
