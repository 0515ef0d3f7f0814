// h5lite.h -- the part of the HDF5 file format the reference's files use,
// read and written without libhdf5.
//
// The reference writes and reads its HDF5 files through libhdf5's default
// ("earliest") format: a version 0 superblock, version 1 object headers and
// groups held in symbol tables (a version 1 B-tree over symbol-table nodes,
// names in a local heap), datasets with contiguous storage.  That is:
//   particles_fields_init.h5 / particle_diagnostics.h5 (src/diagnostics.c:290-387,
//       src/particle_info.c:376-488): /particles_fields/particles, a 1-D array
//       of compound {x,y,z,qm,ux,uy,uz,t} big-endian doubles, and
//       /particles_fields/fields, {Bx,By,Bz,Ex,Ey,Ez};
//   data/poincare_map.h5 (src/poincare_map.c:185-235): /poincare_map/{xpos,
//       ypos,zpos}, 2-D native doubles;
//   the PIC field files the reference reads (src/magnetic_field.c:632-692,
//       src/electric_field.c:447-507, src/data_io.c:22-75): 3-D float datasets
//       cbx, cby, cbz, ex, ey, ez in a group Timestep_<n>.
// The reader takes files written by libhdf5 with that format: superblock
// version 0 or 1 (with or without a user block), version 1 object headers
// with continuation blocks, symbol-table groups, dataspace messages 1 and 2,
// fixed-point, floating-point and compound datatypes (versions 1 to 3),
// layout messages 1 to 3 (compact, contiguous, chunked with a version 1
// B-tree; chunks through the deflate, shuffle and Fletcher-32 filters) and
// contiguous or compact layout version 4.  Files in the newer format
// (superblock 2 and 3, version 2 object headers, link messages) and other
// filters are refused with a message saying so.  The writer emits the
// earliest format, as libhdf5 does by default.
//
// Layout of a written file: superblock, then every group's object header,
// B-tree node, local heap and symbol-table node, then the datasets' object
// headers, then each dataset's contiguous data (16-byte aligned).  The layout
// is a function of the group and dataset names, types and dimensions only, so
// ranks that write disjoint slices of one file compute the same addresses and
// need no exchange: one writes the metadata, each writes its own records.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace tph5 {

constexpr uint64_t kUndef = ~0ull;

// An atomic datatype: class 0 (fixed point) or 1 (IEEE floating point).
struct Atomic {
    int cls = -1;
    uint32_t size = 0;
    bool big_endian = false;
    bool is_signed = false;
};

struct Member {
    std::string name;
    uint32_t offset = 0;
    Atomic type;
};

// A dataset's element type: atomic, or a compound of atomic members.
struct Type {
    int cls = -1;  // 0 fixed, 1 float, 6 compound, -1 anything else
    uint32_t size = 0;
    Atomic atom;                  // cls 0 or 1
    std::vector<Member> members;  // cls 6

    static Type ieee(int bytes, bool big_endian);
    static Type compound_f64(const std::vector<std::string>& names, bool big_endian);
};

// One stage of a chunked dataset's filter pipeline.
struct Filter {
    uint16_t id = 0;  // 1 deflate, 2 shuffle, 3 Fletcher-32 (others are refused on read)
    uint16_t flags = 0;
    std::vector<uint32_t> cd;  // client data
};

struct Dataset {
    std::vector<uint64_t> dims;
    Type type;
    int layout = -1;  // 0 compact, 1 contiguous, 2 chunked
    uint64_t addr = kUndef;
    uint64_t bytes = 0;
    std::vector<uint8_t> compact;  // compact layout: the data
    std::vector<uint8_t> fill;     // the fill value, when the file defines one
    std::vector<uint64_t> chunk;   // chunk extent per dimension
    std::vector<Filter> filters;   // chunked data: applied in order on write, undone in reverse on read
    uint64_t elements() const;
};

// Reader of one file.
class File {
public:
    File() = default;
    File(const File&) = delete;
    File& operator=(const File&) = delete;
    ~File();
    bool open(const char* path);
    // The dataset `name` in group `group` ("/", "", "/a/b" or "a/b").
    bool dataset(const char* group, const char* name, Dataset& ds);
    // The hyperslab [offset, offset + count) of every dimension, as the file's
    // raw element bytes in C order (elements() * type.size bytes for the whole).
    // Chunks stored through deflate (with the system's zlib, loaded at run
    // time), shuffle and Fletcher-32 filters are undone; other filters are
    // refused.
    bool read(const Dataset& ds, const uint64_t* offset, const uint64_t* count, void* raw);
    const std::string& error() const { return err_; }

private:
    struct Msg {
        uint16_t type;
        uint8_t flags;
        std::vector<uint8_t> data;
    };
    int fd_ = -1;
    uint64_t base_ = 0;
    uint64_t size_ = 0;
    uint64_t root_ = kUndef;
    uint64_t visits_ = 0;  // B-tree nodes visited by the current lookup (bounded)
    std::string path_;
    std::string err_;
    bool fail(const char* fmt, ...);
    bool rd(uint64_t addr, void* dst, size_t n);
    bool messages(uint64_t oh, std::vector<Msg>& out);
    bool group_entry(uint64_t group_oh, const std::string& name, uint64_t& oh);
    bool btree_entries(uint64_t node, uint64_t heap_data, uint64_t heap_size, const std::string& name,
                       uint64_t& oh, int depth);
    bool chunk_index(const Dataset& ds, uint64_t node, int depth, std::vector<uint64_t>& keys,
                     std::vector<uint64_t>& addrs, std::vector<uint32_t>& sizes, std::vector<uint32_t>& masks);
    bool unfilter(const Dataset& ds, uint32_t mask, std::vector<uint8_t>& buf, size_t want);
};

// Element conversion, as a C cast from the decoded value: floats exactly,
// integers exactly up to 2^53.
double decode(const Atomic& t, const uint8_t* p);
bool raw_to_double(const Type& t, const uint8_t* raw, size_t n, double* out);
bool raw_to_float(const Type& t, const uint8_t* raw, size_t n, float* out);

// Writer: the groups and datasets of one file, laid out as described above.
struct WDataset {
    std::string name;
    Type type;
    std::vector<uint64_t> dims;
    uint64_t addr = kUndef;  // set by plan()
    uint64_t bytes = 0;
};
struct WGroup {
    std::string name;  // a child of the root group ("" puts the datasets in the root)
    std::vector<WDataset> dsets;
};
struct Plan {
    std::vector<WGroup> groups;
    std::vector<uint8_t> meta;  // bytes [0, meta.size()) of the file
    uint64_t eof = 0;
    std::string err;
    bool plan();  // assigns addresses and encodes meta
    const WDataset* find(const std::string& group, const std::string& name) const;
};
// Opens (creating, never truncating) `path` for writing.
int open_for_write(const char* path, std::string& err);
// Writes the metadata and sets the file's length to plan.eof.
bool write_meta(int fd, const Plan& plan, std::string& err);
// Writes `n` elements (already in the file's byte order) starting at element `first`.
bool write_elements(int fd, const WDataset& d, uint64_t first, uint64_t n, const void* bytes, std::string& err);
// Doubles to IEEE binary64 bytes in the given order.
void put_f64(uint8_t* p, double v, bool big_endian);
// n bytes at byte `at` of an open file (any file), large ranges on several
// threads; false on a read error or the end of the file.
bool read_at(int fd, void* dst, size_t n, uint64_t at);

}  // namespace tph5
