// Minimal HDF5 (classic file format) writer and reader for SpinParser's output files.
//
// The reference writes its observables (.obs), checkpoints (.checkpoint) and deferred-
// measurement archives (.data) with libhdf5 in the classic format: superblock version 0,
// version-1 object headers, groups as symbol tables (v1 B-tree + local heap + symbol-table
// nodes), contiguous float32 datasets, float32[3] array datasets and float32 attributes
// (src/SU2/SU2MeasurementCorrelation.cpp:179-355, src/SU2/SU2EffectiveAction.hpp:79-205).
// The library does not link libhdf5, so this module writes and reads exactly that
// subset with the node sizes libhdf5 uses (group leaf K = 4, internal K = 16), so that any
// HDF5 reader (h5py, the reference's obs.py) opens the files.
//
// Two ways to write:
//   write_file  -- the whole tree, compactly, to a new file (temporary file + rename);
//   append_file -- the root group's metadata and every new or changed group at the end of
//                  an existing file, then the superblock is repointed.  Unchanged groups and
//                  dataset storage are referenced, not copied, so adding a checkpoint to a
//                  multi-GB archive costs the new data plus a few bytes per existing member.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace spn {
namespace h5 {

constexpr uint64_t kUndef = ~uint64_t(0);

struct Attribute {
    std::string name;
    std::vector<uint64_t> dims;  // simple dataspace
    std::vector<float> data;
};

struct Dataset {
    std::string name;
    std::vector<uint64_t> dims;  // simple dataspace
    int array3 = 0;              // 1: element type is float32[3] (lattice positions)
    std::vector<float> data;     // prod(dims) * (array3 ? 3 : 1) values, when loaded
    std::vector<Attribute> attrs;
    // Storage in an existing file (set by the reader).  A dataset with `data` empty and
    // addr != kUndef keeps its storage when the tree is appended to the same file.
    uint64_t addr = kUndef;
    uint64_t nbytes = 0;
    bool compact = false;

    uint64_t count() const;  // number of float values
};

struct Group {
    std::string name;
    std::vector<Group> groups;
    std::vector<Dataset> datasets;
    std::vector<Attribute> attrs;
    // Object of this group in an existing file (set by the reader).  append_file reuses the
    // object of every non-root group that still has it, without rewriting that subtree;
    // code that changes such a group (or anything below it) sets header = kUndef first.
    uint64_t header = kUndef, btree = kUndef, heap = kUndef;

    Group *group(const std::string &n);
    const Group *group(const std::string &n) const;
    Dataset *dataset(const std::string &n);
    const Dataset *dataset(const std::string &n) const;
    const Attribute *attr(const std::string &n) const;
    Group &add_group(const std::string &n);
    // Members in the order HDF5 indexes them (by name, strcmp order): the order of
    // H5Gget_objname_by_idx in the reference.
    std::vector<std::string> member_names() const;
    size_t n_members() const { return groups.size() + datasets.size(); }
};

// An opened file: its metadata tree; dataset values are read on demand.
class File {
public:
    static File open(const std::string &path);
    static bool is_hdf5(const std::string &path);
    Group root;
    std::string path;
    uint64_t eof = 0;
    // Reads the values of a dataset of this file into d.data.
    void load(Dataset &d) const;
    // Loads every dataset of a subtree.
    void load_all(Group &g) const;
};

// Serialises the tree into a complete file image (the root's name is ignored).  Every
// dataset must hold its values.
std::string serialize(const Group &root);

void write_file(const std::string &path, const Group &root);
// `root` is the updated tree of `file` (metadata as returned by File::open, plus additions).
void append_file(const File &file, const Group &root);

}  // namespace h5
}  // namespace spn
