// Checkpoints and observable files of the SU(2) and XYZ cores in the reference's HDF5 layout.
//
// Checkpoints: SU2EffectiveAction::writeCheckpoint / readCheckpoint
// (src/SU2/SU2EffectiveAction.hpp:79-200).  Observables: SU2MeasurementCorrelation's
// _writeOutfileHeader / _writeOutfileCorrelation (src/SU2/SU2MeasurementCorrelation.cpp:179-355).
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <utility>
#include <vector>
#include "h5.hpp"

namespace spn {

struct Lattice;

// A checkpoint group holds "cutoff", "v2" and the named vertex arrays in the given order
// (SU(2): v4dd, v4ss; XYZ: v4dd, v4xx, v4yy, v4zz -- XYZEffectiveAction.hpp:144-149).
// Returns the checkpoint id written, or -1 if the file holds a checkpoint at `cutoff`.
int write_checkpoint_arrays(const std::string &path, bool append, float cutoff, const float *v2, int64_t n_v2,
                            const std::vector<std::pair<std::string, const float *>> &v4, int64_t n_v4);
bool read_checkpoint_arrays(const std::string &path, int id, float &cutoff, float *v2, int64_t n_v2,
                            const std::vector<std::pair<std::string, float *>> &v4, int64_t n_v4);

// Returns the checkpoint id written, or -1 if the file holds a checkpoint at `cutoff`.
int write_checkpoint(const std::string &path, bool append, float cutoff, const float *v2, int64_t n_v2,
                     const float *v4ss, const float *v4dd, int64_t n_v4);

// Returns false if the checkpoint (or one of its datasets) does not exist.
bool read_checkpoint(const std::string &path, int id, float &cutoff, float *v2, int64_t n_v2, float *v4ss,
                     float *v4dd, int64_t n_v4);

// Lattice description stored in every correlation group's "meta" subgroup.
struct ObsMeta {
    std::vector<float> lattice_vectors;  // [n_bravais][3]
    std::vector<float> basis;            // [n_basis][3]
    std::vector<float> sites;            // [n_basis][n_range][3]
    uint64_t n_basis = 0, n_range = 0;
};
ObsMeta make_obs_meta(const Lattice &lat);

// Observable files held in memory and written as whole files.  A file that exists when it
// is first used is loaded, so measurements of an earlier run are kept and duplicates (same
// cutoff) are discarded exactly as the reference discards them.
class ObsStore {
public:
    // Adds one measurement of `group` (e.g. "SU2CorZZ"); false if one at `cutoff` exists.
    bool add(const std::string &path, const std::string &group, const ObsMeta &meta, float cutoff, const float *data);
    void flush();  // writes every modified file
    ~ObsStore();

private:
    struct Entry {
        h5::Group root;
        bool dirty = false;
    };
    Entry &get(const std::string &path);
    std::map<std::string, Entry> files_;
};

}  // namespace spn
