// SU(2) checkpoint and observable files (see su2_files.hpp).
#include "su2_files.hpp"
#include "capi_common.hpp"
#include "error.hpp"
#include "lattice_handle.hpp"
#include "log.hpp"
#include "../../../include/spn_su2.h"
#include <cstring>

namespace spn {

namespace {

h5::Attribute cutoff_attr(float cutoff) {
    h5::Attribute a;
    a.name = "cutoff";
    a.dims = {1};
    a.data = {cutoff};
    return a;
}

h5::Dataset vector_dataset(const std::string &name, const float *p, int64_t n) {
    h5::Dataset d;
    d.name = name;
    d.dims = {uint64_t(n)};
    d.data.assign(p, p + n);
    return d;
}

// Group members that are groups, in index (name) order, and each one's "cutoff" attribute:
// the loop over H5Gget_objname_by_idx in the reference.
bool has_cutoff(const h5::Group &g, float cutoff, int &n_groups) {
    n_groups = 0;
    for (const std::string &name : g.member_names()) {
        const h5::Group *c = g.group(name);
        if (!c) continue;
        ++n_groups;
        const h5::Attribute *a = c->attr("cutoff");
        if (a && !a->data.empty() && a->data[0] == cutoff) return true;
    }
    return false;
}

std::string fmt_cutoff(float c) { return std::to_string(c); }

}  // namespace

int write_checkpoint_arrays(const std::string &path, bool append, float cutoff, const float *v2, int64_t n_v2,
                            const std::vector<std::pair<std::string, const float *>> &v4, int64_t n_v4) {
    const bool existing = append && h5::File::is_hdf5(path);
    h5::File file;
    if (existing) file = h5::File::open(path);
    int id = 0;
    if (has_cutoff(file.root, cutoff, id)) {
        log(LogLevel::Warning, "Found existing checkpoint at cutoff " + fmt_cutoff(cutoff) + ". Skipping checkpoint.");
        return -1;
    }
    h5::Group &g = file.root.add_group("checkpoint_" + std::to_string(id));
    g.attrs.push_back(cutoff_attr(cutoff));
    g.datasets.push_back(vector_dataset("cutoff", &cutoff, 1));
    g.datasets.push_back(vector_dataset("v2", v2, n_v2));
    for (const auto &a : v4) g.datasets.push_back(vector_dataset(a.first, a.second, n_v4));
    if (existing) h5::append_file(file, file.root);
    else h5::write_file(path, file.root);
    return id;
}

bool read_checkpoint_arrays(const std::string &path, int id, float &cutoff, float *v2, int64_t n_v2,
                            const std::vector<std::pair<std::string, float *>> &v4, int64_t n_v4) {
    if (!h5::File::is_hdf5(path)) throw Error(ErrorType::IO, "Could not open data file for reading");
    h5::File file = h5::File::open(path);
    std::string name;
    if (id >= 0) {
        name = "checkpoint_" + std::to_string(id);
    } else {
        std::vector<std::string> members = file.root.member_names();
        for (int i = int(members.size()) - 1; i >= 0; --i)
            if (file.root.group(members[i])) {
                name = "checkpoint_" + std::to_string(i);
                break;
            }
    }
    h5::Group *g = file.root.group(name);
    if (!g) return false;
    struct Want { std::string name; float *dst; int64_t n; };
    float c = 0;
    std::vector<Want> wants = {{"cutoff", &c, 1}, {"v2", v2, n_v2}};
    for (const auto &a : v4) wants.push_back({a.first, a.second, n_v4});
    for (const Want &w : wants) {
        h5::Dataset *d = g->dataset(w.name);
        if (!d) return false;
        if (int64_t(d->count()) != w.n)
            throw Error(ErrorType::Argument, "checkpoint dataset '" + w.name + "' holds " + std::to_string(d->count()) +
                                                 " values, the flow has " + std::to_string(w.n));
    }
    for (const Want &w : wants) {
        h5::Dataset *d = g->dataset(w.name);
        file.load(*d);
        if (w.dst) std::memcpy(w.dst, d->data.data(), size_t(w.n) * sizeof(float));
    }
    cutoff = c;
    return true;
}

// SU2EffectiveAction::writeCheckpoint writes v2, v4dd, v4ss (src/SU2/SU2EffectiveAction.hpp:141-144)
int write_checkpoint(const std::string &path, bool append, float cutoff, const float *v2, int64_t n_v2,
                     const float *v4ss, const float *v4dd, int64_t n_v4) {
    return write_checkpoint_arrays(path, append, cutoff, v2, n_v2, {{"v4dd", v4dd}, {"v4ss", v4ss}}, n_v4);
}

bool read_checkpoint(const std::string &path, int id, float &cutoff, float *v2, int64_t n_v2, float *v4ss,
                     float *v4dd, int64_t n_v4) {
    return read_checkpoint_arrays(path, id, cutoff, v2, n_v2, {{"v4dd", v4dd}, {"v4ss", v4ss}}, n_v4);
}

ObsMeta make_obs_meta(const Lattice &L) {
    ObsMeta m;
    m.n_basis = L.basis.size();
    m.n_range = L.range_ids[0].size();
    for (const Vec3 &a : L.primitives) m.lattice_vectors.insert(m.lattice_vectors.end(), {float(a.x), float(a.y), float(a.z)});
    for (size_t b = 0; b < m.n_basis; ++b) {
        Vec3 p = L.position(L.basis_ids[b]);
        m.basis.insert(m.basis.end(), {float(p.x), float(p.y), float(p.z)});
    }
    for (size_t b = 0; b < m.n_basis; ++b) {
        if (L.range_ids[b].size() != m.n_range)
            throw Error(ErrorType::Unsupported, "basis sites with different range sizes are not supported");
        for (int j : L.range_ids[b]) {
            Vec3 p = L.position(j);
            m.sites.insert(m.sites.end(), {float(p.x), float(p.y), float(p.z)});
        }
    }
    return m;
}

ObsStore::Entry &ObsStore::get(const std::string &path) {
    auto it = files_.find(path);
    if (it != files_.end()) return it->second;
    Entry e;
    if (h5::File::is_hdf5(path)) {
        h5::File f = h5::File::open(path);
        f.load_all(f.root);
        e.root = std::move(f.root);
    }
    return files_.emplace(path, std::move(e)).first->second;
}

bool ObsStore::add(const std::string &path, const std::string &group, const ObsMeta &meta, float cutoff, const float *data) {
    Entry &e = get(path);
    h5::Group *g = e.root.group(group);
    if (!g) g = &e.root.add_group(group);
    if (!g->group("meta")) {
        h5::Group &m = g->add_group("meta");
        h5::Dataset lv, bs, st;
        lv.name = "latticeVectors";
        lv.dims = {meta.lattice_vectors.size() / 3};
        lv.array3 = 1;
        lv.data = meta.lattice_vectors;
        bs.name = "basis";
        bs.dims = {meta.n_basis};
        bs.array3 = 1;
        bs.data = meta.basis;
        st.name = "sites";
        st.dims = {meta.n_basis, meta.n_range};
        st.array3 = 1;
        st.data = meta.sites;
        m.datasets = {bs, lv, st};
        e.dirty = true;
    }
    h5::Group *d = g->group("data");
    if (!d) d = &g->add_group("data");
    int id = 0;
    if (has_cutoff(*d, cutoff, id)) {
        log(LogLevel::Warning, "Found existing correlation measurement at cutoff " + fmt_cutoff(cutoff) + ". Discarding duplicate entry.");
        return false;
    }
    h5::Group &mg = d->add_group("measurement_" + std::to_string(id));
    mg.attrs.push_back(cutoff_attr(cutoff));
    h5::Dataset ds;
    ds.name = "data";
    ds.dims = {meta.n_basis, meta.n_range};
    ds.data.assign(data, data + meta.n_basis * meta.n_range);
    mg.datasets.push_back(std::move(ds));
    e.dirty = true;
    return true;
}

void ObsStore::flush() {
    for (auto &kv : files_) {
        if (!kv.second.dirty) continue;
        h5::write_file(kv.first, kv.second.root);
        kv.second.dirty = false;
    }
}

ObsStore::~ObsStore() {
    try {
        flush();
    } catch (const std::exception &e) {
        log(LogLevel::Error, std::string("could not write observable file: ") + e.what());
    }
}

}  // namespace spn

extern "C" int spn_su2_write_checkpoint(const char *path, int append, float cutoff, int n_v2, const float *v2,
                                        long long n_v4, const float *v4ss, const float *v4dd, int *checkpoint_id) {
    return spn::guarded([&] {
        if (!path || !v2 || !v4ss || !v4dd || n_v2 < 0 || n_v4 < 0)
            throw spn::Error(spn::ErrorType::Argument, "spn_su2_write_checkpoint: bad argument");
        int id = spn::write_checkpoint(path, append != 0, cutoff, v2, n_v2, v4ss, v4dd, n_v4);
        if (checkpoint_id) *checkpoint_id = id;
    });
}

extern "C" int spn_su2_read_checkpoint(const char *path, int checkpoint_id, float *cutoff, int n_v2, float *v2,
                                       long long n_v4, float *v4ss, float *v4dd, int *found) {
    return spn::guarded([&] {
        if (!path || n_v2 < 0 || n_v4 < 0) throw spn::Error(spn::ErrorType::Argument, "spn_su2_read_checkpoint: bad argument");
        float c = 0;
        bool ok = spn::read_checkpoint(path, checkpoint_id, c, v2, n_v2, v4ss, v4dd, n_v4);
        if (ok && cutoff) *cutoff = c;
        if (found) *found = ok ? 1 : 0;
    });
}

extern "C" int spn_su2_write_correlation(const char *path, const spn_lattice *lat, float cutoff, const float *zz,
                                         const float *dd, int *written) {
    return spn::guarded([&] {
        if (!path || !lat || !zz || !dd) throw spn::Error(spn::ErrorType::Argument, "spn_su2_write_correlation: null argument");
        spn::ObsMeta meta = spn::make_obs_meta(lat->lat);
        spn::ObsStore store;
        bool a = store.add(path, "SU2CorZZ", meta, cutoff, zz);
        bool b = store.add(path, "SU2CorDD", meta, cutoff, dd);
        store.flush();
        if (written) *written = (a && b) ? 1 : 0;
    });
}
