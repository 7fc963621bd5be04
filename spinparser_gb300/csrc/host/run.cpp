// Task driver: SpinParser::run and SpinParser::runCore (src/SpinParser.cpp:53-210) with the
// flow (SU(2) or XYZ core) resident on one GPU.
//
// The host side keeps the reference's control flow: parse the task file, build the lattice
// (and always write the .ldf), create the core, then one of three stages depending on the
// recorded calculation status --
//   new / running:   [resume from the .checkpoint] -> cutoff loop {compute_step,
//                    measurements, divergence check, Euler step, periodic checkpoint}
//                    -> final measurement -> final checkpoint + status;
//   postprocessing:  deferred measurements on every archived vertex of the .data file;
//   finished:        nothing to do.
// Measurements follow FrgCore::takeMeasurements (src/FrgCore.hpp:36-67): in the loop only the
// non-deferred ones run, and with any deferred measurement (or --defer) the vertex of every
// cutoff is appended to the .data file for the post-processing stage.
//
// All flow arithmetic runs on the device through the C ABI of this library (spn_su2_*,
// spn_xyz_*); the
// host only moves the state for checkpoints and writes files.  Observable files are kept in
// memory and written whole at every checkpoint, at the end and at least every few seconds;
// measurements after the last checkpoint are recomputed on resume (and duplicates
// discarded), so the files after a resumed run equal those of an uninterrupted one.
#include "capi_common.hpp"
#include "error.hpp"
#include "lattice_handle.hpp"
#include "log.hpp"
#include "su2_files.hpp"
#include "task.hpp"
#include "../../../include/spn_su2.h"
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <dlfcn.h>
#include <memory>
#include <sstream>

namespace spn {

namespace {

constexpr std::time_t kObsFlushSeconds = 10;

void check(int rc) {
    if (rc == 0) return;
    char buf[2048];
    spn_last_error(buf, sizeof(buf));
    ErrorType t = (rc <= int(ErrorType::Argument) && rc >= int(ErrorType::Unsupported)) ? ErrorType(rc) : ErrorType::Internal;
    throw Error(t, buf);
}

// The package's res/ directory: the library lives in <package>/_build/<machine>/.
std::string default_resource_path() {
    Dl_info info;
    if (dladdr(reinterpret_cast<void *>(&spn_run_task), &info) && info.dli_fname) {
        std::string p = info.dli_fname;
        for (int i = 0; i < 3; ++i) {
            size_t s = p.find_last_of('/');
            if (s == std::string::npos) {
                p.clear();
                break;
            }
            p = p.substr(0, s);
        }
        if (!p.empty()) return p + "/res";
    }
    throw Error(ErrorType::Argument, "no resource path given and the library location is unknown");
}

std::string fixed6(double v) {
    char b[64];
    std::snprintf(b, sizeof(b), "%.6f", v);
    return b;
}

// The numerics core behind the driver (FrgCoreFactory::newFrgCore, src/FrgCoreFactory.cpp:25-51):
// SU(2) (spn_su2_*), XYZ (spn_xyz_*) or TRI (spn_tri_*).  The driver holds the state on the host in the
// checkpoint's array order and moves it through these calls.
class Core {
public:
    virtual ~Core() = default;
    virtual const char *id() const = 0;
    // checkpoint dataset names of the vertex arrays, in the reference's order
    virtual std::vector<std::string> arrays() const = 0;
    // observable groups of the correlation measurement, in the reference's write order
    virtual std::vector<std::string> obs_groups() const = 0;
    virtual void initial_state(const spn_lattice *lat, float *v2, std::vector<float *> &v4) = 0;
    virtual void set_state(float c, const float *v2, const std::vector<float *> &v4) = 0;
    virtual void get_state(float &c, float *v2, const std::vector<float *> &v4) = 0;
    virtual void compute_step() = 0;
    virtual bool diverged() = 0;
    virtual void finalize_step(float c) = 0;
    virtual void measure(const std::vector<float *> &out) = 0;  // one [n_corr] array per obs group
    virtual void synchronize() = 0;
    virtual void autotune(float at, float current) = 0;
    int64_t n_v2 = 0, n_v4 = 0;
};

class Su2Core : public Core {
public:
    Su2Core(spn_lattice *lat, const std::vector<float> &freq, float spin, float normalization, int device, int flags)
        : normalization_(normalization) {
        spn_lattice_info info;
        check(spn_lattice_get_info(lat, &info));
        const int nl = info.n_sites;
        const int64_t n_corr = int64_t(info.n_basis) * info.n_range;
        std::vector<int> srid(nl), irid(nl), optr(nl + 1), o1(info.n_overlap), o2(info.n_overlap), rr(info.n_range),
            ri(info.n_range), cr(n_corr);
        check(spn_lattice_get_tables(lat, srid.data(), irid.data(), optr.data(), o1.data(), o2.data(), rr.data(),
                                     ri.data(), cr.data(), nullptr, nullptr, nullptr));
        spn_su2_desc d{};
        d.n_freq = int(freq.size());
        d.freq = freq.data();
        d.n_sites = nl;
        d.sites_rid = srid.data();
        d.inv_sites_rid = irid.data();
        d.overlap_ptr = optr.data();
        d.overlap_rid1 = o1.data();
        d.overlap_rid2 = o2.data();
        d.n_range = info.n_range;
        d.range_rid = rr.data();
        d.range_inv_rid = ri.data();
        d.n_corr = int(n_corr);
        d.corr_rid = cr.data();
        d.spin_length = spin;
        d.device = device;
        d.flags = flags;
        check(spn_su2_create(&d, &h_));
        int nf = 0, ns = 0;
        long long nt = 0;
        check(spn_su2_get_sizes(h_, &nf, &ns, &nt));
        n_v2 = nf;
        n_v4 = int64_t(nt) * ns;
    }
    ~Su2Core() override { spn_su2_destroy(h_); }
    const char *id() const override { return "SU2"; }
    std::vector<std::string> arrays() const override { return {"v4dd", "v4ss"}; }
    std::vector<std::string> obs_groups() const override { return {"SU2CorZZ", "SU2CorDD"}; }
    // SU2EffectiveAction at the first cutoff (src/SU2/SU2EffectiveAction.hpp:38-60)
    void initial_state(const spn_lattice *lat, float *v2, std::vector<float *> &v4) override {
        check(spn_su2_initial_state(lat, int(n_v2), normalization_, v2, v4[1], v4[0]));
    }
    void set_state(float c, const float *v2, const std::vector<float *> &v4) override {
        check(spn_su2_set_state(h_, c, v2, v4[1], v4[0]));
    }
    void get_state(float &c, float *v2, const std::vector<float *> &v4) override {
        check(spn_su2_get_state(h_, &c, v2, v4[1], v4[0]));
    }
    void compute_step() override { check(spn_su2_compute_step(h_)); }
    bool diverged() override {
        int d = 0;
        check(spn_su2_is_diverged(h_, &d));
        return d != 0;
    }
    void finalize_step(float c) override { check(spn_su2_finalize_step(h_, c)); }
    void measure(const std::vector<float *> &out) override {
        check(spn_su2_measure_correlation(h_, out[0], out[1], nullptr, nullptr));
    }
    void synchronize() override { check(spn_su2_synchronize(h_)); }
    void autotune(float at, float current) override {
        int npi = 0, smem = 0, grid = 0;
        check(spn_su2_set_cutoff(h_, at));
        check(spn_su2_autotune(h_, 3, &npi, &smem, &grid));
        check(spn_su2_set_cutoff(h_, current));
        log(LogLevel::Debug, "Vertex flow variant: " + std::to_string(npi) + " node(s) per iteration, schedule in " +
                                 (smem ? "shared" : "global") + " memory, grid " + std::to_string(grid));
    }

private:
    spn_su2 *h_ = nullptr;
    float normalization_;
};

class XyzCore : public Core {
public:
    XyzCore(spn_lattice *lat, const std::vector<float> &freq, float normalization, int device)
        : normalization_(normalization) {
        spn_lattice_info info;
        check(spn_lattice_get_info(lat, &info));
        const int nl = info.n_sites, no = info.n_overlap, nr = info.n_range;
        const int64_t n_corr = int64_t(info.n_basis) * nr;
        std::vector<int> srid(nl), irid(nl), optr(nl + 1), o1(no), o2(no), rr(nr), ri(nr), cr(n_corr);
        std::vector<int> sp(nl), ip(nl), p1(no), p2(no), rp(nr), rip(nr), cp(n_corr);
        check(spn_lattice_get_tables(lat, srid.data(), irid.data(), optr.data(), o1.data(), o2.data(), rr.data(),
                                     ri.data(), cr.data(), nullptr, nullptr, nullptr));
        check(spn_lattice_get_spin_tables(lat, sp.data(), ip.data(), p1.data(), p2.data(), rp.data(), rip.data(),
                                          cp.data()));
        spn_xyz_desc d{};
        d.n_freq = int(freq.size());
        d.freq = freq.data();
        d.n_sites = nl;
        d.sites_rid = srid.data();
        d.sites_perm = sp.data();
        d.inv_sites_rid = irid.data();
        d.inv_sites_perm = ip.data();
        d.overlap_ptr = optr.data();
        d.overlap_rid1 = o1.data();
        d.overlap_rid2 = o2.data();
        d.overlap_perm1 = p1.data();
        d.overlap_perm2 = p2.data();
        d.n_range = nr;
        d.range_rid = rr.data();
        d.range_inv_rid = ri.data();
        d.n_corr = int(n_corr);
        d.corr_rid = cr.data();
        d.corr_perm = cp.data();
        d.device = device;
        check(spn_xyz_create(&d, &h_));
        const int64_t n = int64_t(freq.size());
        n_v2 = n;
        n_v4 = n * n * (n + 1) / 2 * nl;
    }
    ~XyzCore() override { spn_xyz_destroy(h_); }
    const char *id() const override { return "XYZ"; }
    std::vector<std::string> arrays() const override { return {"v4dd", "v4xx", "v4yy", "v4zz"}; }
    std::vector<std::string> obs_groups() const override { return {"XYZCorXX", "XYZCorYY", "XYZCorZZ", "XYZCorDD"}; }
    // XYZEffectiveAction at the first cutoff (src/XYZ/XYZEffectiveAction.hpp:38-60)
    void initial_state(const spn_lattice *lat, float *v2, std::vector<float *> &v4) override {
        check(spn_xyz_initial_state(lat, int(n_v2), normalization_, v2, v4[1], v4[2], v4[3], v4[0]));
    }
    void set_state(float c, const float *v2, const std::vector<float *> &v4) override {
        check(spn_xyz_set_state(h_, c, v2, v4[1], v4[2], v4[3], v4[0]));
    }
    void get_state(float &c, float *v2, const std::vector<float *> &v4) override {
        check(spn_xyz_get_state(h_, &c, v2, v4[1], v4[2], v4[3], v4[0]));
    }
    void compute_step() override { check(spn_xyz_compute_step(h_)); }
    bool diverged() override {
        int d = 0;
        check(spn_xyz_is_diverged(h_, &d));
        return d != 0;
    }
    void finalize_step(float c) override { check(spn_xyz_finalize_step(h_, c)); }
    void measure(const std::vector<float *> &out) override {
        check(spn_xyz_measure_correlation(h_, out[0], out[1], out[2], out[3], nullptr));
    }
    void synchronize() override {
        int d = 0;
        check(spn_xyz_is_diverged(h_, &d));  // synchronises the flow's stream
    }
    void autotune(float, float) override {}

private:
    spn_xyz *h_ = nullptr;
    float normalization_;
};

class TriCore : public Core {
public:
    TriCore(spn_lattice *lat, const std::vector<float> &freq, float normalization, int device)
        : normalization_(normalization) {
        spn_lattice_info info;
        check(spn_lattice_get_info(lat, &info));
        const int nl = info.n_sites, no = info.n_overlap, nr = info.n_range;
        n_corr_ = int64_t(info.n_basis) * nr;
        std::vector<int> srid(nl), irid(nl), optr(nl + 1), o1(no), o2(no), rr(nr), ri(nr), cr(n_corr_);
        std::vector<int> sp(nl), ip(nl), p1(no), p2(no), rp(nr), rip(nr), cp(n_corr_);
        check(spn_lattice_get_tables(lat, srid.data(), irid.data(), optr.data(), o1.data(), o2.data(), rr.data(),
                                     ri.data(), cr.data(), nullptr, nullptr, nullptr));
        check(spn_lattice_get_spin_tables(lat, sp.data(), ip.data(), p1.data(), p2.data(), rp.data(), rip.data(),
                                          cp.data()));
        spn_tri_desc d{};
        d.n_freq = int(freq.size());
        d.freq = freq.data();
        d.n_sites = nl;
        d.sites_rid = srid.data();
        d.sites_perm = sp.data();
        d.inv_sites_rid = irid.data();
        d.inv_sites_perm = ip.data();
        d.overlap_ptr = optr.data();
        d.overlap_rid1 = o1.data();
        d.overlap_rid2 = o2.data();
        d.overlap_perm1 = p1.data();
        d.overlap_perm2 = p2.data();
        d.n_range = nr;
        d.range_rid = rr.data();
        d.range_inv_rid = ri.data();
        d.n_corr = int(n_corr_);
        d.corr_rid = cr.data();
        d.corr_perm = cp.data();
        d.device = device;
        check(spn_tri_create(&d, &h_));
        const int64_t n = int64_t(freq.size());
        n_v2 = n;
        n_v4 = n * n * (n + 1) / 2 * 16 * nl;
        corr_.resize(size_t(10 * n_corr_));
    }
    ~TriCore() override { spn_tri_destroy(h_); }
    const char *id() const override { return "TRI"; }
    // TRIEffectiveAction::writeCheckpoint (src/TRI/TRIEffectiveAction.hpp:146-148)
    std::vector<std::string> arrays() const override { return {"v4"}; }
    // TRIMeasurementCorrelation::takeMeasurement (src/TRI/TRIMeasurementCorrelation.cpp:128-145)
    std::vector<std::string> obs_groups() const override {
        return {"TRICorXX", "TRICorXY", "TRICorXZ", "TRICorYX", "TRICorYY", "TRICorYZ", "TRICorZX", "TRICorZY", "TRICorZZ",
                "TRICorDD"};
    }
    // TRIEffectiveAction at the first cutoff (src/TRI/TRIEffectiveAction.hpp:38-62)
    void initial_state(const spn_lattice *lat, float *v2, std::vector<float *> &v4) override {
        check(spn_tri_initial_state(lat, int(n_v2), normalization_, v2, v4[0]));
    }
    void set_state(float c, const float *v2, const std::vector<float *> &v4) override {
        check(spn_tri_set_state(h_, c, v2, v4[0]));
    }
    void get_state(float &c, float *v2, const std::vector<float *> &v4) override {
        check(spn_tri_get_state(h_, &c, v2, v4[0]));
    }
    void compute_step() override { check(spn_tri_compute_step(h_)); }
    bool diverged() override {
        int d = 0;
        check(spn_tri_is_diverged(h_, &d));
        return d != 0;
    }
    void finalize_step(float c) override { check(spn_tri_finalize_step(h_, c)); }
    void measure(const std::vector<float *> &out) override {
        check(spn_tri_measure_correlation(h_, corr_.data(), nullptr));
        for (size_t q = 0; q < out.size(); ++q)
            if (out[q]) std::memcpy(out[q], corr_.data() + q * n_corr_, sizeof(float) * size_t(n_corr_));
    }
    void synchronize() override {
        int d = 0;
        check(spn_tri_is_diverged(h_, &d));  // synchronises the flow's stream
    }
    void autotune(float, float) override {}

private:
    spn_tri *h_ = nullptr;
    float normalization_;
    int64_t n_corr_ = 0;
    std::vector<float> corr_;
};

class Driver {
public:
    Driver(Task &task, const spn_run_options &o, spn_run_result &res) : task_(task), o_(o), res_(res) {}

    void build(const std::string &resdir) {
        lat_.reset(new spn_lattice);
        lat_->uc = read_unit_cell(resdir, task_.lattice);
        lat_->model = read_spin_model(resdir, task_.model, task_.model_options);
        lat_->lat = build_lattice(lat_->uc, lat_->model, task_.range);
        write_ldf(lat_->lat, lat_->uc, lat_->model, task_.files.ldf);
        log(LogLevel::Info, "Generated lattice model.");

        for (const MeasurementSpec &m : task_.measurements) {
            if (m.name != "correlation") throw Error(ErrorType::Initialization, "Measurement: Unknown measurement type '" + m.name + "'.");
            if (!m.options.empty())
                throw Error(ErrorType::Initialization, "Measurement [correlation]: unknown option '" + m.options[0].first + "'.");
            any_deferred_ = any_deferred_ || m.defer;
        }
        if (task_.symmetry != "SU2" && task_.symmetry != "XYZ" && task_.symmetry != "TRI")
            throw Error(ErrorType::Argument, "Spin model identifier '" + task_.symmetry + "' does not exist.");
        // core options: model options that are not interaction parameters (src/TaskFileParser.cpp:310-317;
        // SU2: spin and normalization, src/SU2/SU2FrgCore.cpp:19-29; XYZ and TRI: normalization,
        // src/XYZ/XYZFrgCore.cpp:19-28, src/TRI/TRIFrgCore.cpp:19-28)
        for (const auto &kv : task_.model_options) {
            if (lat_->model.parameters.count(kv.first)) continue;
            if (kv.first == "spin" && task_.symmetry == "SU2") spin_ = float(parse_number(kv.second));
            else if (kv.first == "normalization") normalization_ = float(parse_number(kv.second));
            else throw Error(ErrorType::Initialization, "Unknown spin model option '" + kv.first + "'.");
        }
        if (std::isnan(normalization_)) normalization_ = task_.symmetry == "SU2" ? 2.0f * spin_ : 1.0f;
        meta_ = make_obs_meta(lat_->lat);
    }

    void print_lattice() const {
        const Lattice &L = lat_->lat;
        log(LogLevel::Info, "Printing lattice debug information.");
        log(LogLevel::Info, "\tNumber of basis sites per unit cell: " + std::to_string(L.basis.size()));
        log(LogLevel::Info, "\tNumber of allocated sites: " + std::to_string(L.n_sites()) + " (" + std::to_string(L.n_sites() * sizeof(int)) + " bytes)");
        log(LogLevel::Info, "\tNumber of sites within range of origin: " + std::to_string(L.range_ids[0].size()));
        log(LogLevel::Info, "\tNumber of parametrized sites: " + std::to_string(L.size));
        log(LogLevel::Info, "\tParametrization is as follows: ");
        log(LogLevel::Info, "\t\tid: (a0, a1, a2, b)");
        for (int i = 0; i < L.size; ++i) {
            const LatticeSite &s = L.sites[i];
            log(LogLevel::Info, "\t\t" + std::to_string(i) + ": (" + std::to_string(s.a0) + ", " + std::to_string(s.a1) + ", " +
                                    std::to_string(s.a2) + ", " + std::to_string(s.b) + ")");
        }
    }

    void create_core() {
        spn_lattice_info info;
        check(spn_lattice_get_info(lat_.get(), &info));
        n_corr_ = int64_t(info.n_basis) * info.n_range;
        if (task_.symmetry == "XYZ") core_.reset(new XyzCore(lat_.get(), task_.frequencies, normalization_, o_.device));
        else if (task_.symmetry == "TRI") core_.reset(new TriCore(lat_.get(), task_.frequencies, normalization_, o_.device));
        else core_.reset(new Su2Core(lat_.get(), task_.frequencies, spin_, normalization_, o_.device, o_.flags));
        v2_.resize(core_->n_v2);
        v4_.assign(core_->arrays().size(), std::vector<float>(core_->n_v4));
        corr_.assign(core_->obs_groups().size(), std::vector<float>(n_corr_));
        std::vector<float *> v4 = v4_ptrs();
        core_->initial_state(lat_.get(), v2_.data(), v4);
        set_state(task_.cutoffs.front());
        log(LogLevel::Info, std::string("Generated FRG core with identifier ") + core_->id() + ".");
    }

    void run() {
        ComputationStatus cs = task_.status;
        const std::vector<float> &cut = task_.cutoffs;
        if (cs.status == CalcStatus::New || cs.status == CalcStatus::Running) {
            size_t k = 0;
            if (cs.status == CalcStatus::Running) {
                float c = 0;
                if (!read_ckpt(task_.files.checkpoint, -1, c))
                    throw Error(ErrorType::IO, "Could not read checkpoint from [" + task_.files.checkpoint + "].");
                set_state(c);
                k = cut.size();
                for (size_t i = 0; i < cut.size(); ++i)
                    if (cut[i] == c) {
                        k = i;
                        break;
                    }
                if (k == cut.size())
                    throw Error(ErrorType::Initialization, "Checkpoint cutoff " + fixed6(c) + " is not a value of the cutoff discretization.");
                log(LogLevel::Info, "Resuming calculation from checkpoint at cutoff " + fixed6(c) + ".");
            }
            if (cs.status == CalcStatus::New) cs.start_time = std::time(nullptr);
            cs.checkpoint_time = std::time(nullptr);
            if (o_.autotune && k + 1 < cut.size()) autotune(cut[k + (cut.size() - k) / 2]);

            auto t0 = std::chrono::steady_clock::now();
            while (k + 1 < cut.size()) {
                log(LogLevel::Debug, "Begin computation of flow.");
                core_->compute_step();
                log(LogLevel::Debug, "Begin computation of measurements.");
                take_measurements(false);
                if (core_->diverged()) {
                    log(LogLevel::Info, "Vertex has diverged. Stopping calculation.");
                    res_.diverged = 1;
                    break;
                }
                ++k;
                core_->finalize_step(cut[k]);
                cutoff_ = cut[k];
                ++res_.steps;
                log(LogLevel::Info, "Current cutoff is at " + fixed6(cutoff_));
                std::time_t now = std::time(nullptr);
                if (now - cs.checkpoint_time > o_.checkpoint_time) {
                    cs.checkpoint_time = now;
                    cs.status = CalcStatus::Running;
                    write_checkpoint_and_status(cs);
                }
                maybe_flush_obs();
            }
            take_measurements(false);
            core_->synchronize();
            res_.flow_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

            if (o_.defer || any_deferred_) {
                cs.status = CalcStatus::Postprocessing;
            } else {
                cs.end_time = std::time(nullptr);
                cs.status = CalcStatus::Finished;
            }
            cs.checkpoint_time = std::time(nullptr);
            write_checkpoint_and_status(cs);
        } else if (cs.status == CalcStatus::Postprocessing) {
            log(LogLevel::Info, "Entering post-processing stage.");
            int n = 0;
            float c = 0;
            while (read_ckpt(task_.files.data, n++, c)) {
                set_state(c);
                log(LogLevel::Info, "Post-processing measurements at cutoff " + std::to_string(c));
                take_measurements(true);
            }
            obs_.flush();
            cs.end_time = std::time(nullptr);
            cs.status = CalcStatus::Finished;
            write_task(task_, cs);
            log(LogLevel::Info, "Post-processing done.");
        } else {
            log(LogLevel::Info, "Nothing left to do. Task had been finished already.");
        }
        obs_.flush();
        res_.status = int(cs.status);
    }

private:
    std::vector<float *> v4_ptrs() {
        std::vector<float *> p;
        for (auto &a : v4_) p.push_back(a.data());
        return p;
    }

    bool read_ckpt(const std::string &path, int id, float &c) {
        std::vector<std::pair<std::string, float *>> a;
        const std::vector<std::string> names = core_->arrays();
        for (size_t q = 0; q < names.size(); ++q) a.emplace_back(names[q], v4_[q].data());
        return read_checkpoint_arrays(path, id, c, v2_.data(), core_->n_v2, a, core_->n_v4);
    }

    void write_ckpt(const std::string &path, bool append) {
        float c = 0;
        core_->get_state(c, v2_.data(), v4_ptrs());
        std::vector<std::pair<std::string, const float *>> a;
        const std::vector<std::string> names = core_->arrays();
        for (size_t q = 0; q < names.size(); ++q) a.emplace_back(names[q], v4_[q].data());
        write_checkpoint_arrays(path, append, c, v2_.data(), core_->n_v2, a, core_->n_v4);
    }

    void set_state(float c) {
        core_->set_state(c, v2_.data(), v4_ptrs());
        cutoff_ = c;
    }

    void autotune(float at) { core_->autotune(at, cutoff_); }

    void take_measurements(bool postprocessing) {
        const std::vector<std::string> groups = core_->obs_groups();
        for (const MeasurementSpec &m : task_.measurements) {
            if (!(cutoff_ <= m.max_cutoff && cutoff_ >= m.min_cutoff)) continue;
            bool deferred = o_.defer || m.defer;
            if (deferred != postprocessing) continue;
            if (measured_cutoff_ != cutoff_) {
                std::vector<float *> out;
                for (auto &a : corr_) out.push_back(a.data());
                core_->measure(out);
                measured_cutoff_ = cutoff_;
                ++res_.measurements;
            }
            for (size_t q = 0; q < groups.size(); ++q) obs_.add(m.output, groups[q], meta_, cutoff_, corr_[q].data());
        }
        if (!postprocessing && (o_.defer || any_deferred_)) write_ckpt(task_.files.data, true);
    }

    // SpinParser::writeCheckpoint (src/SpinParser.cpp:212-220)
    void write_checkpoint_and_status(const ComputationStatus &cs) {
        log(LogLevel::Info, "Writing checkpoint.");
        write_ckpt(task_.files.checkpoint, false);
        obs_.flush();
        last_flush_ = std::time(nullptr);
        write_task(task_, cs);
    }

    void maybe_flush_obs() {
        std::time_t now = std::time(nullptr);
        if (now - last_flush_ >= kObsFlushSeconds) {
            obs_.flush();
            last_flush_ = now;
        }
    }

    Task &task_;
    const spn_run_options &o_;
    spn_run_result &res_;
    std::unique_ptr<spn_lattice> lat_;
    std::unique_ptr<Core> core_;
    ObsMeta meta_;
    ObsStore obs_;
    float spin_ = 0.5f, normalization_ = NAN;
    bool any_deferred_ = false;
    int64_t n_corr_ = 0;
    std::vector<float> v2_;
    std::vector<std::vector<float>> v4_, corr_;  // vertex arrays in checkpoint order; one correlation per group
    float cutoff_ = 0, measured_cutoff_ = -1.0f;
    std::time_t last_flush_ = std::time(nullptr);
};

}  // namespace

void run_task(const std::string &task_path, const spn_run_options &o, spn_run_result &res) {
    set_log_level(o.verbose < 0 ? LogLevel::Warning : (o.verbose > 0 ? LogLevel::Debug : LogLevel::Info));
    const std::string resdir = o.resource_path ? std::string(o.resource_path) : default_resource_path();
    Task task = parse_task(task_path, o.force_restart != 0);
    log(LogLevel::Info, "Task file [" + task_path + "]: " + std::to_string(task.frequencies.size()) + " frequencies, " +
                            std::to_string(task.cutoffs.size()) + " cutoff values.");
    Driver drv(task, o, res);
    drv.build(resdir);
    res.status = int(task.status.status);
    if (o.debug_lattice) {
        drv.print_lattice();
        log(LogLevel::Info, "Lattice debug output complete. Shutting down.");
        return;
    }
    // a finished task needs no device: the reference builds its core anyway, then does nothing
    if (task.status.status != CalcStatus::Finished) drv.create_core();
    log(LogLevel::Info, "Launching FRG numerics core");
    auto t0 = std::chrono::steady_clock::now();
    drv.run();
    log(LogLevel::Info, "Shutting down core. Computation took " +
                            fixed6(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count()) + " seconds. ");
}

}  // namespace spn

extern "C" int spn_run_options_default(spn_run_options *o) {
    return spn::guarded([&] {
        if (!o) throw spn::Error(spn::ErrorType::Argument, "spn_run_options_default: null argument");
        *o = spn_run_options{};
        o->checkpoint_time = 3600;
    });
}

extern "C" int spn_run_task(const char *task_path, const spn_run_options *o, spn_run_result *result) {
    return spn::guarded([&] {
        if (!task_path) throw spn::Error(spn::ErrorType::Argument, "spn_run_task: null task path");
        spn_run_options opts;
        if (o) opts = *o;
        else spn_run_options_default(&opts);
        spn_run_result r{};
        try {
            spn::run_task(task_path, opts, r);
        } catch (const spn::Error &e) {
            spn::log(spn::LogLevel::Error, std::string("Caught exception: ") + e.what());
            if (result) *result = r;
            throw;
        }
        if (result) *result = r;
    });
}
