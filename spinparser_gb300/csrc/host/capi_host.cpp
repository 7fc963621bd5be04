// Host half of the C ABI (include/spn_su2.h): error reporting, lattice construction,
// discretisations and the initial state.  None of these touch the GPU.
#include "capi_common.hpp"
#include "lattice_handle.hpp"
#include "log.hpp"
#include "rpa_schedule.hpp"
#include "../tri_algebra.hpp"
#include "pair_order.hpp"
#include "../../../include/spn_su2.h"
#include <atomic>
#include <cmath>
#include <cstdio>
#include <ctime>
#include <cstring>
#include <map>
#include <string>

namespace spn {
namespace {
thread_local std::string g_last_error;
std::atomic<int> g_log_level{int(LogLevel::Info)};
}
void set_last_error(const std::string &msg) { g_last_error = msg; }

void set_log_level(LogLevel display) { g_log_level = int(display); }

void log(LogLevel level, const std::string &msg) {
    if (int(level) < g_log_level) return;
    static const char *names[] = {"Debug", "Info", "Warning", "Error"};
    std::time_t t = std::time(nullptr);
    std::tm tm{};
    localtime_r(&t, &tm);
    char stamp[32];
    std::strftime(stamp, sizeof(stamp), "%Y-%m-%d %H:%M:%S", &tm);
    std::printf("[%s] %s: %s\n", stamp, names[int(level)], msg.c_str());
    std::fflush(stdout);
}
}  // namespace spn

extern "C" int spn_last_error(char *buf, size_t len) {
    const std::string &m = spn::g_last_error;
    if (buf && len > 0) {
        size_t n = m.size() < len - 1 ? m.size() : len - 1;
        std::memcpy(buf, m.data(), n);
        buf[n] = '\0';
    }
    return int(m.size());
}

extern "C" int spn_lattice_create(const char *resource_dir, const char *lattice_name, int range, const char *model_name,
                                  int n_params, const char *const *param_names, const char *const *param_values,
                                  spn_lattice **out) {
    return spn::guarded([&] {
        if (!resource_dir || !lattice_name || !model_name || !out || n_params < 0 || (n_params > 0 && (!param_names || !param_values)))
            throw spn::Error(spn::ErrorType::Argument, "spn_lattice_create: null argument");
        std::map<std::string, std::string> params;
        for (int i = 0; i < n_params; ++i) {
            if (!param_names[i] || !param_values[i]) throw spn::Error(spn::ErrorType::Argument, "spn_lattice_create: null parameter");
            if (!params.emplace(param_names[i], param_values[i]).second)
                throw spn::Error(spn::ErrorType::Initialization, std::string("Multiple definitions of parameter '") + param_names[i] + "'");
        }
        auto *h = new spn_lattice;
        try {
            h->uc = spn::read_unit_cell(resource_dir, lattice_name);
            h->model = spn::read_spin_model(resource_dir, model_name, params);
            h->lat = spn::build_lattice(h->uc, h->model, range);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

extern "C" int spn_lattice_destroy(spn_lattice *lat) {
    delete lat;
    return SPN_OK;
}

extern "C" int spn_lattice_get_info(const spn_lattice *lat, spn_lattice_info *info) {
    return spn::guarded([&] {
        if (!lat || !info) throw spn::Error(spn::ErrorType::Argument, "spn_lattice_get_info: null argument");
        const spn::Lattice &L = lat->lat;
        info->n_sites = L.size;
        info->n_sites_total = L.n_sites();
        info->n_basis = int(L.basis.size());
        info->n_range = int(L.range_ids[0].size());
        info->n_overlap = int(L.overlap_rid1.size());
        info->n_interactions = int(L.interactions.size());
    });
}

extern "C" int spn_lattice_get_spin_tables(const spn_lattice *lat, int *sites_perm, int *inv_sites_perm,
                                           int *overlap_perm1, int *overlap_perm2, int *range_perm, int *range_inv_perm,
                                           int *corr_perm) {
    return spn::guarded([&] {
        if (!lat) throw spn::Error(spn::ErrorType::Argument, "spn_lattice_get_spin_tables: null lattice");
        const spn::Lattice &L = lat->lat;
        const int nb = int(L.basis.size());
        const int nr = int(L.range_ids[0].size());
        if (sites_perm) {
            auto v = L.sites_perm();
            std::memcpy(sites_perm, v.data(), v.size() * sizeof(int));
        }
        if (inv_sites_perm) {
            auto v = L.inverted_sites_perm();
            std::memcpy(inv_sites_perm, v.data(), v.size() * sizeof(int));
        }
        if (overlap_perm1) std::memcpy(overlap_perm1, L.overlap_perm1.data(), L.overlap_perm1.size() * sizeof(int));
        if (overlap_perm2) std::memcpy(overlap_perm2, L.overlap_perm2.data(), L.overlap_perm2.size() * sizeof(int));
        for (int n = 0; n < nr; ++n) {
            int j = L.range_ids[0][n];
            if (range_perm) range_perm[n] = L.perm(0, j);
            if (range_inv_perm) range_inv_perm[n] = L.perm(j, 0);
        }
        for (int b = 0; b < nb; ++b)
            for (int n = 0; n < nr; ++n)
                if (corr_perm) corr_perm[b * nr + n] = L.perm(L.basis_ids[b], L.range_ids[b][n]);
    });
}

extern "C" int spn_lattice_get_tables(const spn_lattice *lat, int *sites_rid, int *inv_sites_rid, int *overlap_ptr,
                                      int *overlap_rid1, int *overlap_rid2, int *range_rid, int *range_inv_rid,
                                      int *corr_rid, double *site_pos, double *basis_pos, double *lattice_vectors) {
    return spn::guarded([&] {
        if (!lat) throw spn::Error(spn::ErrorType::Argument, "spn_lattice_get_tables: null lattice");
        const spn::Lattice &L = lat->lat;
        const int nb = int(L.basis.size());
        const int nr = int(L.range_ids[0].size());
        for (int b = 0; b < nb; ++b)
            if (int(L.range_ids[b].size()) != nr)
                throw spn::Error(spn::ErrorType::Unsupported, "basis sites with different range sizes are not supported");
        if (sites_rid) {
            auto v = L.sites_rid();
            std::memcpy(sites_rid, v.data(), v.size() * sizeof(int));
        }
        if (inv_sites_rid) {
            auto v = L.inverted_sites_rid();
            std::memcpy(inv_sites_rid, v.data(), v.size() * sizeof(int));
        }
        if (overlap_ptr) std::memcpy(overlap_ptr, L.overlap_ptr.data(), L.overlap_ptr.size() * sizeof(int));
        if (overlap_rid1) std::memcpy(overlap_rid1, L.overlap_rid1.data(), L.overlap_rid1.size() * sizeof(int));
        if (overlap_rid2) std::memcpy(overlap_rid2, L.overlap_rid2.data(), L.overlap_rid2.size() * sizeof(int));
        for (int n = 0; n < nr; ++n) {
            int j = L.range_ids[0][n];
            if (range_rid) range_rid[n] = L.transform(0, j);
            if (range_inv_rid) range_inv_rid[n] = L.transform(j, 0);
        }
        for (int b = 0; b < nb; ++b)
            for (int n = 0; n < nr; ++n) {
                int j = L.range_ids[b][n];
                if (corr_rid) corr_rid[b * nr + n] = L.transform(L.basis_ids[b], j);
                if (site_pos) {
                    spn::Vec3 p = L.position(j);
                    double *o = site_pos + 3 * (size_t(b) * nr + n);
                    o[0] = p.x; o[1] = p.y; o[2] = p.z;
                }
            }
        if (basis_pos)
            for (int b = 0; b < nb; ++b) {
                spn::Vec3 p = L.position(L.basis_ids[b]);
                basis_pos[3 * b] = p.x; basis_pos[3 * b + 1] = p.y; basis_pos[3 * b + 2] = p.z;
            }
        if (lattice_vectors)
            for (int i = 0; i < 3; ++i) {
                lattice_vectors[3 * i] = L.primitives[i].x;
                lattice_vectors[3 * i + 1] = L.primitives[i].y;
                lattice_vectors[3 * i + 2] = L.primitives[i].z;
            }
    });
}

extern "C" int spn_lattice_get_sites(const spn_lattice *lat, int *site_params, int *pair_rid) {
    return spn::guarded([&] {
        if (!lat) throw spn::Error(spn::ErrorType::Argument, "spn_lattice_get_sites: null lattice");
        const spn::Lattice &L = lat->lat;
        if (site_params)
            for (int i = 0; i < L.n_sites(); ++i) {
                site_params[4 * i] = L.sites[i].a0;
                site_params[4 * i + 1] = L.sites[i].a1;
                site_params[4 * i + 2] = L.sites[i].a2;
                site_params[4 * i + 3] = L.sites[i].b;
            }
        if (pair_rid) std::memcpy(pair_rid, L.sym_rid.data(), L.sym_rid.size() * sizeof(int));
    });
}

extern "C" int spn_lattice_get_interactions(const spn_lattice *lat, int *rid, float *coupling) {
    return spn::guarded([&] {
        if (!lat) throw spn::Error(spn::ErrorType::Argument, "spn_lattice_get_interactions: null lattice");
        const auto &I = lat->lat.interactions;
        for (size_t n = 0; n < I.size(); ++n) {
            if (rid) rid[n] = I[n].rid;
            if (coupling)
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) coupling[9 * n + 3 * a + b] = I[n].J[a][b];
        }
    });
}

extern "C" int spn_lattice_write_ldf(const spn_lattice *lat, const char *path) {
    return spn::guarded([&] {
        if (!lat || !path) throw spn::Error(spn::ErrorType::Argument, "spn_lattice_write_ldf: null argument");
        spn::write_ldf(lat->lat, lat->uc, lat->model, path);
    });
}

extern "C" int spn_frequency_exponential(float min, float max, int count, float *out) {
    return spn::guarded([&] {
        if (!out) throw spn::Error(spn::ErrorType::Argument, "spn_frequency_exponential: null output");
        if (!(min > 0)) throw spn::Error(spn::ErrorType::Initialization, "frequency min must be positive");
        if (!(max > min)) throw spn::Error(spn::ErrorType::Initialization, "frequency max must be greater than min");
        if (count <= 1) throw spn::Error(spn::ErrorType::Initialization, "frequency count must be greater than 1");
        float fc = float(count);
        float step = powf(max / min, 1.0f / (fc - 1));
        for (int i = 0; i < count; ++i) out[i] = min * powf(step, float(i));
    });
}

extern "C" int spn_parse_number(const char *text, double *value) {
    return spn::guarded([&] {
        if (!text || !value) throw spn::Error(spn::ErrorType::Argument, "spn_parse_number: null argument");
        *value = spn::parse_number(text);
    });
}

extern "C" int spn_cutoff_exponential(float max, float min, float step, float *out, int cap, int *n) {
    return spn::guarded([&] {
        if (!n || (cap > 0 && !out)) throw spn::Error(spn::ErrorType::Argument, "spn_cutoff_exponential: null output");
        if (!(min > 0)) throw spn::Error(spn::ErrorType::Initialization, "cutoff min must be positive");
        if (!(max > min)) throw spn::Error(spn::ErrorType::Initialization, "cutoff max must be greater than min");
        if (!(step > 0 && step < 1)) throw spn::Error(spn::ErrorType::Initialization, "cutoff step must be in (0,1)");
        int k = 0;
        float v = max;
        while (v > min) {
            if (k < cap) out[k] = v;
            ++k;
            v *= step;
        }
        *n = k;
    });
}

extern "C" int spn_su2_initial_state(const spn_lattice *lat, int n_freq, float normalization, float *v2, float *v4ss,
                                     float *v4dd) {
    return spn::guarded([&] {
        if (!lat || n_freq < 2) throw spn::Error(spn::ErrorType::Argument, "spn_su2_initial_state: bad argument");
        const spn::Lattice &L = lat->lat;
        const long long nl = L.size;
        const long long fn = (long long)n_freq * n_freq * (n_freq + 1) / 2;
        if (v2) std::memset(v2, 0, sizeof(float) * n_freq);
        if (v4dd) std::memset(v4dd, 0, sizeof(float) * size_t(fn * nl));
        if (v4ss) {
            std::memset(v4ss, 0, sizeof(float) * size_t(fn * nl));
            for (long long it = 0; it < fn; ++it)
                for (const auto &ia : L.interactions) v4ss[it * nl + ia.rid] += ia.J[0][0] / normalization;
        }
    });
}

extern "C" int spn_xyz_initial_state(const spn_lattice *lat, int n_freq, float normalization, float *v2, float *v4xx,
                                     float *v4yy, float *v4zz, float *v4dd) {
    return spn::guarded([&] {
        if (!lat || n_freq < 2) throw spn::Error(spn::ErrorType::Argument, "spn_xyz_initial_state: bad argument");
        const spn::Lattice &L = lat->lat;
        const long long nl = L.size;
        const long long fn = (long long)n_freq * n_freq * (n_freq + 1) / 2;
        if (v2) std::memset(v2, 0, sizeof(float) * n_freq);
        if (v4dd) std::memset(v4dd, 0, sizeof(float) * size_t(fn * nl));
        float *comp[3] = {v4xx, v4yy, v4zz};
        for (int c = 0; c < 3; ++c) {
            if (!comp[c]) continue;
            std::memset(comp[c], 0, sizeof(float) * size_t(fn * nl));
            for (long long it = 0; it < fn; ++it)
                for (const auto &ia : L.interactions) comp[c][it * nl + ia.rid] += 0.25f * ia.J[c][c] / normalization;
        }
    });
}

extern "C" int spn_tri_initial_state(const spn_lattice *lat, int n_freq, float normalization, float *v2, float *v4) {
    return spn::guarded([&] {
        if (!lat || n_freq < 2 || !v4) throw spn::Error(spn::ErrorType::Argument, "spn_tri_initial_state: bad argument");
        const spn::Lattice &L = lat->lat;
        const long long nl = L.size;
        const long long fn = (long long)n_freq * n_freq * (n_freq + 1) / 2;
        if (v2) std::memset(v2, 0, sizeof(float) * n_freq);
        std::memset(v4, 0, sizeof(float) * size_t(16 * fn * nl));
        for (long long it = 0; it < fn; ++it)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    for (const auto &ia : L.interactions)
                        v4[(it * 16 + 4 * a + b) * nl + ia.rid] += 0.25f * ia.J[a][b] / normalization;
    });
}

extern "C" int spn_rpa_pair_order(int layout, int n_sites, const int *overlap_ptr, const int *overlap_rid1,
                                  const int *overlap_rid2, const int *overlap_perm1, const int *overlap_perm2, int *order,
                                  long long *collisions) {
    return spn::guarded([&] {
        if ((layout != 0 && layout != 1) || n_sites < 1 || n_sites > 128 || !overlap_ptr || !order)
            throw spn::Error(spn::ErrorType::Argument, "spn_rpa_pair_order: bad argument");
        const int nov = overlap_ptr[n_sites];
        if (nov > 0 && (!overlap_rid1 || !overlap_rid2 || !overlap_perm1 || !overlap_perm2))
            throw spn::Error(spn::ErrorType::Argument, "spn_rpa_pair_order: null pair table");
        for (int i = 0; i < nov; ++i)
            if (overlap_rid1[i] < 0 || overlap_rid1[i] >= n_sites || overlap_rid2[i] < 0 || overlap_rid2[i] >= n_sites ||
                overlap_perm1[i] < 0 || overlap_perm1[i] >= 6 || overlap_perm2[i] < 0 || overlap_perm2[i] >= 6)
                throw spn::Error(spn::ErrorType::Argument, "spn_rpa_pair_order: pair entry out of range");
        const spn::PairBankModel m = layout == 0 ? spn::xyz_rpa_model() : spn::tri_rpa_model();
        const auto words = layout == 0
                               ? spn::xyz_rpa_words(n_sites, overlap_rid1, overlap_rid2, overlap_perm1, overlap_perm2)
                               : spn::tri_rpa_words(n_sites, overlap_rid1, overlap_rid2, overlap_perm1, overlap_perm2);
        const std::vector<int> o = spn::order_pairs_by_banks(n_sites, overlap_ptr, m, words);
        std::memcpy(order, o.data(), o.size() * sizeof(int));
        if (collisions) {
            std::vector<int> natural(static_cast<size_t>(nov));
            for (int i = 0; i < nov; ++i) natural[size_t(i)] = i;
            collisions[0] = spn::pair_bank_collisions(n_sites, overlap_ptr, natural.data(), m, words);
            collisions[1] = spn::pair_bank_collisions(n_sites, overlap_ptr, o.data(), m, words);
        }
    });
}

extern "C" int spn_rpa_lane_schedule(int layout, int n_sites, const int *overlap_ptr, const int *words, int *info,
                                     int *sched, int *count, int *slot_base, int *seg_ptr) {
    return spn::guarded([&] {
        if (layout < 0 || layout > 2 || n_sites < 1 || n_sites > 128 || !overlap_ptr || !info)
            throw spn::Error(spn::ErrorType::Argument, "spn_rpa_lane_schedule: bad argument");
        const int nov = overlap_ptr[n_sites];
        for (int r = 0; r < n_sites; ++r)
            if (overlap_ptr[r + 1] < overlap_ptr[r]) throw spn::Error(spn::ErrorType::Argument, "overlap_ptr must be non-decreasing");
        if (nov > 0 && !words) throw spn::Error(spn::ErrorType::Argument, "spn_rpa_lane_schedule: null words");
        const int last_bit = layout == 1 ? 20 : 26;
        for (int i = 0; i < nov; ++i)
            if (words[i] < 0 || words[i] >= (1 << last_bit) || (words[i] & 127) >= n_sites || ((words[i] >> 7) & 127) >= n_sites)
                throw spn::Error(spn::ErrorType::Argument, "spn_rpa_lane_schedule: pair word out of range");
        const std::vector<int> w(words, words + nov);
        const spn::LaneSchedule s = layout == 1   ? spn::xyz_lane_schedule(n_sites, overlap_ptr, w)
                                    : layout == 2 ? spn::tri_lane_schedule(n_sites, overlap_ptr, w)
                                                  : spn::lane_schedule(n_sites, overlap_ptr, w, 32, last_bit);
        info[0] = s.len;
        info[1] = s.n_seg;
        info[2] = int(s.sched.size());
        info[3] = last_bit;
        if (!sched) return;
        std::memcpy(sched, s.sched.data(), s.sched.size() * sizeof(int));
        if (count) std::memcpy(count, s.count.data(), s.count.size() * sizeof(int));
        if (slot_base) std::memcpy(slot_base, s.slot_base.data(), s.slot_base.size() * sizeof(int));
        if (seg_ptr) std::memcpy(seg_ptr, s.seg_ptr.data(), s.seg_ptr.size() * sizeof(int));
    });
}

extern "C" int spn_tri_tables(int *rows) {
    return spn::guarded([&] {
        if (!rows) throw spn::Error(spn::ErrorType::Argument, "spn_tri_tables: null argument");
        namespace T = spn::tri;
        int n = 0;
        auto put = [&](int tab, int c, int k, int a, int b, int sg) {
            int *r = rows + 6 * n++;
            r[0] = tab; r[1] = c; r[2] = k; r[3] = a; r[4] = b; r[5] = sg;
        };
        for (int c = 0; c < 16; ++c) {
            const int c1 = c >> 2, c2 = c & 3;
            for (int k = 0; k < 16; ++k) put(0, c, k, 15 - k, (15 - k) ^ c ^ 15, T::pp_sign(c, 15 - k));
            for (int k = 0; k < 16; ++k) put(1, c, k, 15 - k, (15 - k) ^ c ^ 15, T::ph_sign(c, 15 - k));
            for (int k = 0; k < 4; ++k) put(2, c, k, 4 * c1 + T::inner(k), 4 * T::inner(k) + c2, T::rpa_sign(c, T::inner(k)));
            for (int k = 0; k < 16; ++k) {
                const int kap = T::inner(k >> 2), lam = T::inner(k & 3);
                put(3, c, k, 4 * c1 + kap, 4 * lam + (c2 ^ kap ^ lam), T::chal_sign(c, kap, lam));
            }
            for (int k = 0; k < 16; ++k) {
                const int l = 15 - k;
                put(4, c, k, l, 4 * (c1 ^ (l >> 2) ^ (l & 3)) + c2, T::ichal_sign(c, l));
            }
            for (int k = 0; k < 4; ++k) {
                const int lam = T::inner(k);
                put(5, c, k, 4 * lam + (c1 ^ c2 ^ lam), 0, T::egg_sign(c, lam));
            }
        }
    });
}

extern "C" int spn_rpa_schedule(int n_sites, const int *overlap_ptr, const int *overlap_rid1, const int *overlap_rid2,
                                int lanes, int *info, int *sched, int *count, int *slot_base, int *seg_ptr) {
    return spn::guarded([&] {
        if (n_sites < 1 || n_sites > 128 || !overlap_ptr || !info || lanes < 1 || lanes > 256)
            throw spn::Error(spn::ErrorType::Argument, "spn_rpa_schedule: bad argument");
        const int nov = overlap_ptr[n_sites];
        for (int r = 0; r < n_sites; ++r)
            if (overlap_ptr[r + 1] < overlap_ptr[r]) throw spn::Error(spn::ErrorType::Argument, "overlap_ptr must be non-decreasing");
        for (int i = 0; i < nov; ++i)
            if (overlap_rid1[i] < 0 || overlap_rid1[i] >= n_sites || overlap_rid2[i] < 0 || overlap_rid2[i] >= n_sites)
                throw spn::Error(spn::ErrorType::Argument, "overlap entry out of range");
        spn::RpaHostSchedule s = spn::build_rpa_schedule(n_sites, overlap_ptr, overlap_rid1, overlap_rid2, lanes);
        info[0] = s.len;
        info[1] = s.n_seg;
        info[2] = int(s.sched.size());
        info[3] = s.packed ? 1 : 0;
        info[4] = s.width;
        if (!sched) return;
        std::memcpy(sched, s.sched.data(), s.sched.size() * sizeof(int));
        if (count) std::memcpy(count, s.count.data(), s.count.size() * sizeof(int));
        if (slot_base) std::memcpy(slot_base, s.slot_base.data(), s.slot_base.size() * sizeof(int));
        if (seg_ptr) std::memcpy(seg_ptr, s.seg_ptr.data(), s.seg_ptr.size() * sizeof(int));
    });
}
