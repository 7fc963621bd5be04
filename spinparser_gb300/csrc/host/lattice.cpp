// Lattice / spin-model construction.  See lattice.hpp for the contract.
//
// Reference behaviour restated here (file:line in the SpinParser sources):
//   * unit-cell reader            src/LatticeModelFactory.cpp:107-181
//   * spin-model reader           src/LatticeModelFactory.cpp:244-365
//   * neighbour / range search    src/LatticeModelFactory.cpp:458-489
//   * site lookup by position     src/LatticeModelFactory.cpp:498-513
//   * automorphism search         src/LatticeModelFactory.cpp:516-730
//   * table construction          src/LatticeModelFactory.cpp:733-985
//   * .ldf debug output           src/LatticeModelFactory.cpp:987-1043
#include "lattice.hpp"
#include "error.hpp"
#include "xml.hpp"
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <dirent.h>
#include <fstream>
#include <regex>
#include <sstream>
#include <iomanip>
#include <sys/stat.h>
#include <unordered_map>

namespace spn {

namespace {

constexpr double kEps = 0.00001;
constexpr double kPi = 3.14159265358979323846;

struct SiteHash {
    size_t operator()(const LatticeSite &s) const {
        size_t h = size_t(uint32_t(s.a0)) * 73856093u;
        h ^= size_t(uint32_t(s.a1)) * 19349663u;
        h ^= size_t(uint32_t(s.a2)) * 83492791u;
        h ^= size_t(uint32_t(s.b)) * 2654435761u;
        return h;
    }
};

// Insertion-ordered set of sites with O(1) membership / index lookup.
struct SiteList {
    std::vector<LatticeSite> v;
    std::unordered_map<LatticeSite, int, SiteHash> idx;
    bool contains(const LatticeSite &s) const { return idx.count(s) != 0; }
    int index_of(const LatticeSite &s) const {
        auto it = idx.find(s);
        return it == idx.end() ? -1 : it->second;
    }
    bool push(const LatticeSite &s) {
        if (contains(s)) return false;
        idx.emplace(s, int(v.size()));
        v.push_back(s);
        return true;
    }
    void rebuild() {
        idx.clear();
        for (int i = 0; i < int(v.size()); ++i) idx.emplace(v[i], i);
    }
};

// Files with extension .xml in a resource directory, sorted by name so that the lookup is
// deterministic (the reference iterates the directory in filesystem order).
std::vector<std::string> xml_files(const std::string &dir) {
    std::vector<std::string> out;
    DIR *d = opendir(dir.c_str());
    if (!d) throw Error(ErrorType::IO, "cannot open resource directory '" + dir + "'");
    while (dirent *e = readdir(d)) {
        std::string name = e->d_name;
        if (name.size() < 4 || name.compare(name.size() - 4, 4, ".xml") != 0) continue;
        std::string path = dir + "/" + name;
        struct stat st;
        if (stat(path.c_str(), &st) == 0 && S_ISREG(st.st_mode)) out.push_back(path);
    }
    closedir(d);
    std::sort(out.begin(), out.end());
    return out;
}

const std::string &req_attr(const XmlNode &n, const char *key, const std::string &what) {
    const std::string *v = n.attr(key);
    if (!v) throw Error(ErrorType::Initialization, what + " '" + key + "' attribute missing.");
    return *v;
}

Vec3 site_position(const LatticeUnitCell &uc, const LatticeSite &s) {
    return double(s.a0) * uc.primitives[0] + double(s.a1) * uc.primitives[1] + double(s.a2) * uc.primitives[2] +
           uc.basis[s.b];
}

// Nearest neighbours through the bond list, in bond order (LatticeBond::getOtherEnd).
std::vector<LatticeSite> neighbours(const LatticeUnitCell &uc, const LatticeSite &s) {
    std::vector<LatticeSite> out;
    for (const auto &bd : uc.bonds) {
        if (bd.from_b != s.b && bd.to_b != s.b) continue;
        if (bd.from_b == s.b) {
            out.emplace_back(s.a0 + bd.da0, s.a1 + bd.da1, s.a2 + bd.da2, bd.to_b);
            if (bd.from_b == bd.to_b) out.emplace_back(s.a0 - bd.da0, s.a1 - bd.da1, s.a2 - bd.da2, bd.from_b);
        } else {
            out.emplace_back(s.a0 - bd.da0, s.a1 - bd.da1, s.a2 - bd.da2, bd.from_b);
        }
    }
    return out;
}

// All sites within `range` bonds of `s`, in the reference's breadth-first order.
SiteList range_around(const LatticeUnitCell &uc, const LatticeSite &s, int range) {
    SiteList sites;
    sites.push(s);
    for (int step = 0; step < range; ++step) {
        SiteList frontier;
        for (const auto &x : sites.v)
            for (const auto &n : neighbours(uc, x)) frontier.push(n);
        for (const auto &n : frontier.v) sites.push(n);
    }
    return sites;
}

struct SiteLocator {
    const LatticeUnitCell &uc;
    Mat3 inv;
    explicit SiteLocator(const LatticeUnitCell &u)
        : uc(u), inv(Mat3::columns(u.primitives[0], u.primitives[1], u.primitives[2]).inverse()) {}
    bool locate(const Vec3 &p, LatticeSite &out) const {
        for (int b = 0; b < int(uc.basis.size()); ++b) {
            Vec3 n = inv * (p - uc.basis[b]);
            if (std::fabs(n.x - std::round(n.x)) < kEps && std::fabs(n.y - std::round(n.y)) < kEps &&
                std::fabs(n.z - std::round(n.z)) < kEps) {
                out = LatticeSite(int(std::lround(n.x)), int(std::lround(n.y)), int(std::lround(n.z)), b);
                return true;
            }
        }
        return false;
    }
};

// The six global spin-component permutations in the reference's enumeration order.
constexpr int kSpinPerm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};

// Lattice automorphisms that map `target` onto the origin (0,0,0,0) and leave all
// couplings invariant up to a global spin permutation.  Candidates are built from
// the same construction as the reference: optional point inversion, translation of
// `target` to the origin, a rotation aligning the first neighbour direction, and a
// rotation about that direction aligning the first non-collinear neighbour.
struct Automorphism {
    Affine T;
    int perm;  // index into kSpinPerm
};

std::vector<Automorphism> lattice_automorphisms(const LatticeUnitCell &uc, const SpinModelUnitCell &model,
                                                const SiteLocator &loc, const LatticeSite &target, bool first_only) {
    const LatticeSite ref(0, 0, 0, 0);
    const Vec3 pref = site_position(uc, ref);

    std::vector<LatticeSite> pre;  // sites whose images must be lattice sites
    auto add_pre = [&](const LatticeSite &s) {
        if (std::find(pre.begin(), pre.end(), s) == pre.end()) pre.push_back(s);
    };
    for (int b = 0; b < int(uc.basis.size()); ++b) add_pre(LatticeSite(0, 0, 0, b));
    for (const auto &bd : uc.bonds) add_pre(LatticeSite(bd.da0, bd.da1, bd.da2, bd.to_b));

    std::vector<LatticeSite> nb = neighbours(uc, target);
    if (nb.size() < 3) throw Error(ErrorType::Initialization, "Could not build lattice. Too few neighbors.");
    const Vec3 pt = site_position(uc, target);
    LatticeSite n1 = nb[0], n2;
    for (size_t i = 1; i < nb.size(); ++i) {
        if (cross(site_position(uc, n1) - pt, site_position(uc, nb[i]) - pt).norm() > kEps) {
            n2 = nb[i];
            break;
        }
        if (i == nb.size() - 1) throw Error(ErrorType::Initialization, "Could not build lattice. Unfavorable lattice geometry.");
    }
    const Vec3 p1 = site_position(uc, n1), p2 = site_position(uc, n2);

    std::vector<Automorphism> found;
    std::vector<LatticeSite> ref_nb = neighbours(uc, ref);
    for (const auto &c1 : ref_nb) {
        for (const auto &c2 : ref_nb) {
            const Vec3 pc1 = site_position(uc, c1), pc2 = site_position(uc, c2);
            if (cross(pc1 - pref, pc2 - pref).norm() < kEps) continue;
            for (int inversion = 0; inversion <= 1; ++inversion) {
                if (first_only && !found.empty()) break;
                Affine T = inversion ? Affine::point_inversion() : Affine::identity();
                T = Affine::translation(pref - T.apply(pt)) * T;

                // align the first neighbour direction with c1
                Vec3 a = (T.apply(p1) - pref).normalized();
                Vec3 bdir = (pc1 - pref).normalized();
                Vec3 axis = cross(a, bdir);
                double angle = std::acos(dot(a, bdir));
                if (axis.norm() < kEps) {
                    if (dot(a, bdir) < 0) {
                        axis = (a.x != 0) ? Vec3(-a.y, a.x, 0) : Vec3(0, -a.z, a.y);
                        angle = kPi;
                    } else {
                        axis = Vec3(1, 0, 0);
                        angle = 0;
                    }
                }
                T = Affine::rotation_about(axis, pref, angle) * T;

                // rotate about the c1 direction to bring the second neighbour into the c1-c2 plane
                Vec3 q = T.apply(p2) - pref;
                Vec3 x = (q - dot(T.apply(p2) - pref, (pc1 - pref).normalized()) * (pc1 - pref).normalized()).normalized();
                Vec3 y = ((pc2 - pref) - dot(pc2 - pref, (pc1 - pref).normalized()) * (pc1 - pref).normalized()).normalized();
                axis = cross(x, y);
                angle = std::acos(dot(x, y));
                if (axis.norm() < kEps) {
                    axis = bdir;
                    angle = (dot(x, y) < 0) ? kPi : 0.0;
                }
                T = Affine::rotation_about(axis, pref, angle) * T;

                double e = (T.apply(pt) - pref).norm();
                if (e > kEps) throw Error(ErrorType::Internal, "Lattice symmetry calculation has failed (target site).");
                e = cross((T.apply(p1) - T.apply(pt)).normalized(), (pc1 - pref).normalized()).norm();
                if (e > kEps) throw Error(ErrorType::Internal, "Lattice symmetry calculation has failed (first neighbour).");
                e = dot(T.apply(p2) - pref, cross(pc1 - pref, pc2 - pref));
                if (std::fabs(e) > kEps) throw Error(ErrorType::Internal, "Lattice symmetry calculation has failed (second neighbour).");

                bool ok = true;
                LatticeSite img;
                for (const auto &p : pre) {
                    if (!loc.locate(T.apply(site_position(uc, p)), img)) {
                        ok = false;
                        break;
                    }
                }
                if (!ok) continue;

                int perm_found = -1;
                for (int pi = 0; pi < 6 && perm_found < 0; ++pi) {
                    bool valid = true;
                    for (const auto &cpl : model.couplings) {
                        LatticeSite ft, tt;  // default (0,0,0,0) when not on the lattice
                        loc.locate(T.apply(site_position(uc, cpl.from)), ft);
                        loc.locate(T.apply(site_position(uc, cpl.to)), tt);
                        float tgt[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                        for (const auto &other : model.couplings) {
                            int c = other.connects(ft, tt);
                            if (c == 1) {
                                for (int s1 = 0; s1 < 3; ++s1)
                                    for (int s2 = 0; s2 < 3; ++s2) tgt[s1][s2] = other.J[s1][s2];
                            } else if (c == -1) {
                                for (int s1 = 0; s1 < 3; ++s1)
                                    for (int s2 = 0; s2 < 3; ++s2) tgt[s1][s2] = other.J[s2][s1];
                            }
                        }
                        for (int s1 = 0; s1 < 3; ++s1)
                            for (int s2 = 0; s2 < 3; ++s2)
                                if (cpl.J[s1][s2] != tgt[kSpinPerm[pi][s1]][kSpinPerm[pi][s2]]) valid = false;
                    }
                    if (valid) perm_found = pi;
                }
                if (perm_found < 0) continue;
                found.push_back(Automorphism{T, perm_found});
            }
        }
    }
    if (found.empty())
        throw Error(ErrorType::Internal, "Lattice symmetry calculation has failed (identity is not a valid symmetry).");
    return found;
}

// Images of `s` (with the spin permutation that accompanies each map), de-duplicated on
// the (site, permutation) pair in order of discovery.
std::vector<std::pair<LatticeSite, int>> orbit(const LatticeUnitCell &uc, const SiteLocator &loc,
                                               const std::vector<Automorphism> &ts, const LatticeSite &s) {
    std::vector<std::pair<LatticeSite, int>> out;
    for (const auto &a : ts) {
        LatticeSite img;
        if (!loc.locate(a.T.apply(site_position(uc, s)), img))
            throw Error(ErrorType::Internal, "Lattice symmetry calculation has failed (image off the lattice).");
        std::pair<LatticeSite, int> e(img, a.perm);
        if (std::find(out.begin(), out.end(), e) == out.end()) out.push_back(e);
    }
    return out;
}

// compose(p, q)[c] = kSpinPerm[p][kSpinPerm[q][c]]: the spin permutation of a map q followed
// by the representative's own p (LatticeModelFactory.cpp:863-865).
int compose_perm(int p, int q) {
    int r[3];
    for (int c = 0; c < 3; ++c) r[c] = kSpinPerm[p][kSpinPerm[q][c]];
    for (int k = 0; k < 6; ++k)
        if (kSpinPerm[k][0] == r[0] && kSpinPerm[k][1] == r[1] && kSpinPerm[k][2] == r[2]) return k;
    return 0;
}

int inverse_perm(int p) {
    int inv[3];
    for (int k = 0; k < 3; ++k) inv[kSpinPerm[p][k]] = k;
    for (int q = 0; q < 6; ++q)
        if (kSpinPerm[q][0] == inv[0] && kSpinPerm[q][1] == inv[1] && kSpinPerm[q][2] == inv[2]) return q;
    return 0;
}

}  // namespace

int SpinCoupling::connects(const LatticeSite &s1, const LatticeSite &s2) const {
    auto from_to = [&](const LatticeSite &x, const LatticeSite &y) {
        return (to.a0 - from.a0) == (y.a0 - x.a0) && (to.a1 - from.a1) == (y.a1 - x.a1) &&
               (to.a2 - from.a2) == (y.a2 - x.a2) && from.b == x.b && to.b == y.b;
    };
    if (from_to(s1, s2)) return 1;
    if (from_to(s2, s1)) return -1;
    return 0;
}

Vec3 Lattice::position(int id) const {
    const LatticeSite &s = sites[id];
    return double(s.a0) * primitives[0] + double(s.a1) * primitives[1] + double(s.a2) * primitives[2] + basis[s.b];
}

std::vector<int> Lattice::sites_rid() const {
    std::vector<int> r(size);
    for (int j = 0; j < size; ++j) r[j] = transform(0, j);
    return r;
}

std::vector<int> Lattice::inverted_sites_rid() const {
    std::vector<int> r(size);
    for (int j = 0; j < size; ++j) r[j] = transform(j, 0);
    return r;
}

std::vector<int> Lattice::sites_perm() const {
    std::vector<int> r(size);
    for (int j = 0; j < size; ++j) r[j] = perm(0, j);
    return r;
}

std::vector<int> Lattice::inverted_sites_perm() const {
    std::vector<int> r(size);
    for (int j = 0; j < size; ++j) r[j] = perm(j, 0);
    return r;
}

double parse_number(const std::string &input) {
    static const std::regex sqrt_re("sqrt\\(([\\.\\d]+)\\)");
    static const std::regex muldiv_re("([\\.\\d]+)([\\*/])([\\.\\d]+)");
    auto fmt = [](double v) {
        std::ostringstream os;
        os << std::fixed << std::setprecision(20) << v;
        return os.str();
    };
    std::string s = input;
    std::smatch m;
    while (std::regex_search(s, m, sqrt_re)) s = m.prefix().str() + fmt(std::sqrt(std::stod(m.str(1)))) + m.suffix().str();
    while (std::regex_search(s, m, muldiv_re)) {
        double a = std::stod(m.str(1)), b = std::stod(m.str(3));
        s = m.prefix().str() + fmt(m.str(2) == "*" ? a * b : a / b) + m.suffix().str();
    }
    try {
        return std::stod(s);
    } catch (const std::exception &) {
        throw Error(ErrorType::Initialization, "cannot parse number '" + input + "'");
    }
}

LatticeUnitCell read_unit_cell(const std::string &dir, const std::string &name) {
    for (const auto &path : xml_files(dir)) {
        XmlNode doc = xml_parse_file(path);
        for (const auto &uc : doc.children) {
            if (uc.name != "unitcell") continue;
            const std::string *nm = uc.attr("name");
            if (!nm) throw Error(ErrorType::Initialization, "Invalid unit cell. Unit cell name is undefined.");
            if (*nm != name) continue;
            if (uc.count("primitive") != 3)
                throw Error(ErrorType::Initialization, "Invalid unit cell. Unit cell must define three primitive vectors.");
            if (uc.count("site") == 0)
                throw Error(ErrorType::Initialization, "Invalid unit cell. Unit cell must contain at least one lattice site.");
            if (uc.count("bond") == 0)
                throw Error(ErrorType::Initialization, "Invalid unit cell. Unit cell must contain at least one lattice bond.");
            LatticeUnitCell out;
            for (const auto &p : uc.children) {
                if (p.name == "primitive" || p.name == "site") {
                    const std::string what = "Invalid unit cell " + p.name + ".";
                    Vec3 v(parse_number(req_attr(p, "x", what)), parse_number(req_attr(p, "y", what)),
                           parse_number(req_attr(p, "z", what)));
                    (p.name == "primitive" ? out.primitives : out.basis).push_back(v);
                } else if (p.name == "bond") {
                    const std::string what = "Invalid unit cell bond.";
                    LatticeBond bd;
                    bd.from_b = std::stoi(req_attr(p, "from", what));
                    bd.to_b = std::stoi(req_attr(p, "to", what));
                    bd.da0 = std::stoi(req_attr(p, "da0", what));
                    bd.da1 = std::stoi(req_attr(p, "da1", what));
                    bd.da2 = std::stoi(req_attr(p, "da2", what));
                    out.bonds.push_back(bd);
                }
            }
            for (const auto &bd : out.bonds)
                if (bd.from_b < 0 || bd.to_b < 0 || bd.from_b >= int(out.basis.size()) || bd.to_b >= int(out.basis.size()))
                    throw Error(ErrorType::Initialization, "Invalid unit cell bond. Basis index out of range.");
            return out;
        }
    }
    throw Error(ErrorType::Initialization, "Invalid lattice unit cell definition: '" + name + "' not found.");
}

SpinModelUnitCell read_spin_model(const std::string &dir, const std::string &name,
                                  const std::map<std::string, std::string> &params) {
    static const std::regex site_re("(-{0,1}\\d+)[, ](-{0,1}\\d+)[, ](-{0,1}\\d+)[, ](\\d+)");
    static const std::regex comp_re("(-?)([xyz])([xyz])");
    for (const auto &path : xml_files(dir)) {
        XmlNode doc = xml_parse_file(path);
        for (const auto &md : doc.children) {
            if (md.name != "model") continue;
            const std::string *nm = md.attr("name");
            if (!nm) throw Error(ErrorType::Initialization, "Invalid spin model. Model name is undefined.");
            if (*nm != name) continue;
            if (md.count("interaction") == 0)
                throw Error(ErrorType::Initialization, "Invalid spin model. Spin model must define at least one interaction.");
            SpinModelUnitCell out;
            for (const auto &it : md.children) {
                if (it.name != "interaction") continue;
                const std::string what = "Invalid interaction.";
                const std::string &param = req_attr(it, "parameter", what);
                const std::string &type = req_attr(it, "type", what);
                const std::string &from = req_attr(it, "from", what);
                const std::string &to = req_attr(it, "to", what);
                std::smatch m1, m2;
                if (!std::regex_match(from, m1, site_re))
                    throw Error(ErrorType::Initialization, "Invalid spin model. Site '" + from + "' is ill-defined.");
                if (!std::regex_match(to, m2, site_re))
                    throw Error(ErrorType::Initialization, "Invalid spin model. Site '" + to + "' is ill-defined.");
                auto pit = params.find(param);
                if (pit == params.end())
                    throw Error(ErrorType::Initialization, "Interaction parameter '" + param + "' is not defined in the taskfile");
                float strength = float(parse_number(pit->second));
                SpinCoupling c;
                c.from = LatticeSite(std::stoi(m1.str(1)), std::stoi(m1.str(2)), std::stoi(m1.str(3)), std::stoi(m1.str(4)));
                c.to = LatticeSite(std::stoi(m2.str(1)), std::stoi(m2.str(2)), std::stoi(m2.str(3)), std::stoi(m2.str(4)));
                if (type == "heisenberg") {
                    c.J[0][0] += strength; c.J[1][1] += strength; c.J[2][2] += strength;
                } else if (type == "xxyy") {
                    c.J[0][0] += strength; c.J[1][1] += strength;
                } else if (type == "gx") {
                    c.J[1][2] += strength; c.J[2][1] += strength;
                } else if (type == "gy") {
                    c.J[2][0] += strength; c.J[0][2] += strength;
                } else if (type == "gz") {
                    c.J[0][1] += strength; c.J[1][0] += strength;
                } else {
                    std::smatch m;
                    if (!std::regex_match(type, m, comp_re))
                        throw Error(ErrorType::Initialization, "Invalid spin model. Unknown interaction type '" + type + "'.");
                    float sign = (m.str(1) == "-") ? -1.0f : 1.0f;
                    int s1 = m.str(2)[0] - 'x', s2 = m.str(3)[0] - 'x';
                    c.J[s1][s2] += sign * strength;
                }
                // merge with an existing coupling of the same bond (either orientation)
                bool merged = false;
                for (auto &e : out.couplings) {
                    if (e.connects(c.from, c.to) == 0) continue;
                    if (e.from == c.from && e.to == c.to) {
                        for (int a = 0; a < 3; ++a)
                            for (int b = 0; b < 3; ++b) e.J[a][b] += c.J[a][b];
                    } else if (e.from == c.to && e.to == c.from) {
                        for (int a = 0; a < 3; ++a)
                            for (int b = 0; b < 3; ++b) e.J[a][b] += c.J[b][a];
                    } else {
                        throw Error(ErrorType::Argument, "Cannnot combine incompatible spin interactions.");
                    }
                    merged = true;
                    break;
                }
                if (!merged) out.couplings.push_back(c);
                out.parameters.insert(param);
            }
            return out;
        }
    }
    throw Error(ErrorType::Initialization, "Invalid spin model definition: '" + name + "' not found.");
}

Lattice build_lattice(const LatticeUnitCell &uc, const SpinModelUnitCell &model, int range) {
    if (uc.primitives.size() != 3 || uc.basis.empty() || uc.bonds.empty())
        throw Error(ErrorType::Initialization, "Invalid unit cell.");
    if (range < 0) throw Error(ErrorType::Argument, "Lattice range must be non-negative.");
    const int nb = int(uc.basis.size());
    SiteLocator loc(uc);

    std::vector<SiteList> hood(nb);
    for (int b = 0; b < nb; ++b) hood[b] = range_around(uc, LatticeSite(0, 0, 0, b), range);

    Lattice lat;
    lat.primitives = uc.primitives;
    lat.basis = uc.basis;

    // representative ids: orbits of the sites around the origin under the automorphisms
    // that fix the origin, numbered in order of first appearance
    const std::vector<Automorphism> fix_origin = lattice_automorphisms(uc, model, loc, LatticeSite(0, 0, 0, 0), false);
    const int n0 = int(hood[0].v.size());
    std::vector<int> cls(n0, -1), cls_perm(n0, 0);
    int rid = 0;
    for (int i = 0; i < n0; ++i) {
        if (cls[i] != -1) continue;
        auto eq = orbit(uc, loc, fix_origin, hood[0].v[i]);
        cls[i] = rid;
        cls_perm[i] = 0;
        for (const auto &e : eq) {
            int j = hood[0].index_of(e.first);
            if (j < 0) throw Error(ErrorType::Internal, "Lattice symmetry calculation has failed (orbit leaves range).");
            if (cls[j] != -1) continue;
            cls[j] = rid;
            cls_perm[j] = inverse_perm(e.second);
        }
        ++rid;
    }
    // Move a representative with identity spin permutation of each class to slot r.  The scan
    // does not stop at the first match: every later identity member is swapped in as well,
    // which fixes which site ends up as the representative.
    for (int r = 0; r < rid; ++r)
        for (int i = 0; i < n0; ++i)
            if (cls[i] == r && cls_perm[i] == 0) {
                std::swap(cls[r], cls[i]);
                std::swap(cls_perm[r], cls_perm[i]);
                std::swap(hood[0].v[r], hood[0].v[i]);
            }
    hood[0].rebuild();
    lat.size = rid;

    SiteList sites;
    for (const auto &s : hood[0].v) sites.push(s);
    for (int b = 0; b < nb; ++b)
        for (const auto &s : hood[b].v) sites.push(s);
    lat.sites = sites.v;
    const int ns = int(sites.v.size());

    lat.basis_ids.resize(nb);
    for (int b = 0; b < nb; ++b) lat.basis_ids[b] = sites.index_of(LatticeSite(0, 0, 0, b));
    lat.range_ids.resize(nb);
    for (int b = 0; b < nb; ++b)
        for (const auto &s : hood[b].v) lat.range_ids[b].push_back(sites.index_of(s));

    lat.sym_rid.assign(size_t(ns) * ns, -1);
    lat.sym_perm.assign(size_t(ns) * ns, 0);
    for (int n = 0; n < n0; ++n) {
        lat.sym_rid[n] = cls[n];
        lat.sym_perm[n] = (unsigned char)cls_perm[n];
    }
    for (int b = 1; b < nb; ++b) {
        const std::vector<Automorphism> to_origin = lattice_automorphisms(uc, model, loc, LatticeSite(0, 0, 0, b), true);
        const int bid = lat.basis_ids[b];
        for (const auto &n : hood[b].v) {
            LatticeSite img;
            if (!loc.locate(to_origin[0].T.apply(site_position(uc, n)), img))
                throw Error(ErrorType::Internal, "Lattice symmetry calculation has failed (image off the lattice).");
            int nid = sites.index_of(n), eid = sites.index_of(img);
            if (eid < 0 || eid >= n0) throw Error(ErrorType::Initialization, "Could not build lattice. Could not find enough symmetries");
            lat.sym_rid[size_t(bid) * ns + nid] = lat.sym_rid[eid];
            lat.sym_perm[size_t(bid) * ns + nid] = (unsigned char)compose_perm(lat.sym_perm[eid], to_origin[0].perm);
        }
    }
    // translate every pair (s1, s2) within range to (basis(s1), s2 - s1)
    for (int s1 = 0; s1 < ns; ++s1) {
        const LatticeSite &x = sites.v[s1];
        const int s1p = lat.basis_ids[x.b];
        for (int s2 = 0; s2 < ns; ++s2) {
            const LatticeSite &y = sites.v[s2];
            LatticeSite d(y.a0 - x.a0, y.a1 - x.a1, y.a2 - x.a2, y.b);
            if (!hood[x.b].contains(d)) continue;
            int s2p = sites.index_of(d);
            lat.sym_rid[size_t(s1) * ns + s2] = lat.sym_rid[size_t(s1p) * ns + s2p];
            lat.sym_perm[size_t(s1) * ns + s2] = lat.sym_perm[size_t(s1p) * ns + s2p];
        }
    }

    // RPA pair lists: for each rid, sites j in range of both the origin and rid
    lat.overlap_ptr.assign(1, 0);
    const LatticeSite &o = sites.v[0];
    for (int r = 0; r < lat.size; ++r) {
        const LatticeSite &x = sites.v[r];
        for (int j = 0; j < ns; ++j) {
            const LatticeSite &y = sites.v[j];
            if (!hood[o.b].contains(y)) continue;
            if (!hood[x.b].contains(LatticeSite(y.a0 - x.a0, y.a1 - x.a1, y.a2 - x.a2, y.b))) continue;
            int r1 = lat.transform(0, j), r2 = lat.transform(j, r);
            if (r1 < 0 || r2 < 0) throw Error(ErrorType::Internal, "Lattice overlap references an unset symmetry entry.");
            lat.overlap_rid1.push_back(r1);
            lat.overlap_rid2.push_back(r2);
            lat.overlap_perm1.push_back(lat.perm(0, j));
            lat.overlap_perm2.push_back(lat.perm(j, r));
        }
        lat.overlap_ptr.push_back(int(lat.overlap_rid1.size()));
    }

    // interactions of the origin with each representative
    for (int r = 0; r < lat.size; ++r) {
        for (const auto &c : model.couplings) {
            int con = c.connects(LatticeSite(0, 0, 0, 0), sites.v[r]);
            if (con == 0) continue;
            RidInteraction ri;
            ri.rid = r;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) ri.J[a][b] = (con == 1) ? c.J[a][b] : c.J[b][a];
            lat.interactions.push_back(ri);
        }
    }
    return lat;
}

void write_ldf(const Lattice &lat, const LatticeUnitCell &uc, const SpinModelUnitCell &model, const std::string &path) {
    std::ofstream f(path);
    if (!f) throw Error(ErrorType::IO, "Could not write lattice debug information to file.");
    char buf[512];
    f << "<lattice>\n";
    const std::vector<int> &r0 = lat.range_ids[0];
    for (int id : r0) {
        Vec3 p = lat.position(id);
        std::snprintf(buf, sizeof buf, "\t<site id=\"%d\" x=\"%f\" y=\"%f\" z=\"%f\" parametrized=\"%s\"/>", id, p.x, p.y, p.z,
                      id < lat.size ? "true" : "false");
        f << buf << "\n";
    }
    for (int i1 : r0)
        for (int i2 : r0)
            for (const auto &bd : uc.bonds) {
                const LatticeSite &s1 = lat.sites[i1], &s2 = lat.sites[i2];
                if (bd.da0 == s2.a0 - s1.a0 && bd.da1 == s2.a1 - s1.a1 && bd.da2 == s2.a2 - s1.a2 && bd.from_b == s1.b &&
                    bd.to_b == s2.b) {
                    std::snprintf(buf, sizeof buf, "\t<bond from=\"%d\" to=\"%d\" />", i1, i2);
                    f << buf << "\n";
                }
            }
    for (int i1 : r0)
        for (int i2 : r0)
            for (const auto &c : model.couplings) {
                const LatticeSite &s1 = lat.sites[i1], &s2 = lat.sites[i2];
                if ((c.to.a0 - c.from.a0) == (s2.a0 - s1.a0) && (c.to.a1 - c.from.a1) == (s2.a1 - s1.a1) &&
                    (c.to.a2 - c.from.a2) == (s2.a2 - s1.a2) && c.from.b == s1.b && c.to.b == s2.b) {
                    std::snprintf(buf, sizeof buf,
                                  "\t<interaction from=\"%d\" to=\"%d\" value=\"[[%f,%f,%f],[%f,%f,%f],[%f,%f,%f]]\" />", i1, i2,
                                  c.J[0][0], c.J[0][1], c.J[0][2], c.J[1][0], c.J[1][1], c.J[1][2], c.J[2][0], c.J[2][1],
                                  c.J[2][2]);
                    f << buf << "\n";
                }
            }
    f << "</lattice>\n";
}

}  // namespace spn
