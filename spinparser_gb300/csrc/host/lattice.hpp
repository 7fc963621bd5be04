// Host-side lattice and spin-model construction: unit-cell / model XML readers and the
// symmetry-reduced lattice tables that the device kernels consume as read-only gather tables.
//
// Restates LatticeModelFactory::newLatticeModel (src/LatticeModelFactory.cpp:733-1047) and
// the Lattice accessors the SU(2) core uses (src/Lattice.hpp:397-551).  The numbering of
// sites and representative ids ("rid") follows the reference exactly, because the .obs
// output enumerates sites in that order and the RPA pair lists are stored in that order.
#pragma once
#include <array>
#include <map>
#include <set>
#include <string>
#include <vector>
#include "geometry.hpp"

namespace spn {

struct LatticeSite {
    int a0 = 0, a1 = 0, a2 = 0, b = 0;
    LatticeSite() = default;
    LatticeSite(int x, int y, int z, int bb) : a0(x), a1(y), a2(z), b(bb) {}
    bool operator==(const LatticeSite &o) const { return a0 == o.a0 && a1 == o.a1 && a2 == o.a2 && b == o.b; }
    bool operator!=(const LatticeSite &o) const { return !(*this == o); }
};

struct LatticeBond {
    int from_b, to_b, da0, da1, da2;
};

struct LatticeUnitCell {
    std::vector<Vec3> primitives;  // three Bravais vectors
    std::vector<Vec3> basis;       // basis site positions
    std::vector<LatticeBond> bonds;
};

struct SpinCoupling {
    LatticeSite from, to;
    float J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    // +1 if (from->to) connects s1->s2 by translation, -1 if it connects s2->s1, else 0
    int connects(const LatticeSite &s1, const LatticeSite &s2) const;
};

struct SpinModelUnitCell {
    std::vector<SpinCoupling> couplings;
    std::set<std::string> parameters;
};

// Interaction of the origin (basis site 0) with representative `rid`.
struct RidInteraction {
    int rid;
    float J[3][3];
};

// Symmetry-reduced lattice.  Indices into `sites` are "site ids"; the first `size` ids are
// the representatives (rid == id) of the pair classes (0, id).
struct Lattice {
    std::vector<Vec3> primitives;
    std::vector<Vec3> basis;
    std::vector<LatticeSite> sites;            // all sites in range of any basis site
    int size = 0;                              // number of representatives (Nl)
    std::vector<int> basis_ids;                // site id of (0,0,0,b)
    std::vector<std::vector<int>> range_ids;   // [b] site ids in range of (0,0,0,b), reference order
    std::vector<int> sym_rid;                  // [id1 * n_sites + id2] -> rid of the pair, -1 if unset
    // [id1 * n_sites + id2] -> spin permutation that accompanies the map of the pair onto its
    // representative, an index into the six permutations (X,Y,Z) (X,Z,Y) (Y,X,Z) (Y,Z,X)
    // (Z,X,Y) (Z,Y,X): component c of the pair is component kSpinPerm[p][c] of the
    // representative (LatticeSiteDescriptor::spinPermutation, src/Lattice.hpp)
    std::vector<unsigned char> sym_perm;
    std::vector<int> overlap_ptr;              // CSR over rid: [size + 1]
    std::vector<int> overlap_rid1, overlap_rid2;
    std::vector<int> overlap_perm1, overlap_perm2;  // permutations of (0, j) and (j, rid) per pair
    std::vector<RidInteraction> interactions;  // SpinModel::interactions (src/SpinModel.hpp)

    int n_sites() const { return int(sites.size()); }
    int transform(int id1, int id2) const { return sym_rid[size_t(id1) * sites.size() + id2]; }
    int perm(int id1, int id2) const { return sym_perm[size_t(id1) * sites.size() + id2]; }
    Vec3 position(int id) const;
    // Lattice::getSites()[j].rid and getInvertedSites()[j].rid
    std::vector<int> sites_rid() const;
    std::vector<int> inverted_sites_rid() const;
    // spin permutations of getSites()[j] and getInvertedSites()[j]
    std::vector<int> sites_perm() const;
    std::vector<int> inverted_sites_perm() const;
};

// Parses numbers the way InputParser::stringToDouble does (src/lib/InputParser.hpp:24-56):
// sqrt(x) terms are substituted first, then a*b and a/b left to right, then std::stod.
double parse_number(const std::string &s);

LatticeUnitCell read_unit_cell(const std::string &resource_dir, const std::string &name);
SpinModelUnitCell read_spin_model(const std::string &resource_dir, const std::string &name,
                                  const std::map<std::string, std::string> &params);

Lattice build_lattice(const LatticeUnitCell &uc, const SpinModelUnitCell &model, int range);

// Lattice debug file (.ldf) as written by the reference (src/LatticeModelFactory.cpp:987-1043).
void write_ldf(const Lattice &lat, const LatticeUnitCell &uc, const SpinModelUnitCell &model, const std::string &path);

}  // namespace spn
