// The opaque spn_lattice handle of the C ABI: the unit cell, the spin model and the
// symmetry-reduced lattice built from them.  Shared by the host entry points and the task
// driver, which builds its lattice through the same handle.
#pragma once
#include "lattice.hpp"

struct spn_lattice {
    spn::LatticeUnitCell uc;
    spn::SpinModelUnitCell model;
    spn::Lattice lat;
};
