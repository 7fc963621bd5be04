// Known-answer tests of the lattice factory's geometry helpers (spinparser_gb300/csrc/host/geometry.hpp)
// with the cases and tolerances of the reference's test/test_Geometry.cpp:16-206: exact equality
// where the reference uses BOOST_CHECK_EQUAL, 1e-10 % (relative) or 1e-10 (absolute, near zero)
// where it uses BOOST_CHECK_CLOSE / BOOST_CHECK_SMALL.  Built and run by tests/test_geometry.py;
// prints one line per failed check and exits with the number of failures.
#include <cmath>
#include <cstdio>

#include "geometry.hpp"

using spn::Affine;
using spn::Mat3;
using spn::Vec3;

static int failures = 0;

static void equal(double got, double want, const char *what) {
    if (!(got == want)) {
        std::printf("%s: %.17g != %.17g\n", what, got, want);
        ++failures;
    }
}

static void close(double got, double want, const char *what) {
    if (!(std::fabs(got - want) <= 1e-12 * std::fabs(want))) {
        std::printf("%s: %.17g not within 1e-10 %% of %.17g\n", what, got, want);
        ++failures;
    }
}

static void small(double got, const char *what) {
    if (!(std::fabs(got) <= 1e-10)) {
        std::printf("%s: %.17g not within 1e-10 of 0\n", what, got);
        ++failures;
    }
}

static void close3(const Vec3 &v, double x, double y, double z, const char *what) {
    const double want[3] = {x, y, z}, got[3] = {v.x, v.y, v.z};
    for (int i = 0; i < 3; ++i) {
        if (want[i] == 0.0) small(got[i], what);
        else close(got[i], want[i], what);
    }
}

int main() {
    // Vec3Normalization (:31-39)
    {
        const Vec3 x(1.0, 2.0, 3.0);
        equal(x.norm(), std::sqrt(14.0), "norm");
        const Vec3 n = x.normalized();
        equal(n.x, 1.0 / std::sqrt(14.0), "normalize x");
        equal(n.y, 2.0 / std::sqrt(14.0), "normalize y");
        equal(n.z, 3.0 / std::sqrt(14.0), "normalize z");
    }
    // Mat3Operations (:93-109): rows (1 1 2) (3 4 5) (6 7 8)
    {
        Mat3 x;
        const double rows[3][3] = {{1.0, 1.0, 2.0}, {3.0, 4.0, 5.0}, {6.0, 7.0, 8.0}};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) x.m[i][j] = rows[i][j];
        equal(x.det(), -3.0, "determinant");
        const Mat3 y = x.inverse();
        const double inv[3][3] = {{1.0, -2.0, 1.0}, {-2.0, 4.0 / 3.0, -1.0 / 3.0}, {1.0, 1.0 / 3.0, -1.0 / 3.0}};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) equal(y.m[i][j], inv[i][j], "inverse");
        // columns() is the transpose of the row layout
        const Mat3 c = Mat3::columns(Vec3(1.0, 3.0, 6.0), Vec3(1.0, 4.0, 7.0), Vec3(2.0, 5.0, 8.0));
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) equal(c.m[i][j], rows[i][j], "columns");
    }
    // Mat4Constructor (:111-151): identity, inversion, translation, rotations
    {
        const Affine id = Affine::identity();
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) equal(id.m[i][j], i == j ? 1.0 : 0.0, "identity");
        close3(Affine::point_inversion().apply(Vec3(1.0, 2.0, 3.0)), -1.0, -2.0, -3.0, "inversion");
        close3(Affine::translation(Vec3(1.0, 2.0, 3.0)).apply(Vec3(1.0, 2.0, 3.0)), 2.0, 4.0, 6.0, "translation");
        close3(Affine::rotation(Vec3(1.0, 1.0, 1.0), 2 * M_PI / 3.0).apply(Vec3(1.0, 0.0, 0.0)), 0.0, 1.0, 0.0,
               "rotation about (1,1,1)");
        close3(Affine::rotation_about(Vec3(0.0, 0.0, 1.0), Vec3(1.0, 0.0, 0.0), M_PI).apply(Vec3(2.0, 0.0, 0.0)), 0.0,
               0.0, 0.0, "rotation about an axis through (1,0,0)");
    }
    // VectorArithmetics (:153-184)
    {
        close(spn::dot(Vec3(1.0, 2.0, 3.0), Vec3(2.0, 3.0, 4.0)), 20.0, "dot");
        close3(spn::cross(Vec3(1.0, 2.0, 3.0), Vec3(2.0, 3.0, 4.0)), -1.0, 2.0, -1.0, "cross");
        close3(Vec3(1.0, 2.0, 3.0) + Vec3(1.0, 2.0, 3.0), 2.0, 4.0, 6.0, "sum");
        close3(Vec3(1.0, 2.0, 3.0) - Vec3(2.0, 3.0, 4.0), -1.0, -1.0, -1.0, "difference");
        close3(-Vec3(1.0, 2.0, 3.0), -1.0, -2.0, -3.0, "negation");
        close3(2.0 * Vec3(1.0, 2.0, 3.0), 2.0, 4.0, 6.0, "scaling");
    }
    // MatrixArithmetics (:186-204)
    {
        const Affine r = Affine::rotation(Vec3(1.0, 1.0, 1.0), M_PI);
        close3((r * r).apply(Vec3(2.0, 3.0, 4.0)), 2.0, 3.0, 4.0, "rotation by pi, twice");
        Mat3 x;
        for (int i = 0; i < 9; ++i) x.m[i / 3][i % 3] = double(i + 1);
        close3(x * Vec3(2.0, 3.0, 4.0), 20.0, 47.0, 74.0, "matrix times vector");
    }
    return failures;
}
