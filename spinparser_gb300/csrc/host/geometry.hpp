// Small double-precision vector / affine-matrix helpers for the lattice symmetry search.
//
// The lattice factory decides whether a candidate isometry maps lattice sites onto lattice
// sites with a 1e-5 tolerance, so the equivalence classes it finds depend on the exact
// floating-point values of the rotation matrices (an acos() argument that rounds above 1
// yields NaN and silently rejects a candidate).  To reproduce the reference's classes bit for
// bit, every formula below evaluates its terms in the same order as the reference geometry
// library (src/lib/Geometry.hpp:36-560): Vec3::norm/normalize (:41-60), dot/cross (:75-90),
// Mat3::inverse via the adjugate (:253-262), Mat4::rotation via Rodrigues' formula
// (:411-438), the point-anchored rotation T(p) R T(-p) (:449-452) and the 4x4 product
// (:456-470).  The host objects are compiled with -ffp-contract=off so no FMA changes a bit.
#pragma once
#include <cmath>

namespace spn {

struct Vec3 {
    double x = 0, y = 0, z = 0;
    Vec3() = default;
    Vec3(double x_, double y_, double z_) : x(x_), y(y_), z(z_) {}
    double norm() const { return std::sqrt(x * x + y * y + z * z); }
    Vec3 normalized() const {
        double n = norm();
        return Vec3(x / n, y / n, z / n);
    }
};

inline Vec3 operator+(const Vec3 &a, const Vec3 &b) { return Vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline Vec3 operator-(const Vec3 &a, const Vec3 &b) { return Vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline Vec3 operator-(const Vec3 &a) { return Vec3(-a.x, -a.y, -a.z); }
inline Vec3 operator*(double s, const Vec3 &a) { return Vec3(s * a.x, s * a.y, s * a.z); }
inline double dot(const Vec3 &a, const Vec3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vec3 cross(const Vec3 &a, const Vec3 &b) {
    return Vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// 3x3 matrix whose columns are the three primitive vectors.
struct Mat3 {
    double m[3][3];
    static Mat3 columns(const Vec3 &a0, const Vec3 &a1, const Vec3 &a2) {
        Mat3 r;
        r.m[0][0] = a0.x; r.m[0][1] = a1.x; r.m[0][2] = a2.x;
        r.m[1][0] = a0.y; r.m[1][1] = a1.y; r.m[1][2] = a2.y;
        r.m[2][0] = a0.z; r.m[2][1] = a1.z; r.m[2][2] = a2.z;
        return r;
    }
    double det() const {
        return -m[0][2] * m[1][1] * m[2][0] + m[0][1] * m[1][2] * m[2][0] + m[0][2] * m[1][0] * m[2][1] -
               m[0][0] * m[1][2] * m[2][1] - m[0][1] * m[1][0] * m[2][2] + m[0][0] * m[1][1] * m[2][2];
    }
    Mat3 inverse() const {
        double adj[9] = {
            -m[1][2] * m[2][1] + m[1][1] * m[2][2], m[0][2] * m[2][1] - m[0][1] * m[2][2],
            -m[0][2] * m[1][1] + m[0][1] * m[1][2], m[1][2] * m[2][0] - m[1][0] * m[2][2],
            -m[0][2] * m[2][0] + m[0][0] * m[2][2], m[0][2] * m[1][0] - m[0][0] * m[1][2],
            -m[1][1] * m[2][0] + m[1][0] * m[2][1], m[0][1] * m[2][0] - m[0][0] * m[2][1],
            -m[0][1] * m[1][0] + m[0][0] * m[1][1]};
        double s = 1 / det();
        Mat3 r;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) r.m[i][j] = s * adj[3 * i + j];
        return r;
    }
    Vec3 operator*(const Vec3 &v) const {
        return Vec3(m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z, m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z,
                    m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z);
    }
};

// Affine 4x4 transformation (last row 0 0 0 1).
struct Affine {
    double m[4][4];
    static Affine diag(double d) {
        Affine r;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) r.m[i][j] = (i == j) ? (i == 3 ? 1.0 : d) : 0.0;
        return r;
    }
    static Affine identity() { return diag(1.0); }
    static Affine point_inversion() { return diag(-1.0); }
    static Affine translation(const Vec3 &v) {
        Affine r = identity();
        r.m[0][3] = v.x; r.m[1][3] = v.y; r.m[2][3] = v.z;
        return r;
    }
    // Rotation by `angle` about `axis` through the origin (Rodrigues' formula).
    static Affine rotation(const Vec3 &axis, double angle) {
        Vec3 a = axis.normalized();
        Affine r = identity();
        r.m[0][0] = a.x * a.x * (1 - cos(angle)) + cos(angle);
        r.m[0][1] = a.x * a.y * (1 - cos(angle)) - a.z * sin(angle);
        r.m[0][2] = a.x * a.z * (1 - cos(angle)) + a.y * sin(angle);
        r.m[1][0] = a.y * a.x * (1 - cos(angle)) + a.z * sin(angle);
        r.m[1][1] = a.y * a.y * (1 - cos(angle)) + cos(angle);
        r.m[1][2] = a.y * a.z * (1 - cos(angle)) - a.x * sin(angle);
        r.m[2][0] = a.z * a.x * (1 - cos(angle)) - a.y * sin(angle);
        r.m[2][1] = a.z * a.y * (1 - cos(angle)) + a.x * sin(angle);
        r.m[2][2] = a.z * a.z * (1 - cos(angle)) + cos(angle);
        return r;
    }
    // Rotation about an axis through `point`: T(point) * R * T(-point).
    static Affine rotation_about(const Vec3 &axis, const Vec3 &point, double angle) {
        return translation(point) * rotation(axis, angle) * translation(-point);
    }
    friend Affine operator*(const Affine &l, const Affine &r) {
        Affine p;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) {
                double acc = 0.0;
                for (int k = 0; k < 4; ++k) acc += l.m[i][k] * r.m[k][j];
                p.m[i][j] = acc;
            }
        return p;
    }
    Vec3 apply(const Vec3 &v) const {
        return Vec3(m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z + m[0][3],
                    m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z + m[1][3],
                    m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z + m[2][3]);
    }
};

}  // namespace spn
