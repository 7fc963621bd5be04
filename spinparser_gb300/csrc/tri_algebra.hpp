// Coefficients of the TRI pf-FRG flow equations (time-reversal-invariant spin models with
// general couplings), host and device.
//
// The TRI vertex has 16 components (a, b) per site, a, b in {0 = X, 1 = Y, 2 = Z, 3 = density}
// (component index 4a + b).  The reference writes its flow equations out term by term
// (src/TRI/TRIFrgCore.cpp:198-2902, TRIMeasurementCorrelation.cpp:199-251); every coefficient
// there is a product of Pauli matrices, sigma_a sigma_b = i^k sigma_(a.b) with sigma_3 = 1, in
// which a component with exactly one density index carries a factor -i.  These functions
// evaluate that algebra; after unrolling they fold to constants.
//   particle-particle ladder (s):  d(c) += pp_sign(c, a) A(a) B(a ^ c ^ 15)
//   particle-hole ladder (u):      d(c) += ph_sign(c, a) A(a) B(a ^ c ^ 15)
//   RPA (t):                       d(mu nu) += 2 rpa_sign(c, k) A(mu k) B(k nu), summed over pairs
//   chalice (t):                   d(mu nu) += chal_sign(c, k, l) A(mu k) L(l, nu ^ k ^ l)
//   inverse chalice (t):           d(mu nu) += ichal_sign(c, l) L(l) B(mu ^ l1 ^ l2, nu)
//   egg (measurement):             chi(c) += f egg_sign(c, l) L(l, c1 ^ c2 ^ l), f = 2 (DD) or 1/2
#pragma once

#if defined(__CUDACC__)
#define SPN_TRI_HD __host__ __device__ __forceinline__
#else
#define SPN_TRI_HD inline
#endif

namespace spn {
namespace tri {

constexpr int kD = 3;  // density component

// sigma_a sigma_b = i^k sigma_c
SPN_TRI_HD constexpr int pauli_c(int a, int b) { return a == kD ? b : (b == kD ? a : (a == b ? kD : 3 - a - b)); }
SPN_TRI_HD constexpr int pauli_k(int a, int b) {
    return (a == kD || b == kD || a == b) ? 0 : (((b - a + 3) % 3 == 1) ? 1 : 3);
}
// power of i of the -i that a mixed spin/density component carries
SPN_TRI_HD constexpr int eta(int a, int b) { return ((a == kD) != (b == kD)) ? 3 : 0; }
// i^k for even k (the algebra gives only real coefficients); 0 for odd k
SPN_TRI_HD constexpr int real_sign(int k) { return (k & 3) == 0 ? 1 : ((k & 3) == 2 ? -1 : 0); }

SPN_TRI_HD constexpr int pp_sign(int c, int a) {
    const int b = a ^ c ^ 15;
    return real_sign(8 + pauli_k(a >> 2, b >> 2) + pauli_k(a & 3, b & 3) + eta(a >> 2, a & 3) + eta(b >> 2, b & 3) -
                     eta(c >> 2, c & 3));
}
SPN_TRI_HD constexpr int ph_sign(int c, int a) {
    const int b = a ^ c ^ 15;
    return real_sign(10 + pauli_k(a >> 2, b >> 2) + pauli_k(b & 3, a & 3) + eta(a >> 2, a & 3) + eta(b >> 2, b & 3) -
                     eta(c >> 2, c & 3));
}
SPN_TRI_HD constexpr int rpa_sign(int c, int k) {
    return real_sign(8 + eta(c >> 2, k) + eta(k, c & 3) - eta(c >> 2, c & 3));
}
// chalice: A(c1, kap) L(lam, rho), rho = c2 ^ kap ^ lam
SPN_TRI_HD constexpr int chal_sign(int c, int kap, int lam) {
    const int c1 = c >> 2, c2 = c & 3, rho = c2 ^ kap ^ lam;
    return real_sign(10 + pauli_k(lam, kap) + pauli_k(pauli_c(lam, kap), rho) + eta(c1, kap) + eta(lam, rho) -
                     eta(c1, c2));
}
// inverse chalice: L(l) B(kap, c2), l = (lam, rho), kap = c1 ^ lam ^ rho
SPN_TRI_HD constexpr int ichal_sign(int c, int l) {
    const int c1 = c >> 2, c2 = c & 3, lam = l >> 2, rho = l & 3, kap = c1 ^ lam ^ rho;
    return real_sign(10 + pauli_k(lam, kap) + pauli_k(pauli_c(lam, kap), rho) + eta(kap, c2) + eta(lam, rho) -
                     eta(c1, c2));
}
// egg diagram of the measurement: tr(sigma_c1 sigma_lam sigma_c2 sigma_rho) / 2, rho = c1 ^ c2 ^ lam
SPN_TRI_HD constexpr int egg_sign(int c, int lam) {
    const int c1 = c >> 2, c2 = c & 3, rho = c1 ^ c2 ^ lam;
    const int r1 = pauli_c(c1, lam), r2 = pauli_c(r1, c2);
    return pauli_c(r2, rho) != kD ? 0
                                  : real_sign(8 + pauli_k(c1, lam) + pauli_k(r1, c2) + pauli_k(r2, rho) + eta(lam, rho));
}

// The reference's order of an inner spin index: density, Z, Y, X.
SPN_TRI_HD constexpr int inner(int n) { return 3 - n; }

}  // namespace tri
}  // namespace spn
