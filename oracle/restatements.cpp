// ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into libvmp.so.
//
// The device kernels evaluate three products of the reference in a shorter
// form than written: they leave out the products with entries that are known
// to be zero and, for the symmetric plane covariance, form only the upper
// triangle.  This file states each device form again on the CPU, in the
// kernels' operation order, beside the dense reference-order form of the
// oracle (mathkit.hpp / oracle.cpp), and counts over many random inputs --
// exact zeros of either sign included -- where the two differ:
//   kind 0: point_crossmat * P_rr * point_crossmat^T (lio_builder.cpp:199-202,
//           240-243); device: hat_sandwich (csrc/common.cuh);
//   kind 1: calcBodyCov's A = range * direction_hat * N and A dvar A^T
//           (commons.cpp:18-45); device: calc_body_cov (csrc/k_points.cu);
//   kind 2: updatePlane's per-point J * pv.cov * J^T (voxel_map.cpp:115-129);
//           device: plane_cov_term (csrc/k_map.cu), upper triangle only.
// Dropping a product with an exact zero removes a +-0 term from a sum: the
// value is unchanged unless every other term is zero too, and then only the
// sign of the zero can change.  counts[] reports that: entries compared,
// value mismatches (must be 0), bit mismatches, bit mismatches whose values
// are not zero (must be 0).  For kind 2 the dense form's lower triangle has
// its own rounding; max_lower returns the largest
// |dense(j,i) - dense(i,j)| / sqrt(dense(i,i) dense(j,j)) over the terms.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>

#include "mathkit.hpp"

namespace orc {
namespace {

typedef Mat<3, 2> M32;
typedef Mat<2, 2> M22;
typedef Mat<6, 6> M66;
typedef Mat<6, 3> M63;

struct Counter {
    long long entries = 0, value_mismatch = 0, bit_mismatch = 0, bit_mismatch_nonzero = 0;
    void compare(double dense, double restated) {
        ++entries;
        if (!(dense == restated)) ++value_mismatch;
        if (std::memcmp(&dense, &restated, sizeof(double)) != 0) {
            ++bit_mismatch;
            if (dense != 0.0) ++bit_mismatch_nonzero;
        }
    }
};

// A value that is an exact zero of random sign with probability pz.
double maybe_zero(std::mt19937_64& rng, double v, double pz) {
    std::uniform_real_distribution<double> u(0.0, 1.0);
    if (u(rng) < pz) return u(rng) < 0.5 ? 0.0 : -0.0;
    return v;
}

// --- device forms, in the kernels' operation order
void hat_sandwich_restated(const V3& p, const M3& M, M3& out) {
    const M3 h = hat(p);
    M3 t;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const int k0 = i == 0 ? 1 : 0, k1 = i == 2 ? 1 : 2;
            t(i, j) = h(i, k0) * M(k0, j) + h(i, k1) * M(k1, j);
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const int k0 = j == 0 ? 1 : 0, k1 = j == 2 ? 1 : 2;
            out(i, j) = t(i, k0) * h(j, k0) + t(i, k1) * h(j, k1);
        }
}

// calcBodyCov's tail from the unit direction d, the range and the basis N.
void body_cov_tail_restated(const V3& d, double range, double range_var, const M22& dvar, const M32& N, M3& cov) {
    const M3 dh = hat(d);
    M32 A, AD;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 2; ++j) {
            const int k0 = i == 0 ? 1 : 0, k1 = i == 2 ? 1 : 2;
            A(i, j) = (range * dh(i, k0)) * N(k0, j) + (range * dh(i, k1)) * N(k1, j);
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 2; ++j) AD(i, j) = A(i, j) * dvar(j, j);
    cov = (d * range_var) * T(d) + AD * T(A);
}
void body_cov_tail_dense(const V3& d, double range, double range_var, const M22& dvar, const M32& N, M3& cov) {
    const M32 A = (range * hat(d)) * N;
    cov = (d * range_var) * T(d) + (A * dvar) * T(A);
}

// Per-point plane covariance term: the device's 21 upper-triangle entries
// (row-major, i <= j) and the dense 6x6.
void plane_term_restated(const V3& p, const V3& mean, int n, const V3& ev, const M3& E, const M3& cov,
                         double up[21]) {
    const V3 pn = v3(E(0, 0), E(1, 0), E(2, 0));
    M3 Mm[3];
    double den[3] = {0.0, 0.0, 0.0};
    for (int m = 1; m < 3; ++m) {
        const V3 vm = v3(E(0, m), E(1, m), E(2, m));
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Mm[m](i, j) = vm[i] * pn[j] + pn[i] * vm[j];
        den[m] = (double)n * (ev[0] - ev[m]);
    }
    const double inv_n = 1.0 / (double)n;
    const V3 d = p - mean;
    double F1[3], F2[3];
    for (int j = 0; j < 3; ++j) {
        const double a0 = d[0] / den[1], a1 = d[1] / den[1], a2 = d[2] / den[1];
        const double b0 = d[0] / den[2], b1 = d[1] / den[2], b2 = d[2] / den[2];
        F1[j] = (a0 * Mm[1](0, j) + a1 * Mm[1](1, j)) + a2 * Mm[1](2, j);
        F2[j] = (b0 * Mm[2](0, j) + b1 * Mm[2](1, j)) + b2 * Mm[2](2, j);
    }
    M3 top;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) top(i, j) = E(i, 1) * F1[j] + E(i, 2) * F2[j];
    const M3 A = top * cov;
    int q = 0;
    for (int i = 0; i < 6; ++i)
        for (int j = i; j < 6; ++j) {
            double v;
            if (i < 3 && j < 3) v = (A(i, 0) * top(j, 0) + A(i, 1) * top(j, 1)) + A(i, 2) * top(j, 2);
            else if (i < 3) v = A(i, j - 3) * inv_n;
            else v = (inv_n * cov(i - 3, j - 3)) * inv_n;
            up[q++] = v;
        }
}
void plane_term_dense(const V3& p, const V3& mean, int n, const V3& ev, const M3& E, const M3& cov, M66& out) {
    const M3 J_Q = M3::Identity() / static_cast<double>(n);
    const V3 pn = v3(E(0, 0), E(1, 0), E(2, 0));
    M3 F = M3::Zero();
    for (int m = 1; m < 3; ++m) {
        const V3 vm = v3(E(0, m), E(1, m), E(2, m));
        const Mat<1, 3> Fm = (T(p - mean) / (n * (ev[0] - ev[m]))) * (vm * T(pn) + pn * T(vm));
        F(m, 0) = Fm(0, 0); F(m, 1) = Fm(0, 1); F(m, 2) = Fm(0, 2);
    }
    M63 J;
    J.setBlock(0, 0, E * F);
    J.setBlock(3, 0, J_Q);
    out = (J * cov) * T(J);
}

M3 random_rotation(std::mt19937_64& rng) {
    std::normal_distribution<double> g(0.0, 1.0);
    double q[4] = {g(rng), g(rng), g(rng), g(rng)};
    const double s = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    const Quat u{q[0] / s, q[1] / s, q[2] / s, q[3] / s};
    return quatToMat(u);
}

// Symmetric positive definite 3x3 like the per-point covariances the map
// receives (A A^T + 1e-4 I), entries sometimes exact zeros.
M3 random_cov(std::mt19937_64& rng, double pz) {
    std::normal_distribution<double> g(0.0, 0.02);
    M3 A;
    for (int i = 0; i < 9; ++i) A[i] = g(rng);
    M3 C = A * T(A) + M3::Identity() * 1e-4;
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j) C(i, j) = C(j, i) = maybe_zero(rng, C(i, j), pz);
    return C;
}

}  // namespace
}  // namespace orc

using namespace orc;

extern "C" void orc_restatement_check(int kind, long long n, unsigned long long seed, long long* counts,
                                      double* max_lower) {
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    Counter c;
    double worst = 0.0;
    for (long long it = 0; it < n; ++it) {
        if (kind == 0) {
            V3 p = v3(maybe_zero(rng, 30.0 * u(rng), 0.15), maybe_zero(rng, 30.0 * u(rng), 0.15),
                      maybe_zero(rng, 10.0 * u(rng), 0.15));
            M3 M = random_cov(rng, 0.1);
            if (it % 7 == 0) M = M * 1e-6;
            M3 a, b = hatSandwich(p, M);
            hat_sandwich_restated(p, M, a);
            for (int i = 0; i < 9; ++i) c.compare(b[i], a[i]);
        } else if (kind == 1) {
            // the direction of a LiDAR point after the z == 0 fix, its range,
            // the basis N as calcBodyCov forms it
            V3 pb = v3(maybe_zero(rng, 40.0 * u(rng), 0.15), maybe_zero(rng, 40.0 * u(rng), 0.15),
                       maybe_zero(rng, 5.0 * u(rng), 0.15));
            if (pb[2] == 0) pb[2] = 0.001;
            const double range = std::sqrt(pb[0] * pb[0] + pb[1] * pb[1] + pb[2] * pb[2]);
            const double s = std::sin(0.1 * 0.017453293);
            M22 dvar; dvar(0, 0) = s * s; dvar(0, 1) = 0; dvar(1, 0) = 0; dvar(1, 1) = s * s;
            const V3 d = normalized(pb);
            const V3 b1 = normalized(v3(1, 1, -(d[0] + d[1]) / d[2]));
            const V3 b2 = normalized(cross(b1, d));
            M32 N;
            for (int i = 0; i < 3; ++i) { N(i, 0) = b1[i]; N(i, 1) = b2[i]; }
            M3 a, b;
            body_cov_tail_restated(d, range, 0.0016, dvar, N, a);
            body_cov_tail_dense(d, range, 0.0016, dvar, N, b);
            for (int i = 0; i < 9; ++i) c.compare(b[i], a[i]);
        } else {
            // a refit: points around a mean, an eigen basis (sometimes axis
            // aligned, i.e. with exact zeros), ascending eigenvalues
            const int npts = 10 + (int)(rng() % 91);
            const V3 mean = v3(50.0 * u(rng), 50.0 * u(rng), 10.0 * u(rng));
            M3 E = random_rotation(rng);
            if (it % 5 == 0) {
                const int perm = (int)(rng() % 6);
                const int idx[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
                E = M3::Zero();
                for (int k = 0; k < 3; ++k) E(idx[perm][k], k) = (rng() & 1) ? 1.0 : -1.0;
            }
            const double l0 = 1e-5 * (1.0 + u(rng)), l1 = 0.01 * (2.0 + u(rng)), l2 = 0.03 * (2.0 + u(rng));
            const V3 ev = v3(l0, l1, l2);
            V3 p = mean + v3(0.25 * u(rng), 0.25 * u(rng), 0.25 * u(rng));
            if (it % 11 == 0) {  // one component of d exactly zero
                const int k = (int)(rng() % 3);
                p[k] = mean[k];
            }
            if (it % 13 == 0) p = mean;  // d == 0
            const M3 cov = random_cov(rng, 0.05);
            double up[21];
            M66 dense;
            plane_term_restated(p, mean, npts, ev, E, cov, up);
            plane_term_dense(p, mean, npts, ev, E, cov, dense);
            int q = 0;
            for (int i = 0; i < 6; ++i)
                for (int j = i; j < 6; ++j) {
                    c.compare(dense(i, j), up[q++]);
                    if (j > i) {
                        const double s = std::sqrt(std::fabs(dense(i, i) * dense(j, j)));
                        const double diff = std::fabs(dense(j, i) - dense(i, j));
                        if (diff > 0.0) worst = std::max(worst, s > 0.0 ? diff / s : INFINITY);
                    }
                }
        }
    }
    counts[0] = c.entries;
    counts[1] = c.value_mismatch;
    counts[2] = c.bit_mismatch;
    counts[3] = c.bit_mismatch_nonzero;
    if (max_lower) *max_lower = worst;
}
