// ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into libvmp.so.
//
// Fixed-size FP64 matrix kit standing in for the Eigen3 / Sophus subset the
// reference calls (Eigen3 and Sophus are not present on this machine and are
// not pinned by the reference: voxel_plus/CMakeLists.txt:28-31).  Restated
// from the published algorithms:
//   * matrix products: coefficient order k = 0..K-1, left to right;
//   * Sophus::SO3::exp / log / hat / leftJacobian (Sophus so3.hpp, epsilon
//     1e-10 for double): exp through the unit quaternion, log through
//     Eigen's rotation-matrix -> quaternion conversion and atan2;
//   * Eigen::Quaternion -> rotation matrix and FromTwoVectors;
//   * Eigen::SelfAdjointEigenSolver<Matrix3d>: cyclic Jacobi, eigenvalues
//     ascending, eigenvectors as columns (signs are arbitrary in Eigen too);
//   * Matrix::inverse() for 23x23: LU with partial pivoting (Eigen's
//     PartialPivLU for fixed sizes above 4).
// Compiled with -ffp-contract=off so that x86-64 and aarch64 hosts produce the
// same bits (no fused multiply-add).
#pragma once
#include <cmath>
#include <cstring>
#include <algorithm>

namespace orc {

template <int R, int C>
struct Mat {
    double v[R * C];
    double& operator()(int i, int j) { return v[i * C + j]; }
    double operator()(int i, int j) const { return v[i * C + j]; }
    double& operator[](int i) { return v[i]; }
    double operator[](int i) const { return v[i]; }
    static Mat Zero() { Mat m; std::memset(m.v, 0, sizeof(m.v)); return m; }
    static Mat Identity() {
        Mat m = Zero();
        for (int i = 0; i < (R < C ? R : C); ++i) m(i, i) = 1.0;
        return m;
    }
    void setZero() { *this = Zero(); }
    void setIdentity() { *this = Identity(); }
    template <int r, int c>
    Mat<r, c> block(int i0, int j0) const {
        Mat<r, c> o;
        for (int i = 0; i < r; ++i)
            for (int j = 0; j < c; ++j) o(i, j) = (*this)(i0 + i, j0 + j);
        return o;
    }
    template <int r, int c>
    void setBlock(int i0, int j0, const Mat<r, c>& b) {
        for (int i = 0; i < r; ++i)
            for (int j = 0; j < c; ++j) (*this)(i0 + i, j0 + j) = b(i, j);
    }
    double trace() const {
        double s = v[0];
        for (int i = 1; i < R; ++i) s += (*this)(i, i);
        return s;
    }
    double maxCoeff() const {
        double m = v[0];
        for (int i = 1; i < R * C; ++i) m = std::max(m, v[i]);
        return m;
    }
};

typedef Mat<3, 1> V3;
typedef Mat<2, 1> V2;
typedef Mat<3, 3> M3;

inline V3 v3(double a, double b, double c) { V3 r; r[0] = a; r[1] = b; r[2] = c; return r; }

template <int R, int C>
inline Mat<R, C> operator+(const Mat<R, C>& a, const Mat<R, C>& b) {
    Mat<R, C> o;
    for (int i = 0; i < R * C; ++i) o.v[i] = a.v[i] + b.v[i];
    return o;
}
template <int R, int C>
inline Mat<R, C> operator-(const Mat<R, C>& a, const Mat<R, C>& b) {
    Mat<R, C> o;
    for (int i = 0; i < R * C; ++i) o.v[i] = a.v[i] - b.v[i];
    return o;
}
template <int R, int C>
inline Mat<R, C> operator-(const Mat<R, C>& a) {
    Mat<R, C> o;
    for (int i = 0; i < R * C; ++i) o.v[i] = -a.v[i];
    return o;
}
template <int R, int C>
inline Mat<R, C>& operator+=(Mat<R, C>& a, const Mat<R, C>& b) {
    for (int i = 0; i < R * C; ++i) a.v[i] += b.v[i];
    return a;
}
template <int R, int C>
inline Mat<R, C>& operator-=(Mat<R, C>& a, const Mat<R, C>& b) {
    for (int i = 0; i < R * C; ++i) a.v[i] -= b.v[i];
    return a;
}
template <int R, int C>
inline Mat<R, C> operator*(const Mat<R, C>& a, double s) {
    Mat<R, C> o;
    for (int i = 0; i < R * C; ++i) o.v[i] = a.v[i] * s;
    return o;
}
template <int R, int C>
inline Mat<R, C> operator*(double s, const Mat<R, C>& a) {
    Mat<R, C> o;
    for (int i = 0; i < R * C; ++i) o.v[i] = s * a.v[i];
    return o;
}
template <int R, int C>
inline Mat<R, C> operator/(const Mat<R, C>& a, double s) {
    Mat<R, C> o;
    for (int i = 0; i < R * C; ++i) o.v[i] = a.v[i] / s;
    return o;
}
template <int R, int C>
inline Mat<R, C>& operator/=(Mat<R, C>& a, double s) {
    for (int i = 0; i < R * C; ++i) a.v[i] /= s;
    return a;
}
template <int R, int K, int C>
inline Mat<R, C> operator*(const Mat<R, K>& a, const Mat<K, C>& b) {
    Mat<R, C> o;
    for (int i = 0; i < R; ++i)
        for (int j = 0; j < C; ++j) {
            double s = a(i, 0) * b(0, j);
            for (int k = 1; k < K; ++k) s += a(i, k) * b(k, j);
            o(i, j) = s;
        }
    return o;
}
template <int R, int C>
inline Mat<C, R> T(const Mat<R, C>& a) {
    Mat<C, R> o;
    for (int i = 0; i < R; ++i)
        for (int j = 0; j < C; ++j) o(j, i) = a(i, j);
    return o;
}
template <int N>
inline double dot(const Mat<N, 1>& a, const Mat<N, 1>& b) {
    double s = a[0] * b[0];
    for (int i = 1; i < N; ++i) s += a[i] * b[i];
    return s;
}
template <int N>
inline double squaredNorm(const Mat<N, 1>& a) { return dot(a, a); }
template <int N>
inline double norm(const Mat<N, 1>& a) { return std::sqrt(squaredNorm(a)); }
template <int N>
inline Mat<N, 1> normalized(const Mat<N, 1>& a) {
    double n = squaredNorm(a);
    if (n > 0.0) return a / std::sqrt(n);
    return a;
}
inline V3 cross(const V3& a, const V3& b) {
    return v3(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}

// ---------------- SO(3) (Sophus so3.hpp) ----------------
constexpr double kSophusEps = 1e-10;

inline M3 hat(const V3& w) {
    M3 m;
    m(0, 0) = 0; m(0, 1) = -w[2]; m(0, 2) = w[1];
    m(1, 0) = w[2]; m(1, 1) = 0; m(1, 2) = -w[0];
    m(2, 0) = -w[1]; m(2, 1) = w[0]; m(2, 2) = 0;
    return m;
}

// point_crossmat * P_rr * point_crossmat.transpose() (lio_builder.cpp:199-202,
// 240-243) as written: t = [w]x M, then t [w]x^T, every entry a dense k = 0..2
// left-to-right sum (the products with [w]x's zero diagonal included).
inline M3 hatSandwich(const V3& w, const M3& M) {
    const M3 h = hat(w);
    return (h * M) * T(h);
}

struct Quat { double w, x, y, z; };

// Eigen QuaternionBase::toRotationMatrix.
inline M3 quatToMat(const Quat& q) {
    const double tx = 2.0 * q.x, ty = 2.0 * q.y, tz = 2.0 * q.z;
    const double twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
    const double txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
    const double tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
    M3 r;
    r(0, 0) = 1.0 - (tyy + tzz); r(0, 1) = txy - twz; r(0, 2) = txz + twy;
    r(1, 0) = txy + twz; r(1, 1) = 1.0 - (txx + tzz); r(1, 2) = tyz - twx;
    r(2, 0) = txz - twy; r(2, 1) = tyz + twx; r(2, 2) = 1.0 - (txx + tyy);
    return r;
}

// Eigen quaternionbase_assign_impl<Matrix3>: rotation matrix -> quaternion.
inline Quat matToQuat(const M3& m) {
    Quat q;
    double t = m(0, 0) + m(1, 1) + m(2, 2);
    if (t > 0.0) {
        t = std::sqrt(t + 1.0);
        q.w = 0.5 * t;
        t = 0.5 / t;
        q.x = (m(2, 1) - m(1, 2)) * t;
        q.y = (m(0, 2) - m(2, 0)) * t;
        q.z = (m(1, 0) - m(0, 1)) * t;
    } else {
        int i = 0;
        if (m(1, 1) > m(0, 0)) i = 1;
        if (m(2, 2) > m(i, i)) i = 2;
        int j = (i + 1) % 3, k = (j + 1) % 3;
        t = std::sqrt(m(i, i) - m(j, j) - m(k, k) + 1.0);
        double c[3];
        c[i] = 0.5 * t;
        t = 0.5 / t;
        q.w = (m(k, j) - m(j, k)) * t;
        c[j] = (m(j, i) + m(i, j)) * t;
        c[k] = (m(k, i) + m(i, k)) * t;
        q.x = c[0]; q.y = c[1]; q.z = c[2];
    }
    return q;
}

// Sophus SO3::expAndTheta -> unit quaternion -> matrix.
inline M3 Exp(const V3& w) {
    double theta_sq = squaredNorm(w);
    double imag, real;
    if (theta_sq < kSophusEps * kSophusEps) {
        double theta_po4 = theta_sq * theta_sq;
        imag = 0.5 - (1.0 / 48.0) * theta_sq + (1.0 / 3840.0) * theta_po4;
        real = 1.0 - (1.0 / 8.0) * theta_sq + (1.0 / 384.0) * theta_po4;
    } else {
        double theta = std::sqrt(theta_sq);
        double half = 0.5 * theta;
        imag = std::sin(half) / theta;
        real = std::cos(half);
    }
    Quat q{real, imag * w[0], imag * w[1], imag * w[2]};
    return quatToMat(q);
}

// Sophus SO3(R).log(): atan-based log on Eigen's quaternion of R.
inline V3 Log(const M3& R) {
    Quat q = matToQuat(R);
    double sq_n = q.x * q.x + q.y * q.y + q.z * q.z;
    double w = q.w;
    double f;
    if (sq_n < kSophusEps * kSophusEps) {
        double sq_w = w * w;
        f = 2.0 / w - (2.0 / 3.0) * sq_n / (w * sq_w);
    } else {
        double n = std::sqrt(sq_n);
        double a = (w < 0.0) ? std::atan2(-n, -w) : std::atan2(n, w);
        f = 2.0 * a / n;
    }
    return v3(f * q.x, f * q.y, f * q.z);
}

// Sophus SO3::leftJacobian.
inline M3 leftJacobian(const V3& w) {
    double theta_sq = squaredNorm(w);
    M3 O = hat(w);
    M3 O2 = O * O;
    if (theta_sq < kSophusEps * kSophusEps) return M3::Identity() + 0.5 * O;
    double theta = std::sqrt(theta_sq);
    return M3::Identity() + (1.0 - std::cos(theta)) / theta_sq * O +
           (theta - std::sin(theta)) / (theta_sq * theta) * O2;
}
// kf::rightJacobian (ieskf.cpp:6-9).
inline M3 rightJacobian(const V3& w) { return T(leftJacobian(w)); }

// Eigen Quaternion::FromTwoVectors(a, b).matrix() (non-opposite branch; the
// opposite branch picks an axis orthogonal to a).
inline M3 fromTwoVectors(const V3& a, const V3& b) {
    V3 v0 = normalized(a), v1 = normalized(b);
    double c = dot(v1, v0);
    Quat q;
    if (c < -1.0 + 1e-12) {
        c = std::max(c, -1.0);
        V3 axis = cross(v0, v3(1, 0, 0));
        if (squaredNorm(axis) < 1e-12) axis = cross(v0, v3(0, 1, 0));
        axis = normalized(axis);
        double w2 = (1.0 + c) * 0.5;
        q.w = std::sqrt(w2);
        double s = std::sqrt(1.0 - w2);
        q.x = axis[0] * s; q.y = axis[1] * s; q.z = axis[2] * s;
        return quatToMat(q);
    }
    V3 axis = cross(v0, v1);
    double s = std::sqrt((1.0 + c) * 2.0);
    double invs = 1.0 / s;
    q.x = axis[0] * invs; q.y = axis[1] * invs; q.z = axis[2] * invs;
    q.w = s * 0.5;
    return quatToMat(q);
}

// Symmetric 3x3 eigen decomposition, cyclic Jacobi; ascending eigenvalues,
// eigenvectors in columns.
inline void eigSym3(const M3& A, V3& evals, M3& evecs) {
    double a[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a[i][j] = A(i, j);
    double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = std::fabs(a[0][1]) + std::fabs(a[0][2]) + std::fabs(a[1][2]);
        double scale = std::fabs(a[0][0]) + std::fabs(a[1][1]) + std::fabs(a[2][2]);
        if (off == 0.0 || off <= 1e-300 || off < 1e-18 * scale) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                double apq = a[p][q];
                if (apq == 0.0) continue;
                double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; ++k) {
                    double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - s * vkq;
                    v[k][q] = s * vkp + c * vkq;
                }
            }
    }
    int idx[3] = {0, 1, 2};
    double d[3] = {a[0][0], a[1][1], a[2][2]};
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (d[idx[j]] < d[idx[i]]) std::swap(idx[i], idx[j]);
    for (int c = 0; c < 3; ++c) {
        evals[c] = d[idx[c]];
        for (int r = 0; r < 3; ++r) evecs(r, c) = v[r][idx[c]];
    }
}

// LU with partial pivoting inverse (Eigen PartialPivLU::inverse).
template <int N>
inline Mat<N, N> inverse(const Mat<N, N>& A) {
    double lu[N][N];
    int perm[N];
    for (int i = 0; i < N; ++i) {
        perm[i] = i;
        for (int j = 0; j < N; ++j) lu[i][j] = A(i, j);
    }
    for (int k = 0; k < N; ++k) {
        int p = k;
        double best = std::fabs(lu[k][k]);
        for (int i = k + 1; i < N; ++i)
            if (std::fabs(lu[i][k]) > best) { best = std::fabs(lu[i][k]); p = i; }
        if (p != k) {
            for (int j = 0; j < N; ++j) std::swap(lu[k][j], lu[p][j]);
            std::swap(perm[k], perm[p]);
        }
        double piv = lu[k][k];
        for (int i = k + 1; i < N; ++i) {
            double f = lu[i][k] / piv;
            lu[i][k] = f;
            for (int j = k + 1; j < N; ++j) lu[i][j] -= f * lu[k][j];
        }
    }
    Mat<N, N> inv;
    for (int c = 0; c < N; ++c) {
        double x[N];
        for (int i = 0; i < N; ++i) x[i] = (perm[i] == c) ? 1.0 : 0.0;
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < i; ++j) x[i] -= lu[i][j] * x[j];
        for (int i = N - 1; i >= 0; --i) {
            for (int j = i + 1; j < N; ++j) x[i] -= lu[i][j] * x[j];
            x[i] /= lu[i][i];
        }
        for (int i = 0; i < N; ++i) inv(i, c) = x[i];
    }
    return inv;
}

// Eigen's Quaternion::setFromTwoVectors (rotation taking a onto b), output
// w x y z: c = a.b of the normalised vectors; axis = a x b, s = sqrt(2 (1 + c)),
// q = (s / 2, axis / s).  For c < -1 + 1e-12 (antiparallel) Eigen takes an
// axis from an SVD; this restatement takes the unit vector of a x e_x (or
// a x e_y when a is along x), rotated by pi.
inline void quatFromTwoVectors(const V3& a0, const V3& b0, double q[4]) {
    const V3 v0 = a0 / std::sqrt(dot(a0, a0));
    const V3 v1 = b0 / std::sqrt(dot(b0, b0));
    const double c = dot(v1, v0);
    if (c < -1.0 + 1e-12) {
        V3 e = std::fabs(v0[0]) < 0.9 ? v3(1, 0, 0) : v3(0, 1, 0);
        V3 ax = cross(v0, e);
        ax = ax / std::sqrt(dot(ax, ax));
        q[0] = 0.0; q[1] = ax[0]; q[2] = ax[1]; q[3] = ax[2];
        return;
    }
    const V3 axis = cross(v0, v1);
    const double s = std::sqrt((1.0 + c) * 2.0);
    const double invs = 1.0 / s;
    q[0] = s * 0.5;
    q[1] = axis[0] * invs;
    q[2] = axis[1] * invs;
    q[3] = axis[2] * invs;
}

}  // namespace orc
