// Seeded synthetic LiDAR-inertial sequences standing in for the reference's
// rosbag input (the demo bag is not available).  The output mimics what the
// reference node hands to LIOBuilder::process after livox2pcl and syncPackage
// (voxel_plus/src/utils.cpp:3-28, voxel_plus/src/lio_node.cpp:137-165):
//   * points in the LiDAR frame, float xyz, per-point time offset in ms
//     (the `curvature` field), every point time distinct and increasing;
//   * the scan end time = start + last point time / 1000;
//   * the package's IMU samples = every sample with t < scan end not yet
//     handed out.
// Scenes (std::mt19937_64, stream s seeded 0x5EED0000 + s):
//   kind 0  room: 20 x 20 x 5 m, 6 walls + 20 random planar boxes,
//           rosette (MID-360-like) pattern, range noise 2 cm;
//   kind 1  urban block: 100 x 100 x 20 m, ground + random facades (boxes
//           rotated about z), 5 % clutter points uniform in boxes,
//           spinning 128-beam pattern, range noise 3 cm;
//   kind 2  corridor: 1 km long planar corridor (walls, floor, ceiling,
//           pillars), spinning 32-beam pattern, range noise 2 cm.
// The trajectory is smooth (sums of sines), static for the first 0.3 s so
// that the IMU initialisation sees gravity only.  IMU: 200 Hz, gyro noise
// 1e-3, accel noise 1e-2, bias random walk.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>
#include <algorithm>

#include "../../include/vmp.h"

namespace {

struct V { double x, y, z; };
inline V add(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V sub(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V mul(V a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dotv(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

struct R33 { double m[9]; };
inline V rmul(const R33& R, V v) {
    return {R.m[0] * v.x + R.m[1] * v.y + R.m[2] * v.z, R.m[3] * v.x + R.m[4] * v.y + R.m[5] * v.z,
            R.m[6] * v.x + R.m[7] * v.y + R.m[8] * v.z};
}
inline V rtmul(const R33& R, V v) {
    return {R.m[0] * v.x + R.m[3] * v.y + R.m[6] * v.z, R.m[1] * v.x + R.m[4] * v.y + R.m[7] * v.z,
            R.m[2] * v.x + R.m[5] * v.y + R.m[8] * v.z};
}
inline R33 rpy(double r, double p, double y) {
    double cr = std::cos(r), sr = std::sin(r), cp = std::cos(p), sp = std::sin(p), cy = std::cos(y), sy = std::sin(y);
    return R33{{cy * cp, cy * sp * sr - sy * cr, cy * sp * cr + sy * sr, sy * cp, sy * sp * sr + cy * cr,
                sy * sp * cr - cy * sr, -sp, cp * sr, cp * cr}};
}
inline R33 rmm(const R33& A, const R33& B) {
    R33 C;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C.m[i * 3 + j] = A.m[i * 3] * B.m[j] + A.m[i * 3 + 1] * B.m[3 + j] + A.m[i * 3 + 2] * B.m[6 + j];
    return C;
}
inline R33 rt(const R33& A) {
    R33 C;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C.m[i * 3 + j] = A.m[j * 3 + i];
    return C;
}
inline V so3log(const R33& R) {
    double c = (R.m[0] + R.m[4] + R.m[8] - 1.0) * 0.5;
    c = std::max(-1.0, std::min(1.0, c));
    double th = std::acos(c);
    V w{R.m[7] - R.m[5], R.m[2] - R.m[6], R.m[3] - R.m[1]};
    double f = th < 1e-9 ? 0.5 : th / (2.0 * std::sin(th));
    return mul(w, f);
}

// An oriented box: centre, half sizes, yaw.  `inside` = the ray starts inside
// (room walls), so the far face is hit.
struct Box { V c; V h; double yaw; bool inside; };

struct Scene {
    std::vector<Box> boxes;
    bool ground = false;
    double ground_z = 0.0;
    std::vector<Box> clutter;  // volumes that hold the clutter points
};

// Ray / oriented-box intersection (slab method in the box frame).
inline bool hitBox(const Box& b, V o, V d, double& t_hit) {
    double cy = std::cos(b.yaw), sy = std::sin(b.yaw);
    V lo = sub(o, b.c);
    V ol{cy * lo.x + sy * lo.y, -sy * lo.x + cy * lo.y, lo.z};
    V dl{cy * d.x + sy * d.y, -sy * d.x + cy * d.y, d.z};
    double t0 = -1e30, t1 = 1e30;
    const double oo[3] = {ol.x, ol.y, ol.z}, dd[3] = {dl.x, dl.y, dl.z}, hh[3] = {b.h.x, b.h.y, b.h.z};
    for (int a = 0; a < 3; ++a) {
        if (std::fabs(dd[a]) < 1e-12) {
            if (oo[a] < -hh[a] || oo[a] > hh[a]) return false;
            continue;
        }
        double ta = (-hh[a] - oo[a]) / dd[a], tb = (hh[a] - oo[a]) / dd[a];
        if (ta > tb) std::swap(ta, tb);
        t0 = std::max(t0, ta);
        t1 = std::min(t1, tb);
    }
    if (t0 > t1) return false;
    if (b.inside) { if (t1 <= 1e-6) return false; t_hit = t1; return true; }
    if (t0 <= 1e-6) return false;
    t_hit = t0;
    return true;
}

}  // namespace

extern "C" {

typedef struct vmp_synth_config {
    int kind;              /* 0 room, 1 urban block, 2 corridor */
    int points_per_scan;   /* nominal rays per scan */
    unsigned long long seed;
    double scan_hz;        /* 10 */
    double imu_hz;         /* 200 */
    double range_sigma;    /* m */
    double max_range;      /* m */
    double min_range;      /* m */
    double speed;          /* trajectory amplitude scale */
    double gyro_noise, acc_noise, bias_walk;
    int beams;             /* spinning patterns */
    double clutter_frac;
} vmp_synth_config;

void vmp_synth_default(vmp_synth_config* c, int kind) {
    std::memset(c, 0, sizeof(*c));
    c->kind = kind;
    c->seed = 0x5EED0000ULL;
    c->scan_hz = 10.0;
    c->imu_hz = 200.0;
    c->gyro_noise = 1e-3;
    c->acc_noise = 1e-2;
    c->bias_walk = 1e-5;
    c->speed = 1.0;
    c->min_range = 0.5;
    if (kind == 0) { c->points_per_scan = 20000; c->range_sigma = 0.02; c->max_range = 40.0; c->beams = 0; c->clutter_frac = 0.0; }
    else if (kind == 1) { c->points_per_scan = 200000; c->range_sigma = 0.03; c->max_range = 100.0; c->beams = 128; c->clutter_frac = 0.05; }
    else { c->points_per_scan = 100000; c->range_sigma = 0.02; c->max_range = 60.0; c->beams = 32; c->clutter_frac = 0.0; }
}

struct vmp_synth {
    vmp_synth_config cfg;
    Scene scene;
    std::mt19937_64 rng;
    double t0 = 100.0;  // first scan start time (s)
    int next_imu = 0;   // next IMU sample index not yet handed out
    V bg{0, 0, 0}, ba{0, 0, 0};
    int bias_step = -1;
    V center{0, 0, 0};
    double amp[3] = {0, 0, 0};
};

static void buildScene(vmp_synth* s) {
    std::mt19937_64& r = s->rng;
    std::uniform_real_distribution<double> U(0.0, 1.0);
    Scene& sc = s->scene;
    if (s->cfg.kind == 0) {
        sc.boxes.push_back(Box{{0, 0, 2.5}, {10, 10, 2.5}, 0.0, true});
        for (int i = 0; i < 20; ++i) {
            V c{-8 + 16 * U(r), -8 + 16 * U(r), 0};
            V h{0.2 + 0.8 * U(r), 0.2 + 0.8 * U(r), 0.3 + 1.2 * U(r)};
            c.z = h.z;
            // keep the trajectory corridor (|x|,|y| < 3) free
            if (std::fabs(c.x) < 3.5 && std::fabs(c.y) < 3.5) { c.x += (c.x < 0 ? -4 : 4); }
            sc.boxes.push_back(Box{c, h, U(r) * 3.14159, false});
        }
        s->center = V{0, 0, 1.5};
        s->amp[0] = 2.5; s->amp[1] = 2.5; s->amp[2] = 0.5;
    } else if (s->cfg.kind == 1) {
        sc.ground = true;
        sc.ground_z = 0.0;
        for (int i = 0; i < 40; ++i) {
            V c{-50 + 100 * U(r), -50 + 100 * U(r), 0};
            if (std::fabs(c.x) < 12 && std::fabs(c.y) < 12) continue;  // keep the drive area open
            V h{2 + 6 * U(r), 2 + 6 * U(r), 3 + 7 * U(r)};
            c.z = h.z;
            sc.boxes.push_back(Box{c, h, U(r) * 3.14159, false});
        }
        for (int i = 0; i < 30; ++i) {
            V c{-40 + 80 * U(r), -40 + 80 * U(r), 0};
            V h{0.5 + U(r), 0.5 + U(r), 0.5 + 0.8 * U(r)};
            c.z = h.z;
            sc.clutter.push_back(Box{c, h, 0.0, false});
        }
        s->center = V{0, 0, 1.8};
        s->amp[0] = 8.0; s->amp[1] = 8.0; s->amp[2] = 0.3;
    } else {
        sc.boxes.push_back(Box{{500, 0, 2.0}, {510, 3.0, 2.0}, 0.0, true});
        for (int i = 0; i < 100; ++i)
            sc.boxes.push_back(Box{{10.0 * i + 5 * U(r), (i % 2 ? 2.2 : -2.2), 2.0}, {0.3, 0.3, 2.0}, 0.0, false});
        s->center = V{0, 0, 1.5};
        s->amp[0] = 0.0; s->amp[1] = 0.8; s->amp[2] = 0.2;
    }
}

// Smooth trajectory; static before t0 + 0.3 s.
static void trajectory(const vmp_synth* s, double t, R33& R, V& p) {
    double tau = t - (s->t0 + 0.3);
    double ramp = 0.0;
    if (tau > 0) ramp = tau < 2.0 ? (tau * tau * tau / 8.0) * (10.0 - 15.0 * tau / 2.0 + 6.0 * tau * tau / 4.0) : 1.0;
    double a = s->cfg.speed;
    double tt = tau > 0 ? tau : 0.0;
    if (s->cfg.kind == 2) {
        // forward along the corridor at ~1.5 m/s
        double u = tau * 0.5;
        double integ = tau <= 0 ? 0.0 : (tau < 2.0 ? 2.0 * (2.5 * u * u * u * u - 3.0 * u * u * u * u * u + u * u * u * u * u * u) : 1.0 + (tau - 2.0));
        double fwd = 1.5 * a * integ;
        p = V{5.0 + fwd, ramp * s->amp[1] * std::sin(0.4 * tt), s->center.z + ramp * s->amp[2] * std::sin(0.7 * tt)};
        R = rpy(ramp * 0.03 * std::sin(1.1 * tt), ramp * 0.02 * std::sin(0.9 * tt), ramp * 0.2 * std::sin(0.3 * tt));
        return;
    }
    p = V{s->center.x + ramp * a * s->amp[0] * std::sin(0.21 * tt), s->center.y + ramp * a * s->amp[1] * std::sin(0.17 * tt + 0.5) - ramp * a * s->amp[1] * std::sin(0.5),
          s->center.z + ramp * a * s->amp[2] * std::sin(0.33 * tt)};
    R = rpy(ramp * 0.05 * std::sin(0.9 * tt), ramp * 0.04 * std::sin(0.7 * tt + 1.0), ramp * a * 0.8 * std::sin(0.12 * tt));
}

static void imuAt(vmp_synth* s, double t, V& acc, V& gyro) {
    const double h = 1e-4;
    R33 R0, R1, Rm;
    V p0, p1, pm;
    trajectory(s, t - h, R0, p0);
    trajectory(s, t + h, R1, p1);
    trajectory(s, t, Rm, pm);
    V a_w = mul(add(sub(p1, mul(pm, 2.0)), p0), 1.0 / (h * h));
    V w = mul(so3log(rmm(rt(R0), R1)), 1.0 / (2 * h));
    V g{0, 0, -9.81};
    acc = rtmul(Rm, sub(a_w, g));
    gyro = w;
}

vmp_synth* vmp_synth_create(const vmp_synth_config* cfg) {
    vmp_synth* s = new vmp_synth();
    s->cfg = *cfg;
    s->rng.seed(cfg->seed);
    buildScene(s);
    return s;
}
void vmp_synth_destroy(vmp_synth* s) { delete s; }

// Ground-truth pose of the sensor at time t (R row-major, p).
void vmp_synth_pose(vmp_synth* s, double t, double* R, double* p) {
    R33 r; V q;
    trajectory(s, t, r, q);
    std::memcpy(R, r.m, sizeof(r.m));
    p[0] = q.x; p[1] = q.y; p[2] = q.z;
}

static double imuTime(const vmp_synth* s, int i) { return s->t0 - 0.2 + i / s->cfg.imu_hz + 0.00037; }

// Package k: scan k (t_start = t0 + k / scan_hz) and the IMU samples up to its
// end.  Returns the number of points (<= max_points).  Packages must be read
// in order (k = 0, 1, 2, ...).
int vmp_synth_package(vmp_synth* s, int k, vmp_point* pts, int max_points, double* t_start, double* t_end,
                      vmp_imu* imus, int max_imu, int* n_imu) {
    const vmp_synth_config& c = s->cfg;
    double ts = s->t0 + k / c.scan_hz;
    double period = 1.0 / c.scan_hz;
    int nrays = c.points_per_scan;
    // per-ray counter-based random numbers: identical output for any thread count
    const unsigned long long scan_key = c.seed * 1315423911ULL + (unsigned long long)k * 2654435761ULL + 17;
    std::vector<vmp_point> rays((size_t)nrays);
    std::vector<unsigned char> keep((size_t)nrays, 0);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int j = 0; j < nrays; ++j) {
        unsigned long long ctr = scan_key ^ (0x9E3779B97F4A7C15ULL * (unsigned long long)(j + 1));
        auto uni = [&ctr]() {
            unsigned long long z = (ctr += 0x9E3779B97F4A7C15ULL);
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
            z ^= z >> 31;
            return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        };
        auto gauss = [&uni]() {
            double u1 = uni(), u2 = uni();
            return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979 * u2);
        };
        double dt = j * (period / nrays);
        double t = ts + dt;
        // beam direction in the sensor frame
        V d;
        if (c.beams <= 0) {
            // rosette: two incommensurate rotations, elevation -7..52 deg
            double u = t * 200.0;
            double az = 2.0 * 3.14159265358979 * (u * 1.0003 + 0.37 * std::sin(2.0 * 3.14159265358979 * u * 0.0731));
            double el = (22.5 + 29.5 * std::sin(2.0 * 3.14159265358979 * u * 0.5171 + 0.3 * std::sin(u * 0.13))) * 3.14159265358979 / 180.0;
            d = V{std::cos(el) * std::cos(az), std::cos(el) * std::sin(az), std::sin(el)};
        } else {
            int beam = j % c.beams;
            int col = j / c.beams;
            int ncol = nrays / c.beams;
            double az = 2.0 * 3.14159265358979 * col / std::max(ncol, 1);
            double el = (-22.5 + 45.0 * beam / std::max(c.beams - 1, 1)) * 3.14159265358979 / 180.0;
            d = V{std::cos(el) * std::cos(az), std::cos(el) * std::sin(az), std::sin(el)};
        }
        R33 R; V p;
        trajectory(s, t, R, p);
        V dw = rmul(R, d);
        double best = 1e30;
        bool hit = false;
        for (const Box& b : s->scene.boxes) {
            double th;
            if (hitBox(b, p, dw, th) && th < best) { best = th; hit = true; }
        }
        if (s->scene.ground && dw.z < -1e-9) {
            double th = (s->scene.ground_z - p.z) / dw.z;
            if (th > 0 && th < best) { best = th; hit = true; }
        }
        double range;
        V pl;
        if (c.clutter_frac > 0 && !s->scene.clutter.empty() && uni() < c.clutter_frac) {
            // non-planar clutter: a random point inside a random clutter volume
            const Box& b = s->scene.clutter[(size_t)(uni() * s->scene.clutter.size()) % s->scene.clutter.size()];
            V q{b.c.x + (2 * uni() - 1) * b.h.x, b.c.y + (2 * uni() - 1) * b.h.y, b.c.z + (2 * uni() - 1) * b.h.z};
            pl = rtmul(R, sub(q, p));
            range = std::sqrt(dotv(pl, pl));
        } else {
            if (!hit) continue;
            range = best + c.range_sigma * gauss();
            pl = mul(d, range);
        }
        if (range < c.min_range || range > c.max_range) continue;
        vmp_point q;
        q.x = (float)pl.x; q.y = (float)pl.y; q.z = (float)pl.z;
        q.t_ms = (float)(dt * 1000.0);
        rays[(size_t)j] = q;
        keep[(size_t)j] = 1;
    }
    std::vector<vmp_point> out;
    out.reserve((size_t)nrays);
    for (int j = 0; j < nrays; ++j)
        if (keep[(size_t)j]) out.push_back(rays[(size_t)j]);
    int n = std::min((int)out.size(), max_points);
    if (n > 0) std::memcpy(pts, out.data(), sizeof(vmp_point) * n);
    *t_start = ts;
    *t_end = ts + (n > 0 ? (double)pts[n - 1].t_ms / double(1000.0) : 0.0);
    // IMU samples with t < t_end not yet handed out
    int m = 0;
    while (true) {
        double ti = imuTime(s, s->next_imu);
        if (ti >= *t_end) break;
        // bias random walk, advanced deterministically per sample index
        while (s->bias_step < s->next_imu) {
            s->bias_step++;
            std::mt19937_64 rb(c.seed ^ (0x9E3779B97F4A7C15ULL * (unsigned long long)(s->bias_step + 1)));
            std::normal_distribution<double> nb(0.0, c.bias_walk);
            s->bg = add(s->bg, V{nb(rb), nb(rb), nb(rb)});
            s->ba = add(s->ba, V{nb(rb), nb(rb), nb(rb)});
        }
        V acc, gyro;
        imuAt(s, ti, acc, gyro);
        std::mt19937_64 rn(c.seed ^ (0xD1B54A32D192ED03ULL * (unsigned long long)(s->next_imu + 7)));
        std::normal_distribution<double> ng(0.0, c.gyro_noise), na(0.0, c.acc_noise);
        if (m < max_imu) {
            imus[m].t = ti;
            imus[m].acc[0] = acc.x + s->ba.x + na(rn); imus[m].acc[1] = acc.y + s->ba.y + na(rn); imus[m].acc[2] = acc.z + s->ba.z + na(rn);
            imus[m].gyro[0] = gyro.x + s->bg.x + ng(rn); imus[m].gyro[1] = gyro.y + s->bg.y + ng(rn); imus[m].gyro[2] = gyro.z + s->bg.z + ng(rn);
            ++m;
        }
        s->next_imu++;
    }
    *n_imu = m;
    return n;
}

}  // extern "C"
