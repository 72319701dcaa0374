"""The C++ LIOBuilder-shaped adapter (include/vmp_lio_builder.hpp) compiles
against mock lio::SyncPackage / LIOConfig types (PCL and Eigen are not needed)
and links libvmp.so; without a GPU its loadConfig reports the missing device."""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include "vmp_lio_builder.hpp"
#include <cstdio>
#include <memory>
struct Pt { float x, y, z, intensity, curvature; };
struct Cloud { std::vector<Pt> points; };
struct Vec3 { double v[3]; double operator[](int i) const { return v[i]; } double operator()(int i) const { return v[i]; } };
struct Mat3 { double m[9]; double operator()(int i, int j) const { return m[i * 3 + j]; } };
struct Imu { Vec3 acc, gyro; double timestamp; };
struct Pkg { std::shared_ptr<Cloud> cloud; std::vector<Imu> imus; double cloud_start_time = 0, cloud_end_time = 0; };
struct Cfg {
    int opti_max_iter = 5; double na = 0.01, ng = 0.01, nba = 1e-4, nbg = 1e-4; int imu_init_num = 20;
    Mat3 r_il{{1, 0, 0, 0, 1, 0, 0, 0, 1}}; Vec3 p_il{{0, 0, 0}}; bool gravity_align = true, estimate_ext = false;
    double scan_resolution = 0.1, voxel_size = 0.5; int update_size_thresh = 10, max_point_thresh = 100;
    double plane_thresh = 0.01, ranging_cov = 0.04, angle_cov = 0.1;
    double merge_thresh_for_angle = 0.1, merge_thresh_for_distance = 0.04; int map_capacity = 100000;
};
int main() {
    vmp_adapter::LIOBuilder b;
    try { b.loadConfig(Cfg{}); } catch (const std::exception& e) { std::printf("nogpu %s\n", e.what()); return 0; }
    Pkg p;
    p.cloud = std::make_shared<Cloud>();
    for (int i = 0; i < 100; ++i) p.cloud->points.push_back(Pt{1.f + i, 2.f, 3.f, 0.f, 0.5f * i});
    for (int i = 0; i < 25; ++i) p.imus.push_back(Imu{{{0, 0, 9.81}}, {{0, 0, 0}}, 0.005 * i});
    p.cloud_end_time = 0.05;
    b.process(p);
    std::vector<Pt> body, world;
    b.lidarToBody(body);
    b.lidarToWorld(world);
    std::printf("ok %d %zu %zu\n", (int)b.status, body.size(), world.size());
    return 0;
}
'''


def test_adapter_compiles_and_links():
    from voxelmapplus_fastlio2_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build_all()
    libdir = os.path.dirname(_lib.LIB_PATH)
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "a.cpp")
        exe = os.path.join(d, "a")
        open(src, "w").write(SRC)
        subprocess.check_call(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-o", exe, src,
                               "-L" + libdir, "-lvmp", "-Wl,-rpath," + libdir])
        out = subprocess.check_output([exe], text=True)
    assert out.startswith("nogpu") or out.startswith("ok"), out
