/*
 * vmp.h -- C ABI of libvmp.so, the GB300 (sm_103a) odometry hot path of a
 * FAST-LIO2 + VoxelMapPlus LiDAR-inertial odometry node.
 *
 * One vmp_stream_t owns the complete device-resident state of one sensor
 * stream: the voxel plane map (hash, voxel records, point slabs, LRU queue),
 * the iterated error-state Kalman filter (state x, covariance P) and the
 * per-point residual records.  Every call enqueues CUDA kernels on the
 * stream's own CUDA stream; there is no CPU fallback: a library that cannot
 * reach a GPU fails vmp_create with VMP_ERR_CUDA.
 *
 * Reference call surface each entry point replaces (paths are relative to the
 * voxel_plus package of liangheming/VoxelMapPlus_FASTLIO2):
 *   vmp_create / vmp_destroy     lio::LIOBuilder::loadConfig   src/map_builder/lio_builder.cpp:5-26
 *   vmp_process                  lio::LIOBuilder::process      src/map_builder/lio_builder.cpp:175-248
 *   vmp_undistort                lio::LIOBuilder::undistortCloud src/map_builder/lio_builder.cpp:65-153
 *   vmp_downsample               pcl::VoxelGrid filter call    src/map_builder/lio_builder.cpp:215-223
 *   vmp_map_index                lio::VoxelMap::index          src/map_builder/voxel_map.cpp:194-198
 *   vmp_map_build                lio::VoxelMap::build          src/map_builder/voxel_map.cpp:200-230
 *   vmp_map_update               lio::VoxelMap::update         src/map_builder/voxel_map.cpp:232-256
 *   vmp_residual_reduce          lio::LIOBuilder::sharedUpdateFunc src/map_builder/lio_builder.cpp:250-311
 *   vmp_ieskf_predict            kf::IESKF::predict            src/map_builder/ieskf.cpp:101-123
 *   vmp_ieskf_update             kf::IESKF::update             src/map_builder/ieskf.cpp:125-156
 *   vmp_get_state / vmp_set_state kf::IESKF::x(), P(), change_x, change_P  src/map_builder/ieskf.h:86-94
 *   vmp_map_export / vmp_map_import  direct featmap access by the node  src/utils.cpp:154-208
 *   vmp_fit_planes               lio::VoxelGrid::updatePlane over all voxels, as VoxelMap::build
 *                                fits them  src/map_builder/voxel_map.cpp:97-136, 200-230
 *
 * Conventions: all matrices are row-major double.  Points are float as in
 * pcl::PointXYZINormal; the per-point time is the field the reference keeps in
 * `curvature` (milliseconds since the scan start, src/utils.cpp:20).
 * No exception crosses the ABI; every entry point returns a vmp_status and
 * vmp_last_error() gives a human-readable reason.  A handle is not
 * re-entrant: one caller thread per handle.
 */
#ifndef VMP_H_
#define VMP_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VMP_ABI_VERSION 2

typedef enum vmp_status {
    VMP_OK = 0,
    VMP_ERR_INVALID_ARG = 1,      /* bad pointer, size or configuration */
    VMP_ERR_OUT_OF_MEMORY = 2,    /* device allocation failed */
    VMP_ERR_ADMISSION_DENIED = 3, /* server HBM budget would be exceeded */
    VMP_ERR_HASH_FULL = 4,        /* voxel hash table has no free slot */
    VMP_ERR_TIMEOUT = 5,          /* a bounded device wait gave up */
    VMP_ERR_CUDA = 6,             /* CUDA runtime error (no GPU, launch failure) */
    VMP_ERR_KEY_RANGE = 7,        /* a voxel index left the packed 21-bit range */
    VMP_ERR_STATE = 8,            /* call not valid in the current stream state */
    VMP_ERR_CAPACITY = 9          /* a per-call size exceeds the configured maximum */
} vmp_status;

/* lio::LIOStatus (lio_builder.h:10-16) */
typedef enum vmp_lio_status {
    VMP_IMU_INIT = 0,
    VMP_MAP_INIT = 1,
    VMP_LIO_MAPPING = 2
} vmp_lio_status;

/* Mirrors lio::LIOConfig (lio_builder.h:17-42): same field names, same
 * defaults (vmp_config_default).  The trailing members size the device
 * buffers and expose the two private kf::IESKF constants (ieskf.h:101-102). */
typedef struct vmp_config {
    int opti_max_iter;            /* 5: read by the node, never applied by the reference */
    double na, ng, nba, nbg;      /* 0.01, 0.01, 1e-4, 1e-4 */
    int imu_init_num;             /* 20 */
    double r_il[9];               /* identity */
    double p_il[3];               /* zero */
    int gravity_align;            /* 1 */
    int estimate_ext;             /* 0 */
    double scan_resolution;       /* 0.1 */
    double voxel_size;            /* 0.5 */
    int update_size_thresh;       /* 10 (must be >= 2) */
    int max_point_thresh;         /* 100 */
    double plane_thresh;          /* 0.01 */
    double ranging_cov;           /* 0.04 */
    double angle_cov;             /* 0.1 (degrees) */
    double merge_thresh_for_angle;    /* 0.1 */
    double merge_thresh_for_distance; /* 0.04 */
    int map_capacity;             /* 100000 */
    /* kf::IESKF private members */
    int ieskf_max_iter;           /* 5 (ieskf.h:101) */
    double ieskf_eps;             /* 0.001 (ieskf.h:102) */
    /* device sizing; no reference counterpart */
    int max_scan_points;          /* raw points accepted per scan (default 262144) */
    int max_imu_per_scan;         /* IMU samples accepted per scan (default 1000, at most 1000) */
    /* reserved[0]: point-slab chunks (0: 2 x records + 1024); reserved[1]:
     * plane-covariance term buffer (0: 4 x max_scan_points + 65536; terms
     * that do not fit are formed by the summation itself); the rest 0 */
    int reserved[6];
} vmp_config;

/* One LiDAR point: xyz in the LiDAR frame and the time offset in ms. */
typedef struct vmp_point {
    float x, y, z, t_ms;
} vmp_point;

/* lio::IMUData (commons.h:12-20) */
typedef struct vmp_imu {
    double t;
    double acc[3];
    double gyro[3];
} vmp_imu;

/* lio::SyncPackage (commons.h:22-28): cloud + its start/end time. */
typedef struct vmp_scan {
    const vmp_point* points;
    int n;
    double t_start;
    double t_end;
} vmp_scan;

/* kf::State (ieskf.h:31-62); rotations row-major. */
typedef struct vmp_state {
    double pos[3];
    double rot[9];
    double rot_ext[9];
    double pos_ext[3];
    double vel[3];
    double bg[3];
    double ba[3];
    double g[3];
} vmp_state;

typedef struct vmp_result {
    int lio_status;       /* vmp_lio_status after the call */
    int iters;            /* IEKF iterations run this scan */
    int effect_num;       /* valid residuals in the last iteration */
    int n_raw;            /* points in the scan */
    int n_down;           /* points after the scan downsample */
    int flags;            /* bit0: no effective point in an iteration */
    long long map_size;   /* live voxels after the scan */
    long long evicted;    /* voxels evicted by this scan */
    vmp_state x;
    double P[23 * 23];
} vmp_result;

/* Sizes of the voxel map (for vmp_map_export buffers). */
typedef struct vmp_map_info {
    long long size;          /* live voxels */
    long long capacity;      /* LRU capacity */
    long long group_counter; /* VoxelGrid::count */
    long long slab_points;   /* buffered points over all voxels */
} vmp_map_info;

/* One voxel of lio::VoxelGrid + its lio::Plane (voxel_map.h:43-103). */
typedef struct vmp_voxel {
    int64_t key[3];
    int32_t n;               /* plane->n */
    int32_t newly_add_point;
    int32_t is_init, is_plane, update_enable, merged;
    uint64_t group_id;
    uint64_t lru_stamp;      /* larger = more recently touched */
    int32_t n_temp;          /* temp_points.size() */
    int32_t pad;
    double mean[3];
    double ppt[9];
    double norm[3];
    double center[3];
    double cov[36];
} vmp_voxel;

typedef struct vmp_stream_s* vmp_stream_t;

void vmp_config_default(vmp_config* cfg);
int vmp_abi_version(void);

vmp_status vmp_create(const vmp_config* cfg, vmp_stream_t* out);
vmp_status vmp_destroy(vmp_stream_t s);
const char* vmp_last_error(vmp_stream_t s);

/* Full per-scan step (LIOBuilder::process).  Host buffers in, result out. */
vmp_status vmp_process(vmp_stream_t s, const vmp_scan* scan, const vmp_imu* imus, int n_imu,
                       vmp_result* out);

/* Same step with the scan and IMU samples already in device memory
 * (device pointers; the call does no host<->device copy of inputs; the
 * result is still written to the host struct). */
vmp_status vmp_process_device(vmp_stream_t s, const vmp_point* d_points, int n, double t_start,
                              double t_end, const vmp_imu* d_imus, int n_imu, vmp_result* out);

/* ---- component entry points (the voxel_plus VoxelMap / IESKF surface) ---- */

/* VoxelMap::index: keys[i*3+0..2] = floor(pts[i]/voxel_size). */
vmp_status vmp_map_index(vmp_stream_t s, const double* pts, int n, int64_t* keys);
/* VoxelMap::build on an empty map: pts n x 3, cov n x 9. */
vmp_status vmp_map_build(vmp_stream_t s, const double* pts, const double* cov, int n);
/* VoxelMap::update: pts n x 3, cov n x 9, applied in order. */
vmp_status vmp_map_update(vmp_stream_t s, const double* pts, const double* cov, int n);
vmp_status vmp_map_info_get(vmp_stream_t s, vmp_map_info* info);
/* Copies up to max voxels, most recently used first (LRU order). */
vmp_status vmp_map_export(vmp_stream_t s, vmp_voxel* out, long long max, long long* n_out);
/* The keys of VoxelMap::featmap in the order of VoxelMap::cache
 * (voxel_map.h:124-125; front = most recently used): keys[i*3+0..2] for up
 * to max voxels, *n_out = live voxels.  24 bytes per voxel instead of a full
 * vmp_voxel, for per-scan key-set checks of large maps. */
vmp_status vmp_map_keys(vmp_stream_t s, int64_t* keys, long long max, long long* n_out);
/* Replaces the map by the given voxels (LRU order as listed, first = most
 * recent) and their buffered points (pts/cov of all voxels concatenated in
 * voxel order, vox[i].n_temp each). */
vmp_status vmp_map_import(vmp_stream_t s, const vmp_voxel* vox, long long n, const double* pts,
                          const double* cov, long long group_counter);
/* Buffered points of the exported voxels, in export order (n_temp each). */
vmp_status vmp_map_export_points(vmp_stream_t s, double* pts, double* cov, long long max_points,
                                 long long* n_out);

/* LIOBuilder::sharedUpdateFunc with an explicit state: pts_l n x 3 (LiDAR
 * frame, after the calcBodyCov z-fix), cov_l n x 9, P 23x23.  Writes the
 * 12x12 H and 12 b of kf::SharedState and the valid-point count.  The
 * per-point residual records persist across calls like residual_info. */
vmp_status vmp_residual_reduce(vmp_stream_t s, const vmp_state* x, const double* P,
                               const double* pts_l, const double* cov_l, int n, double* H,
                               double* b, int* effect_num);

/* IESKF on the stream's device state. */
vmp_status vmp_get_state(vmp_stream_t s, vmp_state* x, double* P);
vmp_status vmp_set_state(vmp_stream_t s, const vmp_state* x, const double* P);
vmp_status vmp_ieskf_predict(vmp_stream_t s, const double acc[3], const double gyro[3], double dt,
                             const double* Q /* 12x12 */);
/* Iterated update with the measurement model of sharedUpdateFunc over the
 * given LiDAR points (after downsample): iters/effect_num reported. */
vmp_status vmp_ieskf_update(vmp_stream_t s, const float* pts_l /* n x 3 */, int n, int* iters,
                            int* effect_num);

/* LIOBuilder::undistortCloud on the stream's filter state: points are sorted
 * by time and compensated in place into out (n points). */
vmp_status vmp_undistort(vmp_stream_t s, const vmp_scan* scan, const vmp_imu* imus, int n_imu,
                         vmp_point* out);
/* pcl::VoxelGrid leaf-centroid downsample at the given leaf size. */
vmp_status vmp_downsample(vmp_stream_t s, const vmp_point* pts, int n, double leaf,
                          vmp_point* out, int* n_out);
/* ---- input decode and output clouds (the steps either side of the path) ----
 * livox_ros_driver2 CustomPoint (CustomPoint.msg) in the field order of the
 * message and of its generated C++ struct (20 bytes with the tail padding),
 * so a CustomMsg's points array can be passed as it is. */
typedef struct vmp_livox_point {
    uint32_t offset_time; /* ns after the message time */
    float x, y, z;        /* m, LiDAR frame */
    uint8_t reflectivity;
    uint8_t tag;
    uint8_t line;
    uint8_t pad;
} vmp_livox_point;
/* livox2pcl (src/utils.cpp:3-28) on the device: keeps the points with
 * line < 4 and tag bits 4-5 equal to 0 or 1, of those every filter_num-th
 * (the first included), of those the ones with
 * range_min^2 < x^2 + y^2 + z^2 < range_max^2 (the sum in float, the test in
 * double); t_ms = offset_time / 1e6 (float), intensity = reflectivity.  The
 * decoded cloud stays in the stream's device scan buffer for
 * vmp_process_decoded.  out / intensity (host, may be NULL) receive the n_out
 * kept points; last_t_ms (may be NULL) the last kept point's t_ms, from which
 * the node's syncPackage forms the package end time (lio_node.cpp:142-146).
 * n <= max_scan_points. */
vmp_status vmp_livox_decode(vmp_stream_t s, const vmp_livox_point* pts, int n, int filter_num, double range_min,
                            double range_max, vmp_point* out, float* intensity, int* n_out, float* last_t_ms);
/* vmp_process on the cloud of the last vmp_livox_decode, without uploading it
 * again (VMP_ERR_STATE when no decoded cloud is pending). */
vmp_status vmp_process_decoded(vmp_stream_t s, double t_start, double t_end, const vmp_imu* imus, int n_imu,
                               vmp_result* out);
/* lidarToBody (frame 0) / lidarToWorld (frame 1) (lio_builder.cpp:155-173)
 * of the last processed scan's undistorted, time-sorted cloud -- the node's
 * sync_pack.cloud after process -- under the state after that scan's update,
 * as a float 4x4 transform in pcl::transformPointCloud's operation order.
 * out (host, max points; x y z t_ms) and intensity (host, may be NULL;
 * reflectivity of decoded scans, 0 otherwise); *n_out = points in the cloud
 * (0 after an IMU-initialisation package). */
vmp_status vmp_output_cloud(vmp_stream_t s, int frame, vmp_point* out, float* intensity, int max, int* n_out);
/* The same into device buffers the caller owns; only enqueues the work on
 * the stream's CUDA stream.  *n_out (host) = points written. */
vmp_status vmp_output_cloud_device(vmp_stream_t s, int frame, vmp_point* d_out, float* d_intensity, int max,
                                   int* n_out);

/* ---- voxel-map export for visualisation ----
 * What voxel2MarkerArray (src/utils.cpp:154-208) reads from the map for one
 * plane marker.  The reference walks the LRU list from its front (most
 * recently touched) and emits the frozen planes (is_plane && !update_enable),
 * at most max_capacity of them. */
typedef struct vmp_plane_marker {
    double center[3];      /* VoxelGrid::center (the mean at the last refit) */
    double norm[3];        /* plane normal */
    double orientation[4]; /* w x y z: Quaterniond::FromTwoVectors((0, 0, 1), norm) (calcVectQuation) */
    double trace;          /* trace of the plane covariance's top-left 3x3 */
    uint8_t rgb[3];        /* mapJet((min(trace, 0.25) / 0.25)^0.2, 0, 1) */
    uint8_t merged;        /* 1: CUBE marker, 0: CYLINDER */
    int32_t pad;
} vmp_plane_marker;
/* The first min(planes, max) frozen plane voxels in LRU order, selected,
 * sorted and formed on the device.  out (host) holds max markers; *n_out =
 * markers written. */
vmp_status vmp_map_planes(vmp_stream_t s, vmp_plane_marker* out, int max, int* n_out);

/* ---- plane voxels of a key cloud (loop closure) ----
 * std_desc::STDManager::buildVoxels (std_matcher/src/std_manager/
 * descriptor.cpp:70-122): the cloud voxelised at voxel_size
 * (VoxelKey::index: floor(p / voxel_size), descriptor.cpp:44-49), per voxel
 * the FP64 sum and sum of outer products of its points in cloud order, and
 * for voxels with more than voxel_min_point points the mean, the eigen
 * decomposition of C = ppt / n - mean mean^T and the plane test
 * lambda_min < voxel_plane_thresh.  One record per voxel, in packed-key order
 * (the reference iterates an unordered_map). */
typedef struct vmp_std_voxel {
    int64_t key[3];
    int32_t n;         /* points in the voxel */
    int32_t valid;     /* n > voxel_min_point: mean and decomposition formed */
    int32_t is_plane;  /* valid and lambda_min < voxel_plane_thresh */
    int32_t pad;
    double sum[3];
    double ppt[9];
    double mean[3];    /* 0 unless valid */
    double lamdas[3];  /* ascending; 0 unless is_plane */
    double norms[9];   /* row-major, eigenvectors as columns in lamdas' order; 0 unless is_plane */
} vmp_std_voxel;
/* pts: n points of `stride` floats each, x y z first (stride 8 for
 * pcl::PointXYZI, 4 for vmp_point).  out (host) holds max records; *n_out =
 * voxels of the cloud.  Allocates and frees device memory per call. */
vmp_status vmp_std_plane_voxels(const float* pts, int stride, int n, double voxel_size, int voxel_min_point,
                                double voxel_plane_thresh, vmp_std_voxel* out, int max, int* n_out);

/* Test hook: a[i] / b[i] computed on the device by the reciprocal-and-
 * correction path the kernels use for divisions that share a divisor, and by
 * the FP64 division (host arrays of n; the two must agree bit for bit). */
vmp_status vmp_test_division(const double* a, const double* b, int n, double* by_recip, double* by_div);

/* Test hook: lio::calcBodyCov (commons.cpp:18-45) of n points on the device
 * (host arrays; pts_out receives the points after the z == 0 fix). */
vmp_status vmp_test_body_cov(const double* pts, int n, double range_inc, double degree_inc, double* pts_out,
                             double* cov);

/* Test hook: point_crossmat * P_rr * point_crossmat^T (lio_builder.cpp:199-202,
 * 240-243) on the device for n points (pts n x 3) and matrices (M n x 9),
 * host arrays; out n x 9. */
vmp_status vmp_test_hat_sandwich(const double* pts, const double* M, int n, double* out);

/* The same leaf-centroid downsample for callers that cannot allocate device
 * memory (no counterpart in the reference): a real-time sensor thread that
 * must not call cudaMalloc/cudaFree, or a host framework whose own allocator
 * owns the GPU's memory.  d_in / d_out are device (or managed) buffers the
 * caller owns, each 16-byte aligned, and they must not overlap (d_out holds
 * up to n points; an in-place call is rejected); *n_out (host) receives the
 * output count.  Host pointers, misaligned or overlapping buffers give
 * VMP_ERR_INVALID_ARG before anything is launched.  The working memory is a
 * fixed 2 MiB __device__ array inside libvmp, held by every GPU that loads
 * the library until exit; at most 65536 input points (VMP_ERR_CAPACITY above
 * that).  The call allocates nothing.  Its first call on a device resolves
 * the array's device address and keeps it for the process, so
 * cudaDeviceReset while libvmp is loaded is not supported.  Calls share the array: calls that
 * overlap on the GPU race and must be serialised by the caller.  cuda_stream
 * may be NULL (default stream); the call returns after that stream
 * finished. */
vmp_status vmp_downsample_noalloc(const vmp_point* d_in, int n, double leaf, vmp_point* d_out, int* n_out,
                                  void* cuda_stream);

/* ---- batched plane fitting ----
 * VoxelGrid::updatePlane (src/map_builder/voxel_map.cpp:97-136) over all
 * points of many voxels at once, as VoxelMap::build fits every voxel after
 * adding its points (voxel_map.cpp:200-230): mean, point covariance
 * C = ppt / n - mean mean^T, ascending eigenvalues, plane test
 * evals[0] <= plane_thresh, and for a plane the normal (sign flipped so that
 * -mean . normal >= 0) and the 6x6 plane covariance sum_p J cov_p J^T with
 * J = [evecs F_p; I / n].  Voxels with fewer than update_point_thresh points
 * are not fitted (only mean and n are set), as updatePlane returns early.
 * A non-plane gets a zero normal and plane covariance (updatePlane returns
 * before forming them).
 * Arithmetic modes: */
enum {
    VMP_FIT_FP64 = 0,  /* the reference's FP64 arithmetic (parallel sums) */
    VMP_FIT_FP32 = 1,  /* plain FP32 throughout, world coordinates */
    VMP_FIT_FP32C = 2  /* FP32 with compensated covariance sums: coordinates
                          relative to the voxel's first point (a subtraction
                          of nearby floats, free of cancellation error) and
                          Kahan-compensated sums of the coordinates and
                          their products */
};
enum { VMP_FIT_FITTED = 1, VMP_FIT_PLANE = 2, VMP_FIT_FLIPPED = 4 };
typedef struct vmp_fit_params {
    int mode;                 /* VMP_FIT_* */
    int update_point_thresh;  /* fits voxels with n >= this (>= 1) */
    double plane_thresh;      /* plane test on the smallest eigenvalue */
} vmp_fit_params;
/* One fitted voxel (296 bytes). */
typedef struct vmp_fit_rec {
    double mean[3];
    double cov[6];        /* C, upper triangle: xx xy xz yy yz zz */
    double evals[3];      /* ascending */
    double norm[3];       /* plane normal after the sign flip (VMP_FIT_FLIPPED: it was negated) */
    double plane_cov[21]; /* 6x6 plane covariance, upper triangle row by row */
    int n;                /* points of the voxel */
    int flags;            /* VMP_FIT_FITTED | VMP_FIT_PLANE | VMP_FIT_FLIPPED */
} vmp_fit_rec;
/* Device-buffer form (allocation-free; cuda_stream may be NULL).  Points are
 * structure-of-arrays floats: xyz = 3 arrays of n_pts (x, then y, then z),
 * cov = 6 arrays of n_pts (xx xy xz yy yz zz of each point's covariance);
 * voxel v owns points offsets[v] .. offsets[v + 1] - 1 (offsets ascending,
 * offsets[0] = 0, offsets[n_vox] = n_pts).  out holds n_vox records.  The
 * call only enqueues work on cuda_stream. */
vmp_status vmp_fit_planes_device(const float* xyz, const float* cov, const long long* offsets, int n_vox,
                                 long long n_pts, const vmp_fit_params* params, vmp_fit_rec* out,
                                 void* cuda_stream);
/* Host-buffer form: copies in, fits, copies the records out and returns
 * after they arrived.  The copies of one quarter of the voxels overlap the fit
 * of the previous quarter; the device buffers are kept for the next call
 * (grown when a call needs more) and calls are serialised. */
vmp_status vmp_fit_planes(const float* xyz, const float* cov, const long long* offsets, int n_vox,
                          long long n_pts, const vmp_fit_params* params, vmp_fit_rec* out);
/* Measurement hook: while on, every fit call records CUDA events around its
 * kernel, waits for them and adds up its device time.  vmp_fit_profile
 * resets the totals. */
vmp_status vmp_fit_profile(int on);
vmp_status vmp_fit_profile_read(double* ms, long long* calls);

/* ---- measurement hooks (no reference counterpart) ----
 * Per-phase device time of vmp_process, from CUDA events recorded on the
 * stream's own CUDA stream.  Slot order: */
enum {
    VMP_PROF_UPLOAD = 0,        /* host->device copy of the scan and IMU samples */
    VMP_PROF_TIME_SORT = 1,     /* stable radix sort of the points by time */
    VMP_PROF_PREDICT = 2,       /* IMU predict chain (IESKF::predict per sample) */
    VMP_PROF_UNDISTORT = 3,     /* per-point motion compensation */
    VMP_PROF_DOWNSAMPLE = 4,    /* leaf-centroid downsample */
    VMP_PROF_BODY_COV = 5,      /* calcBodyCov per downsampled point */
    VMP_PROF_RESIDUAL = 6,      /* residual + H/b block reduction launches that ran an iteration */
    VMP_PROF_RESIDUAL_IDLE = 7, /* residual and step launches after convergence (return at once) */
    VMP_PROF_UPDATE_OTHER = 8,  /* P^-1 before, covariance update after the iterations */
    VMP_PROF_MAP_BATCH = 9,     /* float world transform + point covariances */
    VMP_PROF_MAP_GROUP = 10,    /* keys, hash insert, creation order, sort into voxel segments */
    VMP_PROF_MAP_STATE = 11,    /* per-voxel pushPoint state machine + plane refits */
    VMP_PROF_MAP_FINISH = 12,   /* merges, LRU queue, evictions */
    VMP_PROF_RESULT = 13,       /* result gather + device->host copy */
    VMP_PROF_RESIDUAL_STEP = 14, /* fold of the block partials + IEKF step of an iteration (one CTA) */
    VMP_PROF_SLOTS = 16
};
/* Enables (1) or disables (0) the profiler; either resets the totals. */
vmp_status vmp_profile_enable(vmp_stream_t s, int on);
/* Totals since enable: device ms, launches and points processed per slot
 * (arrays of VMP_PROF_SLOTS; any may be NULL). */
vmp_status vmp_profile_read(vmp_stream_t s, double* ms, long long* launches, long long* items);
/* The cudaStream_t the stream's kernels run on. */
void* vmp_cuda_stream(vmp_stream_t s);
/* Bytes the stream copied host->device and device->host so far. */
vmp_status vmp_io_bytes(vmp_stream_t s, long long* h2d, long long* d2h);
/* Kernel launches issued by the library so far (all streams). */
long long vmp_launch_count(void);
/* Merge resolution: 0 parallel fixed point (default), 1 single-thread replay
 * in point order; both exact.  vmp_last_merge_rounds waits for the stream and
 * returns the rounds of the last batch's fixed point (0 when the replay
 * produced the result). */
vmp_status vmp_set_merge_mode(vmp_stream_t s, int mode);
int vmp_last_merge_rounds(vmp_stream_t s);
/* merge() calls of the last map batch (the points that reached a frozen
 * plane voxel, voxel_map.cpp:70-73); waits for the stream. */
int vmp_last_merge_calls(vmp_stream_t s);
/* Phase times (us) of the last batch's merge fixed point: setup, then per
 * round the call tests and the merging calls, then the write-back; returns
 * how many were written (0: no fixed point ran).  Waits for the stream. */
int vmp_last_merge_profile(vmp_stream_t s, double* us, int max);
/* Test hooks: valid flags of the persistent residual records; the clouds of
 * the last scan (kind 0 undistorted time-sorted cloud, 1 downsampled). */
vmp_status vmp_residual_valid(vmp_stream_t s, unsigned char* valid, int n);
vmp_status vmp_last_cloud(vmp_stream_t s, int kind, vmp_point* out, int max, int* n_out);
/* Steady-state scans run as captured CUDA graphs (default 1): two graph
 * launches around the merge resolution instead of ~90 kernel launches.  The
 * direct launches (0; also used while profiling or when the batch may evict)
 * launch the same kernels with the same grids and give the same results. */
vmp_status vmp_set_graphs(vmp_stream_t s, int on);
/* Test hook: batches that the LRU eviction had to split (an evicted voxel
 * touched again later in the same batch). */
long long vmp_eviction_splits(vmp_stream_t s);
/* Test hook: the bounded wait of the merge resolution's grid barrier.  Two
 * CTAs meet at one barrier; with skip set the second never arrives, the
 * first gives up after spin_limit polls (a 64 ns sleep each), records the failure
 * and returns -- no fault, the context stays usable.  timed_out = 1 when the
 * wait ran out; ms = device time of the launch. */
vmp_status vmp_test_barrier_timeout(int skip, long long spin_limit, int* timed_out, double* ms);
/* Device memory a stream holds (all of it is allocated by vmp_create). */
long long vmp_device_bytes(vmp_stream_t s);
/* How vmp_process waits for its result: 0 (default) polls, lowest latency;
 * 1 the calling thread sleeps until the GPU is done, for many streams driven
 * by more threads than host cores (the server's workers use 1). */
vmp_status vmp_set_wait_mode(vmp_stream_t s, int blocking);

/* ------------------------------------------------------------------ serving
 * Many independent sensor streams on one GPU.  No reference counterpart: the
 * reference runs one LIOBuilder per ROS node (lio_node.cpp:263) and
 * processes its packages one at a time on the timer thread
 * (lio_node.cpp:167-182); a server runs many such streams at once.
 *
 * A server owns its streams (each a vmp_stream_t with its own map, filter
 * and CUDA stream).  vmp_server_open_stream admits a stream while the sum of
 * the admitted streams' device memory stays within the HBM budget and a slot
 * is free, else returns VMP_ERR_ADMISSION_DENIED; vmp_server_open_stream_wait
 * waits instead, admitting the stream as slots and memory free up.  vmp_submit copies a
 * package and returns at once.  Worker threads run each stream's packages in
 * submission order and many streams at once, each on its own CUDA stream,
 * so their kernels overlap on the GPU; a package submitted while others run
 * starts as soon as a worker and its stream are free (continuous batching,
 * not a queue drained batch by batch).  Results come back through vmp_poll.
 * A stream's results do not depend on what else runs: the same packages give
 * the same bits alone and in the mix.
 *
 * Threading: vmp_submit and vmp_poll may be called from any threads. */
typedef struct vmp_server_s* vmp_server_t;

typedef struct vmp_server_config {
    long long hbm_budget_bytes; /* admission limit on the streams' device memory (default 150e9) */
    int max_streams;            /* stream slots (default 64) */
    int workers;                /* host threads driving streams concurrently (default 32) */
    int queue_depth;            /* queued packages per stream before vmp_submit answers VMP_ERR_CAPACITY (default 64) */
    int autotune;               /* 1 (default): tune the launch shape of the served merge resolution online */
    int merge_grid_divisor;     /* served merge launches use SMs / divisor CTAs (0: 16); autotune's start */
    int seg_grid_blocks;        /* working blocks of the voxel-chain kernels while the server runs (0: 152, at most 304); autotune's start */
    int reserved[4];
} vmp_server_config;

typedef struct vmp_server_result {
    long long cookie;  /* as given to vmp_submit */
    int stream_id;
    int status;        /* vmp_status of the package */
    double submit_ms;  /* server clock (ms since vmp_server_create) at vmp_submit */
    double start_ms;   /* when a worker started the package */
    double end_ms;     /* when its result was on the host */
    vmp_result result;
} vmp_server_result;

void vmp_server_config_default(vmp_server_config* c);
/* The autotuner (config.autotune, servers with more than one worker): a
 * coordinate hill climb over three scheduling knobs on windows of 128
 * completed packages, starting after 24 windows (short runs keep the
 * starting shapes, the best measured ones) -- merge_grid_divisor (served
 * merge launches use SMs / d CTAs, d in 4..64; process-wide), max_inflight
 * (packages on the GPU at once: 8, 16, 24 or 32 of the workers) and
 * seg_grid_blocks (blocks of the voxel-chain kernels that take work: 76, 152
 * or 304, the launches' size under a server; process-wide, device-side, back
 * to all blocks when the last server is destroyed).  None changes results, and none needs the
 * streams' scan graphs captured again.  vmp_server_tuning: the merge divisor
 * in use, the windows measured so far and the best rate seen (packages/s);
 * vmp_server_knob: "merge_grid_divisor", "max_inflight", "seg_grid_blocks"
 * or "residual_ctas_per_sm" by name. */
vmp_status vmp_server_tuning(vmp_server_t sv, int* merge_grid_divisor, long long* windows, double* best_rate);
vmp_status vmp_server_knob(vmp_server_t sv, const char* name, int* value);
/* The residual kernel's register budget, by hand: 3 or 4 (default) resident
 * CTAs per SM (process-wide; VMP_RESIDUAL_CTAS_PER_SM gives the value at
 * load).  The
 * results are the same; the streams' scan graphs are captured again at their
 * next scan, which costs milliseconds per stream, so the online tuner leaves
 * this one alone. */
vmp_status vmp_set_residual_ctas_per_sm(int ctas);
/* Test hook: the autotuner's climb on a model instead of a GPU (no CUDA
 * call).  rates[(i * 4 + j) * 3 + k]: packages/s with merge divisor
 * candidate i (4, 8, 16, 32, 64), max_inflight candidate j (8, 16, 24, 32)
 * and seg_grid_blocks candidate k (76, 152, 304); trace (3 x windows ints):
 * the three knobs after each window. */
vmp_status vmp_test_autotune(int merge_divisor, int max_inflight, int seg_blocks, const double* rates, int windows,
                             int* trace);
vmp_status vmp_server_create(const vmp_server_config* c, vmp_server_t* out);
/* Waits for the packages that are running; queued ones are dropped;
 * admission requests still waiting return VMP_ERR_STATE. */
vmp_status vmp_server_destroy(vmp_server_t sv);
/* Admits a stream now or answers VMP_ERR_ADMISSION_DENIED (no free slot, or
 * its device memory would take the open streams past the HBM budget). */
vmp_status vmp_server_open_stream(vmp_server_t sv, const vmp_config* cfg, int* stream_id);
/* The same, waiting: the request queues behind earlier ones (arrival order)
 * until a slot is free and the stream fits the budget beside the open
 * streams -- both free up as vmp_server_close_stream retires streams, while
 * the other streams keep running -- or until timeout_ms passes
 * (VMP_ERR_TIMEOUT; timeout_ms < 0: no limit, 0: as vmp_server_open_stream).
 * A stream larger than the whole budget is denied at once.  The footprint of
 * a configuration is measured by creating the stream once; a creation that
 * runs out of device memory is retried after the next close. */
vmp_status vmp_server_open_stream_wait(vmp_server_t sv, const vmp_config* cfg, int timeout_ms, int* stream_id);
/* Waits until the stream's queued packages are done, then frees it. */
vmp_status vmp_server_close_stream(vmp_server_t sv, int stream_id);
vmp_status vmp_submit(vmp_server_t sv, int stream_id, const vmp_scan* scan, const vmp_imu* imus, int n_imu,
                      long long cookie);
/* The same with the package already in device memory (as vmp_process_device);
 * the buffers must stay valid until the package's result is polled. */
vmp_status vmp_submit_device(vmp_server_t sv, int stream_id, const vmp_point* d_pts, int n, double t_start,
                             double t_end, const vmp_imu* d_imus, int n_imu, long long cookie);
/* A raw Livox CustomMsg point array as the package (the node's lidarCB +
 * syncPackage + process, lio_node.cpp:121-148, 171): copied like vmp_submit;
 * the worker decodes it on the device (vmp_livox_decode: livox2pcl,
 * utils.cpp:3-28), takes the scan's end time as t_start + (last kept point's
 * time in ms) / 1000 (lio_node.cpp:146) and processes the decoded cloud
 * (vmp_process_decoded).  A message that keeps no point gives
 * VMP_ERR_INVALID_ARG in its result. */
vmp_status vmp_submit_livox(vmp_server_t sv, int stream_id, const vmp_livox_point* pts, int n, int filter_num,
                            double range_min, double range_max, double t_start, const vmp_imu* imus, int n_imu,
                            long long cookie);
/* Moves up to max finished results to out (completion order), waiting up to
 * timeout_ms for the first one; returns how many, or -1 on a bad argument. */
int vmp_poll(vmp_server_t sv, vmp_server_result* out, int max, int timeout_ms);
/* Waits until the stream is idle and returns its handle (map export, state
 * reads); the handle stays owned by the server. */
vmp_status vmp_server_stream(vmp_server_t sv, int stream_id, vmp_stream_t* out);
vmp_status vmp_server_info(vmp_server_t sv, long long* budget_used, int* streams_open, int* queued, int* running);
const char* vmp_server_last_error(vmp_server_t sv);

#ifdef __cplusplus
}
#endif

#endif /* VMP_H_ */
