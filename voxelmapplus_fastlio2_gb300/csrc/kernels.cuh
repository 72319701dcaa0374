// Kernel-side interfaces shared between the kernel translation units and the
// host orchestration (vmp_api.cu).
#pragma once
#include "common.cuh"
#include "prims.cuh"

namespace vmp {

// CTAs of the downsample's bounding-box pass (k_minmax_partial); the scratch
// behind DScan::blk_minmax holds kMinMaxBlocks * 6 + 8 floats.
constexpr int kMinMaxBlocks = 152;

// Per-scan device buffers of one stream.
// Per-scan scalars on the device (one host->device copy per scan), so that a
// captured graph of the scan needs no per-scan kernel parameters.
struct DScanHdr {
    int n_raw;
    int n_imu;
    double t_start;
    double t_end;
    int time_unsorted;  // 0 from the host; k_time_keys sets 1 if a point time decreases
    int pad;
};

struct DScan {
    DScanHdr* hdr;         // n_raw / n_imu / package times of the current scan
    // raw scan (input) and its time-sorted, undistorted copy
    float4* raw;           // [max_pts] x, y, z, t_ms
    float4* cloud;         // [max_pts] sorted by time, compensated in place
    float* raw_int;        // [max_pts] intensity of each raw point (0 unless decoded from Livox points)
    float* cloud_int;      // [max_pts] the same in time order
    int* d_n_in;           // [4] decode input count and scratch
    uint32_t* sort_k;      // [max_pts]
    uint32_t* sort_v;      // [max_pts]
    uint32_t* flags;       // [max_pts]
    uint32_t* scan_out;    // [max_pts]
    int* d_n_raw;          // device copy of the raw point count
    // downsample
    float4* down;          // [max_pts]
    int* d_n_down;
    float* minmax;         // [6] + per-block partials
    float* blk_minmax;     // [kMinMaxBlocks * 6 + 8]
    int* ds_params;        // [16] leaf grid parameters / overflow flag
    uint32_t* run_start;   // [max_pts + 1]
    // per downsampled point
    double* pl;            // [max_pts * 3] LiDAR-frame point (after the z == 0 fix)
    double* covl;          // [max_pts * 9] calcBodyCov
    // persistent residual records (residual_info): valid, normal, residual
    uint8_t* rvalid;       // [max_pts]
    double* rnorm;         // [max_pts * 3]
    double* rres;          // [max_pts]
    // map batch (world points + covariances handed to VoxelMap::build/update)
    double* bpts;          // [max_pts * 3]
    double* bcov;          // [max_pts * 9]
    int* d_n_batch;
    // IMU package
    vmp_imu* imus;         // [max_imu]
    DPose* poses;          // [max_imu + 2]
    DStep* steps;          // [max_imu + 2] per-step terms of the predict chain
    // reduction partials
    double* partials;      // [res_blocks * 160]
    unsigned int* done_ctr;
    int max_pts;
    int max_imu;
    int res_blocks;
};

// ---- k_filter.cu
void launch_imu_init(DFilter* f, const vmp_imu* imus, int n, const vmp_config& cfg, double t_end,
                     cudaStream_t st);
void launch_undistort(DFilter* f, DScan& s, int n_max, cudaStream_t st);
// ---- k_predict.cu
// The predict chain: launch_predict_state (the state chain, per-step F / G
// data and the pose cache), then launch_predict_cov (the covariance chain;
// only the residual kernel's gate and the map batch read P);
// launch_predict_chain2 launches both on one stream.
void launch_predict_state(DFilter* f, DScan& s, cudaStream_t st);
void launch_predict_cov(DFilter* f, DScan& s, cudaStream_t st);
void launch_predict_chain2(DFilter* f, DScan& s, cudaStream_t st);
void launch_ieskf_predict_once(DFilter* f, const double* acc, const double* gyro, double dt, cudaStream_t st);
void launch_update_begin(DFilter* f, cudaStream_t st);
// k_residual's shared-memory limit (once per process and device, before any capture).
cudaError_t residual_setup();
// k_residual's register budget (resident CTAs per SM: 3 or 4; same results).
void residual_set_ctas_per_sm(int c);
int residual_ctas_per_sm();
// Bumped whenever a launch shape that captured graphs hold changes.
long long launch_shape_epoch();
// One IEKF iteration: launch_iekf_boxminus (with do_step: x boxminus x_pred
// and its inverse Jacobian; it may run on another stream beside the points),
// launch_residual_points (sharedUpdateFunc over the points, block partials of
// H / b), then launch_residual_step (their fold and, with do_step, the filter
// step).  from_down: LiDAR points from the downsampled cloud (s.down), else
// from s.pl.
void launch_iekf_boxminus(DFilter* f, cudaStream_t st);
void launch_residual_points(DFilter* f, DScan& s, const DMap& m, int n_max, int estimate_ext, cudaStream_t st,
                            int from_down);
void launch_residual_step(DFilter* f, DScan& s, int n_max, int estimate_ext, double eps, cudaStream_t st,
                          int do_step);
void launch_residual_iter(DFilter* f, DScan& s, const DMap& m, int n_max, int estimate_ext, double eps,
                          cudaStream_t st, int do_step, int from_down);
void launch_update_end(DFilter* f, int estimate_ext, cudaStream_t st);

// ---- k_points.cu
void launch_time_sort(DScan& s, int n_max, SortScratch& ss, cudaStream_t st);
void launch_downsample(DScan& s, int n_max, double leaf, SortScratch& ss, ScanScratch& sc, cudaStream_t st);
// livox2pcl on the device: n Livox points at d_in -> s.raw / s.raw_int, count in *s.d_n_raw.
void launch_livox_decode(DScan& s, const vmp_livox_point* d_in, int n, int filter_num, double range_min,
                         double range_max, ScanScratch& sc, cudaStream_t st);
// lidarToBody (frame 0) / lidarToWorld (frame 1) of the first n points of s.cloud.
void launch_output_cloud(const DFilter* f, const DScan& s, int n, int frame, float4* out, float* out_int,
                         cudaStream_t st);
void launch_copy_down(DScan& s, int n_max, cudaStream_t st);
void launch_body_cov(DScan& s, int n_max, double range_inc, double sin_deg, cudaStream_t st);
// world points + covariances for the map: from the downsampled cloud (after
// update) or from the full undistorted cloud (map init)
void launch_map_batch(DFilter* f, DScan& s, int n_max, bool from_full_cloud, double range_inc, double sin_deg,
                      cudaStream_t st);

// ---- graph capture bookkeeping (k_sort.cu)
void set_capture_launch_counter(long long* c);

// ---- k_map.cu
struct MapScratch {
    uint32_t* slot;       // [max_batch] hash slot per point
    uint32_t* rec;        // [max_batch] record per point
    uint32_t* flag;       // [max_batch] creation flags (kept until the batch commits)
    uint32_t* rank;       // [max_batch] creation ranks
    uint32_t* flag2;      // [max_batch] general flags
    uint32_t* rank2;      // [max_batch] general scans
    uint32_t* sk;         // [max_batch] sort keys (record id)
    uint32_t* sv;         // [max_batch] sort values (point index)
    uint32_t* seg_start;  // [max_batch + 1]
    uint32_t* seg_end;    // [max_batch + 1]
    uint32_t* seg_rec;    // [max_batch]
    uint32_t* ev_rec;     // [max_batch] merge event record per point (kNoRec: none)
    uint32_t* ev_list;    // [max_batch] compacted event point indices (ascending)
    uint32_t* last_touch; // [max_batch] 1 if the point is its record's last touch
    uint32_t* victims;    // [max_batch]
    uint32_t* new_pos;    // [max_batch] point index of the j-th creation
    void* merge;          // MergeScratch (k_merge.cu)
    void* seg_snaps;      // [max_batch] refit snapshots (k_map.cu)
    void* covsegs;        // [max_batch] voxels with refits (k_map.cu)
    uint32_t* refit_list; // [max_batch]
    int* seg_cov;         // [max_batch] voxel-with-refits index of a segment
    uint32_t* term_snap;  // [term_cap] refit of each plane covariance term
    double* terms;        // [term_cap][21] plane covariance terms (upper triangles)
    int term_cap;
    int merge_mode;
    int merge_rounds;
    long long merge_d2h;  // bytes read back by the merge rounds (cumulative)
    int* d_n;             // batch size
    int* d_n_new;
    int* d_n_seg;
    int* d_n_ev;
    int* d_n_touch;
    int* d_scratch_int;   // [32]: batch counters; [5]-[7] refit / voxel / term list lengths, [8], [9] work counters
    int max_batch;
    SortScratch sort;
    ScanScratch scan;
};
cudaError_t map_scratch_alloc(MapScratch& ms, int max_batch, int rec_pool, int term_cap);
void map_scratch_free(MapScratch& ms);

// Applies VoxelMap::update (build = false) or VoxelMap::build (build = true)
// to batch points [0, *d_n) of bpts/bcov.
void launch_map_phase_a(DMap& m, MapScratch& ms, const double* bpts, int n_max, cudaStream_t st);
void launch_map_segments(DMap& m, MapScratch& ms, int n_max, cudaStream_t st);
void launch_map_walk(DMap& m, MapScratch& ms, cudaStream_t st);
void launch_map_rollback(DMap& m, MapScratch& ms, int n_max, cudaStream_t st);
void launch_map_phase_b(DMap& m, MapScratch& ms, const double* bpts, const double* bcov, int n_max, bool build,
                        cudaStream_t st);
void launch_map_state(DMap& m, MapScratch& ms, const double* bpts, const double* bcov, int n_max, bool build,
                      cudaStream_t st);
void launch_map_finish(DMap& m, MapScratch& ms, int n_max, bool build, cudaStream_t st);
void launch_map_finish_pre(DMap& m, MapScratch& ms, int n_max, bool build, cudaStream_t st);
void launch_map_finish_post(DMap& m, MapScratch& ms, int n_max, cudaStream_t st);
void launch_rehash(DMap& m, cudaStream_t st);
void launch_queue_compact(DMap& m, uint32_t* flag, uint32_t* rank, uint32_t* tr, uint64_t* ts, int* d_len,
                          int* d_live, int len_max, ScanScratch& sc, cudaStream_t st);
void launch_map_index(const DMap& m, const double* pts, int n, int64_t* keys, cudaStream_t st);
void launch_map_reset(DMap& m, cudaStream_t st);

// ---- k_merge.cu
cudaError_t merge_scratch_alloc(void** out, int max_batch, int rec_pool);
void merge_scratch_free(void* p);
// mode 0: parallel fixed point (sequential replay as fallback); 1: replay only
cudaError_t run_merge_events(DMap& m, MapScratch& ms, void* scratch, int n_max, int mode, int* rounds_out,
                             cudaStream_t st);
int merge_rounds_read(void* scratch, cudaStream_t st);
int merge_profile_read(void* scratch, cudaStream_t st, double* us, int max);
// While at least one multi-worker server exists (on: one more, off: one
// fewer), cooperative merge launches use 1/16 of the SMs and run several at
// once instead of one at a time on all SMs.
void merge_set_throughput_mode(bool on);
bool merge_throughput_mode();
// working blocks of the voxel-chain kernels (0: all); process-wide, device-side
cudaError_t seg_set_grid_blocks(int blocks);
int seg_grid_blocks();
// While that is set (a server runs) the voxel-chain launches have at most this
// many blocks: the largest working-block count the serving tuner picks.
constexpr int kSegServedBlocks = 304;
// Grid of an element-wise (grid-stride) kernel while a server runs: at most
// one block per SM.  A stream's grids are sized for its largest scan, and most
// of those blocks would find no element of a served scan; the results do not
// depend on the grid.  (On the 64-stream mix: 6455 / 6545 / 6597 scans/s with
// at most 608 / 304 / 152 blocks.)
inline int served_grid(int g) { return (g > 152 && seg_grid_blocks() > 0) ? 152 : g; }
// Served merge launches use SMs / d CTAs (process-wide; 16 by default).
void merge_set_grid_divisor(int d);
// Writes the reciprocal table of the voxel state machine on the current
// device (once per device; before any stream of the device runs a map batch).
cudaError_t map_recip_table_init();

}  // namespace vmp
