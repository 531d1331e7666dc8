/*
 * tdm.h -- C ABI of the GB300-native 3DMatch registration hot path.
 *
 * Every entry point returns a tdm_status, never exits and never traps.  Device
 * pointers are caller-owned unless a handle says otherwise; every call is
 * stream-ordered on the tdm_stream it is given (a cudaStream_t; NULL is the
 * legacy default stream).  Calls that must return host-visible sizes say so.
 *
 * Each group cites the reference interface it replaces (andyzeng/3dmatch-toolbox
 * paths).
 */
#ifndef TDM_H
#define TDM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* tdm_stream; /* == cudaStream_t */

typedef enum tdm_status {
  TDM_OK = 0,
  TDM_ERR_INVALID_ARG = 1,
  TDM_ERR_IO = 2,
  TDM_ERR_FORMAT = 3,
  TDM_ERR_OOM = 4,
  TDM_ERR_DEVICE = 5,
  TDM_ERR_TIMEOUT = 6,
  TDM_ERR_CANCELLED = 7,
  TDM_ERR_UNSUPPORTED = 8
} tdm_status;

typedef enum tdm_precision {
  TDM_FP32 = 0, /* CUDA-core FP32: the drop-in form */
  TDM_BF16 = 1, /* tcgen05 BF16 operands, FP32 accumulation */
  TDM_FP8 = 2   /* conv3..conv8 in FP8 E4M3 with per-channel weight scales; conv1/2 + feat BF16 */
} tdm_precision;

/* Voxel grid geometry of core/demo.cu:97-124: dims (x,y,z), origin of voxel
 * (0,0,0), voxel size and truncation margin.  Voxel (x,y,z) is stored at
 * z*dim[1]*dim[0] + y*dim[0] + x. */
typedef struct tdm_grid {
  int32_t dim[3];
  float origin[3];
  float voxel_size;
  float trunc_margin;
} tdm_grid;

/* TDF index-decode modes (core/demo.cu:32-34 decodes the linear voxel index
 * in float32, which is wrong above 2^24 voxels). */
#define TDM_TDF_EXACT 0          /* exact integer decode (default) */
#define TDM_TDF_REFCOMPAT_FLOAT 1 /* reference float32 decode, no contraction */
#define TDM_TDF_REFCOMPAT_FMA 2  /* reference float32 decode with nvcc fmad contraction */

/* ---- library ------------------------------------------------------------ */
const char* tdm_version(void);
/* Message of the last failing call on this host thread. */
const char* tdm_last_error(void);
/* Reads and clears the device-side error word (a bounded wait that ran out,
 * an index that failed a check).  TDM_OK when clean; synchronizes `s`. */
tdm_status tdm_device_status(tdm_stream s);
/* Number of kernels this library has launched in this process (diagnostics;
 * the reference has no counterpart). */
int64_t tdm_launch_count(void);
/* Self-test of the failure path (no reference counterpart; the reference's
 * FatalError exits the process, core/marvin.hpp:132-138).  Launches one small
 * kernel that makes the bounded mbarrier wait of the tcgen05 kernels run out
 * after budget_us (1 .. 1,000,000): it allocates tensor memory, completes one
 * bulk copy, waits on a barrier nothing arrives on, gives up, raises the
 * device error word, frees its tensor memory and returns.  out_dev: 3 int32
 * {copy landed, wait ran out, first copied word (0x5E1F7E57)}.  The next
 * tdm_device_status reports TDM_ERR_TIMEOUT and clears the word; the context
 * stays usable. */
tdm_status tdm_selftest_wait_timeout(uint32_t budget_us, int32_t* out_dev, tdm_stream s);

/* ---- grid + TDF: replaces core/demo.cu:97-158 (ComputeTDF) ---------------- */
/* Grid of core/demo.cu:97-124 from host points (float ops as the reference).
 * Point clouds are expected to be finite.  A NaN coordinate is skipped by the
 * bounds (fminf/fmaxf from +/-inf, as the device form), and a point with any
 * non-finite coordinate is skipped by the occupancy scatter, so the host and
 * device forms give the same grid for any input; an infinite bound is
 * TDM_ERR_INVALID_ARG. */
tdm_status tdm_grid_from_points_host(const float* pts_host, int32_t n, float voxel_size, float trunc_margin,
                                     int32_t pad, tdm_grid* grid_out);
/* Same from device points: min/max reduced on the device, then read back
 * (synchronizes `s`).  ws_dev: tdm_grid_workspace_bytes() bytes. */
size_t tdm_grid_workspace_bytes(void);
tdm_status tdm_grid_from_points(const float* pts_dev, int32_t n, float voxel_size, float trunc_margin, int32_t pad,
                                tdm_grid* grid_out, void* ws_dev, tdm_stream s);
/* TDF of core/demo.cu:22-57 over the whole grid: occupancy scatter of the
 * points, exact windowed squared distance, 1 - d/trunc.  tdf_dev: V floats.
 * ws_dev: tdm_tdf_workspace_bytes(grid) bytes: occupancy, then the in-plane
 * squared distances, one byte per voxel each with x rows padded to 4. */
size_t tdm_tdf_workspace_bytes(const tdm_grid* grid);
/* Exact TDF of evaluation/model-fitting-apc/pointCloud2TDF.m (and
 * deprecated/pointCloud2AccTDF.m): 1 - min(d / trunc_margin, 1) with d the
 * distance from the voxel centre origin + i * voxel_size to the nearest point
 * (float arithmetic; within 1e-6 of the double-precision distance).  No
 * workspace; trunc_margin <= 32 voxels. */
tdm_status tdm_tdf_exact(const float* pts_dev, int32_t n, const tdm_grid* grid, float* tdf_dev, tdm_stream s);
tdm_status tdm_tdf(const float* pts_dev, int32_t n, const tdm_grid* grid, int32_t decode_mode, float* tdf_dev,
                   void* ws_dev, size_t ws_bytes, tdm_stream s);

/* ---- keypoints: replaces core/demo.cu:164-177 ----------------------------- */
/* idx_i = floor(u_i * n_pts), u_i from splitmix64(seed, i) (the reference's
 * random_device stream cannot be replayed, core/utils.hpp:15-20). */
tdm_status tdm_keypoint_indices(uint64_t seed, int32_t n_pts, int32_t k, int32_t* idx_dev, tdm_stream s);
/* keypts = pts[idx]; kp_grid = round((p - origin)/voxel_size) (int32 x,y,z). */
tdm_status tdm_keypoints(const float* pts_dev, int32_t n_pts, const int32_t* idx_dev, int32_t k,
                         const tdm_grid* grid, float* keypts_dev, int32_t* kp_grid_dev, tdm_stream s);

/* ---- patch gather: replaces core/demo.cu:195-218 -------------------------- */
/* patches[k][z][y][x] (30^3, x fastest) = tdf at kp_grid + (x,y,z) - 15; voxels
 * outside the grid read 0. */
tdm_status tdm_gather(const float* tdf_dev, const tdm_grid* grid, const int32_t* kp_grid_dev, int32_t k,
                      float* patches_dev, tdm_stream s);

/* ---- 3D ConvNet: replaces marvin::Net (core/demo.cu:179-231, core/marvin.hpp:
 * 7434 init, 7596-7615 loadWeights, 7632 Malloc, 7653 forward) -------------- */
typedef struct tdm_net tdm_net;
/* Weights by Marvin name ("conv1.weight" [64,1,3,3,3] ... "feat.bias") from a
 * .marvin file (core/marvin.hpp:2581-2612; half/float/double records).
 * use_feat = 0 drops the final 1x1x1 `feat` layer (8-layer form). */
tdm_status tdm_net_create(const char* marvin_path, tdm_precision precision, int32_t use_feat, tdm_net** out);
/* Same from host arrays: weights[l] is [K][C][ks^3] float, biases[l] is [K]. */
tdm_status tdm_net_create_from_host(const float* const* weights, const float* const* biases, tdm_precision precision,
                                    int32_t use_feat, tdm_net** out);
/* patches_dev: b x 27000 float (z,y,x);  desc_dev: b x 512 float. */
tdm_status tdm_net_forward(tdm_net* net, const float* patches_dev, int32_t b, float* desc_dev, tdm_stream s);
/* Net::getResponse(name) (core/marvin.hpp, used at core/demo.cu:185-186): runs
 * the forward up to the named response ("conv1".."conv8", "pool1", "feat") and
 * writes it as float, channels-last [b][D][D][D][C] (Marvin keeps NCDHW). */
tdm_status tdm_net_response(tdm_net* net, const char* name, const float* patches_dev, int32_t b, float* out_dev,
                            tdm_stream s);
/* FP8 form only (no-op otherwise): sets the per-tensor E4M3 activation scales
 * of conv3..conv8's inputs from the largest activations of b calibration
 * patches in the BF16 form (scale = max / 448).  Required before the first
 * FP8 forward.  tdm_net_act_scales returns the 9 scales (index = layer). */
tdm_status tdm_net_calibrate(tdm_net* net, const float* patches_dev, int32_t b, tdm_stream s);
tdm_status tdm_net_act_scales(tdm_net* net, float* scales);
/* A second net with the same weights, precision and FP8 scales (one per
 * concurrent stream: a net's activation workspace serves one call at a time). */
tdm_status tdm_net_clone(const tdm_net* src, tdm_net** out);
/* Device bytes of the activation workspace a forward of b patches allocates. */
size_t tdm_net_workspace_bytes(const tdm_net* net, int32_t b);
/* Patches per internal chunk (bounds the activation workspace; default 2048). */
tdm_status tdm_net_set_max_batch(tdm_net* net, int32_t max_batch);
/* Per-layer device time, the analogue of Marvin's debug_mode tic/toc
 * (core/marvin.hpp:445-456, 7656-7681): when enabled, every layer launch is
 * bracketed by CUDA events on its stream.  tdm_net_layer_times synchronizes and
 * returns accumulated milliseconds and launch counts for 10 slots (0..8 =
 * conv1..conv8, feat; 9 = pool1); reset != 0 clears the totals. */
tdm_status tdm_net_set_timing(tdm_net* net, int32_t enable);
tdm_status tdm_net_layer_times(tdm_net* net, double* ms, int64_t* launches, int32_t reset);
/* Tile autotuner (no reference counterpart: cuDNN picks its own algorithm,
 * core/marvin.hpp:4470).  For the BF16/FP8 forms, times every (N tile,
 * M sub-tiles) shape each tcgen05 layer can run on a forward of b patches
 * (reps timed forwards per shape, per-layer CUDA events) and keeps the
 * fastest per layer.  The accumulation order does not depend on the tile, so
 * the descriptors are the same bits before and after.  No-op for FP32. */
tdm_status tdm_net_autotune(tdm_net* net, const float* patches_dev, int32_t b, int32_t reps, tdm_stream s);
/* Current tile per layer (0..8 = conv1..feat; 0 for the FP32 form). */
tdm_status tdm_net_tiles(const tdm_net* net, int32_t nt[9], int32_t msub[9]);
/* Sets one layer's tile by hand (nt in {64,128,256} dividing the layer's
 * outputs, msub M sub-tiles of 128 rows, 2*msub*nt <= 512 TMEM columns in the
 * grid form), keeping the layer's kernel form when it has that tile. */
tdm_status tdm_net_set_tile(tdm_net* net, int32_t layer, int32_t nt, int32_t msub);
/* Kernel form of a tensor-core layer.  GRID: implicit GEMM over every input
 * position (rows with x, y or z >= Do computed and dropped); DXF: conv2's
 * dx-fused form; GATHER: GEMM over the valid output positions only, each
 * tap's A rows gathered into shared memory (3x3x3 convs conv3..conv7; tiles
 * (256,2), (256,1), (128,2)); XRUN: gathered (b, z, y) rows with whole input
 * x runs, one staged operand shared by the three dx taps (same layers and
 * tiles); GATHER_WT / XRUN_WT: the same with the weights as the MMA's A
 * operand (M = 128 output channels, N = 256 rows; conv3 and conv4, tile
 * (128,2)); DXF_PAIR: conv2's dx-fused form on a pair of CTAs sharing each
 * MMA (M = 256 rows, N = 192: the dx taps of all 64 channels; tile (32,2)).
 * All forms give the same bits. */
typedef enum {
  TDM_CONV_GRID = 0,
  TDM_CONV_DXF = 1,
  TDM_CONV_GATHER = 2,
  TDM_CONV_XRUN = 3,
  TDM_CONV_GATHER_WT = 4,
  TDM_CONV_XRUN_WT = 5,
  TDM_CONV_DXF_PAIR = 6
} tdm_conv_form;
tdm_status tdm_net_tile_forms(const tdm_net* net, int32_t form[9]);
/* Sets tile and form (-1: the current form if it has the tile, else any). */
tdm_status tdm_net_set_tile_form(tdm_net* net, int32_t layer, int32_t nt, int32_t msub, int32_t form);
tdm_status tdm_net_destroy(tdm_net* net);
/* Seeded He-normal weights (N(0, 2/fan_in)), uniform biases in [-0.05, 0.05],
 * written as float32 .marvin records. */
tdm_status tdm_write_seeded_weights(const char* marvin_path, uint64_t seed);

/* ---- mutual nearest neighbours: replaces core/demo.m:51-57 ---------------- */
/* nn_ab[i] = argmin_j |a_i - b_j|, nn_ba likewise; pairs (nn_ba[j], j) for every
 * j with nn_ab[nn_ba[j]] == j, in increasing j.  FP32: exact FP64 refinement of
 * the FP32 candidates (indices equal the exact double-precision NN); BF16:
 * tcgen05 distance GEMM, its 4 best candidates per query re-scored in FP64.
 * da_dev/db_dev 16-byte aligned, dim a multiple of 64.
 * pairs_dev: 2*min(na,nb) int32; n_pairs_dev: 1 int32. */
size_t tdm_mnn_workspace_bytes(int32_t na, int32_t nb, int32_t dim);
tdm_status tdm_match_mnn(const float* da_dev, int32_t na, const float* db_dev, int32_t nb, int32_t dim,
                         tdm_precision precision, int32_t* nn_ab_dev, int32_t* nn_ba_dev, int32_t* pairs_dev,
                         int32_t* n_pairs_dev, void* ws_dev, size_t ws_bytes, tdm_stream s);

/* ---- RANSAC + rigid refit: replaces core/external/sfm/ransacfitRt.m:20-38,
 * core/external/peter/ransac.m:113-232, estimateRt.m ------------------------ */
typedef struct tdm_ransac_params {
  uint64_t seed;      /* sample stream: splitmix64(seed, 3h+j) */
  int32_t iterations; /* trials scored */
  float threshold;    /* inlier if |x - (R y + t)| < threshold (strict) */
  int32_t adaptive;   /* 1: replay ransac.m's adaptive stop (p=0.99) over the trials */
  int32_t max_trials; /* adaptive cap (ransac.m default 50000) */
} tdm_ransac_params;
/* x = R y + t.  x_dev / y_dev: m_max x 3 float; the live count m is read from
 * m_dev (device int32) so the call needs no host round trip.  rt_dev: 12
 * doubles (3x4 row-major, FP64 Kabsch refit on the winner's inliers);
 * inliers_dev: m_max int32; info_dev: 4 int32 = {n_inliers, best_trial,
 * best_count, trials_run}.  Workspace: the best-trial word, then per trial its
 * inlier count and FP32 model. */
size_t tdm_ransac_workspace_bytes(int32_t m_max, int32_t iterations);
tdm_status tdm_ransac(const float* x_dev, const float* y_dev, const int32_t* m_dev, int32_t m_max,
                      const tdm_ransac_params* params, double* rt_dev, int32_t* inliers_dev, int32_t* info_dev,
                      void* ws_dev, size_t ws_bytes, tdm_stream s);
/* tdm_ransac without a caller workspace: no counterpart in the reference (its
 * RANSAC is MATLAB).  For callers that cannot allocate device memory -- a
 * foreign-function binding holding no device allocator, or a serving loop that
 * forbids cudaMalloc after start-up -- the per-trial scratch lives in a fixed
 * device array inside the library (about 6.8 MB per GPU that loads it, kept
 * until the process exits).  Limit: params->iterations <= 131072 trials;
 * larger values return TDM_ERR_INVALID_ARG.  The call allocates nothing.  Its
 * first call on a device looks up the array's device address, so make that
 * first call before any stream capture.  Every call shares the array (each
 * call clears what must start at zero), so calls whose work overlaps on the
 * GPU race and must be serialized by the caller.  Outputs as tdm_ransac. */
tdm_status tdm_ransac_noalloc(const float* x_dev, const float* y_dev, const int32_t* m_dev, int32_t m_max,
                              const tdm_ransac_params* params, double* rt_dev, int32_t* inliers_dev,
                              int32_t* info_dev, tdm_stream s);
/* x[i] = kp_a[pairs[2i]], y[i] = kp_b[pairs[2i+1]] for i < *n_pairs_dev. */
tdm_status tdm_pairs_to_points(const float* kp_a_dev, const float* kp_b_dev, const int32_t* pairs_dev,
                               const int32_t* n_pairs_dev, int32_t max_pairs, float* x_dev, float* y_dev,
                               tdm_stream s);

/* ---- surface overlap of a registered pair: replaces the 1-NN overlap of
 * core/demo.m:66-72 and evaluation/geometric-registration/register2Fragments.m:90-97
 * (multiQueryKNNSearchImpl + sum(dists < 0.05)) ------------------------------ */
/* counts_dev[0] = points of a with a point of Rt*b closer than radius,
 * counts_dev[1] = points of Rt*b with a point of a closer than radius
 * (ratioAligned = counts / sizes).  rt_host: row-major 3x4 double (x_a = R x_b
 * + t), applied in float.  Clouds of 1 .. 524288 points whose coordinates stay
 * within 65536 * 1.05 * radius of the origin (3.4 km at 5 cm).  Exact float
 * distances (d2 < r*r); synchronizes the stream. */
size_t tdm_overlap_workspace_bytes(int32_t na, int32_t nb);
tdm_status tdm_overlap(const float* a_dev, int32_t na, const float* b_dev, int32_t nb, const double rt_host[12],
                       float radius, int32_t* counts_dev, void* ws_dev, size_t ws_bytes, tdm_stream s);

/* ---- ICP refinement: the step register2Fragments.m:70-78 leaves commented
 * out (pcregrigid on 1 cm grid-averaged clouds, inlier ratio 0.3, tolerance
 * [1e-4 m, 9e-5 deg], 50 iterations) ---------------------------------------- */
typedef struct tdm_icp_params {
  float grid;              /* grid-average cell, 0.01 */
  float max_dist;          /* nearest-neighbour search radius, 0.10 */
  float inlier_ratio;      /* closest fraction of the pairs kept, 0.30 */
  int32_t max_iterations;  /* 50 */
  float tol_translation;   /* 1e-4 (m) */
  float tol_rotation_deg;  /* 9e-5 (degrees) */
} tdm_icp_params;
typedef struct tdm_icp_result {
  double rt[12];           /* row-major 3x4, x_fixed = R x_moving + t */
  int32_t iterations;
  int32_t correspondences; /* pairs in the last fit */
  float rmse;              /* of those pairs before the last update (m) */
  int32_t converged;       /* 1 when the tolerances stopped it */
} tdm_icp_result;
/* Point-to-point ICP from init_rt (moving -> fixed).  Deterministic: exact
 * integer Kabsch sums, ties broken by coordinates.  Clouds of 1 .. 524288
 * points; synchronizes the stream once per iteration. */
size_t tdm_icp_workspace_bytes(int32_t n_fixed, int32_t n_moving);
tdm_status tdm_icp(const float* fixed_dev, int32_t n_fixed, const float* moving_dev, int32_t n_moving,
                   const double init_rt_host[12], const tdm_icp_params* params, tdm_icp_result* result, void* ws_dev,
                   size_t ws_bytes, tdm_stream s);

/* ---- TSDF fusion: replaces depth-fusion/demo.cu:18-68 (Integrate) and
 * core/utils.hpp:23-65 (SaveVoxelGrid2SurfacePointCloud) -------------------- */
/* tsdf = 1, weight = 0 (depth-fusion/demo.cu:131-135). */
tdm_status tdm_tsdf_init(float* tsdf_dev, float* weight_dev, const int32_t dim[3], tdm_stream s);
/* uint16 millimetres -> metres, > 6 m -> 0 (depth-fusion/utils.hpp ReadDepth). */
tdm_status tdm_depth_from_mm(const uint16_t* mm_dev, int64_t n, float* depth_dev, tdm_stream s);
/* Integrates n_frames depth maps (n_frames x height x width float metres) in
 * order; cam2base_host: n_frames row-major 4x4 float; K: 3x3 row-major. */
tdm_status tdm_tsdf_integrate(float* tsdf_dev, float* weight_dev, const int32_t dim[3], const float origin[3],
                              float voxel_size, float trunc_margin, const float* depth_dev, int32_t n_frames,
                              int32_t height, int32_t width, const float K[9], const float* cam2base_host,
                              tdm_stream s);
/* Voxel centres with |tsdf| < tsdf_thr and weight > w_thr, in linear index
 * order; writes at most max_pts points, *n_pts_dev = total count. */
size_t tdm_extract_workspace_bytes(const int32_t dim[3]);
tdm_status tdm_tsdf_extract(const float* tsdf_dev, const float* weight_dev, const int32_t dim[3],
                            const float origin[3], float voxel_size, float tsdf_thr, float w_thr, float* pts_dev,
                            int64_t max_pts, int64_t* n_pts_dev, void* ws_dev, size_t ws_bytes, tdm_stream s);

/* ---- whole path: core/demo.cu main + core/demo.m matching/registration ---- */
typedef struct tdm_pipeline tdm_pipeline;
typedef struct tdm_pipeline_config {
  float voxel_size;      /* 0.01 */
  float trunc_voxels;    /* 5 */
  int32_t pad;           /* 15 */
  int32_t max_points;    /* per fragment */
  int32_t max_keypoints; /* per fragment */
  int64_t max_voxels;    /* per fragment grid */
  tdm_precision match_precision;
  tdm_ransac_params ransac;
} tdm_pipeline_config;
typedef struct tdm_pair_result {
  double rt[16];     /* 4x4, x_a = Rt * x_b */
  int32_t n_matches; /* mutual-NN pairs */
  int32_t n_inliers;
  int32_t best_trial;
  int32_t keypoints[2];
  int32_t grid_dim[2][3];
} tdm_pair_result;
tdm_status tdm_pipeline_create(const tdm_pipeline_config* cfg, tdm_net* net, tdm_pipeline** out);
tdm_status tdm_pipeline_destroy(tdm_pipeline* p);
/* demo.cu for one fragment with device-resident points: grid, TDF, keypoints,
 * gather, net.  keypts_dev: k x 3, desc_dev: k x 512 (caller-owned). */
tdm_status tdm_describe_fragment(tdm_pipeline* p, const float* pts_dev, int32_t n, uint64_t kp_seed, int32_t k,
                                 float* keypts_dev, float* desc_dev, tdm_grid* grid_out, tdm_stream s);
/* Whole pair with device-resident points; result copied to host on return. */
tdm_status tdm_register_pair(tdm_pipeline* p, const float* pts_a_dev, int32_t na, const float* pts_b_dev,
                             int32_t nb, uint64_t seed, int32_t k, tdm_pair_result* result, tdm_stream s);
/* Whole pair from host points (host->device copies inside the call). */
tdm_status tdm_register_pair_host(tdm_pipeline* p, const float* pts_a_host, int32_t na, const float* pts_b_host,
                                  int32_t nb, uint64_t seed, int32_t k, tdm_pair_result* result, tdm_stream s);

/* ---- batched description of many fragments (core/demo.cu main, run over a
 * set of fragments at once; the reference runs demo once per fragment,
 * evaluation/geometric-registration/getKeyptsAndDesc.m:43) -----------------
 * Fragments of uneven point and keypoint counts and voxel sizes go through
 * one persistent launch per stage: grids are planned on the device from each
 * fragment's bounds (the same arithmetic as tdm_grid_from_points), and the
 * occupancy, TDF, keypoint and gather kernels walk a device fragment table;
 * the net runs over all patches in chunks.  With use_graph the sequence is
 * captured as a CUDA graph on the first call for a given (points, keypoint
 * and descriptor pointers, fragment count, total keypoints) and replayed
 * afterwards; point counts, voxel sizes and seeds may change between
 * replays.  Results equal tdm_describe_fragment's fragment by fragment. */
typedef struct tdm_batch tdm_batch;
typedef struct tdm_batch_config {
  int32_t max_fragments; /* <= 1024 */
  int64_t max_points;    /* over the batch */
  int64_t max_keypoints; /* over the batch */
  int64_t max_voxels;    /* over the batch (each grid with its x rows padded to a
                          * multiple of 4, then rounded up to 256) */
  float trunc_voxels;    /* truncation in voxels (5) for every fragment */
  int32_t pad;           /* 15 */
  int32_t use_graph;
} tdm_batch_config;
tdm_status tdm_batch_create(const tdm_batch_config* cfg, tdm_net* net, tdm_batch** out);
tdm_status tdm_batch_destroy(tdm_batch* b);
/* Device bytes the batch holds (arenas, table, patch chunk; the net's own
 * workspace not included). */
size_t tdm_batch_device_bytes(const tdm_batch* b);
/* pts_dev: all fragments' points back to back (x,y,z float); host arrays:
 * point_offsets[n_fragments + 1] (fragment f = points [off[f], off[f+1])),
 * voxel_size[f], keypoints[f], seeds[f] (keypoint stream of fragment f, as
 * tdm_keypoint_indices).  keypts_dev: sum(keypoints) x 3 float and desc_dev:
 * sum(keypoints) x 512 float, fragment after fragment.  grids (host,
 * n_fragments) receives each fragment's grid; may be NULL.  Returns after
 * the stream has finished the batch. */
tdm_status tdm_describe_batch(tdm_batch* b, const float* pts_dev, int32_t n_fragments, const int64_t* point_offsets,
                              const float* voxel_size, const int32_t* keypoints, const uint64_t* seeds,
                              float* keypts_dev, float* desc_dev, tdm_grid* grids, tdm_stream s);
/* Kernel launches one call issues (counted on its first, uncaptured run) and
 * whether the last call replayed a captured graph. */
tdm_status tdm_batch_stats(const tdm_batch* b, int64_t* launches_per_call, int32_t* replayed);

/* ---- fragment store: describe once, register many pairs.  The reference
 * describes every fragment of a scene once (demo per fragment,
 * evaluation/geometric-registration/getKeyptsAndDesc.m:34-43, keypts.bin and
 * desc.3dmatch.bin on disk) and registers every pair from those files
 * (runFragmentRegistration.m:27-53 -> register2Fragments.m:18-59).  Here the
 * files are entries of a device arena of a fixed budget, keyed by a caller-
 * chosen 64-bit fragment key (below 2^63); least recently used entries are
 * evicted when a new one does not fit.  A key names one description
 * (points, keypoint seed, keypoint count): describing it again with another
 * seed or count replaces the entry.  Calls on one store may come from
 * several threads; the same key must not be written by two calls at once. --- */
typedef struct tdm_store tdm_store;
typedef struct tdm_store_stats {
  int64_t entries, bytes_used, capacity; /* bytes of the arena */
  int64_t hits, misses, evictions;       /* tdm_store_describe hits / misses */
} tdm_store_stats;
/* One device arena of budget_bytes (each entry takes k x 2,060 bytes, rounded
 * to 256-byte blocks). */
tdm_status tdm_store_create(int64_t budget_bytes, tdm_store** out);
tdm_status tdm_store_destroy(tdm_store* st);
/* tdm_describe_fragment into the store under `key`, unless the key is stored
 * already with this keypoint seed and count (*hit = 1, nothing runs). */
tdm_status tdm_store_describe(tdm_store* st, tdm_pipeline* p, uint64_t key, const float* pts_dev, int32_t n,
                              uint64_t kp_seed, int32_t k, int32_t* hit, tdm_stream s);
/* Copies keypoints (k x 3) and descriptors (k x 512) described elsewhere
 * (e.g. by tdm_describe_batch) into the store under `key`. */
tdm_status tdm_store_put(tdm_store* st, uint64_t key, uint64_t kp_seed, const float* keypts_dev,
                         const float* desc_dev, int32_t k, const tdm_grid* grid, tdm_stream s);
/* Device pointers of a stored fragment, valid until a later call adds to
 * the store (which may evict it) or removes it. */
tdm_status tdm_store_get(tdm_store* st, uint64_t key, const float** keypts_dev, const float** desc_dev, int32_t* k,
                         tdm_grid* grid);
tdm_status tdm_store_remove(tdm_store* st, uint64_t key);
tdm_status tdm_store_get_stats(tdm_store* st, tdm_store_stats* out);
/* core/demo.m:49-64 on two stored fragments: mutual NN of their descriptors,
 * RANSAC on the matched keypoints, refit (the pipeline's match precision and
 * RANSAC parameters; fragments of up to its max_keypoints).  Equals
 * tdm_register_pair when the fragments were described with `seed` and
 * `seed + 1`.  The stream waits for the entries' writers; returns after the
 * result is on the host. */
tdm_status tdm_register_stored(tdm_pipeline* p, tdm_store* st, uint64_t key_a, uint64_t key_b, tdm_pair_result* r,
                               tdm_stream s);

/* ---- serving: pair-registration requests of different sizes as they arrive
 * (the reference registers pairs one by one through files and MATLAB,
 * evaluation/geometric-registration/register2Fragments.m) ----------------------
 * Continuous batching: queued requests are taken in arrival order into waves
 * while they fit the server's device capacity (each request's own points,
 * grid voxels -- from its bounding box -- and keypoints); the fragments of a
 * wave that are not in the server's store are described together by one
 * tdm_describe_batch call (patches of different requests share the net's
 * launches), and a second thread registers the wave's pairs from the store on
 * its own stream while the next wave is described.  Keyed fragments stay in
 * the store for later requests. */
typedef struct tdm_server tdm_server;
typedef struct tdm_server_config {
  tdm_pipeline_config pipeline; /* per-fragment limits of an admitted request; matching and RANSAC */
  int32_t slots;                /* requests per wave at most */
  int64_t hbm_budget_bytes;     /* device bytes the server may hold; sets the wave capacity */
  int64_t store_bytes;          /* part of the budget for the fragment store (0: a tenth) */
} tdm_server_config;
typedef struct tdm_fragment {
  uint64_t key;      /* 0: anonymous (dropped after its pair); else a store key below 2^63 */
  const float* pts;  /* host x,y,z floats (copied at submit); NULL if the key is stored */
  int32_t n;
  uint64_t seed;     /* keypoint stream (tdm_keypoint_indices) */
  int32_t k;         /* keypoints */
} tdm_fragment;
typedef struct tdm_server_stats {
  int64_t requests_done, requests_cancelled, waves, fragments_described;
  int64_t store_hits, store_entries, max_wave_requests, device_bytes;
  double describe_ms, match_ms; /* wall time each stage was busy */
  double overlap_ms;            /* wall time both were busy at once */
} tdm_server_stats;
/* Creates the server: a clone of `net`, a batch, a store and matching
 * buffers sized from the budget (TDM_ERR_OOM when one request of the
 * configured size does not fit), and its two threads. */
tdm_status tdm_server_create(const tdm_server_config* cfg, const tdm_net* net, tdm_server** out);
/* Requests per wave the budget allows (<= cfg.slots). */
int32_t tdm_server_slots(const tdm_server* s);
/* Queues a pair (points copied: the caller's buffers may be reused at once).
 * A request larger than the server's capacity is refused (TDM_ERR_INVALID_ARG). */
tdm_status tdm_server_submit_pair(tdm_server* s, const tdm_fragment* a, const tdm_fragment* b, int64_t* ticket);
/* tdm_register_pair's request: anonymous fragments, keypoints of A from
 * `seed` and of B from `seed + 1`. */
tdm_status tdm_server_submit(tdm_server* s, const float* pts_a_host, int32_t na, const float* pts_b_host, int32_t nb,
                             uint64_t seed, int32_t k, int64_t* ticket);
/* Cancels a request: a queued one is dropped at once, one already on the GPU
 * finishes its kernels and its result is discarded; its wait then returns
 * TDM_ERR_CANCELLED. */
tdm_status tdm_server_cancel(tdm_server* s, int64_t ticket);
/* Waits up to timeout_ms (< 0: no limit) for the ticket's result; latency is
 * submit-to-completion.  TDM_ERR_TIMEOUT leaves the ticket valid. */
tdm_status tdm_server_wait(tdm_server* s, int64_t ticket, int64_t timeout_ms, tdm_pair_result* result,
                           double* latency_ms);
tdm_status tdm_server_get_stats(tdm_server* s, tdm_server_stats* out);
/* Finishes queued requests, then stops the threads and frees the server. */
tdm_status tdm_server_destroy(tdm_server* s);

#ifdef __cplusplus
}
#endif
#endif /* TDM_H */
