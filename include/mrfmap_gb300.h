/*
 * mrfmap_gb300.h -- C ABI of the GB300 MRFMap hot path (libmrfmap_gb300.so).
 *
 * One map = one occupancy volume of 8^3-voxel bricks plus the posed depth
 * views added to it.  Every call is ordered on the map's own CUDA stream;
 * calls that hand results to host memory block until they are ready.
 * Plain pointers and sizes only: poses are 16 floats, row-major 4x4
 * camera-to-world in metres (camera x right, y down, z forward); depth
 * images are rows*cols floats, row-major, row 0 at the top, metres, with
 * NaN / <= 0 meaning "no return".
 *
 * Each entry point cites the reference interface it replaces
 * (paths inside the MRFMap project).
 */
#ifndef MRFMAP_GB300_H
#define MRFMAP_GB300_H
#include <stdint.h>

#if defined(__GNUC__)
#define MRF_API __attribute__((visibility("default")))
#else
#define MRF_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  MRF_OK = 0,
  MRF_ERR_INVALID = 1,   /* bad argument */
  MRF_ERR_CUDA = 2,      /* CUDA runtime error (mrf_last_error has text) */
  MRF_ERR_OOM = 3,       /* device allocation failed */
  MRF_ERR_CAPACITY = 4,  /* a 32-bit index range would overflow */
  MRF_ERR_DEVICE = 5,    /* a kernel raised its error flag (bounds) */
  MRF_ERR_STATE = 6      /* call not valid in the map's state */
} mrf_status;

/* brick activation policy */
#define MRF_ACT_ENDPOINT 0 /* bricks around measured endpoints, 1-voxel halo */
#define MRF_ACT_FULL_RAY 1 /* plus every brick a ray crosses up to the brick run where
                              its Pre pass stops (s + bias(s) > d + 3 sigma(s)) */

/* mrf_infer flags */
#define MRF_JACOBI 1        /* all cameras from one snapshot per iteration */
#define MRF_INCREMENTAL 2   /* keep per-camera messages across calls */
#define MRF_FIX_PRE_RESET 4 /* carry Pre-pass visibility across all bricks */
#define MRF_ASYNC 8         /* enqueue only; do not wait for completion */
#define MRF_PROFILE 16      /* time every kernel with CUDA events (mrf_stats) */
#define MRF_NO_GRAPH 32     /* launch kernels one by one instead of replaying the
                               captured CUDA graph of one iteration */
#define MRF_FULL_RAYS 64    /* read every ray's whole Pre range in every iteration
                               (no static prefixes from their quiet sums; by default
                               a call of 4 or more iterations takes them from the
                               third iteration on when the quiet incidences are at
                               least half of the Pre incidences and average at
                               least 256 per ray) */
#define MRF_QUIET_PREFIX 128 /* take the static prefixes from their quiet sums from
                                the third iteration on whatever their share */

/* Mirrors gvdb_params_t (include/mrfmap/GVDBParams.h:11-28). */
typedef struct mrf_params {
  float res;                /* voxel edge (m) */
  float dims[3];            /* volume extent (m); x,y centred, z from 0 */
  float fx, fy, cx, cy;     /* pinhole intrinsics K */
  int rows, cols;           /* image size */
  float prior;              /* occupancy prior */
  int max_iters;            /* BP iterations when mrf_infer gets iters <= 0 */
  int lookup_n;             /* 3: sigma(z)=p0+p1 z+p2 z^2, 2: linear */
  const float* sigma_lut;   /* ceil(rows/20)*ceil(cols/20)*lookup_n floats */
  const float* bias_lut;    /* same layout; per 20x20-pixel tile */
  float occ_thresh;
  float acc_thresh;
  int activation;           /* MRF_ACT_* */
  int reserved[7];
} mrf_params;

typedef struct mrf_map mrf_map;

typedef struct mrf_stats {
  int64_t n_views;
  int64_t n_bricks;
  int64_t n_rays;          /* rays with at least one incidence */
  int64_t n_inc_pre;       /* incidences traversed by the Pre pass */
  int64_t n_inc_post;      /* ray->voxel messages per iteration (N_inc) */
  int64_t n_pairs;         /* (camera, voxel) pairs (N_cv) */
  int64_t n_pairs_active;  /* pairs with cumulative length > 0.1 */
  int64_t n_vox_touched;   /* distinct voxels with a message (N_vox) */
  int64_t iters_done;      /* iterations run by the last mrf_infer */
  int64_t kernel_launches; /* kernels launched by the last mrf_infer */
  double build_ms;         /* last incidence-list build */
  double infer_ms;         /* last mrf_infer, device time */
  /* MRF_PROFILE: summed device time and launch count per kernel of the last
   * mrf_infer: [0] pair prepare, [1] ray messages, [2] pair update,
   * [3] voxel apply (Jacobi) */
  double kernel_ms[4];
  int64_t kernel_count[4];
  int64_t n_inc_dyn;       /* Post incidences from the first non-zero potential
                              on: the messages recomputed every iteration */
  int64_t n_pairs_dyn;     /* pairs holding at least one of them */
  int64_t n_rays_bp;       /* rays the ray kernel runs over: those with a dynamic
                              incidence (the others' messages are all static) */
  int64_t n_inc_pre_bp;    /* their Pre incidences */
  int64_t builds_full;     /* incidence-list builds of every view so far */
  int64_t builds_appended; /* builds that appended only the views added since
                              the previous build (full-ray maps) */
  int64_t n_inc_from_k4;   /* Pre incidences of those rays from k4 (their first
                              dynamic incidence rounded down to 4) on: what the
                              ray kernel reads in full from the third
                              iteration of a call on */
  int64_t n_loud_prefix;   /* incidences before k4 on voxels with a dynamic
                              incidence in some view: the rest of the static
                              prefixes is summed once per call (0 until the
                              first call of 4 or more iterations counts them) */
  int64_t quiet_prefix_used; /* 1 if the last mrf_infer took the static
                                prefixes from their quiet sums */
  int64_t builds_oom_fallback; /* full builds run because appending the new
                                  views' lists ran out of device memory (the
                                  full build drops the retired views' lists) */
} mrf_stats;

/* Map construction: GVDBInference(...) + GVDBMRFMap::gpuAllocate
 * (src/GVDBInference.cpp:20-37, src/GVDBMRFMap.cpp:23-93). */
MRF_API mrf_status mrf_create(const mrf_params* params, mrf_map** out);
MRF_API void mrf_destroy(mrf_map* map);
/* Device memory of destroyed maps stays pooled (per device) for the next
 * map; this returns the pooled blocks to the driver.  No reference
 * counterpart. */
MRF_API mrf_status mrf_release_cached_memory(void);
/* Bound on the device memory the maps of this process hold on one device
 * (bytes, per device; 0 = no bound, the default).  A call that would grow
 * a buffer past it fails with MRF_ERR_OOM before allocating; the map keeps
 * its views and can be used again once the memory is there (a higher bound,
 * other maps destroyed).  mrf_memory_in_use reports the bytes held on the
 * current device (-1 without one).  No reference counterpart: GVDB's pool
 * grows until the driver refuses. */
MRF_API mrf_status mrf_set_memory_limit(int64_t bytes);
MRF_API int64_t mrf_memory_in_use(void);
/* Test hook, no reference counterpart: sets the map's device error flag from
 * the host, as a traversal kernel does when a ray exceeds 65532 incidences.
 * The next call that checks the flag (an incidence-list build) fails with
 * MRF_ERR_DEVICE and clears it. */
MRF_API mrf_status mrf_test_raise_device_error(mrf_map* map);
/* Test hook, no reference counterpart: the pixels of built view view_id
 * whose rays may cross a brick in slots b0..b1 -- the footprint an appended
 * build re-checks after bricks were activated -- as mask[rows*cols] (0/1,
 * host) and *all (1: the footprint covers the whole image). */
MRF_API mrf_status mrf_test_brick_footprint(mrf_map* map, int view_id, int64_t b0, int64_t b1,
                                            uint8_t* mask, int* all);
/* Test hook, no reference counterpart (host only: no device call, no map):
 * the SM-affine schedule of one view's rays as an incidence build makes it
 * from the view's ray records.  records: n_pix triples {n_pre, n_post,
 * k_dyn} in pixel order (each in [0, 65535]); the rays in BP are those with
 * n_pre > 0 and k_dyn < n_post.  The view's pixels are cut into `regions`
 * runs of consecutive pixels holding equal shares of the BP rays' Pre
 * incidences; region r's home rays, its longest ones up to `share` per cent
 * of its incidences, are home[starts[r] .. starts[r+1]) (longest first,
 * pixel order within a length; starts has regions + 1 entries); the other
 * BP rays are left[0 .. *n_left), longest first.  home and left must hold
 * n_pix entries. */
MRF_API mrf_status mrf_test_region_lists(const int32_t* records, int64_t n_pix, int regions, int share,
                                         uint32_t* home, int64_t* n_home, uint32_t* starts, uint32_t* left,
                                         int64_t* n_left);
/* Test hook, no reference counterpart: the next build that appends new
 * views' lists fails with `status` once their pairs are built (a host-side
 * stand-in for a failing allocation or CUDA call part-way through).  An
 * MRF_ERR_OOM failure makes that build a full one (stats
 * builds_oom_fallback); any other fails the call, and the next build is a
 * full one. */
MRF_API mrf_status mrf_test_fail_next_append(mrf_map* map, mrf_status status);
/* Text of the last error raised on this thread. */
MRF_API const char* mrf_last_error(void);

/* GVDBInference::add_camera_with_depth (src/GVDBInference.cpp:58-64):
 * uploads and cleans the depth image (src/GVDBImage.cpp:13-60) and
 * activates bricks (src/GVDBCamera.cpp:70-112). */
MRF_API mrf_status mrf_add_view(mrf_map* map, const float* pose, const float* depth_host,
                        int* view_id);
/* Same, with the depth image already in device memory: depth_dev must hold
 * params.rows x params.cols floats (the map camera's image; the library
 * cannot check the size of a device buffer).  Views of other sizes go
 * through mrf_add_view_camera. */
MRF_API mrf_status mrf_add_view_device(mrf_map* map, const float* pose, const float* depth_dev,
                               int* view_id);
/* A view with its own pinhole camera (no counterpart in the reference, whose
 * cameras all share gvdb_params_t's rows, cols and K): depth_host holds
 * rows*cols floats.  The sensor tables (params' sigma/bias, tiled over the
 * params' image) are looked up at the pixel's position scaled into the
 * params' image, so one table serves every resolution of the same sensor.
 * Views of any sizes can share a map; mrf_likelihood_view, mrf_render_view
 * and mrf_view_incidences use the view's camera. */
MRF_API mrf_status mrf_add_view_camera(mrf_map* map, const float* pose, const float* depth_host, int rows,
                                       int cols, float fx, float fy, float cx, float cy, int* view_id);
/* A view with its own camera confined to a scene box (no counterpart in the
 * reference): bricks [brick_lo, brick_hi) per axis of the map's brick grid
 * (brick b spans voxels 8b .. 8b+7; voxel v spans metres (v - off) * res
 * with off = dims/2/res for x, y and 0 for z).  The view's rays are traced
 * and its bricks activated inside the box only, so several scenes placed in
 * disjoint boxes of one map share its brick pool, its BP launches (one
 * Jacobi ray launch covers every view of every scene) and its buffers
 * without seeing one another.  A box outside the grid or empty is
 * MRF_ERR_INVALID. */
MRF_API mrf_status mrf_add_view_box(mrf_map* map, const float* pose, const float* depth_host, int rows, int cols,
                                    float fx, float fy, float cx, float cy, const int brick_lo[3],
                                    const int brick_hi[3], int* view_id);
/* A view's camera: rows, cols, and fx, fy, cx, cy in k4 (any may be NULL). */
MRF_API mrf_status mrf_view_camera(mrf_map* map, int view_id, int* rows, int* cols, float* k4);
/* GVDBInference::set_pose (src/GVDBInference.cpp:66-82): moves a view and
 * activates bricks for its new pose. */
MRF_API mrf_status mrf_set_pose(mrf_map* map, int view_id, const float* pose);

/* Takes a view out of the set BP iterates (no reference counterpart: the
 * bounded keyframe window of a long incremental run, whose early keyframes'
 * incidence lists would not fit in memory).  The view's current messages
 * stay in the total log-odds for good and its depth image is released.  Its
 * incidence lists and pairs leave every launch at once; their memory is
 * reclaimed by the next full build, which runs once the retired views'
 * lists reach eight times the live ones, when appending new views runs out
 * of device memory, or before a call that needs every view's structures
 * (Jacobi, warm start).  Its id stays reserved: mrf_infer
 * passes over it and the per-view calls (likelihood, renders, messages,
 * incidences, set_pose) fail with MRF_ERR_STATE.  mrf_reset_state forgets
 * retired views' messages with everything else. */
MRF_API mrf_status mrf_retire_view(mrf_map* map, int view_id);
/* GVDBInference::perform_inference_ids (src/GVDBInference.cpp:100-178):
 * zeroes the messages of the cameras in ids (unless MRF_INCREMENTAL) and
 * runs iters BP iterations over every camera. ids == NULL -> all cameras. */
MRF_API mrf_status mrf_infer(mrf_map* map, const int* ids, int n_ids, int iters, int flags);
/* mrf_infer run to convergence: iterations stop after the first one whose
 * largest belief change (over every voxel) is below tol, checked every
 * check_every iterations, with max_iters as the cap (<= 0: params.max_iters).
 * The reference runs a fixed count (src/GVDBInference.cpp:155); this is
 * what "time to converged map" is measured with.  iters_done and last_delta
 * (the last measured change) may be NULL. */
MRF_API mrf_status mrf_infer_converge(mrf_map* map, const int* ids, int n_ids, int max_iters,
                                      float tol, int check_every, int flags, int* iters_done,
                                      float* last_delta);
/* mrf_infer run until the map reaches a given belief field: iterations stop
 * after the first one whose largest |belief - target| (over every voxel) is
 * at most tol, checked every check_every iterations, max_iters the cap.
 * target_dev is a device array of n_bricks x 512 floats (slot order, as
 * mrf_read_bricks).  No reference counterpart: this is the clock of "time
 * to the converged map" when the converged map is known (a tightly
 * converged plain run).  iters_done and last_dist may be NULL. */
MRF_API mrf_status mrf_infer_until(mrf_map* map, const int* ids, int n_ids, int max_iters,
                                   const float* target_dev, float tol, int check_every, int flags,
                                   int* iters_done, float* last_dist);
/* Warm start (no reference counterpart).  From a predicted total log-odds
 * field logodds[n_bricks x 512] (slot order, as mrf_read_logodds): pairs
 * whose messages are build constants get them exactly, the other pairs of
 * a voxel share the rest of logodds - logit(prior) in proportion to their
 * cumulative lengths; `sweeps` (>= 0) clamped iterations m <- F(logodds -
 * m) then refine the messages (one Jacobi evaluation of every ray factor
 * each), and the total log-odds is rebuilt from them (logit(prior) + sum of
 * messages).  The BP equations and their fixed point are unchanged;
 * continue with MRF_INCREMENTAL so the messages are kept.  The _device form
 * takes a device pointer. */
MRF_API mrf_status mrf_warm_start(mrf_map* map, const float* logodds, int sweeps);
MRF_API mrf_status mrf_warm_start_device(mrf_map* map, const float* logodds_dev, int sweeps);

/* BP state I/O (no reference counterpart; checkpoint / resume of the
 * message state).  mrf_read_messages writes camera view_id's messages as a
 * dense field [n_bricks x 512] (slot order; 0 where the camera has no
 * pair); mrf_write_messages sets them from one; mrf_rebuild_logodds sets
 * the total log-odds to logit(prior) + the sum of every camera's messages
 * (pairs past the length gate) and the beliefs from it. */
MRF_API mrf_status mrf_read_messages(mrf_map* map, int view_id, float* out_dense);
MRF_API mrf_status mrf_write_messages(mrf_map* map, int view_id, const float* dense);
MRF_API mrf_status mrf_rebuild_logodds(mrf_map* map);

/* Warm-start features (no reference counterpart): feat_dev receives
 * [n_bricks x 512 x 4] floats (slot order): the current belief, then
 * log(1 + x) of the voxel's pass-through length, of its potential mass
 * (sum of mu * l) and of its length inside the cameras' potential windows,
 * each summed over the cameras that see it (lengths in voxels). */
MRF_API mrf_status mrf_warm_features(mrf_map* map, float* feat_dev);

/* The warm-start network (no reference counterpart): three 3x3x3
 * convolutions over 8^3 bricks, 4 -> 16 -> 16 -> 1 channels, ReLU between,
 * zeros beyond the brick faces; BF16 tensor-core operands with FP32
 * accumulation; FP32 master parameters (mrf_net_num_params floats:
 * W1[27][4][16] b1[16] W2[27][16][16] b2[16] W3[27][16][1] b3[1], tap =
 * (dx*3 + dy)*3 + dz).  Every pointer is a device pointer; stream is a
 * cudaStream_t (NULL: the default stream); workspace holds
 * mrf_net_workspace_bytes(n_bricks) bytes.
 *   mrf_net_forward: out[n_bricks x 512] predicted log-odds from
 *     feat[n_bricks x 512 x 4].
 *   mrf_net_gradients: loss = sum w (y - target)^2 / norm over the voxels
 *     and its gradient grads[mrf_net_num_params] (deterministic).
 *   mrf_net_adam: one Adam step (bias-corrected, step >= 1). */
MRF_API int64_t mrf_net_num_params(void);
MRF_API int64_t mrf_net_workspace_bytes(int64_t n_bricks);
MRF_API mrf_status mrf_net_forward(const float* params, const float* feat, int64_t n_bricks,
                                   float* out, void* workspace, void* stream);
MRF_API mrf_status mrf_net_gradients(const float* params, const float* feat, const float* target,
                                     const float* weight, int64_t n_bricks, float norm, float* grads,
                                     float* loss, void* workspace, void* stream);
MRF_API mrf_status mrf_net_adam(float* params, const float* grads, float* m1, float* m2, int64_t n,
                                float lr, float beta1, float beta2, float eps, int step, void* stream);

/* Autotuner (no reference counterpart).  The ray-message kernel comes in
 * variants that differ in the cache policy of its streamed loads, in
 * whether a chunk's pair ids are requested one chunk ahead, in the ray
 * schedule (longest first or SM regions) and in the register budget (a
 * 12-block-per-SM target caps a thread at 40 registers); their arithmetic
 * is identical, so the choice never changes a result.
 * The pair reduction has two variants as well (one or two pairs' records
 * requested ahead per thread, at 8 or 5 resident blocks per SM), with the
 * same arithmetic; mrf_autotune times both after choosing the ray variant
 * and keeps the faster (mrf_get_tuning reports it).
 * mrf_autotune times every variant on this map's own incidence lists (reps
 * timed Gauss-Seidel iterations after one warm-up, the map state saved
 * before and restored after each variant), keeps the fastest and returns
 * per-variant milliseconds per iteration in
 * ms_out[0..min(cap, mrf_ray_variants())). */
MRF_API int mrf_ray_variants(void);
MRF_API mrf_status mrf_set_ray_variant(mrf_map* map, int variant);
MRF_API mrf_status mrf_autotune(mrf_map* map, int reps, double* ms_out, int cap, int* chosen);
/* The same with the schedule of the timed iterations in flags (MRF_JACOBI:
 * Jacobi iterations, one ray launch over every view; else Gauss-Seidel). */
MRF_API mrf_status mrf_autotune_flags(mrf_map* map, int reps, int flags, double* ms_out, int cap, int* chosen);

/* SM-region schedule of the ray kernel (no reference counterpart): each
 * SM's region hands its longest rays, up to `percent` of the region's
 * incidences, to the blocks homed on that SM; the rest go to the view's
 * shared leftover queue.  Default 75.  It only moves rays between warps, so
 * results do not change.  mrf_autotune_home_share times `n` shares
 * (1..100) on this map's lists (reps iterations each after a warm-up, the
 * map state restored after each), keeps the fastest, and returns the
 * per-share milliseconds per iteration in ms_out[0..n) (may be NULL).
 * The pair-update tile and the ray chunk are not tuned: both change the
 * order of floating-point sums, and a choice made from timings would make
 * results differ from run to run.  mrf_get_tuning reports the current
 * ray-kernel variant, home share and pair-reduction variant. */
MRF_API mrf_status mrf_set_home_share(mrf_map* map, int percent);
MRF_API mrf_status mrf_autotune_home_share(mrf_map* map, int reps, int flags, const int* shares, int n,
                                           double* ms_out, int* chosen);
MRF_API mrf_status mrf_get_tuning(mrf_map* map, int* ray_variant, int* home_share, int* pair_variant);
MRF_API mrf_status mrf_set_pair_variant(mrf_map* map, int variant);  /* 0 or 1 */

/* Storage precision of the ray kernel's streams (no reference counterpart;
 * the reference stores half2 channels, gvdbkernels.cu:975-978):
 *   MRF_PRECISION_FP32         (default) segment lengths and ln q in fp32
 *   MRF_PRECISION_HALF_STREAMS the ray kernel reads segment lengths and
 *                              gathers ln q as fp16 (round to nearest);
 *                              every product, prefix and sum stays fp32
 *                              (fp64 on long rays), the messages fp32.
 *                              No faster on the bench map (the ray kernel
 *                              is latency-bound); belief error against the
 *                              FP64 oracle 1.5e-6 on a converged 1 cm map,
 *                              but 2.8e-3 in the transient of an incremental
 *                              schedule, so not the default.
 * Changing it keeps the map's state. */
#define MRF_PRECISION_FP32 0
#define MRF_PRECISION_HALF_STREAMS 1
MRF_API mrf_status mrf_set_precision(mrf_map* map, int mode);
/* Extension: log-odds back to the prior, beliefs to 0, messages to 0. */
MRF_API mrf_status mrf_reset_state(mrf_map* map);

/* GVDBInference::get_likelihood_image / compute_likelihood
 * (src/GVDBInference.cpp:180-193).  out_img (rows*cols, host) may be NULL. */
MRF_API mrf_status mrf_likelihood_view(mrf_map* map, int view_id, float* out_img, float* out_sum);
/* GVDBInference::get_likelihood_image_at_pose (src/GVDBInference.cpp:195-240)
 * and GVDBMapLikelihoodEstimator::get_likelihood_image_at_pose
 * (src/GVDBMapLikelihoodEstimator.cpp:294-314); host buffers. */
MRF_API mrf_status mrf_likelihood(mrf_map* map, const float* pose, const float* depth_host,
                          float* out_img, float* out_sum);
/* Same with device buffers: depth_dev in, out_img_dev (may be NULL) and
 * out_sum_dev (one float) out; stream-ordered, does not block. */
MRF_API mrf_status mrf_likelihood_device(mrf_map* map, const float* pose, const float* depth_dev,
                                 float* out_img_dev, float* out_sum_dev);

/* Same as mrf_likelihood_device, but allocates no device memory: no
 * counterpart in the reference.  For callers that may not allocate while
 * scoring (real-time pose-search loops where cudaMalloc can stall the
 * device, hosts whose allocator owns all device memory).  The depth image
 * is cleaned on the fly; the only scratch is a fixed file-scope device array
 * of 4096 FP64 partial sums (32 KiB), so images are limited to 524,288
 * pixels (MRF_ERR_INVALID beyond; 640x480 and 848x480 fit).  All calls share
 * that array: calls overlapping on the GPU race and must be serialized.  The
 * first call in each CUDA context (per device, and again in a context created
 * after the caller destroyed the previous one) looks the array up with
 * cudaGetSymbolAddress; make it before any stream capture.  A map without
 * active bricks scores n * ln(LIKE_EPS), as mrf_likelihood_device does. */
MRF_API mrf_status mrf_likelihood_device_noalloc(mrf_map* map, const float* pose,
                                                 const float* depth_dev, float* out_img_dev,
                                                 float* out_sum_dev);

/* Evaluation renders over the belief field (depth image on the host, image
 * out on the host, rows*cols floats, may be NULL):
 *  MRF_RENDER_EXPECTED_DEPTH  GVDBInference::get_expected_depth_image
 *                             (src/GVDBInference.cpp:242-247)
 *  MRF_RENDER_ACCURACY        get_accuracy_image_at_pose; score = fraction of
 *                             labelled pixels with the density peak within
 *                             1 sigma (src/GVDBInference.cpp:385-429)
 *  MRF_RENDER_SIMPLE_ACCURACY get_simple_accuracy_at_pose with threshold
 *                             (acc_thresh when < 0); score = (TP+TN)/pixels
 *                             (src/GVDBMapLikelihoodEstimator.cpp:365-408)
 *  MRF_RENDER_OCC_THRESH      get_occ_thresh_image_at_pose with threshold
 *                             (occ_thresh when < 0)
 *                             (src/GVDBMapLikelihoodEstimator.cpp:410-434)
 * counts (may be NULL) receives the label histogram of -1, 0, 1, 2. */
#define MRF_RENDER_EXPECTED_DEPTH 0
#define MRF_RENDER_ACCURACY 1
#define MRF_RENDER_SIMPLE_ACCURACY 2
#define MRF_RENDER_OCC_THRESH 3
MRF_API mrf_status mrf_render(mrf_map* map, int mode, const float* pose, const float* depth_host,
                              float threshold, float* out_img, float* out_score, int64_t* counts);
/* Same at a stored view's pose and depth image. */
MRF_API mrf_status mrf_render_view(mrf_map* map, int mode, int view_id, float threshold,
                                   float* out_img, float* out_score, int64_t* counts);

/* GVDBInference::get_diagnostic_image(id, img, 0) and
 * get_diagnostic_image_at_pose (src/GVDBInference.cpp:287-378, kernel
 * src/cuda/gvdbkernels.cu:573-672, 1365-1384): the ray of pixel (x, y) at a
 * pose, traversed through every active brick to the volume exit, one record
 * of ten floats per voxel in out[n_floats] (host): [0] exit distance (m),
 * [1] belief, [2..3] voxel id as uint64 (slot*512 + (x*8+y)*8+z), [4] first
 * return density w = (V_prev - V)/l, [5] visibility V, [6..7] brick slot as
 * uint64, [8] brick-local x, y, z as bytes; out[n_floats-1] holds the number
 * of records; the rest is zero.  n_floats >= 11 (the reference uses the
 * rows*cols image). */
MRF_API mrf_status mrf_pixel_diagnostics(mrf_map* map, const float* pose, int x, int y, float* out,
                                         int64_t n_floats);

/* GVDBMRFMap::get_occupied_bricks(0) (src/GVDBMRFMap.cpp:137-152). */
MRF_API mrf_status mrf_num_bricks(mrf_map* map, int64_t* n_bricks);
/* centres: n*3 floats, brick centres in voxel units (the reference's GVDB
 * world frame); beliefs: n*512 floats, element (x*8+y)*8+z
 * (GVDBMRFMap::get_alphas, src/GVDBMRFMap.cpp:154-208).  Either may be NULL.
 * n must equal mrf_num_bricks (else MRF_ERR_INVALID, as the reference throws). */
MRF_API mrf_status mrf_read_bricks(mrf_map* map, float* centres, float* beliefs, int64_t n);
/* Extension: total log-odds per voxel, same layout. */
MRF_API mrf_status mrf_read_logodds(mrf_map* map, float* logodds, int64_t n);
/* Upper-level node centres (GVDBMRFMap::get_occupied_bricks(lev>0)). */
MRF_API mrf_status mrf_num_nodes(mrf_map* map, int level, int64_t* n);
MRF_API mrf_status mrf_read_nodes(mrf_map* map, int level, float* centres, int64_t n);

/* GVDBMapLikelihoodEstimator::load_map (src/GVDBMapLikelihoodEstimator.cpp:168-240):
 * points n*3 in voxel units, occupancies n floats written into the belief
 * field after activating the bricks around each point. */
MRF_API mrf_status mrf_load_map(mrf_map* map, const float* points, const float* occupancies,
                        int64_t n);

/* Introspection of one view's incidence lists (after building them):
 * meta rows*cols*5 ints per pixel {n_pre, n_post, r0, rinf, inf_gate};
 * vox / len / mu: the view's incidences in ray order (pixel-major), at most
 * cap entries; *n_inc receives the count.  Any output may be NULL. */
MRF_API mrf_status mrf_view_incidences(mrf_map* map, int view_id, int* meta, uint32_t* vox, float* len,
                               float* mu, int64_t cap, int64_t* n_inc);

/* Device pointers of the map state (for zero-copy consumers and benches). */
MRF_API mrf_status mrf_device_beliefs(mrf_map* map, const float** beliefs, int64_t* n_voxels);
MRF_API mrf_status mrf_stats_get(mrf_map* map, mrf_stats* out);
/* The CUDA stream the map enqueues on (cudaStream_t as void*). */
MRF_API mrf_status mrf_get_stream(mrf_map* map, void** stream);
MRF_API mrf_status mrf_synchronize(mrf_map* map);

#ifdef __cplusplus
}
#endif
#endif
