/*
 * mrf_oracle.h -- CPU restatement of MRFMap's forward-ray-sensor-model BP
 * and per-view likelihood.  TEST INFRASTRUCTURE ONLY: the parity tests, the
 * smoke check and the CPU-baseline leg of bench.py call this; the product
 * (libmrfmap_gb300.so) never links or calls it.
 *
 * PARITY UNPINNED against the reference itself: the reference depends on
 * gvdb-voxels, Eigen, yaml-cpp and OpenCV, none of which exist in this
 * build environment, and it ships no tests and no golden outputs.  This file
 * restates the reference's update equations (cited per function) and
 * replaces GVDB's brick traversal with an Amanatides-Woo voxel DDA whose
 * float operations are specified exactly, so the GPU traversal can be
 * checked bit-for-bit against it.
 *
 * Numerics: geometry (ray set-up, DDA, stop rules, potential cut-off,
 * activation) is evaluated in fp32 with every operation rounded separately
 * (build with -ffp-contract=off); the BP and likelihood arithmetic is FP64.
 */
#ifndef MRF_ORACLE_H
#define MRF_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  float res;          /* voxel edge, metres */
  float dims[3];      /* volume extent, metres (x, y centred; z from 0) */
  float fx, fy, cx, cy;
  int rows, cols;
  float prior;        /* occupancy prior */
  int lookup_n;       /* 3 = quadratic, 2 = linear sensor polynomials */
  int n_tiles_u, n_tiles_v;   /* ceil(cols/20), ceil(rows/20) */
  const float* sigma_lut;     /* n_tiles_v*n_tiles_u*lookup_n */
  const float* bias_lut;
} orc_params;

/* activation policies */
#define ORC_ACT_ENDPOINT 0   /* bricks around measured endpoints (reference) */
#define ORC_ACT_FULL_RAY 1   /* + every brick the ray crosses up to its Pre stop */

/* inference flags */
#define ORC_JACOBI        1  /* all cameras from one snapshot per iteration */
#define ORC_INCREMENTAL   2  /* keep per-camera messages across calls */
#define ORC_FIX_PRE_RESET 4  /* carry Pre-pass visibility across all bricks */

typedef struct orc_map orc_map;

orc_map* orc_create(const orc_params* p);
void orc_destroy(orc_map* m);
void orc_set_threads(int n);

/* pose: row-major 4x4 camera-to-world (metres); depth: rows*cols row-major,
 * row 0 = top.  Returns the view id. */
int orc_add_view(orc_map* m, const float* pose, const float* depth, int policy);
/* a view with its own camera (rows x cols, intrinsics); the sensor tables
 * are looked up at the pixel's position scaled into the params' image */
int orc_add_view_camera(orc_map* m, const float* pose, const float* depth, int policy, int rows, int cols,
                        float fx, float fy, float cx, float cy);
/* a view with its own camera confined to a scene box: bricks
 * [brick_lo, brick_hi) per axis; its rays are traced and its bricks
 * activated inside the box only.  Returns the view id, -1 for a bad box. */
int orc_add_view_box(orc_map* m, const float* pose, const float* depth, int policy, int rows, int cols, float fx,
                     float fy, float cx, float cy, const int brick_lo[3], const int brick_hi[3]);
int orc_view_pixels(const orc_map* m, int view);
int orc_set_pose(orc_map* m, int view, const float* pose, int policy);
int orc_num_views(const orc_map* m);
int orc_num_bricks(const orc_map* m);
/* brick coordinates (n x 3 int, brick units) in slot order */
void orc_brick_coords(const orc_map* m, int* out);
int orc_brick_dims(const orc_map* m, int* out3);

/* BP; ids selects which cameras' messages are zeroed (reference semantics);
 * every camera is iterated. iters <= 0 -> use 1. */
void orc_infer(orc_map* m, const int* ids, int n_ids, int iters, int flags);
/* beliefs / log-odds, [n_bricks x 512] in slot order, element (x*8+y)*8+z */
void orc_get_beliefs(const orc_map* m, float* out);
void orc_get_beliefs_f64(const orc_map* m, double* out);
void orc_get_logodds_f64(const orc_map* m, double* out);
/* overwrite the belief field (for external-map likelihood tests) */
void orc_set_beliefs(orc_map* m, const float* in);

/* per-view incidence lists (built on demand).  Returns number of rays with
 * at least one incidence; fills arrays when non-NULL.
 *   ray_pix[r], ray_off[r] (int64), ray_meta[r*5+{n_pre,n_post,r0,rinf,inf_gate}]
 *   inc_vox[i] (voxel id slot*512+local), inc_len[i], inc_s[i], inc_run[i]
 */
int64_t orc_view_num_incidences(orc_map* m, int view);
int orc_view_trace(orc_map* m, int view, int* ray_pix, int64_t* ray_off,
                   int* ray_meta, int* inc_vox, float* inc_len, float* inc_s,
                   unsigned char* inc_run, double* inc_mu);

/* trace one pixel through the current brick set (all active voxels to the
 * volume exit; no stop rule).  Returns count, writes up to max entries. */
int orc_trace_pixel(const orc_map* m, const float* pose, int x, int y,
                    int* vox, float* len, float* s, int max);

/* per-pixel log-likelihood image (rows*cols) of a depth image at a pose under
 * the current belief field; returns the frame sum. */
double orc_likelihood(const orc_map* m, const float* pose, const float* depth,
                      float* out_img);

/* evaluation renders (src/cuda/gvdbkernels.cu:135-181, 183-293, 295-354,
 * 1066-1162, 1332-1363): mode 0 expected depth, 1 accuracy (peak of the
 * first-return density within 1 sigma), 2 simple accuracy (first voxel above
 * thresh), 3 occupancy at the first voxel past the measurement.  counts[4]
 * receives the label histogram of labels -1, 0, 1, 2 (modes 1-3). */
void orc_render(const orc_map* m, int mode, const float* pose, const float* depth, float thresh,
                float* out_img, int64_t* counts);

/* classic log-odds ray insertion of one depth image at a pose (miss along
 * the ray, hit at the endpoint voxel, clamped) into L (one double per
 * active voxel, slot*512+local); single-threaded.  A CPU baseline, not part
 * of MRFMap.  Returns the voxel updates made. */
int64_t orc_insert_logodds(const orc_map* m, const float* pose, const float* depth, float l_hit,
                           float l_miss, float l_min, float l_max, double* L);

/* takes a view out of the iterated set (a bounded keyframe window): its
 * messages stay in the log-odds, it is no longer traced or iterated */
void orc_retire_view(orc_map* m, int view);
/* builds the incidence lists of every view (views in parallel) */
void orc_build_all(orc_map* m);
/* one Gauss-Seidel camera update of camera c (the body of the reference's
 * camera loop, src/GVDBInference.cpp:155-167) on the current state, its
 * messages kept: the unit the CPU baseline is timed on.  Returns the Post
 * incidences processed (-1 for a bad camera). */
int64_t orc_update_camera(orc_map* m, int c, int flags);

/* counters from the last orc_infer: incidence-iterations of Post passes */
int64_t orc_last_updates(const orc_map* m);

#ifdef __cplusplus
}
#endif
#endif
