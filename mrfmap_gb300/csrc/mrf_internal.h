// mrf_internal.h -- structures shared between the C-ABI layer and the kernels.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/mrfmap_gb300.h"

namespace mrf {

constexpr int kBrick = 8;
constexpr int kBrickVox = 512;
constexpr int kLookupPx = 20;          // include/mrfmap/GVDBCommon.cuh:11
constexpr float kFEps = 1e-4f;         // GVDBCommon.cuh:5
constexpr float kLikeEps = 1e-3f;      // GVDBCommon.cuh:8
constexpr float kZMin = 0.1f;          // GVDBCommon.cuh:4
constexpr float kZMax = 10.0f;         // GVDBCommon.cuh:3
constexpr float kMuCutoff = 87.0f;     // 0.5 x^2 above which the fp32 potential is 0
constexpr float kCumLenGate = 0.1f;    // gvdbkernels.cu:408
constexpr int kLongRay = 512;          // rays longer than this carry FP64 sums

// Geometry of one map (volume, camera intrinsics, sensor tables, brick table)
struct Geom {
  float res, inv_res;
  float fx, fy, cx, cy;
  int rows, cols;
  float off[3];      // dims_xy/2/res, 0
  float hi[3];       // dims/res (activation gate)
  int NB[3];         // brick grid
  int E[3];          // 8*NB
  int blo[3], bhi[3];  // voxel box of the traversal and activation: [0, E) for the
                       // map's own camera; a view confined to a scene box
                       // (mrf_add_view_box) has the box's brick-aligned bounds
  float glo[3];      // lower gate of endpoint activation (0, or the box)
  int lookup_n, n_tiles_u, n_tiles_v;
  int lut_rows, lut_cols;  // image size the sensor tables are tiled for
  const float* sigma;   // device
  const float* bias;    // device
  const int* brick_slot;  // device, NB0*NB1*NB2
};

struct Pose {
  float m[16];  // row-major camera-to-world
};

// per-ray record of the incidence lists
struct RayMeta {
  uint32_t off;     // global index of the ray's first incidence
  uint16_t n_pre;   // incidences seen by the Pre pass
  uint16_t n_post;  // incidences receiving a message
  uint16_t r0;      // Pre-pass visibility start
  uint16_t rinf;    // visibility start of the infinity term
  uint32_t flags;   // bit0: infinity term applies; bits 16-31: k_dyn
};
static_assert(sizeof(RayMeta) == 16, "RayMeta layout");

// k_dyn: first Post incidence with a non-zero potential (n_post if none).
// Before it every Post quantity of the ray is exactly zero (tau = 0, F = 0,
// mu1 = 0), so the outgoing probability is exactly the clamp floor F_EPS and
// the message is F_EPS * l: static for the life of the incidence lists.
__host__ __device__ __forceinline__ int ray_kdyn(const RayMeta& m) { return (int)(m.flags >> 16); }
// rays the ray kernel runs over: those with a dynamic incidence.  A ray
// whose Post messages are all static produces nothing (its messages are
// build constants, summed into the pairs), so it is left out of the queues.
__host__ __device__ __forceinline__ bool ray_in_bp(const RayMeta& m) {
  return m.n_pre > 0 && ray_kdyn(m) < m.n_post;
}


constexpr int kMaxRayLen = 65532;        // n_pre fits uint16 after padding to 4
constexpr uint32_t kNoVoxel = 0xFFFFFFFFu;  // padding incidences

// ---- launchers (stream-ordered; return cudaError_t of the launch) --------
cudaError_t launch_clean_depth(const float* in, float* out, int rows, int cols, cudaStream_t s);
cudaError_t launch_activate(const Geom& g, const Pose& P, const float* depth, int policy,
                            uint8_t* flags, cudaStream_t s);
cudaError_t launch_activate_points(const Geom& g, const float* pts, int64_t n, uint8_t* flags,
                                   cudaStream_t s);
cudaError_t launch_new_indicator(const uint8_t* flags, const int* slot, int* ind, int64_t n,
                                 cudaStream_t s);
cudaError_t launch_assign_slots2(const Geom& g, const int* ind, const int* scan, int nb_base,
                                 int* brick_slot, int* brick_coord, int64_t n, cudaStream_t s);
cudaError_t launch_fill_new_voxels(float* L, float* belief, int64_t v0, int64_t v1, float logit_prior,
                                   cudaStream_t s);
cudaError_t launch_set_points(const Geom& g, const float* pts, const float* occ, int64_t n,
                              float* belief, cudaStream_t s);

// traversal: count pass then emit pass.  With check (the view's stored ray
// records) the count pass also sets err[1] when any ray's record would
// differ from the stored one (err holds two ints).
cudaError_t launch_trace_count(const Geom& g, const Pose& P, const float* depth, uint32_t* counts,
                               int* err, cudaStream_t s, const RayMeta* check = nullptr,
                               const uint8_t* only = nullptr, const int* only_all = nullptr);
// pixels of a view whose rays may cross one of the bricks in slots b0..b1
// (mask[pix] = 1; *all = 1 when every pixel must be checked)
cudaError_t launch_brick_footprint(const Geom& g, const Pose& P, const int* coord, uint32_t b0, uint32_t b1,
                                   uint8_t* mask, int* all, cudaStream_t s);
cudaError_t launch_trace_emit(const Geom& g, const Pose& P, const float* depth,
                              const uint32_t* pix_off, uint32_t inc_base, RayMeta* meta,
                              uint32_t* inc_vox, float* inc_len, float* inc_mu, float2* inc_rec,
                              int* err, cudaStream_t s);
// runs of the voxel-sorted incidences (the pairs before renumbering)
cudaError_t launch_vox_heads(const uint32_t* sk, uint32_t n, uint32_t* flag, cudaStream_t s);
// brick-major first-visit pair numbering (mrf_build.cu)
cudaError_t launch_pair_first(const uint32_t* seg, uint32_t np, uint32_t perm_base, const uint32_t* sidx,
                              uint32_t* key, cudaStream_t s);
cudaError_t launch_brick_first(const uint32_t* pair_vox, const uint32_t* key, uint32_t np, uint32_t* bfirst,
                               cudaStream_t s);
cudaError_t launch_brick_keys(const uint32_t* order, uint32_t np, const uint32_t* pair_vox,
                              const uint32_t* bfirst, const uint8_t* loud, int bits, uint32_t* key,
                              cudaStream_t s);
// voxels with a dynamic incidence in any view (vox[k]: the voxel of
// incidence vox_base + k), and the pairs on them
cudaError_t launch_loud_voxels(const RayMeta* meta, int64_t npix, const uint32_t* vox, uint32_t vox_base,
                               uint8_t* loud, cudaStream_t s);
// the same with each incidence's voxel from its pair (vox = pair_vox[inc_pair])
cudaError_t launch_loud_voxels_from_pairs(const RayMeta* meta, int64_t npix, const uint32_t* inc_pair,
                                          const uint32_t* pair_vox, uint8_t* loud, cudaStream_t s);
// flag[v] = 1 for the voxels of the given pairs past the length gate (no reset)
cudaError_t launch_mark_active(const uint32_t* pair_vox, const float* cum, uint32_t np, uint8_t* flag,
                               cudaStream_t s);
cudaError_t launch_count_loud(const uint32_t* pair_vox, uint32_t np, const uint8_t* loud, uint32_t* count,
                              cudaStream_t s);
cudaError_t launch_new_lengths(const uint32_t* order, uint32_t np, const uint32_t* seg, uint32_t* len,
                               uint32_t* slot_of, cudaStream_t s);
cudaError_t launch_move_positions(const uint32_t* sidx, const uint32_t* flag, const uint32_t* scan,
                                  const uint32_t* seg, const uint32_t* slot_of, const uint32_t* start, uint32_t n,
                                  uint32_t inc_base, uint32_t pair_base, uint32_t* out_idx, uint32_t* inc_pair,
                                  cudaStream_t s);
cudaError_t launch_pairs_renumbered(const uint32_t* order, uint32_t np, const uint32_t* vox_old,
                                    const uint32_t* start, uint32_t pair_base, uint32_t perm_base,
                                    uint32_t* pair_vox, uint32_t* seg, cudaStream_t s);
// pairs from the pair-grouped incidences: pair_vox, seg and (when given)
// inc_pair
cudaError_t launch_pairs_from_sorted(const uint32_t* sk, const uint32_t* sidx, const uint32_t* flag,
                                     const uint32_t* scan, uint32_t n, uint32_t pair_base,
                                     uint32_t perm_base, uint32_t inc_base, uint32_t* pair_vox,
                                     uint32_t* seg, uint32_t* inc_pair, cudaStream_t s);
// build records (post length, -(mu l) on dynamic incidences) in sorted order
// build records in pair-grouped order, and each position's dynamic flag
cudaError_t launch_gather_rec(const uint32_t* sidx, uint32_t n, uint32_t inc_base, const float2* rec,
                              float2* out, uint32_t* dflag, cudaStream_t s);
// per pair: cumulative length, summed static messages, dynamic incidences,
// potential mass (from the sorted records)
// long_list: scratch of 1 + np u32 (count, then the pairs with long runs)
cudaError_t launch_pair_stats(const uint32_t* seg, uint32_t p0, uint32_t np, uint32_t perm_base,
                              const float2* srec, float* cum, float* stat, uint32_t* ndyn, float* hit,
                              uint32_t* long_list, cudaStream_t s);
// warm-start initial messages from a predicted log-odds field (voxel CSR)
// (base: per-voxel log-odds without the live views' messages, or NULL for
// the prior lp everywhere)
cudaError_t launch_warm_split(const uint32_t* vseg, const uint32_t* vpairs, const uint32_t* vvox,
                              uint32_t nvox, const float* L_pred, float lp, const float* base, const float* cum,
                              const float* stat, const uint32_t* ndyn, float* m, cudaStream_t s);
// warm-start features per voxel [nvox_slots][4] from the voxel CSR
cudaError_t launch_voxel_features(const uint32_t* vseg, const uint32_t* vpairs, const uint32_t* vvox,
                                  uint32_t nvox, const float* cum, const float* stat, const float* hit,
                                  const float* belief, int64_t n_slots_vox, float* feat, cudaStream_t s);
// dynamic incidences of a view in pair-grouped order (dperm) and the pairs
// that own them (dpair, with their first position dseg)
cudaError_t launch_dyn_scatter(const uint32_t* sidx, const uint32_t* flag, const uint32_t* scan,
                               uint32_t n, uint32_t inc_base, uint32_t dperm_base, uint32_t* dperm,
                               cudaStream_t s);
cudaError_t launch_dpair_flags(const uint32_t* ndyn, uint32_t p0, uint32_t np, uint32_t* flag,
                               cudaStream_t s);
cudaError_t launch_dpairs(const uint32_t* pflag, const uint32_t* pscan, uint32_t p0, uint32_t np,
                          const uint32_t* seg, uint32_t perm_base, const uint32_t* dscan,
                          uint32_t dperm_base, uint32_t dpair_base, uint32_t* dpair, uint32_t* dseg,
                          cudaStream_t s);
cudaError_t launch_iota(uint32_t* out, uint32_t n, cudaStream_t s);
// CUB helpers (scratch-managed by the caller)
size_t scan_temp_bytes(uint32_t n);
cudaError_t exclusive_scan_u32(void* tmp, size_t tmp_bytes, const uint32_t* in, uint32_t* out,
                               uint32_t n, cudaStream_t s);
size_t scan_temp_bytes_i32(int64_t n);
cudaError_t exclusive_scan_i32(void* tmp, size_t tmp_bytes, const int* in, int* out, int64_t n,
                               cudaStream_t s);
size_t sort_temp_bytes(uint32_t n, int bits);
cudaError_t sort_pairs_u32(void* tmp, size_t tmp_bytes, const uint32_t* kin, uint32_t* kout,
                           const uint32_t* vin, uint32_t* vout, uint32_t n, int bits, cudaStream_t s);

// BP
struct BpArrays {
  const RayMeta* meta;
  const uint32_t* inc_pair;
  const float* inc_len;
  const float* inc_mu;
  float* inc_pl;           // p*l per incidence, ray order (dynamic ones only)
  const uint32_t* dperm;   // dynamic incidence at each pair-grouped position
  const uint32_t* dpair;   // pair owning each dynamic run
  const uint32_t* dseg;    // first dynamic position of each run
  const uint4* drun;       // per run: pair id, voxel, cumulative length, static sum
  const uint32_t* pair_vox;
  float* pair_m;
  const float* pair_cum;
  const float* pair_stat;  // sum of the pair's static messages
  const uint32_t* pair_ndyn;
  float* pair_lnq;
  float* pair_dm;
  float* L;
  float* belief;
  // 16-bit streams (MRF_PRECISION_HALF_STREAMS): the ray kernel reads the
  // segment lengths and gathers ln q as fp16; k_pair_prepare writes ln q as
  // fp16 then
  int half_streams;
  int pair_variant;  // pair reduction: 0 one prefetched pair per thread, 1 two
  const float2* quiet_q;     // per ray: quiet sums of the static prefix
  const uint32_t* loud_off;  // per ray: first entry of its loud list (and the next ray's)
  const uint32_t* loud_pid;
  const float* loud_len;
  const uint16_t* loud_pos;
  const __half* inc_len16;
  __half* pair_lnq16;
};
// per-tile partial sums of the pair-update segmented reduction
struct TileCarry {
  uint32_t first_key, last_key;
  float first_sum, last_sum;
  uint32_t flags;
};
uint32_t pair_update_tiles(uint32_t n);
cudaError_t launch_pair_prepare(const BpArrays& a, uint32_t p0, uint32_t p1, int jacobi,
                                cudaStream_t s);
// ray-kernel variants (register budget x load policy; identical arithmetic)
int ray_bp_variants();
// resident blocks per SM of a variant of the persistent ray kernel (queried once)
int ray_bp_resident_blocks(int variant, int half_streams);
// fp32 -> fp16, round to nearest
cudaError_t launch_to_half(const float* in, int64_t n, __half* out, cudaStream_t s);
// the rays of one ray-kernel launch in its schedules: queue[0..n_rays)
// longest first with one zeroed counter; the same rays as nreg regions of
// consecutive pixels, rper regions per view: region r = (view q = r / rper,
// rr = r % rper) has its home rays (longest first) at positions
// rstart[q (rper + 1) + rr] .. rstart[q (rper + 1) + rr + 1] of region (nreg
// zeroed counters), and the views' remaining short rays (longest first):
// view q's lprefix[q + 1] - lprefix[q] leftovers from region[lbase[q]] on,
// nlv views, one zeroed counter
// the static-prefix data of the ray kernel's fast path (iterations from the
// third of a call on): per ray (pixel index) the quiet sums up to r0 and up
// to k4, and the list of the prefix's loud incidences at loff[r]..loff[r+1]
struct QuietPrefix {
  const float2* q;
  const uint32_t* loff;
  const uint32_t* lpid;
  const float* llen;
  const uint16_t* lpos;
};

struct RayWork {
  const RayMeta* queue;
  const uint32_t* queue_ids;   // pixel index of each queue record
  uint32_t n_rays;
  uint32_t* counter;
  const RayMeta* region;
  const uint32_t* region_ids;
  const uint32_t* rstart;
  uint32_t nreg, rper;
  uint32_t* rcounter;
  const uint32_t* lprefix;
  const uint32_t* lbase;
  uint32_t nlv;
  uint32_t* lcounter;
};
// quiet: the static prefix from the quiet sums (a.quiet_q and the loud
// lists must be current)
cudaError_t launch_ray_bp(const BpArrays& a, const RayWork& w, int fix_reset, int num_sms, int variant,
                          bool quiet, cudaStream_t s);
// loud incidences of the static prefixes of rays r_first..r_first+n of one
// view: counts to loff[r] (emit false), or the lists at loff[r] (emit true)
cudaError_t launch_loud_prefix(const RayMeta* meta, uint32_t r_first, uint32_t n, const uint32_t* inc_pair,
                               const float* inc_len, uint32_t pair_base, uint32_t n_loud, uint32_t* loff,
                               uint32_t* lpid, float* llen, uint16_t* lpos, bool emit, cudaStream_t s);
// quiet sums of the static prefixes of rays r_first..r_first+n of one view
cudaError_t launch_quiet_prefix(const BpArrays& a, uint32_t r_first, uint32_t n, uint32_t pair_base,
                                uint32_t n_loud, float2* q, cudaStream_t s);
cudaError_t launch_ray_keys(const RayMeta* meta, uint32_t n, uint32_t* keys, uint32_t* vals,
                            cudaStream_t s);
// queue[i] = meta[order[i]], ids[i] = id_base + order[i], i < n
cudaError_t launch_ray_queue(const RayMeta* meta, const uint32_t* order, uint32_t n, RayMeta* queue,
                             uint32_t* ids, uint32_t id_base, cudaStream_t s);
// dynamic positions k0..k1 hold the runs j0..j1 (dpair/dseg indices);
// tile_first from launch_tile_first over dseg
cudaError_t launch_pair_update(const BpArrays& a, uint32_t k0, uint32_t k1, uint32_t j0, uint32_t j1,
                               const uint32_t* tile_first, TileCarry* carry, int jacobi,
                               cudaStream_t s);
// per-run records of the pair update (from dpair and the pair arrays)
cudaError_t launch_drun(const uint32_t* dpair, uint32_t n, const uint32_t* pair_vox, const float* cum,
                        const float* stat, uint4* drun, cudaStream_t s);
// pairs p0..p1 without dynamic incidences: their constant update, needed
// once after their messages were reset or remapped
cudaError_t launch_static_pairs(const BpArrays& a, uint32_t p0, uint32_t p1, int jacobi,
                                cudaStream_t s);
cudaError_t launch_tile_first(const uint32_t* seg, uint32_t p0, uint32_t p1, uint32_t k0, uint32_t k1,
                              uint32_t* out, cudaStream_t s);
cudaError_t launch_voxel_apply(const uint32_t* vseg, const uint32_t* vpairs, const uint32_t* vvox,
                               uint32_t nvox, const float* pair_dm, float* L, cudaStream_t s);
// flag[v] = 1 for the voxels with a pair past the length gate (the voxels
// whose belief the iterations define), 0 elsewhere
cudaError_t launch_active_voxels(const uint32_t* pair_vox, const float* cum, uint32_t np, uint8_t* flag,
                                 int64_t nvox, cudaStream_t s);
// belief[v] from L[v] where active[v]
cudaError_t launch_belief_refresh(const float* L, const uint8_t* active, int64_t nvox, float* belief,
                                  cudaStream_t s);
cudaError_t launch_voxel_rebuild(const uint32_t* vseg, const uint32_t* vpairs, const uint32_t* vvox,
                                 uint32_t nvox, const float* m, const float* cum, float* L, float* belief,
                                 cudaStream_t s);
// base[pair_vox[p]] += pair_m[p] over one camera's pairs
cudaError_t launch_fold_messages(const uint32_t* pair_vox, const float* pair_m, uint32_t n, float* base,
                                 cudaStream_t s);
cudaError_t launch_remove_messages(const BpArrays& a, uint32_t p0, uint32_t p1, cudaStream_t s);
cudaError_t launch_remap_scatter(const uint32_t* pair_vox, const float* pair_m, uint32_t n,
                                 float* dense, cudaStream_t s);
cudaError_t launch_remap_gather(const uint32_t* pair_vox, float* pair_m, uint32_t n,
                                const float* dense, cudaStream_t s);
cudaError_t launch_fill_f32(float* p, int64_t n, float v, cudaStream_t s);
// out[0] = bits of max |a - b| over n floats (non-negative: the bit order is
// the value order, so an integer max is exact and order-independent)
cudaError_t launch_max_abs_diff(const float* a, const float* b, int64_t n, uint32_t* out,
                                cudaStream_t s);
cudaError_t launch_fill_u32(uint32_t* p, int64_t n, uint32_t v, cudaStream_t s);
// *out = sum of n u32 values, in 64 bits
cudaError_t launch_sum_u32(const uint32_t* v, int64_t n, unsigned long long* out, cudaStream_t s);
// per-view ray-record counters (k_ray_counters): out[0..kRayCounters) zeroed
// on the stream, then summed over meta[0..n)
constexpr int kRayCounters = 7;
cudaError_t launch_ray_counters(const RayMeta* meta, int64_t n, unsigned long long* out, cudaStream_t s);
// out2[0] = pairs past the length gate, out2[1] = distinct voxels they
// reach (flag: nvox bytes of scratch)
cudaError_t launch_touch_counts(const uint32_t* pair_vox, const float* cum, uint32_t np, uint8_t* flag,
                                int64_t nvox, unsigned long long* out2, cudaStream_t s);
cudaError_t launch_vflag(const uint32_t* sk, uint32_t n, uint32_t* flag, cudaStream_t s);
cudaError_t launch_vassign(const uint32_t* sk, const uint32_t* flag, const uint32_t* scan,
                           uint32_t n, uint32_t* vvox, uint32_t* vseg, cudaStream_t s);
cudaError_t launch_scatter_const(const uint32_t* idx, uint32_t n, float v, float* dense,
                                 cudaStream_t s);

// likelihood and readback
cudaError_t launch_likelihood(const Geom& g, const Pose& P, const float* depth, const float* belief,
                              float* out_img, double* partials, int nblocks, cudaStream_t s);
int likelihood_blocks(const Geom& g);
cudaError_t launch_reduce_partials(const double* partials, int n, float* out_sum, cudaStream_t s);

// per-voxel records of one pixel's ray (debug probe; out zeroed by the caller,
// 8-byte aligned, n_floats >= 11)
cudaError_t launch_pixel_diag(const Geom& g, const Pose& P, const float* belief, int x, int y, float* out,
                              int64_t n_floats, cudaStream_t s);
// evaluation renders (mode 0-3, see mrf_render.cu); counts: 4 zeroed u64
cudaError_t launch_render(int mode, const Geom& g, const Pose& P, const float* depth,
                          const float* belief, float thresh, float* out, unsigned long long* counts,
                          cudaStream_t s);

// Map state the likelihood needs, for entry points outside mrf_capi.cu: the
// map's geometry (device brick table and sensor tables), its belief field
// (NULL while the map has no active brick), stream and device.  Makes the
// map's device current.  Allocates nothing.
mrf_status mrf_internal_like_inputs(mrf_map* map, Geom* g, const float** belief,
                                    cudaStream_t* stream, int* device);
void mrf_internal_set_error(const std::string& msg);

}  // namespace mrf
