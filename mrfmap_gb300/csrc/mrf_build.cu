// mrf_build.cu -- per-keyframe work that runs once per brick-set change:
// depth clean-up, brick activation, the 3D-DDA traversal that emits each
// ray's incidence list, and the (camera, voxel) pair / CSR construction.
//
// Reference behaviour restated here (paths inside the MRFMap project):
//   depth clean-up            src/GVDBImage.cpp:32-40
//   endpoint back-projection  src/GVDBImage.cpp:48-56, src/GVDBCamera.cpp:70-100
//   activation radius 1       src/GVDBMRFMap.cpp:117-135
//   per-brick stop rules      src/cuda/gvdbkernels.cu:568, 816, 1035
//   infinity-term gate        src/cuda/gvdbkernels.cu:1196-1208
//   Pre-pass visibility reset src/cuda/gvdbkernels.cu:708-715
#include <cub/cub.cuh>

#include "mrf_geometry.cuh"
#include "mrf_internal.h"

namespace mrf {

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(int64_t n, int t = kThreads) {
  int64_t b = (n + t - 1) / t;
  return (unsigned)(b < 1 ? 1 : b);
}

__global__ void k_clean_depth(const float* __restrict__ in, float* __restrict__ out, int rows,
                              int cols) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * cols) return;
  out[i] = clean_depth_value(in[i], i, rows, cols);
}

__device__ __forceinline__ int floordiv8(int v) { return v >= 0 ? v / 8 : -((-v + 7) / 8); }

__device__ __forceinline__ void mark_point(const Geom& g, float px, float py, float pz,
                                           uint8_t* flags) {
  int lo[3], hi[3];
  float pv[3] = {px, py, pz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    int vi = (int)floorf(pv[a]);
    lo[a] = max(floordiv8(vi - 1), g.blo[a] / kBrick);
    hi[a] = min(floordiv8(vi + 1), g.bhi[a] / kBrick - 1);
  }
  for (int bx = lo[0]; bx <= hi[0]; ++bx)
    for (int by = lo[1]; by <= hi[1]; ++by)
      for (int bz = lo[2]; bz <= hi[2]; ++bz)
        flags[((int64_t)bx * g.NB[1] + by) * g.NB[2] + bz] = 1;
}

__global__ void k_activate(Geom g, Pose P, const float* __restrict__ depth, int policy,
                           uint8_t* __restrict__ flags) {
  int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= g.rows * g.cols) return;
  float d = depth[pix];
  if (!(d > 0.0f)) return;
  int x = pix % g.cols, y = pix / g.cols;
  // back-projection with fx on both axes and integer pixel coordinates
  float f = fd(d, g.fx);
  float X = fm(f, fs((float)x, g.cx));
  float Y = fm(f, fs((float)y, g.cy));
  float pv[3];
  bool inside = true;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float pw = fa(fa(fa(fm(P.m[a * 4 + 0], X), fm(P.m[a * 4 + 1], Y)), fm(P.m[a * 4 + 2], d)),
                  P.m[a * 4 + 3]);
    pv[a] = fa(fm(pw, g.inv_res), g.off[a]);
    if (!(pv[a] >= g.glo[a] && pv[a] < g.hi[a])) inside = false;
  }
  if (inside) mark_point(g, pv[0], pv[1], pv[2], flags);
  if (policy == 1) {
    // every brick the ray crosses up to the brick run where the Pre pass
    // stops (the trace's test: at the exit s of a run's last voxel,
    // s + bias(s) > d + 3 sigma(s)).  The trace then meets only bricks its
    // own view activated before its stop, so bricks other views activate
    // later never change this view's lists.
    const float* sg = lut_at(g, g.sigma, x, y);
    const float* bs = lut_at(g, g.bias, x, y);
    const int n = g.lookup_n;
    Ray ray;
    ray_setup(g, P, x, y, ray);
    Dda r;
    if (dda_init(r, g, ray)) {
      int vx, vy, vz;
      float l, tin, te, s_last = 0.0f;
      int64_t cur = -1;
      while (dda_next(r, g, vx, vy, vz, l, tin, te)) {
        int64_t lin = brick_lin(g, vx, vy, vz);
        if (lin != cur) {
          if (cur >= 0 && fa(s_last, poly_f(bs, n, s_last)) > fa(d, fm(3.0f, poly_f(sg, n, s_last)))) break;
          flags[lin] = 1;
          cur = lin;
        }
        s_last = fm(te, ray.mult);
      }
    }
  }
}

__global__ void k_activate_points(Geom g, const float* __restrict__ pts, int64_t n,
                                  uint8_t* __restrict__ flags) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float px = pts[3 * i], py = pts[3 * i + 1], pz = pts[3 * i + 2];
  if (!(px >= 0.0f && py >= 0.0f && pz >= 0.0f && px < (float)g.E[0] && py < (float)g.E[1] &&
        pz < (float)g.E[2]))
    return;
  mark_point(g, px, py, pz, flags);
}

__global__ void k_new_indicator(const uint8_t* __restrict__ flags, const int* __restrict__ slot,
                                int* __restrict__ ind, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  ind[i] = (flags[i] && slot[i] < 0) ? 1 : 0;
}

__global__ void k_assign_slots(Geom g, const int* __restrict__ ind, const int* __restrict__ scan,
                               int nb_base, int* __restrict__ slot, int* __restrict__ coord,
                               int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !ind[i]) return;
  int s = nb_base + scan[i];
  slot[i] = s;
  int bz = (int)(i % g.NB[2]);
  int by = (int)((i / g.NB[2]) % g.NB[1]);
  int bx = (int)(i / ((int64_t)g.NB[2] * g.NB[1]));
  coord[3 * s + 0] = bx;
  coord[3 * s + 1] = by;
  coord[3 * s + 2] = bz;
}

__global__ void k_fill_new_voxels(float* L, float* belief, int64_t v0, int64_t v1, float lp) {
  int64_t i = v0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v1) return;
  L[i] = lp;
  belief[i] = 0.0f;
}

// set_channel_kernel (gvdbkernels.cu:1040-1064): write occupancies of points
// (voxel units) into the belief field
__global__ void k_set_points(Geom g, const float* __restrict__ pts, const float* __restrict__ occ,
                             int64_t n, float* __restrict__ belief) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float px = pts[3 * i], py = pts[3 * i + 1], pz = pts[3 * i + 2];
  if (!(px >= 0.0f && py >= 0.0f && pz >= 0.0f && px < (float)g.E[0] && py < (float)g.E[1] &&
        pz < (float)g.E[2]))
    return;
  int vx = (int)floorf(px), vy = (int)floorf(py), vz = (int)floorf(pz);
  int s = g.brick_slot[brick_lin(g, vx, vy, vz)];
  if (s < 0) return;
  belief[(int64_t)s * kBrickVox + voxel_local(vx, vy, vz)] = occ[i];
}

// One thread per pixel walks the DDA through the active bricks.  Runs of
// voxels in one brick end with the reference's per-brick stop tests; the
// count pass and the emit pass execute the identical loop.  The emit pass
// keeps the last four incidences in registers (a shift register) and
// stores each aligned group of four as 16-byte vectors: ray offsets are
// multiples of four, so a ray's lists start on a group boundary, and the
// last group is completed with padding.  Every field of an incidence,
// including its build record, is known when it is emitted: the Post range
// ends at a brick-run boundary after which nothing more counts, and an
// incidence is dynamic once a non-zero potential has been seen inside it.
template <bool EMIT>
__global__ void __launch_bounds__(kThreads, 4)
    k_trace(Geom g, Pose P, const float* __restrict__ depth, uint32_t* __restrict__ counts,
            const uint32_t* __restrict__ pix_off, uint32_t inc_base, RayMeta* __restrict__ meta,
            uint32_t* __restrict__ inc_vox, float* __restrict__ inc_len,
            float* __restrict__ inc_mu, float2* __restrict__ inc_rec,
            int* __restrict__ err, const uint8_t* __restrict__ only, const int* __restrict__ only_all) {
  int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= g.rows * g.cols) return;
  // a checking count pass may be limited to the pixels marked in `only`
  // (unless *only_all is set)
  if (only && !*only_all && !only[pix]) return;
  float d = depth[pix];
  int count = 0, n_pre = -1, n_post = -1, r0 = -1, run_start = 0, kmu = -1;
  bool gate = false;
  uint32_t base = EMIT ? pix_off[pix] : 0;
  uint32_t bv[4] = {kNoVoxel, kNoVoxel, kNoVoxel, kNoVoxel};
  float bl[4] = {0.0f, 0.0f, 0.0f, 0.0f}, bm[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  uint32_t bf = 0;  // per slot: bit 0 in the Post range, bit 1 dynamic
  // shift one incidence into the group; store the group when it is whole
  auto push = [&](uint32_t v, float len, float mu, uint32_t f) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      bv[j] = bv[j + 1];
      bl[j] = bl[j + 1];
      bm[j] = bm[j + 1];
    }
    bv[3] = v;
    bl[3] = len;
    bm[3] = mu;
    bf = (bf >> 2) | (f << 6);
  };
  // build record: the length counting towards the cumulative length (Post
  // range only) and, for a dynamic incidence, -(mu * l) (the sign bit marks
  // the class; -0 when mu is 0)
  auto rec = [&](int j, float& pl, float& dl) {
    const uint32_t f = (bf >> (2 * j)) & 3u;
    pl = (f & 1u) ? bl[j] : 0.0f;
    dl = (f & 2u) ? -(bm[j] * pl) : 0.0f;
  };
  auto store = [&](uint32_t k0) {
    *reinterpret_cast<uint4*>(inc_vox + k0) = make_uint4(bv[0], bv[1], bv[2], bv[3]);
    *reinterpret_cast<float4*>(inc_len + k0) = make_float4(bl[0], bl[1], bl[2], bl[3]);
    *reinterpret_cast<float4*>(inc_mu + k0) = make_float4(bm[0], bm[1], bm[2], bm[3]);
    float p0, d0, p1, d1, p2, d2, p3, d3;
    rec(0, p0, d0);
    rec(1, p1, d1);
    rec(2, p2, d2);
    rec(3, p3, d3);
    float4* r = reinterpret_cast<float4*>(inc_rec + k0);
    r[0] = make_float4(p0, d0, p1, d1);
    r[1] = make_float4(p2, d2, p3, d3);
  };
  if (d > 0.0f) {
    int x = pix % g.cols, y = pix / g.cols;
    const float* sg = lut_at(g, g.sigma, x, y);
    const float* bs = lut_at(g, g.bias, x, y);
    const int n = g.lookup_n;
    Ray ray;
    ray_setup(g, P, x, y, ray);
    Dda r;
    if (dda_init(r, g, ray)) {
      int64_t cur = -1;
      int slot = -1;
      bool run_open = false;
      float s_last = 0.0f;
      int vx, vy, vz;
      float l, tin, te;
      while (dda_next(r, g, vx, vy, vz, l, tin, te)) {
        int64_t lin = brick_lin(g, vx, vy, vz);
        if (lin != cur) {
          if (run_open) {
            run_open = false;
            float lhs = fa(s_last, poly_f(bs, n, s_last));
            float rhs = fa(d, fm(3.0f, poly_f(sg, n, s_last)));
            if (n_post < 0 && lhs >= rhs) n_post = count;
            if (lhs > rhs) {
              n_pre = count;
              break;
            }
          }
          cur = lin;
          slot = g.brick_slot[lin];
        }
        if (slot < 0) continue;
        if (count >= kMaxRayLen) {
          atomicOr(err, 1);
          break;
        }
        float s = fm(te, ray.mult);
        if (!run_open) run_start = count;
        if (!EMIT && meta && (r0 < 0 || kmu < 0)) {
          // a checking count pass: the visibility-reset and dynamic starts
          // of the record it compares against
          const bool z = potential_is_zero(sg, bs, n, s, d);
          if (r0 < 0 && !z) r0 = run_start;
          if (kmu < 0 && !z) kmu = count;
        }
        if (EMIT) {
          const bool z = potential_is_zero(sg, bs, n, s, d);
          const float mu = z ? 0.0f : potential(sg, bs, n, s, d);
          if (r0 < 0 && !z) r0 = run_start;
          if (kmu < 0 && !z) kmu = count;
          // in the Post range until n_post is set; dynamic from the first
          // non-zero potential on
          const uint32_t in_post = n_post < 0 ? 1u : 0u;
          const uint32_t f = in_post | ((in_post && kmu >= 0) ? 2u : 0u);
          push((uint32_t)slot * kBrickVox + voxel_local(vx, vy, vz), l, mu, f);
          if ((count & 3) == 3) store(base + (uint32_t)(count - 3));
        }
        run_open = true;
        s_last = s;
        ++count;
      }
      if (n_pre < 0 && run_open) {
        float lhs = fa(s_last, poly_f(bs, n, s_last));
        float rhs = fa(d, fm(3.0f, poly_f(sg, n, s_last)));
        if (n_post < 0 && lhs >= rhs) n_post = count;
        if (lhs > rhs) n_pre = count;
      }
      if (n_pre < 0) {
        n_pre = count;
        if (count > 0) gate = d > fa(s_last, poly_f(bs, n, s_last));
      }
    }
  }
  if (n_pre < 0) n_pre = count;
  if (n_post < 0) n_post = count;
  // each ray's list is padded to a multiple of 4 incidences (16-byte vector
  // loads in the BP kernels); padding carries an invalid voxel id
  const int padded = (n_pre + 3) & ~3;
  if (!EMIT) {
    counts[pix] = (uint32_t)padded;
    if (meta) {
      // the view's stored records: does this trace still give the same list?
      const int kdyn = (kmu >= 0 && kmu < n_post) ? kmu : n_post;
      const RayMeta o = meta[pix];
      const uint32_t flags = (gate ? 1u : 0u) | ((uint32_t)kdyn << 16);
      if (o.n_pre != (uint16_t)n_pre || o.n_post != (uint16_t)n_post ||
          o.r0 != (uint16_t)(r0 >= 0 ? r0 : n_pre) || o.rinf != (uint16_t)(r0 >= 0 ? r0 : run_start) ||
          o.flags != flags)
        err[1] = 1;
    }
  } else {
    // the last group, completed with padding (invalid voxel, zeros)
    if (count & 3) {
      const int k0 = count & ~3;
      for (int k = count; k < padded; ++k) push(kNoVoxel, 0.0f, 0.0f, 0u);
      store(base + (uint32_t)k0);
    }
    const int kdyn = (kmu >= 0 && kmu < n_post) ? kmu : n_post;
    RayMeta m;
    m.off = inc_base + base;
    m.n_pre = (uint16_t)n_pre;
    m.n_post = (uint16_t)n_post;
    m.r0 = (uint16_t)(r0 >= 0 ? r0 : n_pre);
    m.rinf = (uint16_t)(r0 >= 0 ? r0 : run_start);
    m.flags = (gate ? 1u : 0u) | ((uint32_t)kdyn << 16);
    meta[pix] = m;
  }
}

// Pairs, first in voxel order.  The view's incidences are sorted by voxel
// id (stable: increasing incidence index inside a voxel); each run of one
// voxel is a (camera, voxel) pair.  perm[k] is the incidence at
// pair-grouped position k; seg[p] the first position of pair p.  The pairs
// are then renumbered (k_pair_first below) and the positions regrouped.
__global__ void k_vox_heads(const uint32_t* __restrict__ sk, uint32_t n, uint32_t* __restrict__ flag) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) flag[k] = (k == 0 || sk[k] != sk[k - 1]) ? 1u : 0u;
}

__global__ void k_pairs_from_sorted(const uint32_t* __restrict__ sk, const uint32_t* __restrict__ sidx,
                                    const uint32_t* __restrict__ flag,
                                    const uint32_t* __restrict__ scan, uint32_t n,
                                    uint32_t pair_base, uint32_t perm_base, uint32_t inc_base,
                                    uint32_t* __restrict__ pair_vox, uint32_t* __restrict__ seg,
                                    uint32_t* __restrict__ inc_pair) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  uint32_t p = pair_base + scan[k] + flag[k] - 1;
  if (flag[k]) {
    pair_vox[p] = sk[k];
    seg[p] = perm_base + k;
  }
  if (inc_pair) inc_pair[inc_base + sidx[k]] = p;
}

// Pair numbering, brick-major by first visit.  The pairs of a view are
// first found in voxel order (a stable sort of the incidences by voxel);
// they are then renumbered by the first visit of their brick (the lowest
// incidence index -- pixel order, then along the ray -- over the brick's
// pairs) and, within a brick, by their own first visit, and the
// pair-grouped incidence order is rebuilt in the new pair order.  Rays of
// neighbouring pixels cross the same bricks and voxels in the same order,
// so the pair ids met along a ray come in runs of nearby ids (the ray
// kernel's ln q gathers share sectors), while a brick's pairs stay together
// (the per-pair kernels' L accesses stay within the brick).
//   key[p]         = first incidence of pair p (its first sorted position
//                    holds it, the sort being stable)
//   bfirst[brick]  = min key over the brick's pairs
//   order[q]       = old pair of new pair q; slot_of[old] = q
__global__ void k_pair_first(const uint32_t* __restrict__ seg, uint32_t np, uint32_t perm_base,
                             const uint32_t* __restrict__ sidx, uint32_t* __restrict__ key) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < np) key[p] = sidx[seg[p] - perm_base];
}

// pairs come in voxel order, so a warp's lanes mostly share a brick: the
// lanes of one brick reduce among themselves and one of them does the atomic
__global__ void k_brick_first(const uint32_t* __restrict__ pair_vox, const uint32_t* __restrict__ key,
                              uint32_t np, uint32_t* __restrict__ bfirst) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  const bool ok = p < np;
  const uint32_t b = ok ? pair_vox[p] / kBrickVox : 0xFFFFFFFFu;
  const uint32_t k = ok ? key[p] : 0xFFFFFFFFu;
  const unsigned same = __match_any_sync(0xFFFFFFFFu, b);
  const uint32_t m = __reduce_min_sync(same, k);
  if (ok && (threadIdx.x & 31) == (unsigned)(__ffs(same) - 1)) atomicMin(bfirst + b, m);
}

// second sort key: pairs on quiet voxels last (bit `bits` set), then the
// brick's first visit
__global__ void k_brick_keys(const uint32_t* __restrict__ order, uint32_t np,
                             const uint32_t* __restrict__ pair_vox, const uint32_t* __restrict__ bfirst,
                             const uint8_t* __restrict__ loud, int bits, uint32_t* __restrict__ key) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const uint32_t v = pair_vox[order[i]];
  key[i] = bfirst[v / kBrickVox] | (loud[v] ? 0u : (1u << bits));
}

// loud[v] = 1 for every voxel with a dynamic incidence (any view): one
// thread per ray walks its dynamic range [k_dyn, n_post); vox[k] holds the
// voxel of incidence vox_base + k
__global__ void k_loud_voxels(const RayMeta* __restrict__ meta, int64_t npix, const uint32_t* __restrict__ vox,
                              uint32_t vox_base, uint8_t* __restrict__ loud) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= npix) return;
  const RayMeta me = meta[r];
  for (int i = ray_kdyn(me); i < me.n_post; ++i) loud[vox[me.off - vox_base + i]] = 1;
}

__global__ void k_loud_voxels_from_pairs(const RayMeta* __restrict__ meta, int64_t npix,
                                         const uint32_t* __restrict__ inc_pair,
                                         const uint32_t* __restrict__ pair_vox, uint8_t* __restrict__ loud) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= npix) return;
  const RayMeta me = meta[r];
  for (int i = ray_kdyn(me); i < me.n_post; ++i) loud[pair_vox[inc_pair[me.off + i]]] = 1;
}

// *count += number of pairs on loud voxels
__global__ void k_count_loud(const uint32_t* __restrict__ pair_vox, uint32_t np,
                             const uint8_t* __restrict__ loud, uint32_t* __restrict__ count) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  const bool l = p < np && loud[pair_vox[p]];
  const unsigned b = __ballot_sync(0xFFFFFFFFu, l);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(count, (uint32_t)__popc(b));
}

// run lengths in the new order and the old -> new map
__global__ void k_new_lengths(const uint32_t* __restrict__ order, uint32_t np, const uint32_t* __restrict__ seg,
                              uint32_t* __restrict__ len, uint32_t* __restrict__ slot_of) {
  uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= np) return;
  const uint32_t p = order[q];
  len[q] = seg[p + 1] - seg[p];
  slot_of[p] = q;
}

// every sorted position k moves to its pair's new run (out_idx: incidence
// index in the new pair-grouped order), and its incidence gets the new
// pair id
__global__ void k_move_positions(const uint32_t* __restrict__ sidx, const uint32_t* __restrict__ flag,
                                 const uint32_t* __restrict__ scan, const uint32_t* __restrict__ seg,
                                 const uint32_t* __restrict__ slot_of, const uint32_t* __restrict__ start,
                                 uint32_t n, uint32_t inc_base, uint32_t pair_base,
                                 uint32_t* __restrict__ out_idx, uint32_t* __restrict__ inc_pair) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t p = scan[k] + flag[k] - 1;
  const uint32_t q = slot_of[p];
  const uint32_t i = sidx[k];
  out_idx[start[q] + (k - seg[p])] = i;
  inc_pair[inc_base + i] = pair_base + q;
}

// the renumbered pairs: voxel and first pair-grouped position of new pair q
__global__ void k_pairs_renumbered(const uint32_t* __restrict__ order, uint32_t np,
                                   const uint32_t* __restrict__ vox_old, const uint32_t* __restrict__ start,
                                   uint32_t pair_base, uint32_t perm_base, uint32_t* __restrict__ pair_vox,
                                   uint32_t* __restrict__ seg) {
  uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q > np) return;
  if (q < np) pair_vox[pair_base + q] = vox_old[order[q]];
  seg[pair_base + q] = perm_base + start[q];  // start[np] = the view's position count
}

// build records in pair-grouped (sorted) order: one gather per position
__global__ void k_gather_rec(const uint32_t* __restrict__ sidx, uint32_t n, uint32_t inc_base,
                             const float2* __restrict__ rec, float2* __restrict__ out,
                             uint32_t* __restrict__ dflag) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float2 r = rec[inc_base + sidx[k]];
  out[k] = r;
  dflag[k] = signbit(r.y) ? 1u : 0u;  // a dynamic incidence (the record's class bit)
}

// Per pair: cumulative length, the sum of its static messages F_EPS * l
// (each product rounded as the ray kernel rounds it), the number of dynamic
// incidences and the potential mass sum mu * l (a warm-start feature).  The
// sums are carried as unevaluated FP32 pairs (s, e) updated by an
// error-free two-sum (Knuth's TwoSum: e collects every rounding error of
// s), i.e. to about twice FP32's precision, and rounded once through FP64
// at the end, so their value does not depend on the summation order (the
// reference adds with float atomics in no fixed order).  GB300 issues FP64
// at 1/64 of the FP32 rate: plain FP64 accumulation made this kernel
// FP64-bound.  A thread sums a pair's contiguous run of sorted records;
// runs longer than kLongRun (voxels next to a camera, crossed by up to
// ~10^5 rays) are appended to a list and summed by a whole block each.
constexpr uint32_t kLongRun = 512;
constexpr int kStatThreads = 256;

struct F2 {
  float s, e;
  __device__ __forceinline__ void add(float x) {
    const float t = __fadd_rn(s, x);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(x, bp));
    e = __fadd_rn(e, err);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)e; }
};

struct PairSums {
  F2 c, st, h;
  uint32_t nd;
};

__device__ __forceinline__ void add_rec(PairSums& a, const float2 r) {
  a.c.add(r.x);
  if (signbit(r.y)) {
    a.h.add(-r.y);
    ++a.nd;
  } else {
    a.st.add(__fmul_rn(kFEps, r.x));
  }
}

__device__ __forceinline__ void store_sums(uint32_t p, double c, double st, double h, uint32_t nd,
                                           float* __restrict__ cum, float* __restrict__ stat,
                                           uint32_t* __restrict__ ndyn, float* __restrict__ hit) {
  cum[p] = (float)c;
  stat[p] = (float)st;
  ndyn[p] = nd;
  hit[p] = (float)h;
}

__global__ void k_pair_stats(const uint32_t* __restrict__ seg, uint32_t p0, uint32_t np, uint32_t perm_base,
                             const float2* __restrict__ srec, float* __restrict__ cum,
                             float* __restrict__ stat, uint32_t* __restrict__ ndyn,
                             float* __restrict__ hit, uint32_t* __restrict__ long_list) {
  uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= np) return;
  uint32_t p = p0 + q;
  const uint32_t k0 = seg[p] - perm_base, k1 = seg[p + 1] - perm_base;
  if (k1 - k0 > kLongRun) {
    long_list[1 + atomicAdd(long_list, 1u)] = p;
    return;
  }
  PairSums a{{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, 0u};
  for (uint32_t k = k0; k < k1; ++k) add_rec(a, srec[k]);
  store_sums(p, a.c.value(), a.st.value(), a.h.value(), a.nd, cum, stat, ndyn, hit);
}

// one block per listed long run; block sums in a fixed tree order
__global__ void __launch_bounds__(kStatThreads)
    k_pair_stats_long(const uint32_t* __restrict__ seg, uint32_t perm_base, const float2* __restrict__ srec,
                      const uint32_t* __restrict__ long_list, float* __restrict__ cum,
                      float* __restrict__ stat, uint32_t* __restrict__ ndyn, float* __restrict__ hit) {
  __shared__ double sc[kStatThreads], sst[kStatThreads], sh[kStatThreads];
  __shared__ uint32_t snd[kStatThreads];
  const uint32_t n = long_list[0];
  for (uint32_t j = blockIdx.x; j < n; j += gridDim.x) {
    const uint32_t p = long_list[1 + j];
    const uint32_t k0 = seg[p] - perm_base, k1 = seg[p + 1] - perm_base;
    PairSums a{{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, 0u};
    for (uint32_t k = k0 + threadIdx.x; k < k1; k += kStatThreads) add_rec(a, srec[k]);
    sc[threadIdx.x] = a.c.value();
    sst[threadIdx.x] = a.st.value();
    sh[threadIdx.x] = a.h.value();
    snd[threadIdx.x] = a.nd;
    __syncthreads();
    for (int o = kStatThreads / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) {
        sc[threadIdx.x] += sc[threadIdx.x + o];
        sst[threadIdx.x] += sst[threadIdx.x + o];
        sh[threadIdx.x] += sh[threadIdx.x + o];
        snd[threadIdx.x] += snd[threadIdx.x + o];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) store_sums(p, sc[0], sst[0], sh[0], snd[0], cum, stat, ndyn, hit);
    __syncthreads();
  }
}

__global__ void k_dyn_scatter(const uint32_t* __restrict__ sidx, const uint32_t* __restrict__ flag,
                              const uint32_t* __restrict__ scan, uint32_t n, uint32_t inc_base,
                              uint32_t dperm_base, uint32_t* __restrict__ dperm) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n && flag[k]) dperm[dperm_base + scan[k]] = inc_base + sidx[k];
}

__global__ void k_dpair_flags(const uint32_t* __restrict__ ndyn, uint32_t p0, uint32_t np,
                              uint32_t* __restrict__ flag) {
  uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < np) flag[q] = ndyn[p0 + q] ? 1u : 0u;
}

__global__ void k_dpairs(const uint32_t* __restrict__ pflag, const uint32_t* __restrict__ pscan,
                         uint32_t p0, uint32_t np, const uint32_t* __restrict__ seg, uint32_t perm_base,
                         const uint32_t* __restrict__ dscan, uint32_t dperm_base, uint32_t dpair_base,
                         uint32_t* __restrict__ dpair, uint32_t* __restrict__ dseg) {
  uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= np || !pflag[q]) return;
  uint32_t j = dpair_base + pscan[q];
  dpair[j] = p0 + q;
  // the run keeps the pair grouping: it starts at the dynamic rank of the
  // pair's first position
  dseg[j] = dperm_base + dscan[seg[p0 + q] - perm_base];
}

__global__ void k_iota(uint32_t* out, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = i;
}

}  // namespace

cudaError_t launch_clean_depth(const float* in, float* out, int rows, int cols, cudaStream_t s) {
  k_clean_depth<<<grid_for((int64_t)rows * cols), kThreads, 0, s>>>(in, out, rows, cols);
  return cudaGetLastError();
}

cudaError_t launch_activate(const Geom& g, const Pose& P, const float* depth, int policy,
                            uint8_t* flags, cudaStream_t s) {
  k_activate<<<grid_for((int64_t)g.rows * g.cols, 128), 128, 0, s>>>(g, P, depth, policy, flags);
  return cudaGetLastError();
}

cudaError_t launch_activate_points(const Geom& g, const float* pts, int64_t n, uint8_t* flags,
                                   cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_activate_points<<<grid_for(n), kThreads, 0, s>>>(g, pts, n, flags);
  return cudaGetLastError();
}

cudaError_t launch_new_indicator(const uint8_t* flags, const int* slot, int* ind, int64_t n,
                                 cudaStream_t s) {
  k_new_indicator<<<grid_for(n), kThreads, 0, s>>>(flags, slot, ind, n);
  return cudaGetLastError();
}

cudaError_t launch_assign_slots2(const Geom& g, const int* ind, const int* scan, int nb_base,
                                 int* brick_slot, int* brick_coord, int64_t n, cudaStream_t s) {
  k_assign_slots<<<grid_for(n), kThreads, 0, s>>>(g, ind, scan, nb_base, brick_slot, brick_coord, n);
  return cudaGetLastError();
}

cudaError_t launch_fill_new_voxels(float* L, float* belief, int64_t v0, int64_t v1, float lp,
                                   cudaStream_t s) {
  if (v1 <= v0) return cudaSuccess;
  k_fill_new_voxels<<<grid_for(v1 - v0), kThreads, 0, s>>>(L, belief, v0, v1, lp);
  return cudaGetLastError();
}

cudaError_t launch_set_points(const Geom& g, const float* pts, const float* occ, int64_t n,
                              float* belief, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_set_points<<<grid_for(n), kThreads, 0, s>>>(g, pts, occ, n, belief);
  return cudaGetLastError();
}

cudaError_t launch_trace_count(const Geom& g, const Pose& P, const float* depth, uint32_t* counts,
                               int* err, cudaStream_t s, const RayMeta* check, const uint8_t* only,
                               const int* only_all) {
  k_trace<false><<<grid_for((int64_t)g.rows * g.cols), kThreads, 0, s>>>(
      g, P, depth, counts, nullptr, 0, const_cast<RayMeta*>(check), nullptr, nullptr, nullptr, nullptr, err, only,
      only_all);
  return cudaGetLastError();
}

// The pixels of a view whose rays may cross one of the bricks in slots
// b0..b1 (bricks activated after the view's lists were built): each brick's
// eight corners projected through the view's camera (the inverse of
// ray_setup: a pixel's ray projects onto that pixel), the box of the
// projections widened by a pixel against rounding, marked in mask.  A brick
// with a corner at or behind the camera plane, or whose box covers more
// than a quarter of the image, sets *all instead (every pixel is checked).
__global__ void k_brick_footprint(Geom g, Pose P, const int* __restrict__ coord, uint32_t b0, uint32_t b1,
                                  uint8_t* __restrict__ mask, int* __restrict__ all) {
  const uint32_t b = b0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= b1) return;
  const float o0 = fa(fd(P.m[3], g.res), g.off[0]);
  const float o1 = fa(fd(P.m[7], g.res), g.off[1]);
  const float o2 = fa(fd(P.m[11], g.res), g.off[2]);
  const float kx = g.fx / g.cx, ky = g.fy / g.cy;
  float x_lo = 3.0e38f, x_hi = -3.0e38f, y_lo = 3.0e38f, y_hi = -3.0e38f;
  for (int k = 0; k < 8; ++k) {
    const float v0 = (float)(kBrick * (coord[3 * b + 0] + (k & 1))) - o0;
    const float v1 = (float)(kBrick * (coord[3 * b + 1] + ((k >> 1) & 1))) - o1;
    const float v2 = (float)(kBrick * (coord[3 * b + 2] + ((k >> 2) & 1))) - o2;
    const float xc = P.m[0] * v0 + P.m[4] * v1 + P.m[8] * v2;
    const float yc = P.m[1] * v0 + P.m[5] * v1 + P.m[9] * v2;
    const float zc = P.m[2] * v0 + P.m[6] * v1 + P.m[10] * v2;
    if (!(zc > 1e-3f)) {
      atomicExch(all, 1);
      return;
    }
    const float px = (xc / zc * kx + 1.0f) * 0.5f * (float)g.cols - 0.5f;
    const float py = (yc / zc * ky + 1.0f) * 0.5f * (float)g.rows - 0.5f;
    x_lo = fminf(x_lo, px);
    x_hi = fmaxf(x_hi, px);
    y_lo = fminf(y_lo, py);
    y_hi = fmaxf(y_hi, py);
  }
  const int x0 = max(0, (int)floorf(fmaxf(x_lo, -4.0f)) - 1);
  const int x1 = min(g.cols - 1, (int)ceilf(fminf(x_hi, (float)g.cols + 4.0f)) + 1);
  const int y0 = max(0, (int)floorf(fmaxf(y_lo, -4.0f)) - 1);
  const int y1 = min(g.rows - 1, (int)ceilf(fminf(y_hi, (float)g.rows + 4.0f)) + 1);
  if (x0 > x1 || y0 > y1) return;
  if ((int64_t)(x1 - x0 + 1) * (y1 - y0 + 1) * 4 > (int64_t)g.rows * g.cols) {
    atomicExch(all, 1);
    return;
  }
  for (int y = y0; y <= y1; ++y)
    for (int x = x0; x <= x1; ++x) mask[y * g.cols + x] = 1;
}

cudaError_t launch_brick_footprint(const Geom& g, const Pose& P, const int* coord, uint32_t b0, uint32_t b1,
                                   uint8_t* mask, int* all, cudaStream_t s) {
  if (b1 <= b0) return cudaSuccess;
  k_brick_footprint<<<grid_for(b1 - b0), kThreads, 0, s>>>(g, P, coord, b0, b1, mask, all);
  return cudaGetLastError();
}

cudaError_t launch_trace_emit(const Geom& g, const Pose& P, const float* depth,
                              const uint32_t* pix_off, uint32_t inc_base, RayMeta* meta,
                              uint32_t* inc_vox, float* inc_len, float* inc_mu, float2* inc_rec,
                              int* err, cudaStream_t s) {
  k_trace<true><<<grid_for((int64_t)g.rows * g.cols), kThreads, 0, s>>>(
      g, P, depth, nullptr, pix_off, inc_base, meta, inc_vox, inc_len, inc_mu, inc_rec, err, nullptr, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_vox_heads(const uint32_t* sk, uint32_t n, uint32_t* flag, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_vox_heads<<<grid_for(n), kThreads, 0, s>>>(sk, n, flag);
  return cudaGetLastError();
}

cudaError_t launch_pairs_from_sorted(const uint32_t* sk, const uint32_t* sidx, const uint32_t* flag,
                                     const uint32_t* scan, uint32_t n, uint32_t pair_base,
                                     uint32_t perm_base, uint32_t inc_base, uint32_t* pair_vox,
                                     uint32_t* seg, uint32_t* inc_pair, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_pairs_from_sorted<<<grid_for(n), kThreads, 0, s>>>(sk, sidx, flag, scan, n, pair_base, perm_base,
                                                       inc_base, pair_vox, seg, inc_pair);
  return cudaGetLastError();
}

cudaError_t launch_pair_first(const uint32_t* seg, uint32_t np, uint32_t perm_base, const uint32_t* sidx,
                              uint32_t* key, cudaStream_t s) {
  if (!np) return cudaSuccess;
  k_pair_first<<<grid_for(np), kThreads, 0, s>>>(seg, np, perm_base, sidx, key);
  return cudaGetLastError();
}

cudaError_t launch_brick_first(const uint32_t* pair_vox, const uint32_t* key, uint32_t np, uint32_t* bfirst,
                               cudaStream_t s) {
  if (!np) return cudaSuccess;
  k_brick_first<<<grid_for(np), kThreads, 0, s>>>(pair_vox, key, np, bfirst);
  return cudaGetLastError();
}

cudaError_t launch_brick_keys(const uint32_t* order, uint32_t np, const uint32_t* pair_vox,
                              const uint32_t* bfirst, const uint8_t* loud, int bits, uint32_t* key,
                              cudaStream_t s) {
  if (!np) return cudaSuccess;
  k_brick_keys<<<grid_for(np), kThreads, 0, s>>>(order, np, pair_vox, bfirst, loud, bits, key);
  return cudaGetLastError();
}

cudaError_t launch_loud_voxels(const RayMeta* meta, int64_t npix, const uint32_t* vox, uint32_t vox_base,
                               uint8_t* loud, cudaStream_t s) {
  if (npix <= 0) return cudaSuccess;
  k_loud_voxels<<<grid_for(npix), kThreads, 0, s>>>(meta, npix, vox, vox_base, loud);
  return cudaGetLastError();
}

cudaError_t launch_loud_voxels_from_pairs(const RayMeta* meta, int64_t npix, const uint32_t* inc_pair,
                                          const uint32_t* pair_vox, uint8_t* loud, cudaStream_t s) {
  if (npix <= 0) return cudaSuccess;
  k_loud_voxels_from_pairs<<<grid_for(npix), kThreads, 0, s>>>(meta, npix, inc_pair, pair_vox, loud);
  return cudaGetLastError();
}

cudaError_t launch_count_loud(const uint32_t* pair_vox, uint32_t np, const uint8_t* loud, uint32_t* count,
                              cudaStream_t s) {
  if (!np) return cudaSuccess;
  k_count_loud<<<grid_for(np), kThreads, 0, s>>>(pair_vox, np, loud, count);
  return cudaGetLastError();
}

cudaError_t launch_new_lengths(const uint32_t* order, uint32_t np, const uint32_t* seg, uint32_t* len,
                               uint32_t* slot_of, cudaStream_t s) {
  if (!np) return cudaSuccess;
  k_new_lengths<<<grid_for(np), kThreads, 0, s>>>(order, np, seg, len, slot_of);
  return cudaGetLastError();
}

cudaError_t launch_move_positions(const uint32_t* sidx, const uint32_t* flag, const uint32_t* scan,
                                  const uint32_t* seg, const uint32_t* slot_of, const uint32_t* start, uint32_t n,
                                  uint32_t inc_base, uint32_t pair_base, uint32_t* out_idx, uint32_t* inc_pair,
                                  cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_move_positions<<<grid_for(n), kThreads, 0, s>>>(sidx, flag, scan, seg, slot_of, start, n, inc_base,
                                                    pair_base, out_idx, inc_pair);
  return cudaGetLastError();
}

cudaError_t launch_pairs_renumbered(const uint32_t* order, uint32_t np, const uint32_t* vox_old,
                                    const uint32_t* start, uint32_t pair_base, uint32_t perm_base,
                                    uint32_t* pair_vox, uint32_t* seg, cudaStream_t s) {
  k_pairs_renumbered<<<grid_for((int64_t)np + 1), kThreads, 0, s>>>(order, np, vox_old, start, pair_base,
                                                                  perm_base, pair_vox, seg);
  return cudaGetLastError();
}

cudaError_t launch_gather_rec(const uint32_t* sidx, uint32_t n, uint32_t inc_base, const float2* rec,
                              float2* out, uint32_t* dflag, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_gather_rec<<<grid_for(n), kThreads, 0, s>>>(sidx, n, inc_base, rec, out, dflag);
  return cudaGetLastError();
}

cudaError_t launch_pair_stats(const uint32_t* seg, uint32_t p0, uint32_t np, uint32_t perm_base,
                              const float2* srec, float* cum, float* stat, uint32_t* ndyn, float* hit,
                              uint32_t* long_list, cudaStream_t s) {
  if (!np) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(long_list, 0, 4, s);
  if (e != cudaSuccess) return e;
  k_pair_stats<<<grid_for(np), kThreads, 0, s>>>(seg, p0, np, perm_base, srec, cum, stat, ndyn, hit,
                                                 long_list);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_pair_stats_long<<<1024, kStatThreads, 0, s>>>(seg, perm_base, srec, long_list, cum, stat, ndyn, hit);
  return cudaGetLastError();
}

cudaError_t launch_dyn_scatter(const uint32_t* sidx, const uint32_t* flag, const uint32_t* scan,
                               uint32_t n, uint32_t inc_base, uint32_t dperm_base, uint32_t* dperm,
                               cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_dyn_scatter<<<grid_for(n), kThreads, 0, s>>>(sidx, flag, scan, n, inc_base, dperm_base, dperm);
  return cudaGetLastError();
}

cudaError_t launch_dpair_flags(const uint32_t* ndyn, uint32_t p0, uint32_t np, uint32_t* flag,
                               cudaStream_t s) {
  if (!np) return cudaSuccess;
  k_dpair_flags<<<grid_for(np), kThreads, 0, s>>>(ndyn, p0, np, flag);
  return cudaGetLastError();
}

cudaError_t launch_dpairs(const uint32_t* pflag, const uint32_t* pscan, uint32_t p0, uint32_t np,
                          const uint32_t* seg, uint32_t perm_base, const uint32_t* dscan,
                          uint32_t dperm_base, uint32_t dpair_base, uint32_t* dpair, uint32_t* dseg,
                          cudaStream_t s) {
  if (!np) return cudaSuccess;
  k_dpairs<<<grid_for(np), kThreads, 0, s>>>(pflag, pscan, p0, np, seg, perm_base, dscan, dperm_base,
                                            dpair_base, dpair, dseg);
  return cudaGetLastError();
}

cudaError_t launch_iota(uint32_t* out, uint32_t n, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_iota<<<grid_for(n), kThreads, 0, s>>>(out, n);
  return cudaGetLastError();
}

size_t scan_temp_bytes(uint32_t n) {
  size_t b = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, b, (const uint32_t*)nullptr, (uint32_t*)nullptr, (int)n);
  return b;
}

cudaError_t exclusive_scan_u32(void* tmp, size_t tmp_bytes, const uint32_t* in, uint32_t* out,
                               uint32_t n, cudaStream_t s) {
  return cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, in, out, (int)n, s);
}

size_t scan_temp_bytes_i32(int64_t n) {
  size_t b = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, b, (const int*)nullptr, (int*)nullptr, (int)n);
  return b;
}

cudaError_t exclusive_scan_i32(void* tmp, size_t tmp_bytes, const int* in, int* out, int64_t n,
                               cudaStream_t s) {
  return cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, in, out, (int)n, s);
}

size_t sort_temp_bytes(uint32_t n, int bits) {
  size_t b = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, b, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                  (const uint32_t*)nullptr, (uint32_t*)nullptr, (int)n, 0, bits);
  return b;
}

cudaError_t sort_pairs_u32(void* tmp, size_t tmp_bytes, const uint32_t* kin, uint32_t* kout,
                           const uint32_t* vin, uint32_t* vout, uint32_t n, int bits,
                           cudaStream_t s) {
  return cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, kin, kout, vin, vout, (int)n, 0, bits, s);
}

}  // namespace mrf
