// mrf_capi.cu -- the C ABI (include/mrfmap_gb300.h): map object, device
// memory, the build of the incidence lists and the BP schedule.
//
// Layout in HBM (one map):
//   brick table    int32 [NB0*NB1*NB2]       dense brick grid -> pool slot
//   voxel state    fp32 L, fp32 belief        [slots*512], slot-major,
//                                              voxel (x*8+y)*8+z in a slot
//   rays           RayMeta [views*rows*cols]  pixel-major per view
//   incidences     u32 pair, fp32 len, fp32 mu, fp32 p*l   [N_inc]
//                  ray order (pixel-major, then along the ray), each ray
//                  padded to a multiple of 4
//   pairs          u32 voxel, fp32 m, fp32 cum_len, fp32 ln q, fp32 dm,
//                  u32 seg   [N_cv]; per view the pairs on voxels with a
//                  dynamic incidence first, each part brick-major by first
//                  visit along the rays (mrf_build.cu, k_pair_first)
//   grouped        u32 incidence per pair-grouped position [N_pre] (CSR
//                  by pair; the dynamic positions again in dperm)
//   ray queues     RayMeta records in queue order: longest first, and the
//                  SM-affine regions (home rays per region, leftovers)
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <mutex>
#include <thread>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mrfmap_gb300.h"
#include "mrf_internal.h"


using namespace mrf;

namespace {

thread_local std::string g_last_error;

struct Fail {
  mrf_status st;
};

void set_err(const std::string& s) { g_last_error = s; }

#define CK(expr)                                                                          \
  do {                                                                                    \
    cudaError_t _e = (expr);                                                              \
    if (_e != cudaSuccess) {                                                              \
      set_err(std::string(#expr) + ": " + cudaGetErrorString(_e));                        \
      throw Fail{_e == cudaErrorMemoryAllocation ? MRF_ERR_OOM : MRF_ERR_CUDA};           \
    }                                                                                     \
  } while (0)

void fail(mrf_status st, const std::string& msg) {
  set_err(msg);
  throw Fail{st};
}

// Device memory of every map comes from one stream-ordered pool per
// device that keeps freed blocks for reuse (release threshold: never), so a
// map built after another one allocates nothing from the driver and
// destroying a map does not wait on cudaFree.  mrf_release_cached_memory
// hands the pooled blocks back.
constexpr int kMaxDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pools[kMaxDevices] = {};

cudaMemPool_t map_pool() {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) fail(MRF_ERR_INVALID, "device index out of range");
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if (!g_pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    CK(cudaMemPoolCreate(&pool, &props));
    uint64_t keep_all = ~0ull;
    CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep_all));
    g_pools[dev] = pool;
  }
  return g_pools[dev];
}

// Bytes the maps of this process hold per device, and the optional bound
// on them (mrf_set_memory_limit; 0 = none).  A buffer that would grow past
// the bound fails with MRF_ERR_OOM before anything is allocated.
std::atomic<int64_t> g_in_use[kMaxDevices];
std::atomic<int64_t> g_limit{0};

// growable device buffer (stream-ordered on the stream that last sized it)
struct DBuf {
  void* p = nullptr;
  size_t cap = 0;
  int dev = 0;
  cudaStream_t owner = nullptr;
  void reserve(size_t bytes, bool keep, cudaStream_t s) {
    if (bytes <= cap) return;
    size_t nc = std::max(bytes, cap + cap / 2);
    int d = 0;
    CK(cudaGetDevice(&d));
    if (d < 0 || d >= kMaxDevices) fail(MRF_ERR_INVALID, "device index out of range");
    const int64_t lim = g_limit.load();
    if (lim > 0 && g_in_use[d].load() + (int64_t)nc > lim) {
      // a buffer as large as the request itself may still fit where the
      // growth margin does not
      nc = bytes;
      if (g_in_use[d].load() + (int64_t)nc > lim)
        fail(MRF_ERR_OOM, "device memory limit reached (" + std::to_string(g_in_use[d].load()) + " + " +
                              std::to_string(nc) + " bytes > " + std::to_string(lim) + ")");
    }
    void* q = nullptr;
    CK(cudaMallocFromPoolAsync(&q, nc, map_pool(), s));
    g_in_use[d] += (int64_t)nc;
    if (keep && p && cap) CK(cudaMemcpyAsync(q, p, cap, cudaMemcpyDeviceToDevice, s));
    if (p) {
      CK(cudaFreeAsync(p, s));
      g_in_use[dev] -= (int64_t)cap;
    }
    p = q;
    cap = nc;
    dev = d;
    owner = s;
  }
  void release() {
    if (p) {
      cudaFreeAsync(p, owner);
      g_in_use[dev] -= (int64_t)cap;
    }
    p = nullptr;
    cap = 0;
  }
  template <typename T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

struct View {
  Pose pose;
  Geom cam;                  // the map geometry with this view's camera
  int64_t pix_base = 0;      // first pixel of the view in the per-pixel arrays
  DBuf depth;
  uint32_t inc_base = 0, n_inc = 0;
  uint32_t pair_base = 0, n_pairs = 0;
  uint32_t perm_base = 0, n_perm = 0;     // pair-grouped positions of all incidences
  uint32_t dperm_base = 0, n_dperm = 0;   // ... of the dynamic ones
  uint32_t dpair_base = 0, n_dpairs = 0;  // runs of dynamic incidences (one per pair)
  uint32_t order_base = 0, n_active = 0;  // ray queue (longest first)
  uint32_t left_base = 0, n_left = 0;     // leftover queue of the SM-affine schedule
  uint32_t n_loud = 0;                    // pairs on voxels with a dynamic incidence (numbered first)
  uint32_t tile_base = 0;                 // first pair of each pair-update tile
  bool retired = false;                   // out of the window: no lists, no pairs, no depth
  // counters of the view's rays (incidences, rays, Post incidences, dynamic
  // incidences, rays the ray kernel runs over and their Pre incidences)
  int64_t c_npre = 0, c_nrays = 0, c_npost = 0, c_ndyn = 0, c_nrays_bp = 0, c_npre_bp = 0, c_nfast_bp = 0;
};

// pixels a view contributes to the per-pixel arrays (none once retired)
int64_t view_pixels(const View& v) { return v.retired ? 0 : (int64_t)v.cam.rows * v.cam.cols; }

uint32_t u32_checked(int64_t v, const char* what) {
  if (v < 0 || v > (int64_t)0xFFFFFFF0ll) fail(MRF_ERR_CAPACITY, std::string(what) + " exceeds 32-bit range");
  return (uint32_t)v;
}

}  // namespace

constexpr int kHomeShare = 75;  // default per cent of a region's incidences taken by its home blocks

struct mrf_map {
  mrf_params prm;
  std::vector<float> sigma, bias;
  int device = 0, num_sms = 1;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  Geom g{};
  DBuf d_sigma, d_bias, d_slot, d_coord, d_L, d_belief;
  int64_t nb_grid = 0, n_bricks = 0;
  std::vector<int> h_coord;
  int version = 0, built_version = -1;
  int ray_variant = 4;  // ray-kernel variant (mrf_autotune / mrf_set_ray_variant); 4: SM regions,
                        // pair-id prefetch, the fastest on the bench workloads
  uint32_t nreg = 1;    // SM regions per view of the region queues
  // what the last build left: views with lists, per-pixel entries, the ends
  // of the region blocks, the queues and the tiles, the bricks it saw
  int built_views = 0;
  int64_t npix_total = 0, queue_end = 0, tile_end = 0, carry_tiles = 0, vox_active_n = 0, n_perm_total = 0;
  int64_t n_loud_prefix = 0;  // entries of the static prefixes' loud lists
  int64_t loud_count_version = -1, loud_list_version = -1;  // builds the loud lists were counted / made for
  uint32_t region_end = 0;
  int64_t bricks_at_build = -1;
  // holes: retired views' lists still in the arenas; appended: lists added
  // without a full build (the all-view structures of Jacobi are stale);
  // needs_full: the next build must rebuild every view
  bool holes = false, appended = false, needs_full = true;
  // test hook: the next append fails with this status once its pairs are
  // built (0: none)
  int test_append_fail = 0;
  // the build scratch s_vox / s_rec holds the incidences from this index on
  // (0 in a full build; an appended build's first new incidence, so the
  // scratch holds the new views only, not the arenas' retired lists)
  uint32_t scratch_base = 0;
  int64_t dead_inc = 0;
  bool has_messages = false;
  std::vector<View> views;
  // arenas
  DBuf meta, inc_pair, inc_len, inc_mu, inc_pl, pair_vox, pair_m, pair_cum, pair_stat, pair_ndyn, pair_hit,
      pair_q, pair_dm, pair_seg, dperm, s_q0, s_q1, s_q2, s_q3, s_bf, s_loud, s_pv, s_sg, dpair, dseg, drun, carry, ray_order, ray_queue, region_q, rstart, rcounters, counters,
      tile_first, lbase, lsingle, lprefix, queue_ids, region_ids, loud_off, loud_pid, loud_len, loud_pos,
      quiet_q;
  uint32_t jac_tile_base = 0;
  int64_t n_inc = 0, n_pairs = 0, n_dperm = 0, n_dpairs = 0;
  // voxels with a pair past the length gate (their beliefs follow L)
  DBuf vox_active;
  // MRF_PRECISION_HALF_STREAMS: fp16 copies of the segment lengths (per
  // build) and of ln q (written by k_pair_prepare)
  int precision = MRF_PRECISION_FP32;
  int home_share = kHomeShare;  // SM-region schedule: per cent of a region's work on its home blocks
  int pair_variant = 0;  // pair reduction variant (mrf_autotune_flags); same results
  DBuf inc_len16, pair_q16;
  int len16_version = -1;
  // logit(prior) + the messages of retired views, per voxel (kept once a view
  // has been retired; the prior alone before that)
  DBuf d_Lbase;
  bool has_base = false;
  // jacobi voxel CSR
  DBuf vseg, vpairs, vvox;
  uint32_t n_vvox = 0;
  int jacobi_version = -1;
  // scratch
  DBuf s_rec, s_recs, s_pf, s_ps, s_flags, s_ind, s_scan, s_tmp, s_counts, s_offs, s_vox, s_k0, s_k1, s_v0, s_v1,
      s_seg, s_dense, s_err, s_depth_in, s_depth, s_img, s_part, s_sum, s_prev, s_delta, s_snap, s_vcnt;
  mrf_stats stats{};
  // MRF_PROFILE event pool
  std::vector<cudaEvent_t> prof_ev;
  std::vector<int> prof_cat;
  // captured BP iteration per schedule (Jacobi bit, fixed-reset bit, the
  // phase of the iteration in its call (two bits), quiet-prefix bit)
  struct GraphSlot {
    cudaGraphExec_t exec = nullptr;
    int version = -1;
    int64_t launches = 0;
  } graphs[32];

  BpArrays bp() const {
    BpArrays a;
    a.meta = meta.as<RayMeta>();
    a.inc_pair = inc_pair.as<uint32_t>();
    a.inc_len = inc_len.as<float>();
    a.inc_mu = inc_mu.as<float>();
    a.inc_pl = inc_pl.as<float>();
    a.dperm = dperm.as<uint32_t>();
    a.dpair = dpair.as<uint32_t>();
    a.dseg = dseg.as<uint32_t>();
    a.drun = drun.as<uint4>();
    a.pair_vox = pair_vox.as<uint32_t>();
    a.pair_m = pair_m.as<float>();
    a.pair_cum = pair_cum.as<float>();
    a.pair_stat = pair_stat.as<float>();
    a.pair_ndyn = pair_ndyn.as<uint32_t>();
    a.pair_lnq = pair_q.as<float>();
    a.pair_dm = pair_dm.as<float>();
    a.L = d_L.as<float>();
    a.belief = d_belief.as<float>();
    a.half_streams = precision == MRF_PRECISION_HALF_STREAMS ? 1 : 0;
    a.pair_variant = pair_variant;
    a.quiet_q = quiet_q.as<float2>();
    a.loud_off = loud_off.as<uint32_t>();
    a.loud_pid = loud_pid.as<uint32_t>();
    a.loud_len = loud_len.as<float>();
    a.loud_pos = loud_pos.as<uint16_t>();
    a.inc_len16 = inc_len16.as<__half>();
    a.pair_lnq16 = pair_q16.as<__half>();
    return a;
  }
  int64_t hw() const { return (int64_t)prm.rows * prm.cols; }
};

namespace {

void sync(mrf_map* m) { CK(cudaStreamSynchronize(m->stream)); }

template <typename T>
T read1(mrf_map* m, const T* dptr) {
  T v;
  CK(cudaMemcpyAsync(&v, dptr, sizeof(T), cudaMemcpyDeviceToHost, m->stream));
  sync(m);
  return v;
}

void check_device_err(mrf_map* m) {
  int e = read1(m, m->s_err.as<int>());
  if (e) {
    CK(cudaMemsetAsync(m->s_err.p, 0, sizeof(int), m->stream));
    fail(MRF_ERR_DEVICE, "a kernel raised its error flag (ray longer than 65532 incidences)");
  }
}

// ---- activation --------------------------------------------------------
void commit_new_bricks(mrf_map* m) {
  int64_t n = m->nb_grid;
  m->s_ind.reserve((size_t)n * 4, false, m->stream);
  m->s_scan.reserve((size_t)n * 4, false, m->stream);
  CK(launch_new_indicator(m->s_flags.as<uint8_t>(), m->d_slot.as<int>(), m->s_ind.as<int>(), n,
                          m->stream));
  size_t tb = scan_temp_bytes_i32(n);
  m->s_tmp.reserve(tb, false, m->stream);
  CK(exclusive_scan_i32(m->s_tmp.p, tb, m->s_ind.as<int>(), m->s_scan.as<int>(), n, m->stream));
  int last_scan = read1(m, m->s_scan.as<int>() + (n - 1));
  int last_ind = read1(m, m->s_ind.as<int>() + (n - 1));
  int add = last_scan + last_ind;
  if (add == 0) return;
  int64_t nb_new = m->n_bricks + add;
  if ((nb_new * kBrickVox) > (int64_t)0xFFFFFFF0ll) fail(MRF_ERR_CAPACITY, "brick pool exceeds 32-bit voxel ids");
  m->d_coord.reserve((size_t)nb_new * 12, true, m->stream);
  m->d_L.reserve((size_t)nb_new * kBrickVox * 4, true, m->stream);
  m->d_belief.reserve((size_t)nb_new * kBrickVox * 4, true, m->stream);
  CK(launch_assign_slots2(m->g, m->s_ind.as<int>(), m->s_scan.as<int>(), (int)m->n_bricks,
                          m->d_slot.as<int>(), m->d_coord.as<int>(), n, m->stream));
  float lp = logf(m->prm.prior) - logf(1.0f - m->prm.prior);
  CK(launch_fill_new_voxels(m->d_L.as<float>(), m->d_belief.as<float>(), m->n_bricks * kBrickVox,
                            nb_new * kBrickVox, lp, m->stream));
  if (m->has_base) {
    m->d_Lbase.reserve((size_t)nb_new * kBrickVox * 4, true, m->stream);
    CK(launch_fill_f32(m->d_Lbase.as<float>() + m->n_bricks * kBrickVox, add * (int64_t)kBrickVox, lp,
                       m->stream));
  }
  m->h_coord.resize((size_t)nb_new * 3);
  CK(cudaMemcpyAsync(m->h_coord.data() + m->n_bricks * 3, m->d_coord.as<int>() + m->n_bricks * 3,
                     (size_t)add * 12, cudaMemcpyDeviceToHost, m->stream));
  sync(m);
  m->n_bricks = nb_new;
  m->version++;
}

void activate_view(mrf_map* m, const View& v) {
  CK(cudaMemsetAsync(m->s_flags.p, 0, (size_t)m->nb_grid, m->stream));
  m->g.brick_slot = m->d_slot.as<int>();
  Geom g = v.cam;
  g.brick_slot = m->d_slot.as<int>();
  CK(launch_activate(g, v.pose, v.depth.as<float>(), m->prm.activation, m->s_flags.as<uint8_t>(),
                     m->stream));
  commit_new_bricks(m);
}

// ---- incidence lists ---------------------------------------------------
// the pairs and messages of the previous build, kept while a new build
// runs so that every camera's messages move over to its new pairs
struct OldPairs {
  bool remap = false;
  int64_t n_pairs = 0;
  DBuf vox, m;
  std::vector<View> views;  // pair_base / n_pairs of each view
};

void rebuild_lists(mrf_map* m, OldPairs& old);

// A build that fails (device memory bound, device error flag) leaves the
// previous pairs and messages in place, so the next build can still move
// the messages over.
void rebuild(mrf_map* m) {
  OldPairs old;
  old.remap = m->has_messages && m->n_pairs > 0;
  old.n_pairs = m->n_pairs;
  if (old.remap) {
    old.vox = m->pair_vox;
    old.m = m->pair_m;
    m->pair_vox = DBuf{};
    m->pair_m = DBuf{};
    for (auto& v : m->views) {
      View c;
      c.pair_base = v.pair_base;
      c.n_pairs = v.n_pairs;
      old.views.push_back(std::move(c));
    }
  }
  try {
    rebuild_lists(m, old);
  } catch (...) {
    if (old.remap) {
      m->pair_vox.release();
      m->pair_m.release();
      m->pair_vox = old.vox;
      m->pair_m = old.m;
      m->n_pairs = old.n_pairs;
      for (size_t c = 0; c < old.views.size() && c < m->views.size(); ++c) {
        m->views[c].pair_base = old.views[c].pair_base;
        m->views[c].n_pairs = old.views[c].n_pairs;
      }
    }
    throw;
  }
}

// ---- per-view pieces of a build ------------------------------------------

// The counters of the given views' rays, summed on the device from their ray
// records (k_ray_counters), and the records of pixels [hm_base, hm_base +
// hm.size()) copied to the host for the region lists: one synchronisation.
void ray_records_and_counters(mrf_map* m, const std::vector<int>& views, int64_t hm_base,
                              std::vector<RayMeta>& hm) {
  const size_t K = (size_t)kRayCounters;
  m->s_vcnt.reserve(std::max<size_t>(views.size(), 1) * K * 8, false, m->stream);
  unsigned long long* dc = m->s_vcnt.as<unsigned long long>();
  for (size_t k = 0; k < views.size(); ++k) {
    const View& v = m->views[(size_t)views[k]];
    CK(launch_ray_counters(m->meta.as<RayMeta>() + v.pix_base, view_pixels(v), dc + k * K, m->stream));
  }
  std::vector<unsigned long long> hc(views.size() * K, 0ull);
  if (!hc.empty())
    CK(cudaMemcpyAsync(hc.data(), dc, hc.size() * 8, cudaMemcpyDeviceToHost, m->stream));
  if (!hm.empty())
    CK(cudaMemcpyAsync(hm.data(), m->meta.as<RayMeta>() + hm_base, hm.size() * sizeof(RayMeta),
                       cudaMemcpyDeviceToHost, m->stream));
  sync(m);
  check_device_err(m);
  for (size_t k = 0; k < views.size(); ++k) {
    View& v = m->views[(size_t)views[k]];
    const unsigned long long* c = hc.data() + k * K;
    v.c_npre = (int64_t)c[0];
    v.c_nrays = (int64_t)c[1];
    v.c_npost = (int64_t)c[2];
    v.c_ndyn = (int64_t)c[3];
    v.c_nrays_bp = (int64_t)c[4];
    v.c_npre_bp = (int64_t)c[5];
    v.c_nfast_bp = (int64_t)c[6];
  }
}

// The pairs of view c: its incidences (at v.inc_base; voxel ids in s_vox and
// build records in s_rec at the same positions) sorted by voxel (stable),
// one pair per run, the pairs renumbered brick-major by first visit
// (mrf_build.cu, k_pair_first; pairs on voxels flagged in s_loud first) and
// the incidences regrouped in the new pair order; then the pair statistics
// and the dynamic runs.  Numbered from the totals' current ends, which
// advance.
void view_pairs(mrf_map* m, int c, int bits, int64_t& pair_total, int64_t& perm_total, int64_t& dperm_total,
                int64_t& dpair_total) {
  View& v = m->views[c];
  uint32_t n = v.n_inc;
  uint32_t nr = (uint32_t)v.c_npre;
  v.pair_base = (uint32_t)pair_total;
  v.perm_base = (uint32_t)perm_total;
  v.dperm_base = (uint32_t)dperm_total;
  v.dpair_base = (uint32_t)dpair_total;
  v.n_pairs = 0;
  v.n_perm = 0;
  v.n_dperm = 0;
  v.n_dpairs = 0;
  v.n_loud = 0;
  if (nr == 0) return;
    m->s_k0.reserve((size_t)n * 4 + 4, false, m->stream);
    m->s_k1.reserve((size_t)n * 4 + 4, false, m->stream);
    m->s_v0.reserve((size_t)n * 4 + 4, false, m->stream);
    m->s_v1.reserve((size_t)n * 4 + 4, false, m->stream);
    CK(launch_iota(m->s_v0.as<uint32_t>(), n, m->stream));
    size_t t2 = sort_temp_bytes(n, bits);
    m->s_tmp.reserve(t2, false, m->stream);
    // padding incidences carry kNoVoxel, whose low bits exceed every voxel id
    CK(sort_pairs_u32(m->s_tmp.p, t2, m->s_vox.as<uint32_t>() + (v.inc_base - m->scratch_base), m->s_k1.as<uint32_t>(),
                      m->s_v0.as<uint32_t>(), m->s_v1.as<uint32_t>(), n, bits, m->stream));
    size_t t1 = scan_temp_bytes(nr + 1);
    m->s_tmp.reserve(t1, false, m->stream);
    // voxel-order pairs: runs of the sorted voxel keys
    CK(launch_vox_heads(m->s_k1.as<uint32_t>(), nr, m->s_k0.as<uint32_t>(), m->stream));
    CK(cudaMemsetAsync(m->s_k0.as<uint32_t>() + nr, 0, 4, m->stream));
    CK(exclusive_scan_u32(m->s_tmp.p, t1, m->s_k0.as<uint32_t>(), m->s_v0.as<uint32_t>(), nr + 1,
                          m->stream));
    const uint32_t np = read1(m, m->s_v0.as<uint32_t>() + nr);
    u32_checked(pair_total + np + 1, "pair count");
    size_t pb = (size_t)(pair_total + np + 1);
    m->pair_vox.reserve(pb * 4, true, m->stream);
    m->pair_m.reserve(pb * 4, true, m->stream);
    m->pair_cum.reserve(pb * 4, true, m->stream);
    m->pair_stat.reserve(pb * 4, true, m->stream);
    m->pair_ndyn.reserve(pb * 4, true, m->stream);
    m->pair_hit.reserve(pb * 4, true, m->stream);
    m->pair_seg.reserve(pb * 4, true, m->stream);
    {
      const uint32_t np0 = np;
      const size_t q4 = (size_t)np0 * 4 + 4;
      m->s_pv.reserve(q4, false, m->stream);
      m->s_sg.reserve(q4, false, m->stream);
      uint32_t* pv = m->s_pv.as<uint32_t>();
      uint32_t* sg = m->s_sg.as<uint32_t>();
      CK(launch_pairs_from_sorted(m->s_k1.as<uint32_t>(), m->s_v1.as<uint32_t>(), m->s_k0.as<uint32_t>(),
                                  m->s_v0.as<uint32_t>(), nr, 0, 0, v.inc_base, pv, sg, nullptr, m->stream));
      CK(launch_fill_u32(sg + np0, 1, nr, m->stream));
      // first visits: of each pair, and of each brick (min over its pairs)
      m->s_q0.reserve(q4, false, m->stream);
      m->s_q1.reserve(q4, false, m->stream);
      m->s_q2.reserve(q4, false, m->stream);
      m->s_q3.reserve(q4, false, m->stream);
      m->s_bf.reserve((size_t)m->n_bricks * 4 + 4, false, m->stream);
      uint32_t* q0 = m->s_q0.as<uint32_t>();
      uint32_t* q1 = m->s_q1.as<uint32_t>();
      uint32_t* q2 = m->s_q2.as<uint32_t>();
      uint32_t* q3 = m->s_q3.as<uint32_t>();
      CK(launch_pair_first(sg, np0, 0, m->s_v1.as<uint32_t>(), q0, m->stream));
      CK(launch_fill_u32(m->s_bf.as<uint32_t>(), m->n_bricks, 0xFFFFFFFFu, m->stream));
      CK(launch_brick_first(pv, q0, np0, m->s_bf.as<uint32_t>(), m->stream));
      // order: by own first visit, then (stable) by (quiet voxel, the
      // brick's first visit)
      int ibits = 1;
      while (ibits < 31 && ((uint64_t)1 << ibits) < (uint64_t)n) ++ibits;
      size_t t4 = std::max(sort_temp_bytes(np0, ibits), sort_temp_bytes(np0, ibits + 1));
      m->s_tmp.reserve(std::max(t4, t1), false, m->stream);
      CK(launch_iota(q2, np0, m->stream));
      CK(sort_pairs_u32(m->s_tmp.p, t4, q0, q1, q2, q3, np0, ibits, m->stream));  // q3: by own visit
      CK(launch_brick_keys(q3, np0, pv, m->s_bf.as<uint32_t>(), m->s_loud.as<uint8_t>(), ibits, q0,
                           m->stream));
      CK(sort_pairs_u32(m->s_tmp.p, t4, q0, q1, q3, q2, np0, ibits + 1, m->stream));  // q2: new order
      // new runs: lengths in the new order, their starts, the old -> new map
      CK(launch_new_lengths(q2, np0, sg, q0, q3, m->stream));
      CK(cudaMemsetAsync(q0 + np0, 0, 4, m->stream));
      size_t t5 = scan_temp_bytes(np0 + 1);
      m->s_tmp.reserve(t5, false, m->stream);
      CK(exclusive_scan_u32(m->s_tmp.p, t5, q0, q1, np0 + 1, m->stream));
      // the sorted positions in the new pair order (and each incidence's
      // new pair id), the renumbered pairs' voxels and runs
      m->s_recs.reserve((size_t)nr * 8, false, m->stream);
      uint32_t* nidx = m->s_recs.as<uint32_t>();
      CK(launch_move_positions(m->s_v1.as<uint32_t>(), m->s_k0.as<uint32_t>(), m->s_v0.as<uint32_t>(), sg, q3,
                               q1, nr, v.inc_base, v.pair_base, nidx, m->inc_pair.as<uint32_t>(), m->stream));
      CK(launch_pairs_renumbered(q2, np0, pv, q1, v.pair_base, v.perm_base, m->pair_vox.as<uint32_t>(),
                                 m->pair_seg.as<uint32_t>(), m->stream));
      std::swap(m->s_v1, m->s_recs);  // the moved positions become the sorted order
      m->s_v1.reserve((size_t)n * 4 + 4, true, m->stream);
    }
    CK(cudaMemsetAsync(m->s_k1.p, 0, 4, m->stream));
    CK(launch_count_loud(m->pair_vox.as<uint32_t>() + v.pair_base, np, m->s_loud.as<uint8_t>(),
                         m->s_k1.as<uint32_t>(), m->stream));
    v.n_loud = read1(m, m->s_k1.as<uint32_t>());
    m->s_recs.reserve((size_t)nr * 8, false, m->stream);
    CK(launch_gather_rec(m->s_v1.as<uint32_t>(), nr, v.inc_base - m->scratch_base, m->s_rec.as<float2>(),
                         m->s_recs.as<float2>(), m->s_k0.as<uint32_t>(), m->stream));
    m->s_pf.reserve((size_t)np * 4 + 4, false, m->stream);
    CK(launch_pair_stats(m->pair_seg.as<uint32_t>(), v.pair_base, np, v.perm_base, m->s_recs.as<float2>(),
                         m->pair_cum.as<float>(), m->pair_stat.as<float>(), m->pair_ndyn.as<uint32_t>(),
                         m->pair_hit.as<float>(), m->s_pf.as<uint32_t>(), m->stream));
    // dynamic incidences in pair-grouped order (a stable compaction of the
    // sorted positions) and the run of each pair that has any
    CK(cudaMemsetAsync(m->s_k0.as<uint32_t>() + nr, 0, 4, m->stream));
    CK(exclusive_scan_u32(m->s_tmp.p, t1, m->s_k0.as<uint32_t>(), m->s_v0.as<uint32_t>(), nr + 1,
                          m->stream));
    uint32_t nd = read1(m, m->s_v0.as<uint32_t>() + nr);
    CK(launch_dyn_scatter(m->s_v1.as<uint32_t>(), m->s_k0.as<uint32_t>(), m->s_v0.as<uint32_t>(), nr,
                          v.inc_base, v.dperm_base, m->dperm.as<uint32_t>(), m->stream));
    m->s_pf.reserve((size_t)np * 4 + 4, false, m->stream);
    m->s_ps.reserve((size_t)np * 4 + 4, false, m->stream);
    CK(launch_dpair_flags(m->pair_ndyn.as<uint32_t>(), v.pair_base, np, m->s_pf.as<uint32_t>(),
                          m->stream));
    CK(cudaMemsetAsync(m->s_pf.as<uint32_t>() + np, 0, 4, m->stream));
    size_t t3 = scan_temp_bytes(np + 1);
    m->s_tmp.reserve(t3, false, m->stream);
    CK(exclusive_scan_u32(m->s_tmp.p, t3, m->s_pf.as<uint32_t>(), m->s_ps.as<uint32_t>(), np + 1,
                          m->stream));
    uint32_t ndp = read1(m, m->s_ps.as<uint32_t>() + np);
    size_t db = (size_t)(dpair_total + ndp + 1);
    m->dpair.reserve(db * 4, true, m->stream);
    m->dseg.reserve(db * 4, true, m->stream);
    CK(launch_dpairs(m->s_pf.as<uint32_t>(), m->s_ps.as<uint32_t>(), v.pair_base, np,
                     m->pair_seg.as<uint32_t>(), v.perm_base, m->s_v0.as<uint32_t>(), v.dperm_base,
                     v.dpair_base, m->dpair.as<uint32_t>(), m->dseg.as<uint32_t>(), m->stream));
    CK(launch_fill_u32(m->dseg.as<uint32_t>() + v.dpair_base + ndp, 1, v.dperm_base + nd, m->stream));
    v.n_pairs = np;
    v.n_perm = nr;
    v.n_dperm = nd;
    v.n_dpairs = ndp;
    pair_total += np;
    perm_total += nr;
    dperm_total += nd;
    dpair_total += ndp;
}

// A view's rays in the SM-affine schedule: R regions of consecutive pixels
// holding equal shares of the view's Pre incidences; a region's home rays
// (its longest rays up to kHomeShare of its incidences, longest first) are
// taken by the blocks homed on it, every region's remaining short rays go to
// the view's leftover queue (longest first) that the blocks drain
// afterwards, which evens out the regions' finishing times (the home share,
// 75 % unless mrf_set_home_share or mrf_autotune_home_share chose another;
// it moves rays between warps only, never a result).  Built on
// the host in linear time: a counting sort by length feeds the regions'
// buckets in order, so each bucket is longest first.  Pixel indices are
// absolute (v.pix_base + i); starts are positions in home.
struct RegionLists {
  std::vector<uint32_t> home, left, starts;
};
void region_lists(const View& v, const RayMeta* vm, int R, int64_t share, RegionLists& out) {
  const int64_t hw = view_pixels(v);
  std::vector<uint32_t> lcount(65536, 0u), reg((size_t)hw, 0u), bucket_off((size_t)R + 1, 0u);
  int64_t work = 0;
  for (int64_t i = 0; i < hw; ++i) {
    if (!ray_in_bp(vm[i])) continue;
    work += vm[i].n_pre;
    ++lcount[65535 - vm[i].n_pre];
  }
  // region of each active pixel: equal shares of the view's work
  int64_t acc = 0;
  for (int64_t i = 0; i < hw; ++i) {
    if (!ray_in_bp(vm[i])) continue;
    const uint32_t r = (uint32_t)std::min<int64_t>(R - 1, acc * R / std::max<int64_t>(work, 1));
    reg[(size_t)i] = r;
    ++bucket_off[r + 1];
    acc += vm[i].n_pre;
  }
  for (int r = 0; r < R; ++r) bucket_off[r + 1] += bucket_off[r];
  // the view's active rays longest first (pixel order within a length)
  uint32_t pos = 0;
  for (int k = 0; k < 65536; ++k) {
    const uint32_t c0 = lcount[k];
    lcount[k] = pos;
    pos += c0;
  }
  std::vector<uint32_t> lsorted(pos), buckets(pos), fill(bucket_off.begin(), bucket_off.end() - 1);
  for (int64_t i = 0; i < hw; ++i)
    if (ray_in_bp(vm[i])) lsorted[lcount[65535 - vm[i].n_pre]++] = (uint32_t)i;
  for (uint32_t i : lsorted) buckets[fill[reg[i]]++] = i;
  // home = each region's longest rays up to `share` per cent of its work
  std::vector<uint8_t> is_home((size_t)hw, 0);
  out.home.reserve(pos);
  for (int r = 0; r < R; ++r) {
    int64_t rw = 0, hwk = 0;
    for (uint32_t k = bucket_off[r]; k < bucket_off[r + 1]; ++k) rw += vm[buckets[k]].n_pre;
    out.starts.push_back((uint32_t)out.home.size());
    for (uint32_t k = bucket_off[r]; k < bucket_off[r + 1] && hwk * 100 < rw * share; ++k) {
      const uint32_t i = buckets[k];
      is_home[i] = 1;
      hwk += vm[i].n_pre;
      out.home.push_back((uint32_t)(v.pix_base + i));
    }
  }
  // leftovers longest first
  for (uint32_t i : lsorted)
    if (!is_home[i]) out.left.push_back((uint32_t)(v.pix_base + i));
}

// region lists of several views in parallel host threads (at most one per
// core, the views taken in turn); hm holds the ray records of every view in
// `views` at their pix_base
void region_lists_parallel(mrf_map* m, const std::vector<int>& views, const std::vector<RayMeta>& hm,
                           int64_t hm_base, std::vector<RegionLists>& lists) {
  const int R = std::max(1, m->num_sms);
  const int nv = (int)views.size();
  const int nt = std::max(1, std::min<int>(nv, (int)std::thread::hardware_concurrency()));
  std::atomic<int> next{0};
  std::vector<std::thread> pool;
  std::vector<char> failed((size_t)nv, 0);
  for (int t = 0; t < nt; ++t)
    pool.emplace_back([&] {
      for (int k = next++; k < nv; k = next++) {
        try {
          const View& v = m->views[views[k]];
          region_lists(v, hm.data() + (v.pix_base - hm_base), R, m->home_share, lists[(size_t)views[k]]);
        } catch (...) {
          failed[(size_t)k] = 1;
        }
      }
    });
  for (auto& t : pool) t.join();
  for (char f : failed)
    if (f) fail(MRF_ERR_OOM, "host memory for the region queues");
}

// Per-view blocks [home rays][leftovers] of views (in that order) laid out
// in region_q from position `at` on, their ray records gathered from meta;
// per view: rstart row c*(R+1) (R region starts and the end of the home
// block, absolute), lbase[c] (first leftover) and lsingle {0, n_left} at 2c.
// Returns the end position.
uint32_t region_blocks(mrf_map* m, const std::vector<int>& views, const std::vector<RegionLists>& lists,
                       uint32_t at) {
  const int R = std::max(1, m->num_sms);
  const int V = (int)m->views.size();
  m->rstart.reserve((size_t)V * (R + 1) * 4 + 4, true, m->stream);
  m->lbase.reserve((size_t)V * 4 + 4, true, m->stream);
  m->lsingle.reserve((size_t)V * 8 + 8, true, m->stream);
  std::vector<uint32_t> pix;
  // each view's row of region starts, leftover base and leftover counter
  // pair, staged on the host until the synchronisation below
  const size_t nv = views.size();
  std::vector<uint32_t> rows(nv * ((size_t)R + 1)), lbs(nv), lss(2 * nv);
  for (size_t k = 0; k < nv; ++k) {
    const int c = views[k];
    View& v = m->views[c];
    const RegionLists& l = lists[(size_t)c];
    uint32_t* row = rows.data() + k * ((size_t)R + 1);
    const uint32_t b = at + (uint32_t)pix.size();
    for (int r = 0; r < R; ++r) row[r] = b + (r < (int)l.starts.size() ? l.starts[(size_t)r] : 0u);
    row[R] = b + (uint32_t)l.home.size();
    v.left_base = b + (uint32_t)l.home.size();
    v.n_left = (uint32_t)l.left.size();
    pix.insert(pix.end(), l.home.begin(), l.home.end());
    pix.insert(pix.end(), l.left.begin(), l.left.end());
    lbs[k] = v.left_base;
    lss[2 * k] = 0u;
    lss[2 * k + 1] = v.n_left;
    CK(cudaMemcpyAsync(m->rstart.as<uint32_t>() + (size_t)c * (R + 1), row, (size_t)(R + 1) * 4,
                       cudaMemcpyHostToDevice, m->stream));
    CK(cudaMemcpyAsync(m->lbase.as<uint32_t>() + c, &lbs[k], 4, cudaMemcpyHostToDevice, m->stream));
    CK(cudaMemcpyAsync(m->lsingle.as<uint32_t>() + 2 * (size_t)c, &lss[2 * k], 8, cudaMemcpyHostToDevice,
                       m->stream));
  }
  const uint32_t end = at + (uint32_t)pix.size();
  m->region_q.reserve(std::max<size_t>(end, 1) * sizeof(RayMeta), true, m->stream);
  m->region_ids.reserve(std::max<size_t>(end, 1) * 4, true, m->stream);
  if (!pix.empty()) {
    m->ray_order.reserve(pix.size() * 4, false, m->stream);
    CK(cudaMemcpyAsync(m->ray_order.p, pix.data(), pix.size() * 4, cudaMemcpyHostToDevice, m->stream));
    CK(launch_ray_queue(m->meta.as<RayMeta>(), m->ray_order.as<uint32_t>(), (uint32_t)pix.size(),
                        m->region_q.as<RayMeta>() + at, m->region_ids.as<uint32_t>() + at, 0u, m->stream));
  }
  sync(m);  // the host staging vectors go out of scope
  return end;
}

// the leftover prefix of every view (V + 1 entries) for a launch over all
// views (Jacobi)
void leftover_prefix(mrf_map* m) {
  const int V = (int)m->views.size();
  std::vector<uint32_t> pre((size_t)V + 1, 0u);
  for (int c = 0; c < V; ++c) pre[(size_t)c + 1] = pre[(size_t)c] + m->views[c].n_left;
  m->lprefix.reserve(pre.size() * 4, false, m->stream);
  CK(cudaMemcpyAsync(m->lprefix.p, pre.data(), pre.size() * 4, cudaMemcpyHostToDevice, m->stream));
  sync(m);
}

// the region blocks of every built view again, from their ray records (the
// home share changed); the incidence lists stay as they are.  The caller
// drops the captured graphs.
void rebuild_regions(mrf_map* m) {
  const int B = m->built_views;
  if (m->built_version < 0 || B == 0 || m->npix_total == 0) return;
  std::vector<RayMeta> hm((size_t)m->npix_total);
  CK(cudaMemcpyAsync(hm.data(), m->meta.p, hm.size() * sizeof(RayMeta), cudaMemcpyDeviceToHost, m->stream));
  sync(m);
  std::vector<int> live, built;
  for (int c = 0; c < B; ++c) {
    built.push_back(c);
    if (!m->views[c].retired) live.push_back(c);
  }
  std::vector<RegionLists> lists(m->views.size());
  region_lists_parallel(m, live, hm, 0, lists);
  for (int c : built)
    if (m->views[c].retired) {
      m->views[c].n_left = 0;
      m->views[c].left_base = 0;
    }
  m->region_end = region_blocks(m, built, lists, 0u);
  leftover_prefix(m);
}

// view c's active rays longest first (17-bit key radix sort on the GPU),
// their records copied into queue order at ray_queue + v.order_base
void view_ray_queue(mrf_map* m, int c) {
  View& v = m->views[c];
  const int64_t hw = view_pixels(v);
  const int64_t act = hw ? v.c_nrays_bp : 0;  // the rays in BP (ray_in_bp)
  v.n_active = (uint32_t)act;
  if (hw == 0) return;
  m->s_k0.reserve((size_t)hw * 4 + 4, false, m->stream);
  m->s_k1.reserve((size_t)hw * 4 + 4, false, m->stream);
  m->s_v0.reserve((size_t)hw * 4 + 4, false, m->stream);
  m->s_v1.reserve((size_t)hw * 4 + 4, false, m->stream);
  CK(launch_ray_keys(m->meta.as<RayMeta>() + v.pix_base, (uint32_t)hw, m->s_k0.as<uint32_t>(),
                     m->s_v0.as<uint32_t>(), m->stream));
  size_t t = sort_temp_bytes((uint32_t)hw, 17);
  m->s_tmp.reserve(t, false, m->stream);
  CK(sort_pairs_u32(m->s_tmp.p, t, m->s_k0.as<uint32_t>(), m->s_k1.as<uint32_t>(), m->s_v0.as<uint32_t>(),
                    m->s_v1.as<uint32_t>(), (uint32_t)hw, 17, m->stream));
  CK(launch_ray_queue(m->meta.as<RayMeta>() + v.pix_base, m->s_v1.as<uint32_t>(), (uint32_t)act,
                      m->ray_queue.as<RayMeta>() + v.order_base, m->queue_ids.as<uint32_t>() + v.order_base,
                      (uint32_t)v.pix_base, m->stream));
}

// the statistics of the live views
void stats_from_views(mrf_map* m) {
  int64_t nrays = 0, npre = 0, npost = 0, ndyn = 0, nrays_bp = 0, npre_bp = 0, np = 0, ndp = 0, nfast = 0;
  for (const View& v : m->views) {
    if (v.retired) continue;
    nrays += v.c_nrays;
    npre += v.c_npre;
    npost += v.c_npost;
    ndyn += v.c_ndyn;
    nrays_bp += v.c_nrays_bp;
    npre_bp += v.c_npre_bp;
    nfast += v.c_nfast_bp;
    np += v.n_pairs;
    ndp += v.n_dpairs;
  }
  m->stats.n_rays = nrays;
  m->stats.n_inc_pre = npre;
  m->stats.n_inc_post = npost;
  m->stats.n_pairs = np;
  m->stats.n_inc_dyn = ndyn;
  m->stats.n_pairs_dyn = ndp;
  m->stats.n_rays_bp = nrays_bp;
  m->stats.n_inc_pre_bp = npre_bp;
  m->stats.n_inc_from_k4 = nfast;
  m->stats.n_loud_prefix = m->loud_count_version == m->built_version ? m->n_loud_prefix : 0;
}

int voxel_id_bits(const mrf_map* m) {
  int bits = 1;
  while (bits < 32 && ((uint64_t)1 << bits) <= (uint64_t)(m->n_bricks * kBrickVox)) ++bits;
  return bits;
}

// Incidence counts of the given views: view k's pixel counts at
// s_counts + coff[k] (its hw entries and a sentinel) and their exclusive scan
// at s_offs + coff[k]; each view's total is summed in 64 bits and the running
// total (from `before` incidences already in the arenas) checked against the
// 32-bit index range before any offset is used.  Returns the views' counts.
std::vector<uint32_t> count_views(mrf_map* m, const std::vector<int>& views, int64_t before,
                                  std::vector<int64_t>& coff) {
  int64_t tot_px = 0;
  coff.assign(views.size(), 0);
  for (size_t k = 0; k < views.size(); ++k) {
    coff[k] = tot_px;
    tot_px += view_pixels(m->views[views[k]]) + 1;
  }
  m->s_counts.reserve((size_t)std::max<int64_t>(tot_px, 1) * 4, false, m->stream);
  m->s_offs.reserve((size_t)std::max<int64_t>(tot_px, 1) * 4, false, m->stream);
  m->s_delta.reserve(64, false, m->stream);
  std::vector<uint32_t> n(views.size(), 0u);
  unsigned long long run = (unsigned long long)before;
  for (size_t k = 0; k < views.size(); ++k) {
    const View& v = m->views[views[k]];
    const int64_t hw = view_pixels(v);
    uint32_t* cnt = m->s_counts.as<uint32_t>() + coff[k];
    if (hw) CK(launch_trace_count(v.cam, v.pose, v.depth.as<float>(), cnt, m->s_err.as<int>(), m->stream));
    CK(launch_sum_u32(cnt, hw, m->s_delta.as<unsigned long long>(), m->stream));
    const unsigned long long total = read1(m, m->s_delta.as<unsigned long long>());
    run += total;
    if (run > 0xFFFFFFF0ull)
      fail(MRF_ERR_CAPACITY, "incidence count " + std::to_string(run) +
                                 " exceeds the 32-bit incidence index range (fewer or smaller views per map)");
    CK(cudaMemsetAsync(cnt + hw, 0, 4, m->stream));
    size_t tb = scan_temp_bytes((uint32_t)(hw + 1));
    m->s_tmp.reserve(tb, false, m->stream);
    CK(exclusive_scan_u32(m->s_tmp.p, tb, cnt, m->s_offs.as<uint32_t>() + coff[k], (uint32_t)(hw + 1),
                          m->stream));
    n[k] = (uint32_t)total;
  }
  check_device_err(m);
  return n;
}

// the emit pass of view c at v.inc_base (pix_off: its scanned counts)
void emit_view(mrf_map* m, int c, const uint32_t* pix_off) {
  View& v = m->views[c];
  CK(launch_trace_emit(v.cam, v.pose, v.depth.as<float>(), pix_off, v.inc_base,
                       m->meta.as<RayMeta>() + v.pix_base, m->s_vox.as<uint32_t>() + (v.inc_base - m->scratch_base),
                       m->inc_len.as<float>() + v.inc_base, m->inc_mu.as<float>() + v.inc_base,
                       m->s_rec.as<float2>() + (v.inc_base - m->scratch_base), m->s_err.as<int>(), m->stream));
}

// tiles of view c's pair update, from position tb of tile_first
void view_tiles(mrf_map* m, int c, uint32_t tb) {
  View& v = m->views[c];
  v.tile_base = tb;
  CK(launch_tile_first(m->dseg.as<uint32_t>(), v.dpair_base, v.dpair_base + v.n_dpairs, v.dperm_base,
                       v.dperm_base + v.n_dperm, m->tile_first.as<uint32_t>() + tb, m->stream));
}

// The loud lists of the static prefixes of every live view's queued rays
// (npix pixel records in meta): counts per ray, one scan over all pixels,
// then the lists (pair id, length, position) -- the data the ray kernel's
// fast path gathers every iteration, and room for the quiet sums.
void count_loud_lists(mrf_map* m) {
  const int64_t npix = m->npix_total;
  m->loud_off.reserve((size_t)(npix + 1) * 4, false, m->stream);
  CK(cudaMemsetAsync(m->loud_off.p, 0, (size_t)(npix + 1) * 4, m->stream));
  const RayMeta* meta = m->meta.as<RayMeta>();
  for (const View& v : m->views) {
    if (v.retired || v.n_inc == 0) continue;
    CK(launch_loud_prefix(meta, (uint32_t)v.pix_base, (uint32_t)view_pixels(v), m->inc_pair.as<uint32_t>(),
                          m->inc_len.as<float>(), v.pair_base, v.n_loud, m->loud_off.as<uint32_t>(), nullptr,
                          nullptr, nullptr, false, m->stream));
  }
  m->s_offs.reserve((size_t)(npix + 1) * 4, false, m->stream);
  const size_t t = scan_temp_bytes((uint32_t)(npix + 1));
  m->s_tmp.reserve(t, false, m->stream);
  CK(exclusive_scan_u32(m->s_tmp.p, t, m->loud_off.as<uint32_t>(), m->s_offs.as<uint32_t>(), (uint32_t)(npix + 1),
                        m->stream));
  std::swap(m->loud_off, m->s_offs);
  m->n_loud_prefix = read1(m, m->loud_off.as<uint32_t>() + npix);
  m->stats.n_loud_prefix = m->n_loud_prefix;
}

void emit_loud_lists(mrf_map* m) {
  const int64_t npix = m->npix_total;
  const uint32_t total = (uint32_t)m->n_loud_prefix;
  const RayMeta* meta = m->meta.as<RayMeta>();
  m->quiet_q.reserve((size_t)std::max<int64_t>(npix, 1) * 8, false, m->stream);
  m->loud_pid.reserve((size_t)std::max<uint32_t>(total, 1) * 4, false, m->stream);
  m->loud_len.reserve((size_t)std::max<uint32_t>(total, 1) * 4, false, m->stream);
  m->loud_pos.reserve((size_t)std::max<uint32_t>(total, 1) * 2, false, m->stream);
  for (const View& v : m->views) {
    if (v.retired || v.n_inc == 0) continue;
    CK(launch_loud_prefix(meta, (uint32_t)v.pix_base, (uint32_t)view_pixels(v), m->inc_pair.as<uint32_t>(),
                          m->inc_len.as<float>(), v.pair_base, v.n_loud, m->loud_off.as<uint32_t>(),
                          m->loud_pid.as<uint32_t>(), m->loud_len.as<float>(), m->loud_pos.as<uint16_t>(), true,
                          m->stream));
  }
}

// Whether a call of `iters` iterations takes the static prefixes from
// their quiet sums from its third iteration on: only when at least two
// iterations use them (the quiet sums cost about one pass over the static
// prefixes), the quiet incidences are at least half of the Pre incidences
// and they average at least two 128-incidence chunks per ray (else the
// per-ray overhead outweighs the saved gathers: maps of short rays, or of
// rays near many surfaces).  Counts the loud lists of the current build
// when needed and makes them when the answer is yes.
constexpr int64_t kQuietPerRay = 256;
bool quiet_path(mrf_map* m, int64_t iters, int flags) {
  const bool force = (flags & MRF_QUIET_PREFIX) != 0;
  if (iters < (force ? 3 : 4) || (flags & MRF_FULL_RAYS) || m->n_inc <= 0 || m->npix_total <= 0) return false;
  const int64_t pre = m->stats.n_inc_pre_bp, k4 = m->stats.n_inc_from_k4, rays = m->stats.n_rays_bp;
  if (!force && (rays <= 0 || pre - k4 < kQuietPerRay * rays)) return false;  // no count needed
  if (m->loud_count_version != m->built_version) {
    count_loud_lists(m);
    m->loud_count_version = m->built_version;
    m->loud_list_version = -1;
  }
  const int64_t quiet = pre - k4 - m->n_loud_prefix;
  if (!force && (quiet * 2 < pre || quiet < kQuietPerRay * rays)) return false;
  if (m->loud_list_version != m->built_version) {
    emit_loud_lists(m);
    m->loud_list_version = m->built_version;
  }
  return true;
}

// the quiet sums of every live view's static prefixes from the current
// ln q (valid from the third iteration of a call on, when the quiet pairs'
// ln q no longer change)
void quiet_prefix_all(mrf_map* m, const BpArrays& a) {
  for (const View& v : m->views) {
    if (v.retired || v.n_inc == 0) continue;
    CK(launch_quiet_prefix(a, (uint32_t)v.pix_base, (uint32_t)view_pixels(v), v.pair_base, v.n_loud,
                           m->quiet_q.as<float2>(), m->stream));
  }
}

void rebuild_lists(mrf_map* m, OldPairs& old) {
  const int V = (int)m->views.size();
  m->g.brick_slot = m->d_slot.as<int>();
  // per-pixel arrays of all live views back to back (views may differ in size)
  int64_t npix = 0;
  for (View& v : m->views) {
    v.pix_base = npix;
    v.cam.brick_slot = m->g.brick_slot;
    npix += view_pixels(v);
  }
  u32_checked(npix, "pixel count");
  CK(cudaEventRecord(m->ev0, m->stream));
  const bool remap = old.remap;
  DBuf& old_vox = old.vox;
  DBuf& old_m = old.m;
  const std::vector<View>& old_views = old.views;
  // 1. counts of every pixel of every live view, one scan per view ->
  //    offsets (totals in 64 bits: a wrapped total would size the arenas
  //    too small for the emit pass)
  std::vector<int> live;
  for (int c = 0; c < V; ++c) {
    m->views[c].n_inc = 0;
    if (!m->views[c].retired) live.push_back(c);
  }
  std::vector<int64_t> coff;
  const std::vector<uint32_t> cnt = count_views(m, live, 0, coff);
  int64_t n_inc = 0;
  for (int c = 0; c < V; ++c) {
    View& v = m->views[c];
    v.inc_base = (uint32_t)n_inc;
    const auto it = std::find(live.begin(), live.end(), c);
    if (it != live.end()) {
      v.n_inc = cnt[(size_t)(it - live.begin())];
      n_inc += v.n_inc;
    }
  }
  // 2. arenas
  {
    const size_t ib = (size_t)std::max<int64_t>(n_inc, 1) * 4;
    m->meta.reserve((size_t)std::max<int64_t>(npix, 1) * sizeof(RayMeta), false, m->stream);
    m->inc_pair.reserve(ib, false, m->stream);
    m->inc_len.reserve(ib, false, m->stream);
    m->inc_mu.reserve(ib, false, m->stream);
    m->dperm.reserve(ib, false, m->stream);
    m->inc_pl.reserve(ib, false, m->stream);
    m->s_vox.reserve(ib, false, m->stream);
    m->s_rec.reserve(ib * 2, false, m->stream);
    m->scratch_base = 0;
  }
  // 3. emit
  for (size_t k = 0; k < live.size(); ++k) emit_view(m, live[k], m->s_offs.as<uint32_t>() + coff[k]);
  // per-view counters from the ray records
  std::vector<RayMeta> hm((size_t)npix);
  {
    std::vector<int> all_views((size_t)V);
    for (int c = 0; c < V; ++c) all_views[(size_t)c] = c;
    ray_records_and_counters(m, all_views, 0, hm);
  }
  // voxels with a dynamic incidence in any view ("loud"; the others are
  // quiet, see enqueue_iteration)
  m->s_loud.reserve((size_t)std::max<int64_t>(m->n_bricks * kBrickVox, 1), false, m->stream);
  CK(cudaMemsetAsync(m->s_loud.p, 0, (size_t)std::max<int64_t>(m->n_bricks * kBrickVox, 1), m->stream));
  CK(launch_loud_voxels(m->meta.as<RayMeta>(), npix, m->s_vox.as<uint32_t>(), 0u, m->s_loud.as<uint8_t>(),
                        m->stream));
  // the region lists of the SM-affine schedule are host work on the ray
  // records alone: built on host threads while the GPU builds the pairs
  std::vector<RegionLists> lists((size_t)V);
  bool lists_failed = false;
  std::thread lists_thread([&] {
    try {
      region_lists_parallel(m, live, hm, 0, lists);
    } catch (...) {
      lists_failed = true;
    }
  });
  // 4. pairs per view
  const int bits = voxel_id_bits(m);
  int64_t pair_total = 0, perm_total = 0, dperm_total = 0, dpair_total = 0;
  try {
    for (int c = 0; c < V; ++c) view_pairs(m, c, bits, pair_total, perm_total, dperm_total, dpair_total);
  } catch (...) {
    lists_thread.join();
    throw;
  }
  lists_thread.join();
  if (lists_failed) fail(MRF_ERR_OOM, "host memory for the region queues");
  // 5. ray queues: per view the active rays longest first, and the
  //    SM-affine region blocks
  {
    m->ray_queue.reserve((size_t)std::max<int64_t>(npix, 1) * sizeof(RayMeta), false, m->stream);
    m->queue_ids.reserve((size_t)std::max<int64_t>(npix, 1) * 4, false, m->stream);
    int64_t base = 0;
    for (int c = 0; c < V; ++c) {
      View& v = m->views[c];
      v.order_base = (uint32_t)base;
      view_ray_queue(m, c);
      base += v.n_active;
    }
    m->queue_end = base;
    m->counters.reserve((size_t)(V + 1) * 4, false, m->stream);
    const int R = std::max(1, m->num_sms);
    m->nreg = (uint32_t)R;
    m->rcounters.reserve(((size_t)2 * V * R + 2 * (size_t)V + 2) * 4, false, m->stream);
    // retired views: empty rows
    for (int c = 0; c < V; ++c) {
      View& v = m->views[c];
      if (v.retired) {
        v.n_left = 0;
        v.left_base = 0;
      }
    }
    std::vector<int> all;
    for (int c = 0; c < V; ++c) all.push_back(c);
    m->region_end = region_blocks(m, all, lists, 0u);
    leftover_prefix(m);
  }
  m->n_inc = n_inc;
  m->n_pairs = pair_total;
  m->n_perm_total = perm_total;
  m->n_dperm = dperm_total;
  m->n_dpairs = dpair_total;
  size_t pb = (size_t)std::max<int64_t>(pair_total + 1, 1);
  m->pair_vox.reserve(pb * 4, true, m->stream);
  m->pair_m.reserve(pb * 4, true, m->stream);
  m->pair_cum.reserve(pb * 4, true, m->stream);
  m->pair_stat.reserve(pb * 4, true, m->stream);
  m->pair_ndyn.reserve(pb * 4, true, m->stream);
  m->pair_hit.reserve(pb * 4, true, m->stream);
  m->pair_seg.reserve(pb * 4, true, m->stream);
  m->dpair.reserve((size_t)(dpair_total + 1) * 4, true, m->stream);
  m->dseg.reserve((size_t)(dpair_total + 1) * 4, true, m->stream);
  if (dpair_total == 0) CK(launch_fill_u32(m->dseg.as<uint32_t>(), 1, 0u, m->stream));
  m->drun.reserve((size_t)(dpair_total + 1) * 16, false, m->stream);
  CK(launch_drun(m->dpair.as<uint32_t>(), (uint32_t)dpair_total, m->pair_vox.as<uint32_t>(),
                 m->pair_cum.as<float>(), m->pair_stat.as<float>(), m->drun.as<uint4>(), m->stream));
  m->pair_q.reserve(pb * 4, false, m->stream);
  m->pair_dm.reserve(pb * 4, false, m->stream);
  CK(launch_fill_f32(m->pair_m.as<float>(), pair_total, 0.0f, m->stream));
  {
    // tile carries of the pair update: enough for any view or all of them;
    // first pair of every tile, per view (Gauss-Seidel) and over all views
    // (Jacobi)
    int64_t tiles = (int64_t)pair_update_tiles((uint32_t)std::min<int64_t>(dperm_total, 0xFFFFFFF0ll)) + V + 1;
    m->carry_tiles = tiles;
    m->carry.reserve((size_t)tiles * sizeof(TileCarry), false, m->stream);
    m->tile_first.reserve((size_t)(2 * tiles + 2) * 4, false, m->stream);
    uint32_t tb = 0;
    for (int c = 0; c < V; ++c) {
      view_tiles(m, c, tb);
      tb += pair_update_tiles(m->views[c].n_dperm);
    }
    m->jac_tile_base = tb;
    CK(launch_tile_first(m->dseg.as<uint32_t>(), 0, (uint32_t)dpair_total, 0, (uint32_t)dperm_total,
                         m->tile_first.as<uint32_t>() + tb, m->stream));
    m->tile_end = tb + pair_update_tiles((uint32_t)std::min<int64_t>(dperm_total, 0xFFFFFFF0ll)) + 1;
  }
  // 6. carry messages of every camera over to its new pairs
  if (remap) {
    int64_t nv = m->n_bricks * kBrickVox;
    m->s_dense.reserve((size_t)nv * 4, false, m->stream);
    CK(cudaMemsetAsync(m->s_dense.p, 0, (size_t)nv * 4, m->stream));
    for (int c = 0; c < V && c < (int)old_views.size(); ++c) {
      const View& o = old_views[c];
      const View& v = m->views[c];
      CK(launch_remap_scatter(old_vox.as<uint32_t>() + o.pair_base, old_m.as<float>() + o.pair_base,
                              o.n_pairs, m->s_dense.as<float>(), m->stream));
      CK(launch_remap_gather(m->pair_vox.as<uint32_t>() + v.pair_base,
                             m->pair_m.as<float>() + v.pair_base, v.n_pairs,
                             m->s_dense.as<float>(), m->stream));
      CK(launch_scatter_const(old_vox.as<uint32_t>() + o.pair_base, o.n_pairs, 0.0f,
                              m->s_dense.as<float>(), m->stream));
    }
    sync(m);
    old_vox.release();
    old_m.release();
    old.remap = false;  // the new pairs hold the messages from here on
  }
  {
    const int64_t nv = m->n_bricks * kBrickVox;
    m->vox_active.reserve((size_t)std::max<int64_t>(nv, 1), false, m->stream);
    CK(launch_active_voxels(m->pair_vox.as<uint32_t>(), m->pair_cum.as<float>(), (uint32_t)pair_total,
                            m->vox_active.as<uint8_t>(), nv, m->stream));
    m->vox_active_n = nv;
  }
  CK(cudaEventRecord(m->ev1, m->stream));
  sync(m);
  check_device_err(m);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, m->ev0, m->ev1);
  m->stats.build_ms = ms;
  m->built_version = m->version;
  m->jacobi_version = -1;
  m->built_views = V;
  m->npix_total = npix;
  m->bricks_at_build = m->n_bricks;
  m->holes = false;
  m->needs_full = false;
  m->dead_inc = 0;
  stats_from_views(m);
}

// Appends the lists of the views added since the last build (a full-ray
// map only; see ensure_built), leaving the other views' lists, pairs and
// messages as they are: every brick a full-ray view's rays cross before
// their stop was activated by the view itself, so bricks activated later
// change no old list -- which a count pass over the old views, compared
// with their stored ray records, confirms whenever the brick set grew.
// Returns false (nothing changed) when a full build is needed instead.
bool append_lists(mrf_map* m) {
  const int V = (int)m->views.size();
  CK(cudaEventRecord(m->ev0, m->stream));
  m->g.brick_slot = m->d_slot.as<int>();
  for (View& v : m->views) v.cam.brick_slot = m->g.brick_slot;
  if (m->n_bricks != m->bricks_at_build) {
    // err[1]: the count pass's mismatch flag (err[0], the kernels' error
    // flag, is left as it is and checked below).  Only the pixels whose
    // rays may cross a brick activated since the last build are traced
    // again (their footprint through each view's camera); err[2] tells the
    // pass to check every pixel of the view.
    CK(cudaMemsetAsync(m->s_err.as<int>() + 1, 0, 4, m->stream));
    const uint32_t b0 = (uint32_t)std::max<int64_t>(m->bricks_at_build, 0), b1 = (uint32_t)m->n_bricks;
    for (int c = 0; c < m->built_views; ++c) {
      const View& v = m->views[c];
      const int64_t hw = view_pixels(v);
      if (!hw) continue;
      m->s_counts.reserve((size_t)hw * 4 + 4, false, m->stream);
      m->s_dense.reserve((size_t)hw + 16, false, m->stream);
      CK(cudaMemsetAsync(m->s_dense.p, 0, (size_t)hw, m->stream));
      CK(cudaMemsetAsync(m->s_err.as<int>() + 2, 0, 4, m->stream));
      CK(launch_brick_footprint(v.cam, v.pose, m->d_coord.as<int>(), b0, b1, m->s_dense.as<uint8_t>(),
                                m->s_err.as<int>() + 2, m->stream));
      CK(launch_trace_count(v.cam, v.pose, v.depth.as<float>(), m->s_counts.as<uint32_t>(), m->s_err.as<int>(),
                            m->stream, m->meta.as<RayMeta>() + v.pix_base, m->s_dense.as<uint8_t>(),
                            m->s_err.as<int>() + 2));
    }
    int flags[2] = {0, 0};
    CK(cudaMemcpyAsync(flags, m->s_err.p, 8, cudaMemcpyDeviceToHost, m->stream));
    sync(m);
    check_device_err(m);
    if (flags[1]) {
      CK(cudaMemsetAsync(m->s_err.as<int>() + 1, 0, 4, m->stream));
      return false;
    }
  }
  std::vector<int> added;
  for (int c = m->built_views; c < V; ++c)
    if (!m->views[c].retired) added.push_back(c);
  // 1-3. counts, arenas (kept), emit of the new views
  int64_t npix = m->npix_total, n_inc = m->n_inc;
  for (int c = m->built_views; c < V; ++c) {
    View& v = m->views[c];
    v.pix_base = npix;
    v.inc_base = (uint32_t)n_inc;
    v.n_inc = 0;
    npix += view_pixels(v);
  }
  u32_checked(npix, "pixel count");
  std::vector<int64_t> coff;
  const std::vector<uint32_t> cnt = count_views(m, added, n_inc, coff);
  for (size_t k = 0; k < added.size(); ++k) {
    View& v = m->views[added[k]];
    v.inc_base = (uint32_t)n_inc;
    v.n_inc = cnt[k];
    n_inc += cnt[k];
  }
  for (int c = m->built_views; c < V; ++c)
    if (m->views[c].retired) m->views[c].inc_base = (uint32_t)n_inc;
  {
    const size_t ib = (size_t)std::max<int64_t>(n_inc, 1) * 4;
    m->meta.reserve((size_t)std::max<int64_t>(npix, 1) * sizeof(RayMeta), true, m->stream);
    m->inc_len.reserve(ib, true, m->stream);
    m->inc_mu.reserve(ib, true, m->stream);
    m->inc_pair.reserve(ib, true, m->stream);
    m->inc_pl.reserve(ib, true, m->stream);
    m->dperm.reserve((size_t)(m->n_dperm + (n_inc - m->n_inc)) * 4 + 4, true, m->stream);
    // scratch of the build: the new views' incidences only, from the first
    // new one on (the arenas' retired lists need none)
    m->scratch_base = (uint32_t)m->n_inc;
    const size_t sb = (size_t)std::max<int64_t>(n_inc - m->n_inc, 1) * 4;
    m->s_vox.reserve(sb, false, m->stream);
    m->s_rec.reserve(sb * 2, false, m->stream);
  }
  for (size_t k = 0; k < added.size(); ++k) emit_view(m, added[k], m->s_offs.as<uint32_t>() + coff[k]);
  // the new views' ray records on the host, and their counters
  const int64_t hw_new = npix - m->npix_total;
  std::vector<RayMeta> hm((size_t)std::max<int64_t>(hw_new, 0));
  ray_records_and_counters(m, added, m->npix_total, hm);
  // the new views' region lists: host work on their ray records, on host
  // threads while the GPU builds their pairs
  std::vector<RegionLists> lists((size_t)V);
  bool lists_failed = false;
  std::thread lists_thread([&] {
    try {
      region_lists_parallel(m, added, hm, m->npix_total, lists);
    } catch (...) {
      lists_failed = true;
    }
  });
  struct Joiner {
    std::thread& t;
    ~Joiner() {
      if (t.joinable()) t.join();
    }
  } joiner{lists_thread};
  // loud voxels of every live view: the old views' from their pairs, the
  // new ones' from the voxel ids of the emit pass
  const int64_t nvox = m->n_bricks * kBrickVox;
  m->s_loud.reserve((size_t)std::max<int64_t>(nvox, 1), false, m->stream);
  CK(cudaMemsetAsync(m->s_loud.p, 0, (size_t)std::max<int64_t>(nvox, 1), m->stream));
  for (int c = 0; c < m->built_views; ++c) {
    const View& v = m->views[c];
    if (v.retired || !v.n_inc) continue;
    CK(launch_loud_voxels_from_pairs(m->meta.as<RayMeta>() + v.pix_base, view_pixels(v), m->inc_pair.as<uint32_t>(),
                                     m->pair_vox.as<uint32_t>(), m->s_loud.as<uint8_t>(), m->stream));
  }
  for (int c : added)
    CK(launch_loud_voxels(m->meta.as<RayMeta>() + m->views[c].pix_base, view_pixels(m->views[c]),
                          m->s_vox.as<uint32_t>(), m->scratch_base, m->s_loud.as<uint8_t>(), m->stream));
  // an old view's quiet pairs (numbered after its loud ones) must all stay
  // quiet: where one became loud, the view prepares every pair
  m->s_k1.reserve(64, false, m->stream);
  for (int c = 0; c < m->built_views; ++c) {
    View& v = m->views[c];
    if (v.retired || v.n_loud >= v.n_pairs) continue;
    CK(cudaMemsetAsync(m->s_k1.p, 0, 4, m->stream));
    CK(launch_count_loud(m->pair_vox.as<uint32_t>() + v.pair_base + v.n_loud, v.n_pairs - v.n_loud,
                         m->s_loud.as<uint8_t>(), m->s_k1.as<uint32_t>(), m->stream));
    if (read1(m, m->s_k1.as<uint32_t>())) v.n_loud = v.n_pairs;
  }
  // 4. pairs of the new views, numbered after the existing ones
  const int bits = voxel_id_bits(m);
  int64_t pair_total = m->n_pairs, perm_total = m->n_perm_total, dperm_total = m->n_dperm,
          dpair_total = m->n_dpairs;
  const int64_t pair0 = pair_total, dpair0 = dpair_total;
  for (int c : added) view_pairs(m, c, bits, pair_total, perm_total, dperm_total, dpair_total);
  if (m->test_append_fail) {
    const mrf_status st = (mrf_status)m->test_append_fail;
    m->test_append_fail = 0;
    fail(st, "append of the new views' lists: injected failure (mrf_test_fail_next_append)");
  }
  // 5. ray queues and region blocks of the new views
  {
    int64_t base = 0;
    for (int c = 0; c < m->built_views; ++c) base = std::max<int64_t>(base, (int64_t)m->views[c].order_base + m->views[c].n_active);
    base = std::max<int64_t>(base, m->queue_end);
    m->ray_queue.reserve((size_t)std::max<int64_t>(base + hw_new, 1) * sizeof(RayMeta), true, m->stream);
    m->queue_ids.reserve((size_t)std::max<int64_t>(base + hw_new, 1) * 4, true, m->stream);
    for (int c = m->built_views; c < V; ++c) {
      View& v = m->views[c];
      v.order_base = (uint32_t)base;
      view_ray_queue(m, c);
      base += v.n_active;
    }
    m->queue_end = base;
    const int R = std::max(1, m->num_sms);
    m->counters.reserve((size_t)(V + 1) * 4, false, m->stream);
    m->rcounters.reserve(((size_t)2 * V * R + 2 * (size_t)V + 2) * 4, false, m->stream);
    lists_thread.join();
    if (lists_failed) fail(MRF_ERR_OOM, "host memory for the region queues");
    std::vector<int> newv;
    for (int c = m->built_views; c < V; ++c) {
      if (m->views[c].retired) {
        m->views[c].n_left = 0;
        m->views[c].left_base = 0;
      }
      newv.push_back(c);
    }
    m->region_end = region_blocks(m, newv, lists, m->region_end);
  }
  m->n_inc = n_inc;
  m->n_pairs = pair_total;
  m->n_perm_total = perm_total;
  m->n_dperm = dperm_total;
  m->n_dpairs = dpair_total;
  const size_t pb = (size_t)std::max<int64_t>(pair_total + 1, 1);
  m->pair_vox.reserve(pb * 4, true, m->stream);
  m->pair_m.reserve(pb * 4, true, m->stream);
  m->pair_cum.reserve(pb * 4, true, m->stream);
  m->pair_stat.reserve(pb * 4, true, m->stream);
  m->pair_ndyn.reserve(pb * 4, true, m->stream);
  m->pair_hit.reserve(pb * 4, true, m->stream);
  m->pair_seg.reserve(pb * 4, true, m->stream);
  m->dpair.reserve((size_t)(dpair_total + 1) * 4, true, m->stream);
  m->dseg.reserve((size_t)(dpair_total + 1) * 4, true, m->stream);
  m->drun.reserve((size_t)(dpair_total + 1) * 16, true, m->stream);
  CK(launch_drun(m->dpair.as<uint32_t>() + dpair0, (uint32_t)(dpair_total - dpair0), m->pair_vox.as<uint32_t>(),
                 m->pair_cum.as<float>(), m->pair_stat.as<float>(), m->drun.as<uint4>() + dpair0, m->stream));
  m->pair_q.reserve(pb * 4, false, m->stream);
  m->pair_dm.reserve(pb * 4, false, m->stream);
  CK(launch_fill_f32(m->pair_m.as<float>() + pair0, pair_total - pair0, 0.0f, m->stream));
  // tiles of the new views at the end of tile_first; the carries sized for
  // the largest launch
  {
    int64_t need = m->tile_end;
    for (int c = m->built_views; c < V; ++c) need += pair_update_tiles(m->views[c].n_dperm) + 1;
    m->tile_first.reserve((size_t)(need + 2) * 4, true, m->stream);
    uint32_t tb = (uint32_t)m->tile_end;
    int64_t most = m->carry_tiles;
    for (int c = m->built_views; c < V; ++c) {
      view_tiles(m, c, tb);
      tb += pair_update_tiles(m->views[c].n_dperm) + 1;
      most = std::max<int64_t>(most, (int64_t)pair_update_tiles(m->views[c].n_dperm) + 1);
    }
    m->tile_end = tb;
    m->carry_tiles = most;
    m->carry.reserve((size_t)most * sizeof(TileCarry), false, m->stream);
  }
  // active voxels: the new bricks' voxels start at 0, the new pairs add theirs
  m->vox_active.reserve((size_t)std::max<int64_t>(nvox, 1), true, m->stream);
  if (nvox > m->vox_active_n)
    CK(cudaMemsetAsync(m->vox_active.as<uint8_t>() + m->vox_active_n, 0, (size_t)(nvox - m->vox_active_n), m->stream));
  m->vox_active_n = nvox;
  CK(launch_mark_active(m->pair_vox.as<uint32_t>() + pair0, m->pair_cum.as<float>() + pair0,
                        (uint32_t)(pair_total - pair0), m->vox_active.as<uint8_t>(), m->stream));
  CK(cudaEventRecord(m->ev1, m->stream));
  sync(m);
  check_device_err(m);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, m->ev0, m->ev1);
  m->stats.build_ms = ms;
  m->built_version = m->version;
  m->jacobi_version = -1;
  m->built_views = V;
  m->npix_total = npix;
  m->bricks_at_build = m->n_bricks;
  stats_from_views(m);
  return true;
}

void build_jacobi_csr(mrf_map* m) {
  uint32_t np = (uint32_t)m->n_pairs;
  m->vpairs.reserve((size_t)np * 4 + 4, false, m->stream);
  m->vvox.reserve((size_t)np * 4 + 4, false, m->stream);
  m->vseg.reserve((size_t)np * 4 + 8, false, m->stream);
  m->s_k0.reserve((size_t)np * 4 + 4, false, m->stream);
  m->s_v0.reserve((size_t)np * 4 + 4, false, m->stream);
  m->s_k1.reserve((size_t)np * 4 + 4, false, m->stream);
  m->s_v1.reserve((size_t)np * 4 + 4, false, m->stream);
  if (np == 0) {
    m->n_vvox = 0;
    m->jacobi_version = m->built_version;
    return;
  }
  CK(launch_iota(m->s_v0.as<uint32_t>(), np, m->stream));
  int bits = 1;
  while (bits < 32 && ((uint64_t)1 << bits) <= (uint64_t)(m->n_bricks * kBrickVox)) ++bits;
  size_t t = sort_temp_bytes(np, bits);
  m->s_tmp.reserve(t, false, m->stream);
  CK(sort_pairs_u32(m->s_tmp.p, t, m->pair_vox.as<uint32_t>(), m->s_k1.as<uint32_t>(),
                    m->s_v0.as<uint32_t>(), m->vpairs.as<uint32_t>(), np, bits, m->stream));
  CK(launch_vflag(m->s_k1.as<uint32_t>(), np, m->s_k0.as<uint32_t>(), m->stream));
  CK(cudaMemsetAsync(m->s_k0.as<uint32_t>() + np, 0, 4, m->stream));
  size_t t2 = scan_temp_bytes(np + 1);
  m->s_tmp.reserve(t2, false, m->stream);
  CK(exclusive_scan_u32(m->s_tmp.p, t2, m->s_k0.as<uint32_t>(), m->s_v1.as<uint32_t>(), np + 1,
                        m->stream));
  uint32_t nv = read1(m, m->s_v1.as<uint32_t>() + np);
  CK(launch_vassign(m->s_k1.as<uint32_t>(), m->s_k0.as<uint32_t>(), m->s_v1.as<uint32_t>(), np,
                    m->vvox.as<uint32_t>(), m->vseg.as<uint32_t>(), m->stream));
  CK(cudaMemcpyAsync(m->vseg.as<uint32_t>() + nv, &np, 4, cudaMemcpyHostToDevice, m->stream));
  sync(m);
  m->n_vvox = nv;
  m->jacobi_version = m->built_version;
}

// Lists of views added since the last build are appended when that is exact
// (full-ray activation: see append_lists) and the arenas are not mostly
// retired views' data; otherwise, and after set_pose or load_map, every
// view is rebuilt (which also drops the retired views' data).
void ensure_built(mrf_map* m);

// the all-view structures (Jacobi queues and tiles, the voxel CSR) need
// one full build with no retired views' data in the arenas
void ensure_compact(mrf_map* m) {
  if (m->holes || m->appended) {
    m->needs_full = true;
    m->version++;
  }
  ensure_built(m);
}

// Retired views' lists stay in the arenas until they reach kDeadRatio times
// the live ones; the next build is then a full one, which drops them.  Only
// memory grows with them: no per-frame pass reads a retired view's data.
constexpr int64_t kDeadRatio = 8;

void ensure_built(mrf_map* m) {
  if (m->built_version != m->version) {
    const bool can_append = !m->needs_full && m->built_version >= 0 &&
                            m->prm.activation == MRF_ACT_FULL_RAY && m->built_views <= (int)m->views.size() &&
                            m->dead_inc * (kDeadRatio + 1) <= m->n_inc * kDeadRatio;
    bool done = false;
    if (can_append) {
      // a part-done append: the next build starts over, and the views it
      // was adding carry no pairs (their message range was never written)
      // into that build's message remap
      auto abandon = [&] {
        m->needs_full = true;
        for (size_t c = (size_t)std::max(m->built_views, 0); c < m->views.size(); ++c) {
          m->views[c].pair_base = 0;
          m->views[c].n_pairs = 0;
        }
      };
      try {
        done = append_lists(m);
      } catch (const Fail& e) {
        abandon();
        // out of memory: the retired views' lists fill it, and the full
        // build below drops them and reuses the buffers
        if (e.st != MRF_ERR_OOM) throw;
        ++m->stats.builds_oom_fallback;
      } catch (...) {
        abandon();
        throw;
      }
      if (done) {
        m->appended = true;
        m->len16_version = -1;
        ++m->stats.builds_appended;
      }
    }
    if (!done) {
      rebuild(m);
      m->appended = false;
      m->len16_version = -1;
      ++m->stats.builds_full;
    }
  }
  // the fp16 streams of the current lists
  if (m->precision == MRF_PRECISION_HALF_STREAMS && m->len16_version != m->built_version) {
    m->inc_len16.reserve((size_t)std::max<int64_t>(m->n_inc, 1) * 2, false, m->stream);
    m->pair_q16.reserve((size_t)std::max<int64_t>(m->n_pairs, 1) * 2, false, m->stream);
    CK(launch_to_half(m->inc_len.as<float>(), m->n_inc, m->inc_len16.as<__half>(), m->stream));
    m->len16_version = m->built_version;
  }
}

struct Profiler {
  mrf_map* m;
  bool on;
  size_t n = 0;
  void begin(int cat) {
    if (!on) return;
    while (m->prof_ev.size() < 2 * (n + 1)) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      m->prof_ev.push_back(e);
    }
    if (m->prof_cat.size() < n + 1) m->prof_cat.resize(n + 1);
    m->prof_cat[n] = cat;
    CK(cudaEventRecord(m->prof_ev[2 * n], m->stream));
  }
  void end() {
    if (!on) return;
    CK(cudaEventRecord(m->prof_ev[2 * n + 1], m->stream));
    ++n;
  }
  void collect() {
    for (int k = 0; k < 4; ++k) {
      m->stats.kernel_ms[k] = 0.0;
      m->stats.kernel_count[k] = 0;
    }
    for (size_t i = 0; i < n; ++i) {
      float ms = 0.0f;
      CK(cudaEventElapsedTime(&ms, m->prof_ev[2 * i], m->prof_ev[2 * i + 1]));
      m->stats.kernel_ms[m->prof_cat[i]] += ms;
      m->stats.kernel_count[m->prof_cat[i]] += 1;
    }
  }
};

// one BP iteration over every camera (src/GVDBInference.cpp:155-167):
// Gauss-Seidel camera by camera, or Jacobi over all cameras at once.  The
// pairs without dynamic incidences get their (constant) update in the first
// iteration of each mrf_infer call only: afterwards it would leave every
// value unchanged (L + (m_new - m_new) = L).
// the rays of view c, and of all views (c = -1; the views' queues and
// regions are contiguous), with their counters
RayWork ray_work(mrf_map* m, int c) {
  const int V = (int)m->views.size();
  const uint32_t R = m->nreg;
  RayWork w{};
  w.region = m->region_q.as<RayMeta>();
  w.region_ids = m->region_ids.as<uint32_t>();
  w.rper = R;
  uint32_t* lc = m->rcounters.as<uint32_t>() + (size_t)2 * V * R;  // leftover counters
  if (c >= 0) {
    const View& v = m->views[c];
    w.queue = m->ray_queue.as<RayMeta>() + v.order_base;
    w.queue_ids = m->queue_ids.as<uint32_t>() + v.order_base;
    w.n_rays = v.n_active;
    w.counter = m->counters.as<uint32_t>() + c;
    w.rstart = m->rstart.as<uint32_t>() + (size_t)c * (R + 1);
    w.nreg = R;
    w.rcounter = m->rcounters.as<uint32_t>() + (size_t)c * R;
    w.lprefix = m->lsingle.as<uint32_t>() + 2 * (size_t)c;
    w.lbase = m->lbase.as<uint32_t>() + c;
    w.nlv = 1;
    w.lcounter = lc + c;
  } else {
    w.queue = m->ray_queue.as<RayMeta>();
    w.queue_ids = m->queue_ids.as<uint32_t>();
    for (const View& v : m->views) w.n_rays += v.n_active;
    w.counter = m->counters.as<uint32_t>() + V;
    w.rstart = m->rstart.as<uint32_t>();
    w.nreg = (uint32_t)V * R;
    w.rcounter = m->rcounters.as<uint32_t>() + (size_t)V * R;
    w.lprefix = m->lprefix.as<uint32_t>();
    w.lbase = m->lbase.as<uint32_t>();
    w.nlv = (uint32_t)V;
    w.lcounter = lc + V;
  }
  return w;
}

void zero_counters(mrf_map* m) {
  const size_t V = m->views.size();
  CK(cudaMemsetAsync(m->counters.p, 0, (V + 1) * 4, m->stream));
  CK(cudaMemsetAsync(m->rcounters.p, 0, (2 * V * m->nreg + V + 1) * 4, m->stream));
}

// phase 0: the first iteration of a call (static-pair updates); phase 1:
// the second; phase 2: later ones.  From phase 2 on the ln q of a pair
// whose voxel has no dynamic incidence in any view (a quiet voxel, whose
// pairs are numbered after the others) cannot change: its total log-odds
// moves only through static-pair updates, which happen in the first
// iteration, and the second iteration's prepare has seen them all.  Those
// pairs' ln q is then left as it is.
void enqueue_iteration(mrf_map* m, const BpArrays& a, bool jacobi, int fix, int phase, bool quiet,
                       Profiler& prof, int64_t& launches) {
  const int V = (int)m->views.size();
  const bool first = phase == 0;
  zero_counters(m);
  if (!jacobi) {
    for (int c = 0; c < V; ++c) {
      const View& v = m->views[c];
      if (v.n_inc == 0) continue;
      prof.begin(0);
      CK(launch_pair_prepare(a, v.pair_base, v.pair_base + (phase >= 2 ? v.n_loud : v.n_pairs), 0,
                             m->stream));
      prof.end();
      prof.begin(1);
      CK(launch_ray_bp(a, ray_work(m, c), fix, m->num_sms, m->ray_variant, quiet && phase >= 2, m->stream));
      prof.end();
      prof.begin(2);
      if (v.n_dperm) {
        CK(launch_pair_update(a, v.dperm_base, v.dperm_base + v.n_dperm, v.dpair_base,
                              v.dpair_base + v.n_dpairs, m->tile_first.as<uint32_t>() + v.tile_base,
                              m->carry.as<TileCarry>(), 0, m->stream));
        launches += 2;
      }
      if (first) {
        CK(launch_static_pairs(a, v.pair_base, v.pair_base + v.n_pairs, 0, m->stream));
        ++launches;
      }
      prof.end();
      launches += 2;
    }
  } else {
    uint32_t P = (uint32_t)m->n_pairs;
    prof.begin(0);
    CK(launch_pair_prepare(a, 0, P, 1, m->stream));
    prof.end();
    prof.begin(1);
    // the queues of all views are contiguous: one launch over all rays
    CK(launch_ray_bp(a, ray_work(m, -1), fix, m->num_sms, m->ray_variant, quiet && phase >= 2, m->stream));
    prof.end();
    prof.begin(2);
    CK(launch_pair_update(a, 0, (uint32_t)m->n_dperm, 0, (uint32_t)m->n_dpairs,
                          m->tile_first.as<uint32_t>() + m->jac_tile_base, m->carry.as<TileCarry>(),
                          1, m->stream));
    if (first) CK(launch_static_pairs(a, 0, P, 1, m->stream));
    prof.end();
    prof.begin(3);
    CK(launch_voxel_apply(m->vseg.as<uint32_t>(), m->vpairs.as<uint32_t>(), m->vvox.as<uint32_t>(),
                          m->n_vvox, m->pair_dm.as<float>(), m->d_L.as<float>(), m->stream));
    prof.end();
    launches += 5 + (first ? 1 : 0);
  }
}

// The iteration is captured once per incidence build and schedule into a
// CUDA graph and replayed iters times.
cudaGraphExec_t iteration_graph(mrf_map* m, const BpArrays& a, bool jacobi, int fix, int phase, bool quiet,
                                int64_t& launches_per_iter) {
  int key = (jacobi ? 1 : 0) | (fix ? 2 : 0) | (phase << 2) | (quiet ? 16 : 0);
  auto& slot = m->graphs[key];
  if (slot.exec && slot.version == m->built_version) {
    launches_per_iter = slot.launches;
    return slot.exec;
  }
  if (slot.exec) {
    cudaGraphExecDestroy(slot.exec);
    slot.exec = nullptr;
  }
  Profiler off{m, false};
  int64_t launches = 0;
  cudaGraph_t graph = nullptr;
  CK(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
  try {
    enqueue_iteration(m, a, jacobi, fix, phase, quiet, off, launches);
  } catch (...) {
    cudaStreamEndCapture(m->stream, &graph);
    if (graph) cudaGraphDestroy(graph);
    throw;
  }
  CK(cudaStreamEndCapture(m->stream, &graph));
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  CK(e);
  slot.exec = exec;
  slot.version = m->built_version;
  slot.launches = launches;
  launches_per_iter = launches;
  return exec;
}

// beliefs of the voxels the iterations update, from their total log-odds
void refresh_beliefs(mrf_map* m) {
  CK(launch_belief_refresh(m->d_L.as<float>(), m->vox_active.as<uint8_t>(), m->n_bricks * kBrickVox,
                           m->d_belief.as<float>(), m->stream));
}

// tol > 0: stop after the first iteration whose largest belief change is
// below tol -- or, with a target field, whose largest distance to the
// target is at most tol (checked every check_every iterations; iters is the
// cap)
void run_infer(mrf_map* m, const int* ids, int n_ids, int iters, int flags, float tol = -1.0f,
               int check_every = 1, float* last_delta = nullptr, const float* target = nullptr) {
  const bool jacobi = flags & MRF_JACOBI;
  if (jacobi)
    ensure_compact(m);
  else
    ensure_built(m);
  if (jacobi && m->jacobi_version != m->built_version) build_jacobi_csr(m);
  const int V = (int)m->views.size();
  if (iters <= 0) iters = m->prm.max_iters > 0 ? m->prm.max_iters : 1;
  if (check_every < 1) check_every = 1;
  const bool quiet = quiet_path(m, iters, flags);  // before bp(): it may allocate the loud lists
  m->stats.quiet_prefix_used = quiet ? 1 : 0;
  BpArrays a = m->bp();
  int64_t launches = 0;
  Profiler prof{m, (flags & MRF_PROFILE) != 0};
  CK(cudaEventRecord(m->ev0, m->stream));
  if (!(flags & MRF_INCREMENTAL)) {
    // src/GVDBInference.cpp:128-133: the selected cameras start from zero
    for (int k = 0; k < (ids ? n_ids : V); ++k) {
      int c = ids ? ids[k] : k;
      if (c < 0 || c >= V) continue;
      const View& v = m->views[c];
      if (v.n_pairs == 0) continue;
      CK(launch_fill_f32(m->pair_m.as<float>() + v.pair_base, v.n_pairs, 0.0f, m->stream));
      ++launches;
    }
  }
  const int fix = (flags & MRF_FIX_PRE_RESET) ? 1 : 0;
  const bool conv = tol > 0.0f;
  const int64_t nvox = m->n_bricks * kBrickVox;
  if (conv) {
    m->s_prev.reserve((size_t)std::max<int64_t>(nvox, 1) * 4, false, m->stream);
    m->s_delta.reserve(64, false, m->stream);
  }
  float delta = -1.0f;
  int done = 0;
  if (m->n_inc > 0) {
    const bool direct = prof.on || (flags & MRF_NO_GRAPH);
    int64_t per[3] = {0, 0, 0};
    cudaGraphExec_t exec[3] = {nullptr, nullptr, nullptr};
    if (!direct)
      for (int ph = 0; ph < 3 && ph < iters; ++ph)
        exec[ph] = iteration_graph(m, a, jacobi, fix, ph, quiet, per[ph]);
    for (int it = 0; it < iters; ++it) {
      const bool check = conv && ((it + 1) % check_every == 0 || it + 1 == iters);
      if (check && !target) {
        refresh_beliefs(m);
        CK(cudaMemcpyAsync(m->s_prev.p, m->d_belief.p, (size_t)nvox * 4, cudaMemcpyDeviceToDevice,
                           m->stream));
      }
      const int ph = std::min(it, 2);
      if (it == 2 && quiet) {
        // from here on the ray kernel takes the static prefixes from
        // their quiet sums
        prof.begin(1);
        quiet_prefix_all(m, a);
        prof.end();
      }
      if (direct) {
        enqueue_iteration(m, a, jacobi, fix, ph, quiet, prof, launches);
      } else {
        CK(cudaGraphLaunch(exec[ph], m->stream));
        launches += per[ph];
      }
      done = it + 1;
      if (check) {
        refresh_beliefs(m);
        CK(launch_max_abs_diff(m->d_belief.as<float>(), target ? target : m->s_prev.as<float>(), nvox,
                               m->s_delta.as<uint32_t>(), m->stream));
        ++launches;
        uint32_t bits = 0;
        CK(cudaMemcpyAsync(&bits, m->s_delta.p, 4, cudaMemcpyDeviceToHost, m->stream));
        sync(m);
        std::memcpy(&delta, &bits, 4);
        if (target ? delta <= tol : delta < tol) break;
      }
    }
  }
  // the iteration kernels update L only; the beliefs follow once per call
  if (done > 0) {
    refresh_beliefs(m);
    ++launches;
  }
  CK(cudaEventRecord(m->ev1, m->stream));
  m->has_messages = true;
  m->stats.iters_done = done;
  m->stats.kernel_launches = launches;
  if (last_delta) *last_delta = delta;
  if (!(flags & MRF_ASYNC) || prof.on || conv) {
    sync(m);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, m->ev0, m->ev1);
    m->stats.infer_ms = ms;
    prof.collect();
  }
}

Geom make_geom(const mrf_params& p) {
  Geom g{};
  g.res = p.res;
  g.inv_res = 1.0f / p.res;
  g.fx = p.fx;
  g.fy = p.fy;
  g.cx = p.cx;
  g.cy = p.cy;
  g.rows = p.rows;
  g.cols = p.cols;
  for (int a = 0; a < 3; ++a) {
    float gg = p.dims[a] / p.res;
    g.hi[a] = gg;
    int G = (int)ceilf(gg);
    g.NB[a] = (G + 1 + kBrick - 1) / kBrick;
    g.E[a] = kBrick * g.NB[a];
    g.blo[a] = 0;
    g.bhi[a] = g.E[a];
    g.glo[a] = 0.0f;
  }
  g.off[0] = (p.dims[0] * 0.5f) / p.res;
  g.off[1] = (p.dims[1] * 0.5f) / p.res;
  g.off[2] = 0.0f;
  g.lookup_n = p.lookup_n;
  g.n_tiles_u = (p.cols + kLookupPx - 1) / kLookupPx;
  g.n_tiles_v = (p.rows + kLookupPx - 1) / kLookupPx;
  g.lut_rows = p.rows;
  g.lut_cols = p.cols;
  return g;
}

void set_pose(Pose& P, const float* pose) {
  for (int i = 0; i < 16; ++i) P.m[i] = pose[i];
}

mrf_status guard(mrf_map* m) {
  if (!m) {
    set_err("null map");
    return MRF_ERR_INVALID;
  }
  cudaSetDevice(m->device);
  return MRF_OK;
}

template <typename F>
mrf_status wrap(F&& f) {
  try {
    f();
    return MRF_OK;
  } catch (const Fail& e) {
    return e.st;
  } catch (const std::exception& e) {
    set_err(e.what());
    return MRF_ERR_INVALID;
  }
}

void destroy_bufs(mrf_map* m) {
  DBuf* all[] = {&m->d_sigma, &m->d_bias, &m->d_slot, &m->d_coord, &m->d_L, &m->d_belief,
                 &m->meta, &m->inc_pair, &m->inc_len, &m->inc_mu, &m->inc_pl, &m->pair_vox,
                 &m->pair_m, &m->pair_cum, &m->pair_stat, &m->pair_ndyn, &m->pair_hit, &m->pair_q,
                 &m->pair_dm,
                 &m->pair_seg, &m->dperm, &m->dpair, &m->dseg, &m->drun,
                 &m->carry, &m->ray_order, &m->ray_queue, &m->region_q, &m->rstart, &m->rcounters, &m->counters, &m->tile_first,
                 &m->lbase, &m->lsingle, &m->lprefix, &m->queue_ids, &m->region_ids, &m->loud_off,
                 &m->loud_pid, &m->loud_len, &m->loud_pos, &m->quiet_q,
                 &m->vseg, &m->vpairs, &m->vvox, &m->vox_active, &m->d_Lbase, &m->inc_len16, &m->pair_q16,
                 &m->s_rec, &m->s_recs, &m->s_pf, &m->s_ps,
                 &m->s_flags, &m->s_ind, &m->s_scan,
                 &m->s_q0, &m->s_q1, &m->s_q2, &m->s_q3, &m->s_bf, &m->s_loud, &m->s_pv, &m->s_sg,
                 &m->s_tmp, &m->s_counts, &m->s_offs, &m->s_vox, &m->s_k0, &m->s_k1, &m->s_v0,
                 &m->s_v1, &m->s_seg, &m->s_dense, &m->s_err, &m->s_depth_in, &m->s_depth,
                 &m->s_img, &m->s_part, &m->s_sum, &m->s_prev, &m->s_delta, &m->s_snap, &m->s_vcnt};
  for (DBuf* b : all) b->release();
  for (auto& v : m->views) v.depth.release();
}

// cam: the camera geometry (a view's, or the map's for an arbitrary pose)
void likelihood_dev(mrf_map* m, const Pose& P, const float* depth_clean, float* img_dev,
                    float* sum_dev, const Geom* cam = nullptr) {
  Geom g = cam ? *cam : m->g;
  g.brick_slot = m->d_slot.as<int>();
  int nb = likelihood_blocks(g);
  m->s_part.reserve((size_t)nb * 8, false, m->stream);
  const float* bel = m->d_belief.as<float>();
  if (m->n_bricks == 0) {
    // an empty map still needs a valid pointer for the kernel signature
    m->s_dense.reserve(4, false, m->stream);
    bel = m->s_dense.as<float>();
  }
  CK(launch_likelihood(g, P, depth_clean, bel, img_dev, m->s_part.as<double>(), nb, m->stream));
  CK(launch_reduce_partials(m->s_part.as<double>(), nb, sum_dev, m->stream));
}

}  // namespace

namespace mrf {

mrf_status mrf_internal_like_inputs(mrf_map* m, Geom* g, const float** belief, cudaStream_t* stream,
                                    int* device) {
  if (!m) {
    set_err("null map");
    return MRF_ERR_INVALID;
  }
  if (cudaSetDevice(m->device) != cudaSuccess) {
    set_err("cudaSetDevice failed");
    return MRF_ERR_CUDA;
  }
  *g = m->g;
  g->brick_slot = m->d_slot.as<int>();
  // no belief field before the first active brick (every brick-table probe
  // misses then, so the field is never read)
  *belief = m->n_bricks ? m->d_belief.as<float>() : nullptr;
  *stream = m->stream;
  *device = m->device;
  return MRF_OK;
}

void mrf_internal_set_error(const std::string& msg) { set_err(msg); }

}  // namespace mrf

extern "C" {

const char* mrf_last_error(void) { return g_last_error.c_str(); }

mrf_status mrf_create(const mrf_params* params, mrf_map** out) {
  if (!params || !out) {
    set_err("null argument");
    return MRF_ERR_INVALID;
  }
  *out = nullptr;
  const mrf_params& p = *params;
  if (!(p.res > 0.0f) || p.rows <= 0 || p.cols <= 0 || !(p.fx > 0.0f) || !(p.fy > 0.0f) ||
      !(p.cx > 0.0f) || !(p.cy > 0.0f) || (p.lookup_n != 2 && p.lookup_n != 3) || !p.sigma_lut ||
      !p.bias_lut || !(p.prior > 0.0f && p.prior < 1.0f) ||
      (p.activation != MRF_ACT_ENDPOINT && p.activation != MRF_ACT_FULL_RAY)) {
    set_err("invalid mrf_params");
    return MRF_ERR_INVALID;
  }
  for (int a = 0; a < 3; ++a)
    if (!(p.dims[a] > 0.0f)) {
      set_err("invalid dims");
      return MRF_ERR_INVALID;
    }
  mrf_map* m = new mrf_map();
  mrf_status st = wrap([&] {
    m->prm = p;
    int nl = ((p.rows + kLookupPx - 1) / kLookupPx) * ((p.cols + kLookupPx - 1) / kLookupPx) *
             p.lookup_n;
    if (nl > 3096) fail(MRF_ERR_INVALID, "sensor lookup table larger than 3096 floats");
    m->sigma.assign(p.sigma_lut, p.sigma_lut + nl);
    m->bias.assign(p.bias_lut, p.bias_lut + nl);
    m->prm.sigma_lut = m->sigma.data();
    m->prm.bias_lut = m->bias.data();
    CK(cudaGetDevice(&m->device));
    CK(cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, m->device));
    for (int k = 0; k < ray_bp_variants(); ++k) {
      ray_bp_resident_blocks(k, 0);
      ray_bp_resident_blocks(k, 1);
    }
    CK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&m->ev0));
    CK(cudaEventCreate(&m->ev1));
    m->g = make_geom(p);
    m->nb_grid = (int64_t)m->g.NB[0] * m->g.NB[1] * m->g.NB[2];
    m->d_sigma.reserve((size_t)nl * 4, false, m->stream);
    m->d_bias.reserve((size_t)nl * 4, false, m->stream);
    CK(cudaMemcpyAsync(m->d_sigma.p, m->sigma.data(), (size_t)nl * 4, cudaMemcpyHostToDevice, m->stream));
    CK(cudaMemcpyAsync(m->d_bias.p, m->bias.data(), (size_t)nl * 4, cudaMemcpyHostToDevice, m->stream));
    m->g.sigma = m->d_sigma.as<float>();
    m->g.bias = m->d_bias.as<float>();
    m->d_slot.reserve((size_t)m->nb_grid * 4, false, m->stream);
    CK(cudaMemsetAsync(m->d_slot.p, 0xFF, (size_t)m->nb_grid * 4, m->stream));
    m->s_flags.reserve((size_t)m->nb_grid, false, m->stream);
    m->s_err.reserve(16, false, m->stream);
    CK(cudaMemsetAsync(m->s_err.p, 0, 16, m->stream));
    m->s_sum.reserve(16, false, m->stream);
    m->g.brick_slot = m->d_slot.as<int>();
    sync(m);
  });
  if (st != MRF_OK) {
    destroy_bufs(m);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return st;
  }
  *out = m;
  return MRF_OK;
}

void mrf_destroy(mrf_map* m) {
  if (!m) return;
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  destroy_bufs(m);
  if (m->stream) cudaStreamSynchronize(m->stream);
  for (cudaEvent_t e : m->prof_ev) cudaEventDestroy(e);
  for (auto& g : m->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  if (m->ev0) cudaEventDestroy(m->ev0);
  if (m->ev1) cudaEventDestroy(m->ev1);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

mrf_status mrf_release_cached_memory(void) {
  std::lock_guard<std::mutex> lk(g_pool_mu);
  for (int d = 0; d < kMaxDevices; ++d) {
    if (!g_pools[d]) continue;
    cudaError_t e = cudaMemPoolTrimTo(g_pools[d], 0);
    if (e != cudaSuccess) {
      set_err(std::string("cudaMemPoolTrimTo: ") + cudaGetErrorString(e));
      return MRF_ERR_CUDA;
    }
  }
  return MRF_OK;
}

mrf_status mrf_set_memory_limit(int64_t bytes) {
  if (bytes < 0) {
    set_err("negative memory limit");
    return MRF_ERR_INVALID;
  }
  g_limit.store(bytes);
  return MRF_OK;
}

int64_t mrf_memory_in_use(void) {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) return -1;
  return g_in_use[d].load();
}

mrf_status mrf_test_brick_footprint(mrf_map* m, int view_id, int64_t b0, int64_t b1, uint8_t* mask, int* all) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (view_id < 0 || view_id >= (int)m->views.size() || !mask || !all || b0 < 0 || b1 < b0 || b1 > m->n_bricks) {
    set_err("invalid footprint arguments");
    return MRF_ERR_INVALID;
  }
  return wrap([&] {
    const View& v = m->views[view_id];
    if (v.retired) fail(MRF_ERR_STATE, "view retired");
    const int64_t hw = (int64_t)v.cam.rows * v.cam.cols;
    m->s_dense.reserve((size_t)hw + 16, false, m->stream);
    CK(cudaMemsetAsync(m->s_dense.p, 0, (size_t)hw, m->stream));
    CK(cudaMemsetAsync(m->s_err.as<int>() + 2, 0, 4, m->stream));
    CK(launch_brick_footprint(v.cam, v.pose, m->d_coord.as<int>(), (uint32_t)b0, (uint32_t)b1,
                              m->s_dense.as<uint8_t>(), m->s_err.as<int>() + 2, m->stream));
    CK(cudaMemcpyAsync(mask, m->s_dense.p, (size_t)hw, cudaMemcpyDeviceToHost, m->stream));
    CK(cudaMemcpyAsync(all, m->s_err.as<int>() + 2, 4, cudaMemcpyDeviceToHost, m->stream));
    sync(m);
  });
}

mrf_status mrf_test_raise_device_error(mrf_map* m) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  return wrap([&] {
    const int one = 1;
    CK(cudaMemcpyAsync(m->s_err.p, &one, sizeof(int), cudaMemcpyHostToDevice, m->stream));
    sync(m);
  });
}

mrf_status mrf_test_region_lists(const int32_t* records, int64_t n_pix, int regions, int share, uint32_t* home,
                                 int64_t* n_home, uint32_t* starts, uint32_t* left, int64_t* n_left) {
  if (!records || n_pix < 0 || n_pix > (int64_t)0x7FFFFFFF || regions < 1 || share < 0 || share > 100 || !home ||
      !n_home || !starts || !left || !n_left) {
    set_err("mrf_test_region_lists: invalid arguments");
    return MRF_ERR_INVALID;
  }
  return wrap([&] {
    std::vector<RayMeta> hm((size_t)n_pix);
    for (int64_t i = 0; i < n_pix; ++i) {
      const int32_t* r = records + 3 * i;
      for (int k = 0; k < 3; ++k)
        if (r[k] < 0 || r[k] > 65535) fail(MRF_ERR_INVALID, "mrf_test_region_lists: fields must lie in [0, 65535]");
      RayMeta me{};
      me.n_pre = (uint16_t)r[0];
      me.n_post = (uint16_t)r[1];
      me.flags = (uint32_t)r[2] << 16;
      hm[(size_t)i] = me;
    }
    View v;
    v.cam.rows = 1;
    v.cam.cols = (int)n_pix;
    v.pix_base = 0;
    v.retired = false;
    RegionLists l;
    region_lists(v, hm.data(), regions, share, l);
    std::copy(l.home.begin(), l.home.end(), home);
    std::copy(l.left.begin(), l.left.end(), left);
    for (int r = 0; r < regions; ++r) starts[r] = r < (int)l.starts.size() ? l.starts[(size_t)r] : 0u;
    starts[regions] = (uint32_t)l.home.size();
    *n_home = (int64_t)l.home.size();
    *n_left = (int64_t)l.left.size();
  });
}

mrf_status mrf_test_fail_next_append(mrf_map* m, mrf_status status) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (status == MRF_OK) {
    set_err("mrf_test_fail_next_append: a failure status is needed");
    return MRF_ERR_INVALID;
  }
  m->test_append_fail = (int)status;
  return MRF_OK;
}

static mrf_status add_view_impl(mrf_map* m, const float* pose, const float* depth, bool device,
                                int* view_id, const int* cam_size = nullptr, const float* cam_k = nullptr,
                                const int* box_lo = nullptr, const int* box_hi = nullptr) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (!pose || !depth) {
    set_err("null pose or depth");
    return MRF_ERR_INVALID;
  }
  if (box_lo)
    for (int a = 0; a < 3; ++a)
      if (box_lo[a] < 0 || box_hi[a] > m->g.NB[a] || box_lo[a] >= box_hi[a]) {
        set_err("scene box outside the brick grid or empty");
        return MRF_ERR_INVALID;
      }
  if (cam_size && (cam_size[0] < 1 || cam_size[1] < 1 || (int64_t)cam_size[0] * cam_size[1] > (1 << 26) ||
                   !(cam_k[0] > 0.0f) || !(cam_k[1] > 0.0f))) {
    set_err("invalid camera");
    return MRF_ERR_INVALID;
  }
  return wrap([&] {
    View v;
    set_pose(v.pose, pose);
    v.cam = m->g;
    if (cam_size) {
      v.cam.rows = cam_size[0];
      v.cam.cols = cam_size[1];
      v.cam.fx = cam_k[0];
      v.cam.fy = cam_k[1];
      v.cam.cx = cam_k[2];
      v.cam.cy = cam_k[3];
    }
    if (box_lo)
      for (int a = 0; a < 3; ++a) {
        v.cam.blo[a] = kBrick * box_lo[a];
        v.cam.bhi[a] = kBrick * box_hi[a];
        v.cam.glo[a] = (float)v.cam.blo[a];
        v.cam.hi[a] = std::min(m->g.hi[a], (float)v.cam.bhi[a]);
      }
    const int64_t HW = (int64_t)v.cam.rows * v.cam.cols;
    v.depth.reserve((size_t)HW * 4, false, m->stream);
    const float* src = depth;
    if (!device) {
      m->s_depth_in.reserve((size_t)HW * 4, false, m->stream);
      CK(cudaMemcpyAsync(m->s_depth_in.p, depth, (size_t)HW * 4, cudaMemcpyHostToDevice, m->stream));
      src = m->s_depth_in.as<float>();
    }
    CK(launch_clean_depth(src, v.depth.as<float>(), v.cam.rows, v.cam.cols, m->stream));
    activate_view(m, v);
    m->views.push_back(std::move(v));
    m->version++;  // the view set changed: incidence lists must be rebuilt
    m->stats.n_views = (int64_t)m->views.size();
    m->stats.n_bricks = m->n_bricks;
    if (view_id) *view_id = (int)m->views.size() - 1;
  });
}

mrf_status mrf_add_view(mrf_map* m, const float* pose, const float* depth_host, int* view_id) {
  return add_view_impl(m, pose, depth_host, false, view_id);
}

mrf_status mrf_add_view_device(mrf_map* m, const float* pose, const float* depth_dev, int* view_id) {
  return add_view_impl(m, pose, depth_dev, true, view_id);
}

mrf_status mrf_add_view_camera(mrf_map* m, const float* pose, const float* depth_host, int rows, int cols,
                               float fx, float fy, float cx, float cy, int* view_id) {
  const int size[2] = {rows, cols};
  const float k[4] = {fx, fy, cx, cy};
  return add_view_impl(m, pose, depth_host, false, view_id, size, k);
}

mrf_status mrf_add_view_box(mrf_map* m, const float* pose, const float* depth_host, int rows, int cols, float fx,
                            float fy, float cx, float cy, const int brick_lo[3], const int brick_hi[3],
                            int* view_id) {
  if (!brick_lo || !brick_hi) {
    set_err("null scene box");
    return MRF_ERR_INVALID;
  }
  const int size[2] = {rows, cols};
  const float k[4] = {fx, fy, cx, cy};
  return add_view_impl(m, pose, depth_host, false, view_id, size, k, brick_lo, brick_hi);
}

mrf_status mrf_view_camera(mrf_map* m, int view_id, int* rows, int* cols, float* k4) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (view_id < 0 || view_id >= (int)m->views.size()) {
    set_err("invalid view id");
    return MRF_ERR_INVALID;
  }
  const Geom& c = m->views[view_id].cam;
  if (rows) *rows = c.rows;
  if (cols) *cols = c.cols;
  if (k4) {
    k4[0] = c.fx;
    k4[1] = c.fy;
    k4[2] = c.cx;
    k4[3] = c.cy;
  }
  return MRF_OK;
}

mrf_status mrf_set_pose(mrf_map* m, int view_id, const float* pose) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (!pose || view_id < 0 || view_id >= (int)m->views.size()) {
    set_err("invalid view id or pose");
    return MRF_ERR_INVALID;
  }
  if (m->views[view_id].retired) {
    set_err("view retired (mrf_retire_view)");
    return MRF_ERR_STATE;
  }
  return wrap([&] {
    // take the camera's messages out of the total log-odds before it moves
    // (src/GVDBInference.cpp:66-82 removes its ray contributions first)
    const View& v = m->views[view_id];
    if (m->has_messages && v.n_pairs)
      CK(launch_remove_messages(m->bp(), v.pair_base, v.pair_base + v.n_pairs, m->stream));
    set_pose(m->views[view_id].pose, pose);
    activate_view(m, m->views[view_id]);
    m->version++;
    m->needs_full = true;  // the moved view's lists are traced anew
    m->stats.n_bricks = m->n_bricks;
  });
}

mrf_status mrf_retire_view(mrf_map* m, int view_id) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (view_id < 0 || view_id >= (int)m->views.size()) {
    set_err("invalid view id");
    return MRF_ERR_INVALID;
  }
  View& v = m->views[view_id];
  if (v.retired) return MRF_OK;
  return wrap([&] {
    const int64_t nvox = m->n_bricks * kBrickVox;
    if (!m->has_base && nvox) {
      const float lp = logf(m->prm.prior) - logf(1.0f - m->prm.prior);
      m->d_Lbase.reserve((size_t)nvox * 4, false, m->stream);
      CK(launch_fill_f32(m->d_Lbase.as<float>(), nvox, lp, m->stream));
      m->has_base = true;
    }
    // its messages stay in L; the base keeps them for the calls that rebuild
    // L from the prior and the live views' messages
    if (m->has_messages && v.n_pairs)
      CK(launch_fold_messages(m->pair_vox.as<uint32_t>() + v.pair_base, m->pair_m.as<float>() + v.pair_base,
                              v.n_pairs, m->d_Lbase.as<float>(), m->stream));
    sync(m);
    v.depth.release();
    v.retired = true;
    // its lists and pairs are out of every launch from now on; their space
    // in the arenas is reclaimed by the next full build
    if (v.n_inc) m->holes = true;
    m->dead_inc += v.n_inc;
    v.n_inc = v.n_pairs = v.n_perm = v.n_dperm = v.n_dpairs = v.n_active = v.n_left = v.n_loud = 0;
    m->version++;
  });
}

mrf_status mrf_infer(mrf_map* m, const int* ids, int n_ids, int iters, int flags) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (n_ids < 0 || (n_ids > 0 && !ids)) {
    set_err("invalid ids");
    return MRF_ERR_INVALID;
  }
  return wrap([&] { run_infer(m, ids, ids ? n_ids : 0, iters, flags); });
}

mrf_status mrf_infer_converge(mrf_map* m, const int* ids, int n_ids, int max_iters, float tol,
                              int check_every, int flags, int* iters_done, float* last_delta) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (n_ids < 0 || (n_ids > 0 && !ids) || !(tol > 0.0f)) {
    set_err("invalid ids or tolerance");
    return MRF_ERR_INVALID;
  }
  return wrap([&] {
    run_infer(m, ids, ids ? n_ids : 0, max_iters, flags, tol, check_every, last_delta);
    if (iters_done) *iters_done = (int)m->stats.iters_done;
  });
}

mrf_status mrf_infer_until(mrf_map* m, const int* ids, int n_ids, int max_iters, const float* target_dev,
                           float tol, int check_every, int flags, int* iters_done, float* last_dist) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (n_ids < 0 || (n_ids > 0 && !ids) || !(tol >= 0.0f) || !target_dev) {
    set_err("invalid ids, tolerance or target");
    return MRF_ERR_INVALID;
  }
  return wrap([&] {
    run_infer(m, ids, ids ? n_ids : 0, max_iters, flags, tol > 0.0f ? tol : 1e-30f, check_every, last_dist,
              target_dev);
    if (iters_done) *iters_done = (int)m->stats.iters_done;
  });
}

// The total log-odds without the live views' messages: the prior, plus the
// messages of retired views once there are any (their beliefs, which only
// those messages set, stay as they are).  Live views' messages are added
// back by k_voxel_rebuild.
static void start_logodds(mrf_map* m, float lp) {
  const int64_t nvox = m->n_bricks * kBrickVox;
  if (m->has_base)
    CK(cudaMemcpyAsync(m->d_L.p, m->d_Lbase.p, (size_t)nvox * 4, cudaMemcpyDeviceToDevice, m->stream));
  else
    CK(launch_fill_new_voxels(m->d_L.as<float>(), m->d_belief.as<float>(), 0, nvox, lp, m->stream));
}

// Warm start.  The messages start from a split of the predicted field
// L_pred: pairs without dynamic incidences get their exact (constant)
// message, the dynamic pairs of a voxel share the rest of
// L_pred - logit(prior) in proportion to their cumulative lengths.  Then,
// with the total log-odds held at L_pred, `sweeps` clamped iterations
// m <- F(L_pred - m) refine them (each one Jacobi evaluation of every ray
// factor).  Finally the total log-odds is rebuilt from the messages,
// L = logit(prior) + sum m, so the state is a consistent BP state: the
// equations and their fixed point are those of the plain start.
static void warm_start_impl(mrf_map* m, const float* L_pred, bool device_ptr, int sweeps) {
  ensure_compact(m);
  if (m->jacobi_version != m->built_version) build_jacobi_csr(m);
  const int64_t nvox = m->n_bricks * kBrickVox;
  if (nvox == 0 || m->n_inc == 0) return;
  if (sweeps < 0) sweeps = 0;
  const float lp = logf(m->prm.prior) - logf(1.0f - m->prm.prior);
  CK(cudaMemcpyAsync(m->d_L.p, L_pred, (size_t)nvox * 4,
                     device_ptr ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, m->stream));
  CK(launch_warm_split(m->vseg.as<uint32_t>(), m->vpairs.as<uint32_t>(), m->vvox.as<uint32_t>(), m->n_vvox,
                       m->d_L.as<float>(), lp, m->has_base ? m->d_Lbase.as<float>() : nullptr,
                       m->pair_cum.as<float>(), m->pair_stat.as<float>(), m->pair_ndyn.as<uint32_t>(),
                       m->pair_m.as<float>(), m->stream));
  BpArrays a = m->bp();
  const int V = (int)m->views.size();
  const uint32_t P = (uint32_t)m->n_pairs;
  for (int k = 0; k < sweeps; ++k) {
    zero_counters(m);
    CK(launch_pair_prepare(a, 0, P, 1, m->stream));
    CK(launch_ray_bp(a, ray_work(m, -1), 0, m->num_sms, m->ray_variant, false, m->stream));
    CK(launch_pair_update(a, 0, (uint32_t)m->n_dperm, 0, (uint32_t)m->n_dpairs,
                          m->tile_first.as<uint32_t>() + m->jac_tile_base, m->carry.as<TileCarry>(),
                          1, m->stream));
  }
  start_logodds(m, lp);
  CK(launch_voxel_rebuild(m->vseg.as<uint32_t>(), m->vpairs.as<uint32_t>(), m->vvox.as<uint32_t>(),
                          m->n_vvox, m->pair_m.as<float>(), m->pair_cum.as<float>(),
                          m->d_L.as<float>(), m->d_belief.as<float>(), m->stream));
  m->has_messages = true;
  sync(m);
  check_device_err(m);
}

// BP state I/O: one camera's messages as a dense field over the voxel slots
// (0 where the camera has no pair), and the reverse.
mrf_status mrf_read_messages(mrf_map* m, int view_id, float* out_dense) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (view_id < 0 || view_id >= (int)m->views.size() || !out_dense) {
    set_err("invalid view id or null argument");
    return MRF_ERR_INVALID;
  }
  if (m->views[view_id].retired) {
    set_err("view retired (mrf_retire_view)");
    return MRF_ERR_STATE;
  }
  return wrap([&] {
    ensure_built(m);
    const int64_t nvox = m->n_bricks * kBrickVox;
    if (nvox == 0) return;
    const View& v = m->views[view_id];
    m->s_dense.reserve((size_t)nvox * 4, false, m->stream);
    CK(cudaMemsetAsync(m->s_dense.p, 0, (size_t)nvox * 4, m->stream));
    CK(launch_remap_scatter(m->pair_vox.as<uint32_t>() + v.pair_base, m->pair_m.as<float>() + v.pair_base,
                            v.n_pairs, m->s_dense.as<float>(), m->stream));
    CK(cudaMemcpyAsync(out_dense, m->s_dense.p, (size_t)nvox * 4, cudaMemcpyDeviceToHost, m->stream));
    sync(m);
  });
}

mrf_status mrf_write_messages(mrf_map* m, int view_id, const float* dense) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (view_id < 0 || view_id >= (int)m->views.size() || !dense) {
    set_err("invalid view id or null argument");
    return MRF_ERR_INVALID;
  }
  if (m->views[view_id].retired) {
    set_err("view retired (mrf_retire_view)");
    return MRF_ERR_STATE;
  }
  return wrap([&] {
    ensure_built(m);
    const int64_t nvox = m->n_bricks * kBrickVox;
    if (nvox == 0) return;
    const View& v = m->views[view_id];
    m->s_dense.reserve((size_t)nvox * 4, false, m->stream);
    CK(cudaMemcpyAsync(m->s_dense.p, dense, (size_t)nvox * 4, cudaMemcpyHostToDevice, m->stream));
    CK(launch_remap_gather(m->pair_vox.as<uint32_t>() + v.pair_base, m->pair_m.as<float>() + v.pair_base,
                           v.n_pairs, m->s_dense.as<float>(), m->stream));
    m->has_messages = true;
    sync(m);
  });
}

mrf_status mrf_rebuild_logodds(mrf_map* m) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  return wrap([&] {
    ensure_compact(m);
    if (m->jacobi_version != m->built_version) build_jacobi_csr(m);
    const int64_t nvox = m->n_bricks * kBrickVox;
    if (nvox == 0) return;
    const float lp = logf(m->prm.prior) - logf(1.0f - m->prm.prior);
    start_logodds(m, lp);
    CK(launch_voxel_rebuild(m->vseg.as<uint32_t>(), m->vpairs.as<uint32_t>(), m->vvox.as<uint32_t>(),
                            m->n_vvox, m->pair_m.as<float>(), m->pair_cum.as<float>(),
                            m->d_L.as<float>(), m->d_belief.as<float>(), m->stream));
    sync(m);
  });
}

mrf_status mrf_warm_features(mrf_map* m, float* feat_dev) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (!feat_dev) {
    set_err("null argument");
    return MRF_ERR_INVALID;
  }
  return wrap([&] {
    ensure_compact(m);
    if (m->jacobi_version != m->built_version) build_jacobi_csr(m);
    const int64_t nvox = m->n_bricks * kBrickVox;
    CK(launch_voxel_features(m->vseg.as<uint32_t>(), m->vpairs.as<uint32_t>(), m->vvox.as<uint32_t>(),
                             m->n_vvox, m->pair_cum.as<float>(), m->pair_stat.as<float>(),
                             m->pair_hit.as<float>(), m->d_belief.as<float>(), nvox, feat_dev,
                             m->stream));
    sync(m);
  });
}

mrf_status mrf_warm_start(mrf_map* m, const float* logodds, int sweeps) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (!logodds) {
    set_err("null argument");
    return MRF_ERR_INVALID;
  }
  return wrap([&] { warm_start_impl(m, logodds, false, sweeps); });
}

mrf_status mrf_warm_start_device(mrf_map* m, const float* logodds_dev, int sweeps) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (!logodds_dev) {
    set_err("null argument");
    return MRF_ERR_INVALID;
  }
  return wrap([&] { warm_start_impl(m, logodds_dev, true, sweeps); });
}

int mrf_ray_variants(void) { return ray_bp_variants(); }

static void drop_graphs(mrf_map* m) {
  for (auto& g : m->graphs) g.version = -1;
}

mrf_status mrf_set_precision(mrf_map* m, int mode) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (mode != MRF_PRECISION_FP32 && mode != MRF_PRECISION_HALF_STREAMS) {
    set_err("invalid precision mode");
    return MRF_ERR_INVALID;
  }
  if (mode != m->precision) {
    m->precision = mode;
    m->len16_version = -1;
    drop_graphs(m);
  }
  return MRF_OK;
}

mrf_status mrf_set_ray_variant(mrf_map* m, int variant) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (variant < 0 || variant >= ray_bp_variants()) {
    set_err("invalid ray-kernel variant");
    return MRF_ERR_INVALID;
  }
  m->ray_variant = variant;
  drop_graphs(m);
  return MRF_OK;
}

// reps timed iterations (after one warm-up) of the map's current schedule,
// the BP state saved before and restored after: milliseconds per iteration
static double time_schedule(mrf_map* m, bool jacobi, int reps) {
  if (m->n_inc <= 0) return 0.0;
  // the iterations of a long call (the third on)
  const bool quiet = quiet_path(m, 1 << 30, jacobi ? MRF_JACOBI : 0);
  BpArrays a = m->bp();
  const size_t nv = (size_t)m->n_bricks * kBrickVox * 4, npb = (size_t)m->n_pairs * 4;
  m->s_snap.reserve(2 * nv + npb, false, m->stream);
  char* snap = static_cast<char*>(m->s_snap.p);
  CK(cudaMemcpyAsync(snap, m->d_L.p, nv, cudaMemcpyDeviceToDevice, m->stream));
  CK(cudaMemcpyAsync(snap + nv, m->d_belief.p, nv, cudaMemcpyDeviceToDevice, m->stream));
  CK(cudaMemcpyAsync(snap + 2 * nv, m->pair_m.p, npb, cudaMemcpyDeviceToDevice, m->stream));
  Profiler off{m, false};
  int64_t launches = 0;
  if (quiet) quiet_prefix_all(m, a);
  for (int r = 0; r <= reps; ++r) {
    if (r == 1) CK(cudaEventRecord(m->ev0, m->stream));
    enqueue_iteration(m, a, jacobi, 0, 2, quiet, off, launches);
  }
  CK(cudaEventRecord(m->ev1, m->stream));
  sync(m);
  float t = 0.0f;
  CK(cudaEventElapsedTime(&t, m->ev0, m->ev1));
  CK(cudaMemcpyAsync(m->d_L.p, snap, nv, cudaMemcpyDeviceToDevice, m->stream));
  CK(cudaMemcpyAsync(m->d_belief.p, snap + nv, nv, cudaMemcpyDeviceToDevice, m->stream));
  CK(cudaMemcpyAsync(m->pair_m.p, snap + 2 * nv, npb, cudaMemcpyDeviceToDevice, m->stream));
  sync(m);
  return t / reps;
}

mrf_status mrf_set_home_share(mrf_map* m, int percent) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (percent < 1 || percent > 100) {
    set_err("home share must be 1..100 per cent");
    return MRF_ERR_INVALID;
  }
  if (percent == m->home_share) return MRF_OK;
  return wrap([&] {
    m->home_share = percent;
    rebuild_regions(m);
    drop_graphs(m);
  });
}

mrf_status mrf_set_pair_variant(mrf_map* m, int variant) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (variant < 0 || variant > 1) {
    set_err("invalid pair-reduction variant");
    return MRF_ERR_INVALID;
  }
  m->pair_variant = variant;
  drop_graphs(m);
  return MRF_OK;
}

mrf_status mrf_get_tuning(mrf_map* m, int* ray_variant, int* home_share, int* pair_variant) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (ray_variant) *ray_variant = m->ray_variant;
  if (home_share) *home_share = m->home_share;
  if (pair_variant) *pair_variant = m->pair_variant;
  return MRF_OK;
}

mrf_status mrf_autotune_home_share(mrf_map* m, int reps, int flags, const int* shares, int n, double* ms_out,
                                   int* chosen) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (reps < 1 || n < 1 || !shares) {
    set_err("invalid autotune arguments");
    return MRF_ERR_INVALID;
  }
  for (int k = 0; k < n; ++k)
    if (shares[k] < 1 || shares[k] > 100) {
      set_err("home share must be 1..100 per cent");
      return MRF_ERR_INVALID;
    }
  const bool jacobi = (flags & MRF_JACOBI) != 0;
  return wrap([&] {
    if (jacobi)
      ensure_compact(m);
    else
      ensure_built(m);
    if (jacobi && m->jacobi_version != m->built_version) build_jacobi_csr(m);
    std::vector<double> ms((size_t)n, 0.0);
    for (int k = 0; k < n; ++k) {
      m->home_share = shares[k];
      rebuild_regions(m);
      drop_graphs(m);
      ms[(size_t)k] = time_schedule(m, jacobi, reps);
    }
    int best = 0;
    for (int k = 1; k < n; ++k)
      if (ms[(size_t)k] < ms[(size_t)best]) best = k;
    m->home_share = shares[best];
    rebuild_regions(m);
    drop_graphs(m);
    if (ms_out)
      for (int k = 0; k < n; ++k) ms_out[k] = ms[(size_t)k];
    if (chosen) *chosen = shares[best];
  });
}

mrf_status mrf_autotune(mrf_map* m, int reps, double* ms_out, int cap, int* chosen) {
  return mrf_autotune_flags(m, reps, 0, ms_out, cap, chosen);
}

mrf_status mrf_autotune_flags(mrf_map* m, int reps, int flags, double* ms_out, int cap, int* chosen) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (reps < 1 || cap < 0 || (cap > 0 && !ms_out)) {
    set_err("invalid autotune arguments");
    return MRF_ERR_INVALID;
  }
  const bool jacobi = (flags & MRF_JACOBI) != 0;
  return wrap([&] {
    if (jacobi)
      ensure_compact(m);
    else
      ensure_built(m);
    if (jacobi && m->jacobi_version != m->built_version) build_jacobi_csr(m);
    const int V = (int)m->views.size();
    const int NV = ray_bp_variants();
    const bool quiet = quiet_path(m, 1 << 30, flags);  // the iterations of a long call
    BpArrays a = m->bp();
    std::vector<double> ms(NV, 0.0);
    if (m->n_inc > 0) {
      // Each variant runs whole Gauss-Seidel iterations (the ray kernel's
      // cache policy also changes what the pair kernels after it find in
      // L2); the map state is saved first and restored after every variant.
      const size_t nv = (size_t)m->n_bricks * kBrickVox * 4, npb = (size_t)m->n_pairs * 4;
      m->s_snap.reserve(2 * nv + npb, false, m->stream);
      char* snap = static_cast<char*>(m->s_snap.p);
      CK(cudaMemcpyAsync(snap, m->d_L.p, nv, cudaMemcpyDeviceToDevice, m->stream));
      CK(cudaMemcpyAsync(snap + nv, m->d_belief.p, nv, cudaMemcpyDeviceToDevice, m->stream));
      CK(cudaMemcpyAsync(snap + 2 * nv, m->pair_m.p, npb, cudaMemcpyDeviceToDevice, m->stream));
      const int keep = m->ray_variant;
      Profiler off{m, false};
      int64_t launches = 0;
      if (quiet) quiet_prefix_all(m, a);
      for (int k = 0; k < NV; ++k) {
        m->ray_variant = k;
        for (int r = 0; r <= reps; ++r) {
          if (r == 1) CK(cudaEventRecord(m->ev0, m->stream));
          enqueue_iteration(m, a, jacobi, 0, 2, quiet, off, launches);
        }
        CK(cudaEventRecord(m->ev1, m->stream));
        sync(m);
        float t = 0.0f;
        CK(cudaEventElapsedTime(&t, m->ev0, m->ev1));
        ms[k] = t / reps;
        CK(cudaMemcpyAsync(m->d_L.p, snap, nv, cudaMemcpyDeviceToDevice, m->stream));
        CK(cudaMemcpyAsync(m->d_belief.p, snap + nv, nv, cudaMemcpyDeviceToDevice, m->stream));
        CK(cudaMemcpyAsync(m->pair_m.p, snap + 2 * nv, npb, cudaMemcpyDeviceToDevice, m->stream));
      }
      m->ray_variant = keep;
      sync(m);
    }
    int best = 0;
    for (int k = 1; k < NV; ++k)
      if (ms[k] < ms[best]) best = k;
    for (int k = 0; k < NV && k < cap; ++k) ms_out[k] = ms[k];
    m->ray_variant = best;
    drop_graphs(m);
    // then the pair reduction's variant with that ray kernel
    if (m->n_inc > 0) {
      double pms[2];
      for (int k = 0; k < 2; ++k) {
        m->pair_variant = k;
        drop_graphs(m);
        pms[k] = time_schedule(m, jacobi, reps);
      }
      m->pair_variant = pms[1] < pms[0] ? 1 : 0;
      drop_graphs(m);
    }
    if (chosen) *chosen = best;
  });
}

mrf_status mrf_reset_state(mrf_map* m) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  return wrap([&] {
    float lp = logf(m->prm.prior) - logf(1.0f - m->prm.prior);
    CK(launch_fill_new_voxels(m->d_L.as<float>(), m->d_belief.as<float>(), 0,
                              m->n_bricks * kBrickVox, lp, m->stream));
    if (m->has_base) CK(launch_fill_f32(m->d_Lbase.as<float>(), m->n_bricks * kBrickVox, lp, m->stream));
    if (m->n_pairs) CK(launch_fill_f32(m->pair_m.as<float>(), m->n_pairs, 0.0f, m->stream));
  });
}

mrf_status mrf_likelihood_device(mrf_map* m, const float* pose, const float* depth_dev,
                                 float* out_img_dev, float* out_sum_dev) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (!pose || !depth_dev || !out_sum_dev) {
    set_err("null argument");
    return MRF_ERR_INVALID;
  }
  return wrap([&] {
    Pose P;
    set_pose(P, pose);
    const int64_t HW = m->hw();
    m->s_depth.reserve((size_t)HW * 4, false, m->stream);
    CK(launch_clean_depth(depth_dev, m->s_depth.as<float>(), m->prm.rows, m->prm.cols, m->stream));
    likelihood_dev(m, P, m->s_depth.as<float>(), out_img_dev, out_sum_dev);
  });
}

static mrf_status likelihood_host(mrf_map* m, const Pose& P, const float* depth_clean_dev,
                                  float* out_img, float* out_sum, const Geom* cam = nullptr) {
  return wrap([&] {
    const int64_t HW = cam ? (int64_t)cam->rows * cam->cols : m->hw();
    float* img = nullptr;
    if (out_img) {
      m->s_img.reserve((size_t)HW * 4, false, m->stream);
      img = m->s_img.as<float>();
    }
    likelihood_dev(m, P, depth_clean_dev, img, m->s_sum.as<float>(), cam);
    float sum = 0.0f;
    CK(cudaMemcpyAsync(&sum, m->s_sum.p, 4, cudaMemcpyDeviceToHost, m->stream));
    if (out_img) CK(cudaMemcpyAsync(out_img, img, (size_t)HW * 4, cudaMemcpyDeviceToHost, m->stream));
    sync(m);
    if (out_sum) *out_sum = sum;
  });
}

mrf_status mrf_likelihood(mrf_map* m, const float* pose, const float* depth_host, float* out_img,
                          float* out_sum) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (!pose || !depth_host) {
    set_err("null argument");
    return MRF_ERR_INVALID;
  }
  mrf_status st = wrap([&] {
    const int64_t HW = m->hw();
    m->s_depth_in.reserve((size_t)HW * 4, false, m->stream);
    m->s_depth.reserve((size_t)HW * 4, false, m->stream);
    CK(cudaMemcpyAsync(m->s_depth_in.p, depth_host, (size_t)HW * 4, cudaMemcpyHostToDevice, m->stream));
    CK(launch_clean_depth(m->s_depth_in.as<float>(), m->s_depth.as<float>(), m->prm.rows,
                          m->prm.cols, m->stream));
  });
  if (st != MRF_OK) return st;
  Pose P;
  set_pose(P, pose);
  return likelihood_host(m, P, m->s_depth.as<float>(), out_img, out_sum);
}

mrf_status mrf_likelihood_view(mrf_map* m, int view_id, float* out_img, float* out_sum) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (view_id < 0 || view_id >= (int)m->views.size()) {
    set_err("invalid view id");
    return MRF_ERR_INVALID;
  }
  if (m->views[view_id].retired) {
    set_err("view retired (mrf_retire_view)");
    return MRF_ERR_STATE;
  }
  const View& v = m->views[view_id];
  return likelihood_host(m, v.pose, v.depth.as<float>(), out_img, out_sum, &v.cam);
}

static mrf_status render_impl(mrf_map* m, int mode, const Pose& P, const float* depth_clean_dev,
                              float threshold, float* out_img, float* out_score, int64_t* counts,
                              const Geom* cam = nullptr) {
  if (mode < 0 || mode > 3) {
    set_err("invalid render mode");
    return MRF_ERR_INVALID;
  }
  return wrap([&] {
    Geom g = cam ? *cam : m->g;
    const int64_t HW = (int64_t)g.rows * g.cols;
    if (threshold < 0.0f)
      threshold = mode == MRF_RENDER_SIMPLE_ACCURACY ? m->prm.acc_thresh : m->prm.occ_thresh;
    m->s_img.reserve((size_t)HW * 4, false, m->stream);
    m->s_part.reserve(64, false, m->stream);
    CK(cudaMemsetAsync(m->s_part.p, 0, 32, m->stream));
    g.brick_slot = m->d_slot.as<int>();
    const float* bel = m->d_belief.as<float>();
    if (m->n_bricks == 0) {
      m->s_dense.reserve(4, false, m->stream);
      bel = m->s_dense.as<float>();
    }
    CK(launch_render(mode, g, P, depth_clean_dev, bel, threshold, m->s_img.as<float>(),
                     reinterpret_cast<unsigned long long*>(m->s_part.p), m->stream));
    unsigned long long h[4] = {0, 0, 0, 0};
    CK(cudaMemcpyAsync(h, m->s_part.p, 32, cudaMemcpyDeviceToHost, m->stream));
    if (out_img)
      CK(cudaMemcpyAsync(out_img, m->s_img.p, (size_t)HW * 4, cudaMemcpyDeviceToHost, m->stream));
    sync(m);
    if (counts)
      for (int k = 0; k < 4; ++k) counts[k] = (int64_t)h[k];
    if (out_score) {
      double n = (double)HW;
      // src/cuda/gvdbhelper.cu:16-62: accuracy = #1 / (pixels - #(-1));
      // simple accuracy = (TP + TN) / pixels with TP = #1, TN = #(-1)
      if (mode == MRF_RENDER_ACCURACY)
        *out_score = (n - h[0]) > 0 ? (float)(h[2] / (n - (double)h[0])) : 0.0f;
      else if (mode == MRF_RENDER_SIMPLE_ACCURACY)
        *out_score = (float)(((double)h[2] + (double)h[0]) / n);
      else
        *out_score = 0.0f;
    }
  });
}

mrf_status mrf_render(mrf_map* m, int mode, const float* pose, const float* depth_host,
                      float threshold, float* out_img, float* out_score, int64_t* counts) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (!pose || !depth_host) {
    set_err("null argument");
    return MRF_ERR_INVALID;
  }
  mrf_status st = wrap([&] {
    const int64_t HW = m->hw();
    m->s_depth_in.reserve((size_t)HW * 4, false, m->stream);
    m->s_depth.reserve((size_t)HW * 4, false, m->stream);
    CK(cudaMemcpyAsync(m->s_depth_in.p, depth_host, (size_t)HW * 4, cudaMemcpyHostToDevice, m->stream));
    CK(launch_clean_depth(m->s_depth_in.as<float>(), m->s_depth.as<float>(), m->prm.rows,
                          m->prm.cols, m->stream));
  });
  if (st != MRF_OK) return st;
  Pose P;
  set_pose(P, pose);
  return render_impl(m, mode, P, m->s_depth.as<float>(), threshold, out_img, out_score, counts);
}

mrf_status mrf_render_view(mrf_map* m, int mode, int view_id, float threshold, float* out_img,
                           float* out_score, int64_t* counts) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (view_id < 0 || view_id >= (int)m->views.size()) {
    set_err("invalid view id");
    return MRF_ERR_INVALID;
  }
  if (m->views[view_id].retired) {
    set_err("view retired (mrf_retire_view)");
    return MRF_ERR_STATE;
  }
  const View& v = m->views[view_id];
  return render_impl(m, mode, v.pose, v.depth.as<float>(), threshold, out_img, out_score, counts, &v.cam);
}

mrf_status mrf_pixel_diagnostics(mrf_map* m, const float* pose, int x, int y, float* out, int64_t n_floats) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (!pose || !out || n_floats < 11 || x < 0 || y < 0 || x >= m->prm.cols || y >= m->prm.rows) {
    set_err("invalid pixel diagnostics arguments");
    return MRF_ERR_INVALID;
  }
  return wrap([&] {
    Pose P;
    set_pose(P, pose);
    m->s_img.reserve((size_t)n_floats * 4, false, m->stream);
    CK(cudaMemsetAsync(m->s_img.p, 0, (size_t)n_floats * 4, m->stream));
    m->g.brick_slot = m->d_slot.as<int>();
    const float* bel = m->d_belief.as<float>();
    if (m->n_bricks == 0) {
      m->s_dense.reserve(4, false, m->stream);
      bel = m->s_dense.as<float>();
    }
    CK(launch_pixel_diag(m->g, P, bel, x, y, m->s_img.as<float>(), n_floats, m->stream));
    CK(cudaMemcpyAsync(out, m->s_img.p, (size_t)n_floats * 4, cudaMemcpyDeviceToHost, m->stream));
    sync(m);
  });
}

mrf_status mrf_num_bricks(mrf_map* m, int64_t* n) {
  if (guard(m) != MRF_OK || !n) return MRF_ERR_INVALID;
  *n = m->n_bricks;
  return MRF_OK;
}

mrf_status mrf_read_bricks(mrf_map* m, float* centres, float* beliefs, int64_t n) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (n != m->n_bricks) {
    set_err("Dimensions for the alphas array are incorrect!");
    return MRF_ERR_INVALID;
  }
  return wrap([&] {
    if (centres)
      for (int64_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) centres[i * 3 + a] = (float)(m->h_coord[i * 3 + a] * kBrick + kBrick / 2);
    if (beliefs && n) {
      CK(cudaMemcpyAsync(beliefs, m->d_belief.p, (size_t)n * kBrickVox * 4, cudaMemcpyDeviceToHost,
                         m->stream));
      sync(m);
    }
  });
}

mrf_status mrf_read_logodds(mrf_map* m, float* logodds, int64_t n) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (n != m->n_bricks || !logodds) {
    set_err("invalid size");
    return MRF_ERR_INVALID;
  }
  return wrap([&] {
    if (n) {
      CK(cudaMemcpyAsync(logodds, m->d_L.p, (size_t)n * kBrickVox * 4, cudaMemcpyDeviceToHost,
                         m->stream));
      sync(m);
    }
  });
}

static void node_list(mrf_map* m, int level, std::vector<int>& out) {
  // level-l nodes span 8^(l+1) voxels per axis (gvdb_map_config 3,3,3,3,3)
  int64_t span = 1;
  for (int l = 0; l < level; ++l) span *= 8;
  std::vector<int64_t> keys;
  keys.reserve((size_t)m->n_bricks);
  for (int64_t i = 0; i < m->n_bricks; ++i) {
    int64_t c[3];
    for (int a = 0; a < 3; ++a) c[a] = m->h_coord[i * 3 + a] / span;
    keys.push_back((c[0] << 40) | (c[1] << 20) | c[2]);
  }
  std::vector<int64_t> seen;
  for (int64_t k : keys)
    if (std::find(seen.begin(), seen.end(), k) == seen.end()) seen.push_back(k);
  out.clear();
  for (int64_t k : seen) {
    out.push_back((int)(k >> 40));
    out.push_back((int)((k >> 20) & 0xFFFFF));
    out.push_back((int)(k & 0xFFFFF));
  }
}

mrf_status mrf_num_nodes(mrf_map* m, int level, int64_t* n) {
  if (guard(m) != MRF_OK || !n || level < 0 || level > 4) return MRF_ERR_INVALID;
  if (level == 0) {
    *n = m->n_bricks;
    return MRF_OK;
  }
  std::vector<int> nodes;
  node_list(m, level, nodes);
  *n = (int64_t)nodes.size() / 3;
  return MRF_OK;
}

mrf_status mrf_read_nodes(mrf_map* m, int level, float* centres, int64_t n) {
  if (guard(m) != MRF_OK || !centres || level < 0 || level > 4) return MRF_ERR_INVALID;
  if (level == 0) return mrf_read_bricks(m, centres, nullptr, n);
  std::vector<int> nodes;
  node_list(m, level, nodes);
  if ((int64_t)nodes.size() / 3 != n) {
    set_err("invalid size");
    return MRF_ERR_INVALID;
  }
  int64_t span = kBrick;
  for (int l = 0; l < level; ++l) span *= 8;
  for (int64_t i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) centres[i * 3 + a] = (float)(nodes[i * 3 + a] * span + span / 2);
  return MRF_OK;
}

mrf_status mrf_load_map(mrf_map* m, const float* points, const float* occ, int64_t n) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (n < 0 || (n > 0 && (!points || !occ))) {
    set_err("invalid points");
    return MRF_ERR_INVALID;
  }
  DBuf pts, oc;  // released on every exit, failures included
  mrf_status st = wrap([&] {
    if (n == 0) return;
    pts.reserve((size_t)n * 12, false, m->stream);
    oc.reserve((size_t)n * 4, false, m->stream);
    CK(cudaMemcpyAsync(pts.p, points, (size_t)n * 12, cudaMemcpyHostToDevice, m->stream));
    CK(cudaMemcpyAsync(oc.p, occ, (size_t)n * 4, cudaMemcpyHostToDevice, m->stream));
    CK(cudaMemsetAsync(m->s_flags.p, 0, (size_t)m->nb_grid, m->stream));
    m->g.brick_slot = m->d_slot.as<int>();
    CK(launch_activate_points(m->g, pts.as<float>(), n, m->s_flags.as<uint8_t>(), m->stream));
    commit_new_bricks(m);
    m->needs_full = true;
    m->g.brick_slot = m->d_slot.as<int>();
    CK(launch_set_points(m->g, pts.as<float>(), oc.as<float>(), n, m->d_belief.as<float>(), m->stream));
    sync(m);
    m->stats.n_bricks = m->n_bricks;
  });
  pts.release();
  oc.release();
  return st;
}

mrf_status mrf_view_incidences(mrf_map* m, int view_id, int* meta, uint32_t* vox, float* len,
                               float* mu, int64_t cap, int64_t* n_inc) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  if (view_id < 0 || view_id >= (int)m->views.size() || cap < 0) {
    set_err("invalid view id");
    return MRF_ERR_INVALID;
  }
  if (m->views[view_id].retired) {
    set_err("view retired (mrf_retire_view)");
    return MRF_ERR_STATE;
  }
  return wrap([&] {
    ensure_built(m);
    const View& v = m->views[view_id];
    const int64_t HW = (int64_t)v.cam.rows * v.cam.cols;
    std::vector<RayMeta> hm((size_t)HW);
    CK(cudaMemcpyAsync(hm.data(), m->meta.as<RayMeta>() + v.pix_base, (size_t)HW * sizeof(RayMeta),
                       cudaMemcpyDeviceToHost, m->stream));
    sync(m);
    int64_t total = 0;
    for (int64_t i = 0; i < HW; ++i) {
      total += hm[i].n_pre;
      if (meta) {
        meta[i * 5 + 0] = hm[i].n_pre;
        meta[i * 5 + 1] = hm[i].n_post;
        meta[i * 5 + 2] = hm[i].r0;
        meta[i * 5 + 3] = hm[i].rinf;
        meta[i * 5 + 4] = (int)(hm[i].flags & 1u);
      }
    }
    if (n_inc) *n_inc = total;
    if (cap <= 0 || v.n_inc == 0 || (!len && !mu && !vox)) return;
    // device lists are padded per ray: copy the view's range, then compact
    std::vector<float> hl(v.n_inc), hmu(v.n_inc);
    std::vector<uint32_t> ip(v.n_inc), pv(v.n_pairs);
    CK(cudaMemcpyAsync(hl.data(), m->inc_len.as<float>() + v.inc_base, (size_t)v.n_inc * 4,
                       cudaMemcpyDeviceToHost, m->stream));
    CK(cudaMemcpyAsync(hmu.data(), m->inc_mu.as<float>() + v.inc_base, (size_t)v.n_inc * 4,
                       cudaMemcpyDeviceToHost, m->stream));
    CK(cudaMemcpyAsync(ip.data(), m->inc_pair.as<uint32_t>() + v.inc_base, (size_t)v.n_inc * 4,
                       cudaMemcpyDeviceToHost, m->stream));
    if (v.n_pairs)
      CK(cudaMemcpyAsync(pv.data(), m->pair_vox.as<uint32_t>() + v.pair_base, (size_t)v.n_pairs * 4,
                         cudaMemcpyDeviceToHost, m->stream));
    sync(m);
    int64_t k = 0;
    for (int64_t i = 0; i < HW && k < cap; ++i) {
      int64_t o = (int64_t)hm[i].off - v.inc_base;
      for (int j = 0; j < hm[i].n_pre && k < cap; ++j, ++k) {
        if (len) len[k] = hl[o + j];
        if (mu) mu[k] = hmu[o + j];
        if (vox) vox[k] = pv[ip[o + j] - v.pair_base];
      }
    }
  });
}

mrf_status mrf_device_beliefs(mrf_map* m, const float** beliefs, int64_t* n_voxels) {
  if (guard(m) != MRF_OK || !beliefs || !n_voxels) return MRF_ERR_INVALID;
  *beliefs = m->d_belief.as<float>();
  *n_voxels = m->n_bricks * kBrickVox;
  return MRF_OK;
}

mrf_status mrf_stats_get(mrf_map* m, mrf_stats* out) {
  if (guard(m) != MRF_OK || !out) return MRF_ERR_INVALID;
  mrf_status st = wrap([&] {
    ensure_built(m);
    // pairs past the length gate and the distinct voxels they reach
    const int64_t nvox = m->n_bricks * kBrickVox;
    m->s_loud.reserve((size_t)std::max<int64_t>(nvox, 1), false, m->stream);
    m->s_delta.reserve(64, false, m->stream);
    CK(launch_touch_counts(m->pair_vox.as<uint32_t>(), m->pair_cum.as<float>(), (uint32_t)m->n_pairs,
                           m->s_loud.as<uint8_t>(), nvox, m->s_delta.as<unsigned long long>(), m->stream));
    unsigned long long cnt[2] = {0, 0};
    CK(cudaMemcpyAsync(cnt, m->s_delta.p, 16, cudaMemcpyDeviceToHost, m->stream));
    sync(m);
    m->stats.n_pairs_active = (int64_t)cnt[0];
    m->stats.n_vox_touched = (int64_t)cnt[1];
    m->stats.n_views = (int64_t)m->views.size();
    m->stats.n_bricks = m->n_bricks;
  });
  *out = m->stats;
  return st;
}

mrf_status mrf_get_stream(mrf_map* m, void** stream) {
  if (guard(m) != MRF_OK || !stream) return MRF_ERR_INVALID;
  *stream = (void*)m->stream;
  return MRF_OK;
}

mrf_status mrf_synchronize(mrf_map* m) {
  if (guard(m) != MRF_OK) return MRF_ERR_INVALID;
  return wrap([&] { sync(m); });
}

}  // extern "C"
