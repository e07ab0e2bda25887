// mrf_bp.cu -- the BP hot loop over the incidence lists.
//
//   k_pair_prepare : per (camera, voxel) pair, the cavity probability
//                    q = P(empty) excluding the camera's own message
//                    (src/cuda/gvdbkernels.cu:764-773)
//   k_ray_bp       : per ray, Pre pass (tau accumulation with the reference's
//                    per-brick visibility reset, gvdbkernels.cu:689-819), the
//                    infinity term (gvdbkernels.cu:1196-1208) and the Post pass
//                    (ray->voxel messages, gvdbkernels.cu:824-1038), all as
//                    warp-wide log-domain prefix scans
//   k_pair_update  : per pair, the length-weighted message average, new
//                    log-odds message, total log-odds and belief
//                    (gvdbkernels.cu:457-479); a segmented sum over the
//                    pair-grouped permutation of the dynamic incidences --
//                    no atomics, fixed summation order
#include <cuda_fp16.h>

#include <algorithm>

#include "mrf_internal.h"

namespace mrf {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T u = __shfl_up_sync(kFull, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// kPrepPer pairs per thread, strided by the block so that every load stays
// coalesced and a thread keeps kPrepPer independent L gathers in flight
constexpr int kPrepThreads = 256;
constexpr int kPrepPer = 4;

__global__ void __launch_bounds__(kPrepThreads)
    k_pair_prepare(const uint32_t* __restrict__ pair_vox, const float* __restrict__ m,
                   const float* __restrict__ L, float* __restrict__ lnq, __half* __restrict__ lnq16,
                   float* __restrict__ dm, uint32_t p0, uint32_t p1) {
  const uint32_t base = p0 + blockIdx.x * (kPrepThreads * kPrepPer) + threadIdx.x;
  float eta[kPrepPer];
#pragma unroll
  for (int k = 0; k < kPrepPer; ++k) {
    const uint32_t p = base + k * kPrepThreads;
    eta[k] = p < p1 ? L[pair_vox[p]] - m[p] : 0.0f;
  }
#pragma unroll
  for (int k = 0; k < kPrepPer; ++k) {
    const uint32_t p = base + k * kPrepThreads;
    if (p >= p1) break;
    float qq = clampf(1.0f / (1.0f + expf(eta[k])), kFEps, 1.0f - kFEps);
    if (lnq16)
      lnq16[p] = __float2half_rn(logf(qq));  // 16-bit streams: the ray kernel gathers halves
    else
      lnq[p] = logf(qq);
    if (dm) dm[p] = __int_as_float(0x7fc00000);  // Jacobi: NaN until the pair updates
  }
}

// ---- ray messages ----------------------------------------------------------
// One warp per ray.  Each lane owns kE = 4 consecutive incidences of a
// chunk of 128 (ray offsets are padded to multiples of 4, so the streams load
// as 16-byte vectors): the prefix over the ray is a serial sum inside the
// lane plus one warp scan per chunk, and a lane keeps 4 gathers in flight.
//
// Pass 1 forms the visibility exponent A_i = sum_{j<=i} l_j ln q_j,
// V_i = exp(A_i), q_i and the Pre total T over the whole ray.  Pass 2 turns
// (V_i mu_i, q_i, l_i) and T into the messages p_i * l_i of the dynamic
// range [k_dyn, n_post) only: before k_dyn every potential is zero, so
// tau_i = 0, F_i = 0, mu1_i = 0 and p_i is exactly the clamp floor F_EPS
// (static messages, summed once per build into the pairs).  Potentials are
// loaded from k_dyn (rounded down to a vector) on.  Pass 2 re-reads the
// dynamic range (a sixth of the incidences, mostly still in L1/L2) from
// A_{k_dyn - 1} instead of keeping pass 1's slice in registers: the kernel
// then fits 40 registers, twelve resident blocks per SM.  On rays longer
// than kLongRay the Pre total T is summed across lanes in FP64 and the
// running difference T - F of pass 2 is carried in FP64; each lane's share
// of T is a compensated FP32 sum.  (GB300 issues FP64 at 1/64 of the FP32
// rate, so FP64 stays out of the per-incidence arithmetic.)
//
// The ln q gathers are the kernel's cost.  Pairs are numbered brick-major
// by first visit (mrf_build.cu), so consecutive incidences of a ray gather
// from nearby addresses and neighbouring rays from the same ones.
//
// Pre visibility restarts at r0 (the reference restores its carried state
// only once the accumulated tau is non-zero, gvdbkernels.cu:708-715):
// V^pre_i = exp(A_i - A_{r0-1}) = V_i * exp(-A_{r0-1}); Post uses V_i.
constexpr int kRayWarps = 4;
constexpr int kE = 4;                    // incidences per lane of a chunk
constexpr int kChunk = 32 * kE;          // 128
constexpr float kUnderflowGuard = -60.0f;

template <typename T>
__device__ __forceinline__ T warp_excl_scan(T v, int lane) {
  T incl = warp_incl_scan(v, lane);
  return incl - v;
}

// one lane's slice of a chunk (KE incidences).  ln q is kept; q itself is
// formed only where a potential is non-zero or a message is computed.
template <int KE>
struct Slice {
  float A[KE], lq[KE], mu[KE], len[KE];
};

// streamed incidence arrays: read-only path (kPol 0) or evict-first
// streaming loads (kPol 1) that leave L2 to the ln q gathers
template <int kPol, typename T>
__device__ __forceinline__ T ld_stream(const T* p) {
  if (kPol) return __ldcs(p);
  return __ldg(p);
}

template <typename T>
__device__ __forceinline__ T from_bits(uint32_t u);
template <>
__device__ __forceinline__ uint32_t from_bits<uint32_t>(uint32_t u) { return u; }
template <>
__device__ __forceinline__ float from_bits<float>(uint32_t u) { return __uint_as_float(u); }

// KE consecutive values at element i (i a multiple of KE; KE = 2 or a
// multiple of 4): 8-byte or 16-byte vector loads, zeros when !ok
template <int KE, int kPol, typename T>
__device__ __forceinline__ void ld_vec(T (&out)[KE], const T* __restrict__ base, int i, bool ok) {
  static_assert(sizeof(T) == 4, "4-byte elements");
  if constexpr (KE % 4 == 0) {
#pragma unroll
    for (int v = 0; v < KE / 4; ++v) {
      uint4 u = make_uint4(0u, 0u, 0u, 0u);
      if (ok) u = ld_stream<kPol>(reinterpret_cast<const uint4*>(base + i + 4 * v));
      out[4 * v + 0] = from_bits<T>(u.x);
      out[4 * v + 1] = from_bits<T>(u.y);
      out[4 * v + 2] = from_bits<T>(u.z);
      out[4 * v + 3] = from_bits<T>(u.w);
    }
  } else {
    static_assert(KE == 2, "short chunks hold two incidences per lane");
    uint2 u = make_uint2(0u, 0u);
    if (ok) u = ld_stream<kPol>(reinterpret_cast<const uint2*>(base + i));
    out[0] = from_bits<T>(u.x);
    out[1] = from_bits<T>(u.y);
  }
}

// a lane's KE pair ids at i0 (those >= n read as zero)
template <int KE, int kPol>
__device__ __forceinline__ void load_pids(uint32_t (&pid)[KE], uint32_t off, int i0, int n,
                                          const uint32_t* __restrict__ inc_pair) {
  if constexpr (KE % 4 == 0) {
#pragma unroll
    for (int v = 0; v < KE / 4; ++v) {
      uint32_t t[4];
      ld_vec<4, kPol>(t, inc_pair + off, i0 + 4 * v, i0 + 4 * v < n);
#pragma unroll
      for (int j = 0; j < 4; ++j) pid[4 * v + j] = t[j];
    }
  } else {
    ld_vec<KE, kPol>(pid, inc_pair + off, i0, i0 < n);
  }
}

// ln q of a lane's KE incidences (those >= n read as zero; kWhole: the
// whole chunk lies inside the ray and nothing is checked)
__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__half v) { return __half2float(v); }

template <int KE, bool kWhole, typename TQ>
__device__ __forceinline__ void gather_lq(float (&lq)[KE], const uint32_t (&pid)[KE], int i0, int n,
                                          const TQ* __restrict__ lnq) {
#pragma unroll
  for (int j = 0; j < KE; ++j) lq[j] = (kWhole || i0 + j < n) ? to_f(__ldg(lnq + pid[j])) : 0.0f;
}

// VW lengths at element i of base (fp32: one 16-byte vector; fp16: one
// 8-byte vector of four halves), zeros when !ok
template <int VW, int kPol>
__device__ __forceinline__ void ld_len(float (&out)[VW], const float* __restrict__ base, int i, bool ok) {
  ld_vec<VW, kPol>(out, base, i, ok);
}
template <int VW, int kPol>
__device__ __forceinline__ void ld_len(float (&out)[VW], const __half* __restrict__ base, int i, bool ok) {
  static_assert(VW == 4, "fp16 lengths load four at a time");
  uint2 u = make_uint2(0u, 0u);
  if (ok) u = ld_stream<kPol>(reinterpret_cast<const uint2*>(base + i));
  const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
  const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
  out[0] = a.x;
  out[1] = a.y;
  out[2] = b.x;
  out[3] = b.y;
}

// with the lane's ln q gathered: loads lengths (and potentials at and after
// kmu, a multiple of 4; below it they are known zeros), forms prefix
// exponents from carryA; returns the chunk total of l ln q
// (kLenIn: the lengths were loaded ahead into len_in)
template <int KE, int kPol, bool kWhole, bool kLenIn = false, typename TL = float>
__device__ __forceinline__ float slice_from_lq(Slice<KE>& s, const float (&lq)[KE], uint32_t off, int i0,
                                               int n, int kmu, float carryA, int lane,
                                               const TL* __restrict__ inc_len,
                                               const float* __restrict__ inc_mu,
                                               const float* len_in = nullptr) {
  constexpr int VW = KE % 4 == 0 ? 4 : KE;  // vector width
#pragma unroll
  for (int v = 0; v < KE / VW; ++v) {
    const int i = i0 + VW * v;
    float l[VW], m[VW];
    if constexpr (kLenIn) {
#pragma unroll
      for (int j = 0; j < VW; ++j) l[j] = len_in[VW * v + j];
    } else {
      ld_len<VW, kPol>(l, inc_len + off, i, kWhole || i < n);
    }
    ld_vec<VW, kPol>(m, inc_mu + off, i, (kWhole || i < n) && i >= kmu);
#pragma unroll
    for (int j = 0; j < VW; ++j) {
      s.len[VW * v + j] = l[j];
      s.mu[VW * v + j] = m[j];
    }
  }
  float run = 0.0f;
#pragma unroll
  for (int j = 0; j < KE; ++j) {
    const bool ok = kWhole || i0 + j < n;
    s.lq[j] = ok ? lq[j] : 0.0f;
    if (!ok) {
      s.len[j] = 0.0f;
      s.mu[j] = 0.0f;
    }
    run += s.len[j] * lq[j];
    s.A[j] = run;  // lane-local inclusive prefix, rebased below
  }
  float ex = warp_excl_scan(run, lane);
  float b = carryA + ex;
#pragma unroll
  for (int j = 0; j < KE; ++j) s.A[j] += b;
  return __shfl_sync(kFull, ex + run, 31);
}

template <int KE, int kPol, bool kWhole, bool kLenIn = false, typename TL = float, typename TQ = float>
__device__ __forceinline__ float slice_from_pids(Slice<KE>& s, const uint32_t (&pid)[KE], uint32_t off,
                                                 int i0, int n, int kmu, float carryA, int lane,
                                                 const TL* __restrict__ inc_len,
                                                 const float* __restrict__ inc_mu,
                                                 const TQ* __restrict__ lnq,
                                                 const float* len_in = nullptr) {
  float lq[KE];
  gather_lq<KE, kWhole>(lq, pid, i0, n, lnq);
  return slice_from_lq<KE, kPol, kWhole, kLenIn, TL>(s, lq, off, i0, n, kmu, carryA, lane, inc_len, inc_mu,
                                                    len_in);
}

template <int KE, int kPol, bool kWhole, typename TL, typename TQ>
__device__ __forceinline__ float load_slice(Slice<KE>& s, uint32_t off, int i0, int n, int kmu,
                                            float carryA, int lane,
                                            const uint32_t* __restrict__ inc_pair,
                                            const TL* __restrict__ inc_len,
                                            const float* __restrict__ inc_mu,
                                            const TQ* __restrict__ lnq) {
  uint32_t pid[KE];
  load_pids<KE, kPol>(pid, off, i0, kWhole ? i0 + KE : n, inc_pair);
  return slice_from_pids<KE, kPol, kWhole, false, TL, TQ>(s, pid, off, i0, n, kmu, carryA, lane, inc_len,
                                                          inc_mu, lnq);
}

// A at chunk-relative index idx (0 <= idx < 32 * KE), broadcast to the warp
template <int KE>
__device__ __forceinline__ float slice_value(const Slice<KE>& s, int idx) {
  const int jj = idx % KE;
  float mine = 0.0f;
#pragma unroll
  for (int j = 0; j < KE; ++j)
    if (j == jj) mine = s.A[j];
  return __shfl_sync(kFull, mine, idx / KE);
}

// pass 2 on one lane's slice: messages p*l for positions i0..i0+KE-1; the
// vectors starting inside [k4, n_post) are written (k4 a multiple of 4).
// cF is F at the chunk start and D = T - cF, formed in the ray's
// accumulation type by the caller; returns the chunk's total of tau.
template <int KE, bool kWhole>
__device__ __forceinline__ float emit_slice(const float (&vmu)[KE], const float (&q)[KE],
                                            const float (&len)[KE], int i0, int k4, int n_post,
                                            float cF, float D, int lane, uint32_t off,
                                            float* __restrict__ inc_pl) {
  float tau[KE], eloc[KE];
  float run = 0.0f;
#pragma unroll
  for (int j = 0; j < KE; ++j) {
    tau[j] = (kWhole || i0 + j < n_post) ? vmu[j] * (1.0f - q[j]) : 0.0f;
    eloc[j] = run;
    run += tau[j];
  }
  float ex = warp_excl_scan(run, lane);
  float out[KE];
#pragma unroll
  for (int j = 0; j < KE; ++j) {
    float fin = ex + eloc[j];
    float F = cF + fin;
    float R = (D - fin) - tau[j];
    float mu1 = F + vmu[j];
    float mu0 = F + __fdividef(R, q[j]);
    float p = clampf(__fdividef(mu1, mu1 + mu0 + 1e-7f), kFEps, 1.0f - kFEps);
    out[j] = (kWhole || i0 + j < n_post) ? p * len[j] : 0.0f;
  }
  constexpr int VW = KE % 4 == 0 ? 4 : KE;
#pragma unroll
  for (int v = 0; v < KE / VW; ++v) {
    const int i = i0 + VW * v;
    if (i >= k4 && (kWhole || i < n_post)) {
      if constexpr (VW == 4)
        *reinterpret_cast<float4*>(inc_pl + off + i) =
            make_float4(out[4 * v], out[4 * v + 1], out[4 * v + 2], out[4 * v + 3]);
      else
        *reinterpret_cast<float2*>(inc_pl + off + i) = make_float2(out[2 * v], out[2 * v + 1]);
    }
  }
  return __shfl_sync(kFull, ex + run, 31);
}

// Pass-1 bookkeeping of one slice: A_{r0-1}, A_{rinf-1} and A_{k4-1} where
// those positions fall inside it
template <int KE>
__device__ __forceinline__ void pre_marks(const Slice<KE>& s, int base, int r0, int rinf, int k4,
                                          float& Ar0, float& Arinf, float& Ak) {
  constexpr int CH = 32 * KE;
  if (r0 - 1 >= base && r0 - 1 < base + CH) Ar0 = slice_value<KE>(s, r0 - 1 - base);
  if (rinf - 1 >= base && rinf - 1 < base + CH) Arinf = slice_value<KE>(s, rinf - 1 - base);
  if (k4 - 1 >= base && k4 - 1 < base + CH) Ak = slice_value<KE>(s, k4 - 1 - base);
}

// the lane's share of the Pre total from one slice that may hold non-zero
// potentials, added to a compensated FP32 sum (ts, tc): the error of the
// lane's sum stays at a few ulps however long the ray is
template <int KE>
__device__ __forceinline__ void pre_total(const Slice<KE>& s, int i0, int r0, float Ar0, float& ts,
                                          float& tc) {
  // exp(-A_{r0-1}) rescales Post visibility to Pre visibility unless the
  // Post visibility may have underflowed (then exponentiate the difference)
  const bool direct = Ar0 < kUnderflowGuard;
  const float scale = direct ? 0.0f : __expf(-Ar0);
  float w = 0.0f;
#pragma unroll
  for (int j = 0; j < KE; ++j) {
    if (i0 + j >= r0 && s.mu[j] != 0.0f) {
      float vp = direct ? __expf(s.A[j] - Ar0) : __expf(s.A[j]) * scale;
      w += vp * (1.0f - __expf(s.lq[j])) * s.mu[j];
    }
  }
  const float y = w - tc;
  const float t = ts + y;
  tc = (t - ts) - y;
  ts = t;
}

template <typename Acc, int kPol, int kPf, typename TL, typename TQ>
__device__ __forceinline__ void ray_bp_warp(const RayMeta& me, uint32_t rid, const QuietPrefix& qp,
                                            const uint32_t* __restrict__ inc_pair,
                                            const TL* __restrict__ inc_len,
                                            const float* __restrict__ inc_mu,
                                            const TQ* __restrict__ lnq, float* __restrict__ inc_pl,
                                            int fix_reset, int lane) {
  const int n_pre = me.n_pre, n_post = me.n_post;
  const int r0 = fix_reset ? 0 : me.r0;
  const int rinf = fix_reset ? 0 : me.rinf;
  const int kdyn = ray_kdyn(me);
  const int k4 = kdyn & ~3;
  const uint32_t off = me.off;
  float carryA = 0.0f, Ar0 = 0.0f, Arinf = 0.0f, Ak = 0.0f;
  // ---- the static prefix [0, k4) from its quiet sums --------------------
  // Its quiet incidences (pairs on voxels without a dynamic incidence in
  // any view) keep their ln q from the third iteration of a call on, so
  // their sums up to r0 and up to k4 were formed once (k_quiet_prefix);
  // only the prefix's loud incidences are gathered here.  A ray in the
  // queues has a non-zero potential, so its rinf equals r0.
  const int start = qp.q ? k4 : 0;
  // kPf >= 1: the first chunk's pair ids are requested before the static
  // prefix's loads, so the two chains of dependent loads overlap
  uint32_t pid_next[kE];
  float len_next[kE];
  if (kPf) load_pids<kE, kPol>(pid_next, off, start + kE * lane, n_pre, inc_pair);
  if (kPf == 2) ld_len<kE, kPol>(len_next, inc_len + off, start + kE * lane, start + kE * lane < n_pre);
  if (qp.q) {
    const float2 qv = qp.q[rid];
    const uint32_t e0 = qp.loff[rid], e1 = qp.loff[rid + 1];
    float la = 0.0f, lk = 0.0f;
    for (uint32_t e = e0 + lane; e < e1; e += 32) {
      const float c = qp.llen[e] * to_f(__ldg(lnq + qp.lpid[e]));
      lk += c;
      if ((int)qp.lpos[e] < r0) la += c;
    }
    lk = warp_sum(lk);
    la = warp_sum(la);
    carryA = qv.y + lk;
    Ak = carryA;
    if (!fix_reset && r0 <= k4) {
      Ar0 = qv.x + la;
      Arinf = Ar0;
    }
  }
  // ---- pass 1: prefixes, Pre total ---------------------------------------
  // Chunks of 128 (a chunk costs the same instructions however many of its
  // lanes hold incidences: measured against 256-incidence chunks and against
  // 256-incidence chunks with 64- or 128-incidence tails, this was fastest).
  // Chunks wholly inside the ray skip the bounds checks; chunks wholly
  // before k4 hold no potential and skip the Pre-total work.  kPf 1: the
  // next chunk's pair ids are requested before this chunk's ln q gathers;
  // kPf 2: its lengths as well.
  float ts = 0.0f, tc = 0.0f;
  Slice<kE> s;
  {
    float len[kE];
    for (int base = start; base < n_pre; base += kChunk) {
      const int i0 = base + kE * lane;
      uint32_t pid[kE];
      if (kPf) {
#pragma unroll
        for (int j = 0; j < kE; ++j) pid[j] = pid_next[j];
        if (kPf == 2) {
#pragma unroll
          for (int j = 0; j < kE; ++j) len[j] = len_next[j];
        }
        if (base + kChunk < n_pre) {
          load_pids<kE, kPol>(pid_next, off, i0 + kChunk, n_pre, inc_pair);
          if (kPf == 2) ld_len<kE, kPol>(len_next, inc_len + off, i0 + kChunk, i0 + kChunk < n_pre);
        }
      } else {
        load_pids<kE, kPol>(pid, off, i0, n_pre, inc_pair);
      }
      const float tot =
          base + kChunk <= n_pre
              ? slice_from_pids<kE, kPol, true, kPf == 2>(s, pid, off, i0, n_pre, k4, carryA, lane, inc_len,
                                                          inc_mu, lnq, len)
              : slice_from_pids<kE, kPol, false, kPf == 2>(s, pid, off, i0, n_pre, k4, carryA, lane,
                                                           inc_len, inc_mu, lnq, len);
      pre_marks<kE>(s, base, r0, rinf, k4, Ar0, Arinf, Ak);
      if (base + kChunk > k4) pre_total<kE>(s, i0, r0, Ar0, ts, tc);
      carryA += tot;
    }
  }
  // the lanes' compensated shares, summed in Acc once per ray (FP64 on
  // rays longer than kLongRay)
  Acc T = warp_sum((Acc)ts - (Acc)tc);
  // infinity term: visibility at the end of Pre (gvdbkernels.cu:1196-1208)
  if (me.flags & 1u) T += (Acc)__expf(carryA - Arinf);
  if (kdyn >= n_post) return;  // every message of the ray is static
  // ---- pass 2: dynamic messages ------------------------------------------
  // F is zero before k_dyn, so the running F starts at zero at k4; the
  // long-range difference T - F is carried in Acc, one subtraction per chunk
  Acc Dd = T;
  float cF = 0.0f;
  float carryA2 = Ak;
  for (int base = k4; base < n_post; base += kChunk) {
    const int i0 = base + kE * lane;
    const bool full = base + kChunk <= n_post;
    const float tot2 =
        full ? load_slice<kE, kPol, true>(s, off, i0, n_post, k4, carryA2, lane, inc_pair, inc_len, inc_mu,
                                          lnq)
             : load_slice<kE, kPol, false>(s, off, i0, n_post, k4, carryA2, lane, inc_pair, inc_len,
                                           inc_mu, lnq);
    carryA2 += tot2;
    float vmu[kE], q[kE];
#pragma unroll
    for (int j = 0; j < kE; ++j) {
      vmu[j] = __expf(s.A[j]) * s.mu[j];
      q[j] = __expf(s.lq[j]);
    }
    const float D = (float)Dd;
    const float ct = full ? emit_slice<kE, true>(vmu, q, s.len, i0, k4, n_post, cF, D, lane, off, inc_pl)
                          : emit_slice<kE, false>(vmu, q, s.len, i0, k4, n_post, cF, D, lane, off, inc_pl);
    Dd -= (Acc)ct;
    cF += ct;
  }
}

// Persistent launch: each warp takes the next ray from a work counter.
// kReg false: one queue, rays longest first (sorted once per incidence
// build, their RayMeta records copied into queue order), so the long rays
// start early and the short ones fill the tail.  kReg true (SM-affine):
// the view's pixels are cut into regions of consecutive pixels holding
// equal shares of its incidences, one region per SM (block b serves
// regions b mod G, + G, ..., G = min(grid, regions); a persistent grid is
// placed on the SMs in block order, so a region's blocks share an SM); a
// warp takes the home rays of its regions, then drains the view's leftover
// queue of short rays.  The warps of one SM trace neighbouring rays at the
// same time -- rays that cross the same voxels, so their ln q gathers hit
// the SM's L1.  Which warp handles a ray does not change its result.  Variants differ only in register budget (kMinBlocks
// resident blocks per SM), load policy and schedule: their arithmetic is
// identical, so the autotuner's choice never changes a result.
template <int kMinBlocks, int kPol, int kPf, bool kReg, typename TL, typename TQ>
__global__ void __launch_bounds__(kRayWarps * 32, kMinBlocks) k_ray_bp(const RayMeta* __restrict__ queue,
                                                           uint32_t n_rays,
                                                           const uint32_t* __restrict__ rstart,
                                                           uint32_t nreg, uint32_t rper,
                                                           const uint32_t* __restrict__ lprefix,
                                                           const uint32_t* __restrict__ lbase,
                                                           uint32_t nlv,
                                                           uint32_t* __restrict__ lcounter,
                                                           uint32_t* __restrict__ counter,
                                                           const uint32_t* __restrict__ inc_pair,
                                                           const TL* __restrict__ inc_len,
                                                           const float* __restrict__ inc_mu,
                                                           const TQ* __restrict__ lnq,
                                                           float* __restrict__ inc_pl,
                                                           const uint32_t* __restrict__ ids,
                                                           QuietPrefix qp, int fix_reset) {
  const int lane = threadIdx.x & 31;
  auto ray_at = [&](uint32_t i) {
    const RayMeta me = queue[i];
    const uint32_t rid = qp.q ? ids[i] : 0u;
    if (me.n_pre <= kLongRay)
      ray_bp_warp<float, kPol, kPf, TL, TQ>(me, rid, qp, inc_pair, inc_len, inc_mu, lnq, inc_pl, fix_reset,
                                            lane);
    else
      ray_bp_warp<double, kPol, kPf, TL, TQ>(me, rid, qp, inc_pair, inc_len, inc_mu, lnq, inc_pl, fix_reset,
                                             lane);
  };
  if constexpr (kReg) {
    // counter[r]: tickets of region r, whose home rays are positions
    // rstart[q (rper + 1) + rr] .. rstart[q (rper + 1) + rr + 1] (view q =
    // r / rper, rr = r % rper).  Block b serves regions b mod G, + G, ...
    // (G = min(grid, regions): every region has a home block).
    const uint32_t G = min(gridDim.x, nreg);
    for (uint32_t r = blockIdx.x % G; r < nreg; r += G) {
      const uint32_t q = r / rper;
      const uint32_t* rs = rstart + (size_t)q * (rper + 1) + (r - q * rper);
      const uint32_t a = rs[0], nr = rs[1] - a;
      // the next ticket is taken before the current ray runs, so its
      // atomic's latency hides behind the ray's work
      uint32_t idx = 0;
      if (lane == 0) idx = atomicAdd(counter + r, 1u);
      idx = __shfl_sync(kFull, idx, 0);
      while (idx < nr) {
        const uint32_t cur = a + idx;
        if (lane == 0) idx = atomicAdd(counter + r, 1u);
        idx = __shfl_sync(kFull, idx, 0);
        ray_at(cur);
      }
    }
    // the views' leftovers, one ticket counter over all of them: ticket t
    // is view q's (t - lprefix[q])-th leftover for the last q with
    // lprefix[q] <= t
    const uint32_t n_left = lprefix[nlv];
    auto leftover = [&]() {
      uint32_t pos = 0xFFFFFFFFu;
      if (lane == 0) {
        const uint32_t t = atomicAdd(lcounter, 1u);
        if (t < n_left) {
          uint32_t lo = 0, hi = nlv;
          while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (lprefix[mid] <= t) lo = mid;
            else hi = mid;
          }
          pos = lbase[lo] + (t - lprefix[lo]);
        }
      }
      return __shfl_sync(kFull, pos, 0);
    };
    uint32_t pos = leftover();
    while (pos != 0xFFFFFFFFu) {
      const uint32_t cur = pos;
      pos = leftover();
      ray_at(cur);
    }
  } else {
    uint32_t idx = 0;
    if (lane == 0) idx = atomicAdd(counter, 1u);
    idx = __shfl_sync(kFull, idx, 0);
    while (idx < n_rays) {
      const uint32_t cur = idx;
      if (lane == 0) idx = atomicAdd(counter, 1u);
      idx = __shfl_sync(kFull, idx, 0);
      ray_at(cur);
    }
  }
}

// queue records: queue[i] = meta[base + order[i]] (order: view-local ray
// indices, longest first)
__global__ void k_ray_queue(const RayMeta* __restrict__ meta, const uint32_t* __restrict__ order,
                            uint32_t n, RayMeta* __restrict__ queue, uint32_t* __restrict__ ids,
                            uint32_t id_base) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    queue[i] = meta[order[i]];
    ids[i] = id_base + order[i];
  }
}

// The static prefix of each queued ray of one view (rays r0..r0+n of the
// pixel arrays; a warp per ray): the loud incidences in [0, k4) -- those
// whose pair is among the view's first n_loud, the pairs on voxels with a
// dynamic incidence in any view -- counted (emit false) or listed at
// loff[r] (emit true: pair id, length, position), in ray order.
template <bool kEmit>
__global__ void k_loud_prefix(const RayMeta* __restrict__ meta, uint32_t r_first, uint32_t n,
                              const uint32_t* __restrict__ inc_pair, const float* __restrict__ inc_len,
                              uint32_t pair_base, uint32_t n_loud, uint32_t* __restrict__ loff,
                              uint32_t* __restrict__ lpid, float* __restrict__ llen,
                              uint16_t* __restrict__ lpos) {
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= n) return;
  const uint32_t r = r_first + w;
  const RayMeta me = meta[r];
  uint32_t cnt = 0;
  uint32_t at = kEmit ? loff[r] : 0u;
  if (ray_in_bp(me)) {
    const int k4 = ray_kdyn(me) & ~3;
    for (int b = 0; b < k4; b += 32) {
      const int j = b + lane;
      const uint32_t p = j < k4 ? inc_pair[me.off + j] : 0u;
      const bool loud = j < k4 && p - pair_base < n_loud;
      const unsigned m = __ballot_sync(kFull, loud);
      if (kEmit && loud) {
        const uint32_t e = at + (uint32_t)__popc(m & ((1u << lane) - 1u));
        lpid[e] = p;
        llen[e] = inc_len[me.off + j];
        lpos[e] = (uint16_t)j;
      }
      at += (uint32_t)__popc(m);
      cnt += (uint32_t)__popc(m);
    }
  }
  if (!kEmit && lane == 0) loff[r] = cnt;
}

// The quiet sums of the static prefix of each queued ray of one view (a
// warp per ray): sum of l ln q over the quiet incidences j < min(r0, k4)
// and j < k4, written to q[r] -- valid while the quiet pairs' ln q stay
// fixed, from the third iteration of a call on.  Lane-strided partial
// sums and a butterfly warp sum: a fixed order.
template <typename TQ>
__global__ void k_quiet_prefix(const RayMeta* __restrict__ meta, uint32_t r_first, uint32_t n,
                               const uint32_t* __restrict__ inc_pair, const float* __restrict__ inc_len,
                               const TQ* __restrict__ lnq, uint32_t pair_base, uint32_t n_loud,
                               float2* __restrict__ q) {
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= n) return;
  const uint32_t r = r_first + w;
  const RayMeta me = meta[r];
  if (!ray_in_bp(me)) return;
  const int k4 = ray_kdyn(me) & ~3;
  const int ra = min((int)me.r0, k4);
  float qa = 0.0f, qk = 0.0f;
  for (int j = lane; j < k4; j += 32) {
    const uint32_t p = inc_pair[me.off + j];
    if (p - pair_base >= n_loud) {
      const float c = inc_len[me.off + j] * to_f(__ldg(lnq + p));
      qk += c;
      if (j < ra) qa += c;
    }
  }
  qa = warp_sum(qa);
  qk = warp_sum(qk);
  if (lane == 0) q[r] = make_float2(qa, qk);
}

// ray queue of one build: active rays sorted by decreasing length
__global__ void k_ray_keys(const RayMeta* __restrict__ meta, uint32_t n, uint32_t* __restrict__ keys,
                           uint32_t* __restrict__ vals) {
  uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const RayMeta me = meta[r];
  keys[r] = ray_in_bp(me) ? 0xFFFFu - me.n_pre : 0x10000u;  // rays left out sort last
  vals[r] = r;
}

// Pair update: a load-balanced segmented reduction over the pair-grouped
// permutation of the messages, fused with the per-pair update.  One block
// takes a tile of kTile consecutive positions: it gathers the tile's messages
// into shared memory (coalesced permutation reads, kTile independent gathers
// in flight) together with the segment bounds of the pairs the tile
// touches; each thread then sums whole pairs sequentially from shared memory
// (a fixed order) and updates the pairs that lie inside the tile.  Segments
// that cross tile edges leave partial sums that k_pair_fixup adds in tile
// order.  Any segment length balances: voxels next to the camera are crossed
// by thousands of rays.
constexpr int kTileThreads = 256;
constexpr int kTile = 4 * kTileThreads;
constexpr uint32_t kOpenStart = 1u, kOpenEnd = 2u, kSingle = 4u;

// a dynamic run's update with its old message mo and the voxel's old total
// Lo already loaded (the gate c > kCumLenGate already checked)
__device__ __forceinline__ void apply_run_loaded(const uint4 r, float mo, float Lo, float acc_dyn,
                                                 float* __restrict__ m, float* __restrict__ L,
                                                 float* __restrict__ dm, int jacobi) {
  const uint32_t p = r.x, v = r.y;
  const float c = __uint_as_float(r.z);
  float a = clampf((__uint_as_float(r.w) + acc_dyn) / c, kFEps, 1.0f - kFEps);
  float mn = logf(a) - logf(1.0f - a);
  m[p] = mn;
  if (jacobi) {
    dm[p] = mn - mo;
    return;
  }
  L[v] = Lo + (mn - mo);
}

// factor->voxel update of one pair (gvdbkernels.cu:457-479).  The belief
// 1 - clamp(1 / (1 + e^L)) is not written here: k_belief_refresh derives it
// from L once the iterations of a call are done.
__device__ __forceinline__ void apply_pair(uint32_t p, float acc, const uint32_t* __restrict__ pair_vox,
                                           float* __restrict__ m, const float* __restrict__ cum,
                                           float* __restrict__ L, float* __restrict__ dm, int jacobi) {
  const float c = cum[p];
  const float mo = m[p];
  const uint32_t v = pair_vox[p];
  if (!(c > kCumLenGate)) return;  // gvdbkernels.cu:408: the pair never updates
  float a = clampf(acc / c, kFEps, 1.0f - kFEps);
  float mn = logf(a) - logf(1.0f - a);
  m[p] = mn;
  if (jacobi) {
    dm[p] = mn - mo;
    return;
  }
  L[v] = L[v] + (mn - mo);
}

// the same for a dynamic run, whose pair id, voxel, cumulative length and
// static-message sum are stored together (one 16-byte load; the voxel's L
// gather does not wait on a pair-id lookup)
__device__ __forceinline__ void apply_run(const uint4 r, float acc_dyn, float* __restrict__ m,
                                          float* __restrict__ L, float* __restrict__ dm, int jacobi) {
  const uint32_t p = r.x, v = r.y;
  const float c = __uint_as_float(r.z);
  if (!(c > kCumLenGate)) return;  // gvdbkernels.cu:408: the pair never updates
  apply_run_loaded(r, m[p], jacobi ? 0.0f : L[v], acc_dyn, m, L, dm, jacobi);
}

// kTwo false: one prefetched pair per thread, 32 registers (8 blocks per
// SM); true: two, 48 registers (5 blocks per SM).  Same arithmetic.
template <bool kTwo>
__global__ void __launch_bounds__(kTileThreads, kTwo ? 5 : 8)
    k_pair_reduce(const uint32_t* __restrict__ perm, const float* __restrict__ pl,
                  const uint32_t* __restrict__ seg, const uint32_t* __restrict__ tile_first,
                  uint32_t k0, uint32_t k1, uint32_t p_end, TileCarry* __restrict__ carry,
                  const uint4* __restrict__ drun, float* __restrict__ m, float* __restrict__ L,
                  float* __restrict__ dm, int jacobi) {
  __shared__ float sv[kTile];
  __shared__ uint32_t sseg[kTile + 2];
  const int t = threadIdx.x;
  const uint32_t base = k0 + blockIdx.x * kTile;
  const uint32_t n = min((uint32_t)kTile, k1 - base);
  const uint32_t end = base + n;
  const uint32_t pf = tile_first[blockIdx.x];
  // a tile touches at most n pairs: their starts and the next pair's start
  const uint32_t nseg = min(n + 1, p_end - pf) + 1;
  // the run records of this thread's first two pairs (q = t, t + 256; a
  // tile of 1024 positions holds about 340 pairs), and those pairs' messages
  // and voxel totals, are requested before the message gathers so that no
  // dependent load waits after the barrier.  The tile's pairs end at the
  // next tile's first pair.
  const uint32_t last = blockIdx.x + 1 < gridDim.x ? tile_first[blockIdx.x + 1] : p_end - 1;
  uint4 r0 = make_uint4(0u, 0u, 0u, 0u), r1 = make_uint4(0u, 0u, 0u, 0u);
  float mo0 = 0.0f, Lo0 = 0.0f, mo1 = 0.0f, Lo1 = 0.0f;
  const bool pre = t < n && pf + t < p_end;
  const bool pre1 = kTwo && t + kTileThreads < n && pf + t + kTileThreads <= min(last, p_end - 1);
  if (pre) r0 = drun[pf + t];
  if (pre1) r1 = drun[pf + t + kTileThreads];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    uint32_t i = j * kTileThreads + t;
    if (i < n) sv[i] = pl[perm[base + i]];
  }
  for (uint32_t q = t; q < nseg; q += kTileThreads) sseg[q] = seg[pf + q];
  const bool gate0 = pre && __uint_as_float(r0.z) > kCumLenGate;
  if (gate0) {
    mo0 = m[r0.x];
    if (!jacobi) Lo0 = L[r0.y];
  }
  const bool gate1 = pre1 && __uint_as_float(r1.z) > kCumLenGate;
  if (gate1) {
    mo1 = m[r1.x];
    if (!jacobi) Lo1 = L[r1.y];
  }
  __syncthreads();
  for (uint32_t q = t; q < n && pf + q < p_end && sseg[q] < end; q += kTileThreads) {
    const uint32_t s0 = sseg[q], s1 = sseg[q + 1];
    const uint32_t a = max(s0, base) - base, b = min(s1, end) - base;
    float acc = 0.0f;
    for (uint32_t i = a; i < b; ++i) acc += sv[i];
    const bool open_start = s0 < base, open_end = s1 > end;
    if (!open_start && !open_end) {
      if (q == t) {
        if (gate0) apply_run_loaded(r0, mo0, Lo0, acc, m, L, dm, jacobi);
      } else if (q == t + kTileThreads && pre1) {
        if (gate1) apply_run_loaded(r1, mo1, Lo1, acc, m, L, dm, jacobi);
      } else {
        apply_run(drun[pf + q], acc, m, L, dm, jacobi);
      }
      continue;
    }
    TileCarry& c = carry[blockIdx.x];
    if (open_start) {
      c.first_key = pf + q;
      c.first_sum = acc;
    }
    if (open_end) {
      c.last_key = pf + q;
      c.last_sum = acc;
    }
  }
  if (t == 0) {
    // the first pair is open at the start iff it began before the tile; the
    // last pair (the one holding position end-1) is open iff it goes on
    // ql = last q with sseg[q] < end (binary search over the loaded starts)
    uint32_t lo = 0, hi = min(n, p_end - pf);
    while (hi - lo > 1) {
      uint32_t mid = (lo + hi) >> 1;
      if (sseg[mid] < end) lo = mid;
      else hi = mid;
    }
    const uint32_t ql = lo;
    uint32_t f = 0;
    if (sseg[0] < base) f |= kOpenStart;
    if (sseg[ql + 1] > end) f |= kOpenEnd;
    if (ql == 0) f |= kSingle;
    carry[blockIdx.x].flags = f;
  }
}

// first pair of every tile of a position range (pairs are sorted, so it is
// the pair whose segment holds the tile's first position)
__global__ void k_tile_first(const uint32_t* __restrict__ seg, uint32_t p0, uint32_t p1, uint32_t k0,
                             uint32_t ntiles, uint32_t* __restrict__ out) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  uint32_t pos = k0 + t * kTile;
  uint32_t lo = p0, hi = p1;  // last p with seg[p] <= pos
  while (hi - lo > 1) {
    uint32_t mid = lo + ((hi - lo) >> 1);
    if (seg[mid] <= pos) lo = mid;
    else hi = mid;
  }
  out[t] = lo;
}

// segments crossing tile edges: the tile where such a segment starts walks
// forward adding each following tile's partial, in tile order
__global__ void k_pair_fixup(const TileCarry* __restrict__ carry, uint32_t ntiles,
                             const uint4* __restrict__ drun, float* __restrict__ m,
                             float* __restrict__ L, float* __restrict__ dm, int jacobi) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  TileCarry c = carry[t];
  if (!(c.flags & kOpenEnd)) return;
  if ((c.flags & kSingle) && (c.flags & kOpenStart)) return;  // not where the segment starts
  float sum = c.last_sum;
  uint32_t key = c.last_key;
  for (uint32_t u = t + 1; u < ntiles; ++u) {
    TileCarry d = carry[u];
    sum += d.first_sum;
    if ((d.flags & kSingle) && (d.flags & kOpenEnd)) continue;
    break;
  }
  apply_run(drun[key], sum, m, L, dm, jacobi);
}

// per dynamic run: {pair id, voxel, cumulative length, static-message sum}
__global__ void k_drun(const uint32_t* __restrict__ dpair, uint32_t n, const uint32_t* __restrict__ pair_vox,
                       const float* __restrict__ cum, const float* __restrict__ stat,
                       uint4* __restrict__ drun) {
  uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const uint32_t p = dpair[j];
  drun[j] = make_uint4(p, pair_vox[p], __float_as_uint(cum[p]), __float_as_uint(stat[p]));
}

// pairs whose incidences are all static: a = (sum of F_EPS * l) / cum is a
// build constant, so their update changes the state only right after their
// messages were zeroed or remapped
__global__ void k_static_pairs(uint32_t p0, uint32_t p1, const uint32_t* __restrict__ ndyn,
                               const float* __restrict__ stat, const uint32_t* __restrict__ pair_vox,
                               float* __restrict__ m, const float* __restrict__ cum,
                               float* __restrict__ L, float* __restrict__ dm, int jacobi) {
  uint32_t p = p0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= p1 || ndyn[p]) return;
  apply_pair(p, stat[p], pair_vox, m, cum, L, dm, jacobi);
}

// Jacobi: total log-odds of each voxel moves by the sum of its cameras'
// message changes (pairs of a voxel grouped by a voxel-sorted CSR)
__global__ void k_voxel_apply(const uint32_t* __restrict__ vseg, const uint32_t* __restrict__ vpairs,
                              const uint32_t* __restrict__ vvox, uint32_t nvox,
                              const float* __restrict__ dm, float* __restrict__ L) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvox) return;
  float s = 0.0f;
  bool any = false;
  for (uint32_t k = vseg[i]; k < vseg[i + 1]; ++k) {
    float d = dm[vpairs[k]];
    if (d == d) {  // pairs below the length gate carry NaN and are skipped
      s += d;
      any = true;
    }
  }
  if (!any) return;
  uint32_t v = vvox[i];
  L[v] = L[v] + s;
}

// beliefs of the voxels the iterations update (those with a pair past the
// length gate in some camera), from their total log-odds: the per-voxel
// belief of gvdbkernels.cu:474-477, written once per call instead of at
// every message update
__global__ void k_belief_refresh(const float* __restrict__ L, const uint8_t* __restrict__ active, int64_t n,
                                 float* __restrict__ belief) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (active[i]) belief[i] = 1.0f - clampf(1.0f / (1.0f + expf(L[i])), kFEps, 1.0f - kFEps);
}

__global__ void k_max_abs_diff(const float* __restrict__ a, const float* __restrict__ b, int64_t n,
                               uint32_t* __restrict__ out) {
  float mx = 0.0f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    mx = fmaxf(mx, fabsf(a[i] - b[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(mx));
}

// total log-odds of each voxel rebuilt from its messages (voxel CSR):
// L = L (already the prior) + sum m over the pairs that pass the length gate
__global__ void k_voxel_rebuild(const uint32_t* __restrict__ vseg, const uint32_t* __restrict__ vpairs,
                                const uint32_t* __restrict__ vvox, uint32_t nvox,
                                const float* __restrict__ m, const float* __restrict__ cum,
                                float* __restrict__ L, float* __restrict__ belief) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvox) return;
  float s = 0.0f;
  bool any = false;
  for (uint32_t k = vseg[i]; k < vseg[i + 1]; ++k) {
    const uint32_t p = vpairs[k];
    if (cum[p] > kCumLenGate) {
      s += m[p];
      any = true;
    }
  }
  if (!any) return;
  uint32_t v = vvox[i];
  float Lv = L[v] + s;
  L[v] = Lv;
  belief[v] = 1.0f - clampf(1.0f / (1.0f + expf(Lv)), kFEps, 1.0f - kFEps);
}

// Warm-start initial messages of every voxel's pairs from a predicted total
// log-odds: pairs without dynamic incidences get their exact constant
// message; the rest of (L_pred - logit(prior)) is shared among the dynamic
// pairs in proportion to their cumulative length.  Pairs below the length
// gate keep 0 (they never update).
__global__ void k_warm_split(const uint32_t* __restrict__ vseg, const uint32_t* __restrict__ vpairs,
                             const uint32_t* __restrict__ vvox, uint32_t nvox,
                             const float* __restrict__ L_pred, float lp, const float* __restrict__ base,
                             const float* __restrict__ cum, const float* __restrict__ stat,
                             const uint32_t* __restrict__ ndyn, float* __restrict__ m) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvox) return;
  float fixed = 0.0f, dyn_len = 0.0f;
  for (uint32_t k = vseg[i]; k < vseg[i + 1]; ++k) {
    const uint32_t p = vpairs[k];
    const float c = cum[p];
    if (!(c > kCumLenGate)) continue;
    if (ndyn[p]) {
      dyn_len += c;
    } else {
      float a = clampf(stat[p] / c, kFEps, 1.0f - kFEps);
      fixed += logf(a) - logf(1.0f - a);
    }
  }
  const float rest = L_pred[vvox[i]] - (base ? base[vvox[i]] : lp) - fixed;
  for (uint32_t k = vseg[i]; k < vseg[i + 1]; ++k) {
    const uint32_t p = vpairs[k];
    const float c = cum[p];
    float mv = 0.0f;
    if (c > kCumLenGate) {
      if (ndyn[p]) {
        mv = rest * (c / dyn_len);
      } else {
        float a = clampf(stat[p] / c, kFEps, 1.0f - kFEps);
        mv = logf(a) - logf(1.0f - a);
      }
    }
    m[p] = mv;
  }
}

// Warm-start features of every voxel slot, [slot*512 + local][4]:
// 0 current belief, 1 log(1 + pass-through length), 2 log(1 + potential
// mass sum mu*l), 3 log(1 + length inside the potential windows); lengths
// in voxels, summed over the voxel's cameras in pair order.
__global__ void k_feat_belief(const float* __restrict__ belief, int64_t n, float* __restrict__ feat) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  *reinterpret_cast<float4*>(feat + 4 * i) = make_float4(belief[i], 0.0f, 0.0f, 0.0f);
}

__global__ void k_voxel_features(const uint32_t* __restrict__ vseg, const uint32_t* __restrict__ vpairs,
                                 const uint32_t* __restrict__ vvox, uint32_t nvox,
                                 const float* __restrict__ cum, const float* __restrict__ stat,
                                 const float* __restrict__ hit, float* __restrict__ feat) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvox) return;
  float pass = 0.0f, mass = 0.0f, win = 0.0f;
  for (uint32_t k = vseg[i]; k < vseg[i + 1]; ++k) {
    const uint32_t p = vpairs[k];
    const float sl = stat[p] * (1.0f / kFEps);
    pass += sl;
    mass += hit[p];
    win += fmaxf(cum[p] - sl, 0.0f);
  }
  float* f = feat + 4 * (int64_t)vvox[i];
  f[1] = log1pf(pass);
  f[2] = log1pf(mass);
  f[3] = log1pf(win);
}

// moving a camera: take its messages out of the total log-odds
__global__ void k_remove_messages(const uint32_t* __restrict__ pair_vox, float* __restrict__ m,
                                  uint32_t p0, uint32_t p1, float* __restrict__ L,
                                  float* __restrict__ belief) {
  uint32_t p = p0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= p1) return;
  float mo = m[p];
  if (mo == 0.0f) return;
  uint32_t v = pair_vox[p];
  float Lv = L[v] - mo;
  L[v] = Lv;
  belief[v] = 1.0f - clampf(1.0f / (1.0f + expf(Lv)), kFEps, 1.0f - kFEps);
  m[p] = 0.0f;
}

// a retired camera's messages added to the base log-odds (one pair per
// voxel within a camera: no two threads share a voxel)
__global__ void k_fold_messages(const uint32_t* __restrict__ pv, const float* __restrict__ m, uint32_t n,
                                float* __restrict__ base) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n && m[p] != 0.0f) base[pv[p]] += m[p];
}

__global__ void k_remap_scatter(const uint32_t* __restrict__ pv, const float* __restrict__ m,
                                uint32_t n, float* __restrict__ dense) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) dense[pv[p]] = m[p];
}

__global__ void k_remap_gather(const uint32_t* __restrict__ pv, float* __restrict__ m, uint32_t n,
                               const float* __restrict__ dense) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) m[p] = dense[pv[p]];
}

__global__ void k_fill_u32(uint32_t* p, int64_t n, uint32_t v) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

__global__ void k_fill(float* p, int64_t n, float v) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

__global__ void k_vflag(const uint32_t* __restrict__ sk, uint32_t n, uint32_t* __restrict__ flag) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) flag[k] = (k == 0 || sk[k] != sk[k - 1]) ? 1u : 0u;
}

__global__ void k_vassign(const uint32_t* __restrict__ sk, const uint32_t* __restrict__ flag,
                          const uint32_t* __restrict__ scan, uint32_t n, uint32_t* __restrict__ vvox,
                          uint32_t* __restrict__ vseg) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n || !flag[k]) return;
  vvox[scan[k]] = sk[k];
  vseg[scan[k]] = k;
}

__global__ void k_scatter_const(const uint32_t* __restrict__ idx, uint32_t n, float v,
                                float* __restrict__ dense) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) dense[idx[p]] = v;
}

// pairs past the length gate (the ones that ever update): counted, and
// their voxels flagged
__global__ void k_touch_pairs(const uint32_t* __restrict__ pair_vox, const float* __restrict__ cum,
                              uint32_t np, uint8_t* __restrict__ flag,
                              unsigned long long* __restrict__ n_active) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = p < np && cum[p] > kCumLenGate;
  if (act) flag[pair_vox[p]] = 1;
  const unsigned b = __ballot_sync(kFull, act);
  if (n_active && (threadIdx.x & 31) == 0 && b) atomicAdd(n_active, (unsigned long long)__popc(b));
}

// 64-bit total of n u32 counts (the incidence total of a build, checked
// against the 32-bit index range before any offset is formed from it)
__global__ void k_sum_u32(const uint32_t* __restrict__ v, int64_t n, unsigned long long* __restrict__ out) {
  unsigned long long c = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    c += v[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(kFull, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// the per-view counters of a view's ray records, kRayCounters 64-bit totals:
// Pre incidences, rays with any, Post incidences, dynamic Post incidences
// (those from k_dyn on), rays in BP, their Pre incidences, and their Pre
// incidences from the quiet-prefix boundary (k_dyn rounded down to 4) on.
// Integer sums: the totals do not depend on the order of the atomics.
__global__ void k_ray_counters(const RayMeta* __restrict__ meta, int64_t n, unsigned long long* __restrict__ out) {
  unsigned long long c[kRayCounters] = {};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const RayMeta r = meta[i];
    const int kd = ray_kdyn(r);
    c[0] += r.n_pre;
    c[1] += r.n_pre > 0;
    c[2] += r.n_post;
    c[3] += (unsigned)(r.n_post - min(kd, (int)r.n_post));
    if (ray_in_bp(r)) {
      c[4] += 1;
      c[5] += r.n_pre;
      c[6] += (unsigned long long)(long long)((int)r.n_pre - (kd & ~3));  // two's complement: a signed total
    }
  }
#pragma unroll
  for (int k = 0; k < kRayCounters; ++k) {
    unsigned long long v = c[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(out + k, v);
  }
}

__global__ void k_count_flags(const uint8_t* __restrict__ flag, int64_t n, unsigned long long* __restrict__ out) {
  unsigned c = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    c += flag[i] != 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(kFull, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, (unsigned long long)c);
}

inline unsigned blocks(int64_t n, int t) { return (unsigned)std::max<int64_t>(1, (n + t - 1) / t); }

}  // namespace

cudaError_t launch_pair_prepare(const BpArrays& a, uint32_t p0, uint32_t p1, int jacobi,
                                cudaStream_t s) {
  if (p1 <= p0) return cudaSuccess;
  k_pair_prepare<<<blocks(p1 - p0, kPrepThreads * kPrepPer), kPrepThreads, 0, s>>>(
      a.pair_vox, a.pair_m, a.L, a.pair_lnq, a.half_streams ? a.pair_lnq16 : nullptr,
      jacobi ? a.pair_dm : nullptr, p0, p1);
  return cudaGetLastError();
}


// ray-kernel variants: (id, resident-block target, load policy, chunk
// prefetch, schedule: 0 longest first, 1 SM regions)
#define MRF_RAY_VARIANTS(X) \
  X(0, 0, 0, 0, 0) X(1, 0, 0, 1, 0) X(2, 0, 0, 2, 0) X(3, 0, 0, 0, 1) X(4, 0, 0, 1, 1) X(5, 0, 0, 2, 1) \
  X(6, 12, 0, 1, 1) X(7, 12, 1, 1, 1)
constexpr int kRayVariants = 8;

int ray_bp_variants() { return kRayVariants; }

namespace {
template <typename K>
int resident_of(K kernel) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel,
                                                    kRayWarps * 32, 0) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  return per_sm;
}
}  // namespace

int ray_bp_resident_blocks(int variant, int half_streams) {
  static int resident[2][kRayVariants] = {{0}};
  if (variant < 0 || variant >= kRayVariants) return 1;
  const int h = half_streams ? 1 : 0;
  if (!resident[h][variant]) {
    switch (variant) {
#define X(id, mb, pol, pf, sc)                                                                        \
  case id:                                                                                            \
    resident[h][variant] = h ? resident_of(k_ray_bp<mb, pol, pf, (sc > 0), __half, __half>)          \
                             : resident_of(k_ray_bp<mb, pol, pf, (sc > 0), float, float>);           \
    break;
      MRF_RAY_VARIANTS(X)
#undef X
    }
  }
  return resident[h][variant];
}

cudaError_t launch_ray_bp(const BpArrays& a, const RayWork& w, int fix_reset, int num_sms, int variant,
                          bool quiet, cudaStream_t s) {
  if (!w.n_rays) return cudaSuccess;
  QuietPrefix qp{};
  if (quiet) {
    qp.q = a.quiet_q;
    qp.loff = a.loud_off;
    qp.lpid = a.loud_pid;
    qp.llen = a.loud_len;
    qp.lpos = a.loud_pos;
  }
  if (variant < 0 || variant >= kRayVariants) return cudaErrorInvalidValue;
  int64_t b = std::min<int64_t>((int64_t)num_sms * ray_bp_resident_blocks(variant, a.half_streams),
                                (w.n_rays + kRayWarps - 1) / kRayWarps);
  const unsigned grid = (unsigned)std::max<int64_t>(b, 1);
  switch (variant) {
#define X(id, mb, pol, pf, sc)                                                                    \
  case id:                                                                                        \
    if (a.half_streams)                                                                           \
      k_ray_bp<mb, pol, pf, (sc > 0), __half, __half><<<grid, kRayWarps * 32, 0, s>>>(            \
          sc == 0 ? w.queue : w.region, w.n_rays, w.rstart, w.nreg, w.rper, w.lprefix, w.lbase,    \
          w.nlv, w.lcounter, sc == 0 ? w.counter : w.rcounter, a.inc_pair, a.inc_len16, a.inc_mu,  \
          a.pair_lnq16, a.inc_pl, sc == 0 ? w.queue_ids : w.region_ids, qp, fix_reset);            \
    else                                                                                          \
      k_ray_bp<mb, pol, pf, (sc > 0), float, float><<<grid, kRayWarps * 32, 0, s>>>(              \
          sc == 0 ? w.queue : w.region, w.n_rays, w.rstart, w.nreg, w.rper, w.lprefix, w.lbase,    \
          w.nlv, w.lcounter, sc == 0 ? w.counter : w.rcounter, a.inc_pair, a.inc_len, a.inc_mu,    \
          a.pair_lnq, a.inc_pl, sc == 0 ? w.queue_ids : w.region_ids, qp, fix_reset);              \
    break;
    MRF_RAY_VARIANTS(X)
#undef X
  }
  return cudaGetLastError();
}

cudaError_t launch_ray_keys(const RayMeta* meta, uint32_t n, uint32_t* keys, uint32_t* vals,
                            cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_ray_keys<<<blocks(n, 256), 256, 0, s>>>(meta, n, keys, vals);
  return cudaGetLastError();
}

cudaError_t launch_ray_queue(const RayMeta* meta, const uint32_t* order, uint32_t n, RayMeta* queue,
                             uint32_t* ids, uint32_t id_base, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_ray_queue<<<blocks(n, 256), 256, 0, s>>>(meta, order, n, queue, ids, id_base);
  return cudaGetLastError();
}

cudaError_t launch_loud_prefix(const RayMeta* meta, uint32_t r_first, uint32_t n, const uint32_t* inc_pair,
                               const float* inc_len, uint32_t pair_base, uint32_t n_loud, uint32_t* loff,
                               uint32_t* lpid, float* llen, uint16_t* lpos, bool emit, cudaStream_t s) {
  if (!n) return cudaSuccess;
  const unsigned g = blocks((uint64_t)n * 32, 256);
  if (emit)
    k_loud_prefix<true><<<g, 256, 0, s>>>(meta, r_first, n, inc_pair, inc_len, pair_base, n_loud, loff, lpid,
                                          llen, lpos);
  else
    k_loud_prefix<false><<<g, 256, 0, s>>>(meta, r_first, n, inc_pair, inc_len, pair_base, n_loud, loff,
                                           lpid, llen, lpos);
  return cudaGetLastError();
}

cudaError_t launch_quiet_prefix(const BpArrays& a, uint32_t r_first, uint32_t n, uint32_t pair_base,
                                uint32_t n_loud, float2* q, cudaStream_t s) {
  if (!n) return cudaSuccess;
  const unsigned g = blocks((uint64_t)n * 32, 256);
  if (a.half_streams)
    k_quiet_prefix<__half><<<g, 256, 0, s>>>(a.meta, r_first, n, a.inc_pair, a.inc_len, a.pair_lnq16, pair_base,
                                             n_loud, q);
  else
    k_quiet_prefix<float><<<g, 256, 0, s>>>(a.meta, r_first, n, a.inc_pair, a.inc_len, a.pair_lnq, pair_base,
                                            n_loud, q);
  return cudaGetLastError();
}

cudaError_t launch_pair_update(const BpArrays& a, uint32_t k0, uint32_t k1, uint32_t j0, uint32_t j1,
                               const uint32_t* tile_first, TileCarry* carry, int jacobi,
                               cudaStream_t s) {
  (void)j0;
  if (k1 <= k0) return cudaSuccess;
  uint32_t ntiles = (k1 - k0 + kTile - 1) / kTile;
  if (a.pair_variant)
    k_pair_reduce<true><<<ntiles, kTileThreads, 0, s>>>(a.dperm, a.inc_pl, a.dseg, tile_first, k0, k1, j1,
                                                        carry, a.drun, a.pair_m, a.L, a.pair_dm, jacobi);
  else
    k_pair_reduce<false><<<ntiles, kTileThreads, 0, s>>>(a.dperm, a.inc_pl, a.dseg, tile_first, k0, k1, j1,
                                                         carry, a.drun, a.pair_m, a.L, a.pair_dm, jacobi);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_pair_fixup<<<blocks(ntiles, 256), 256, 0, s>>>(carry, ntiles, a.drun, a.pair_m, a.L, a.pair_dm,
                                                   jacobi);
  return cudaGetLastError();
}

cudaError_t launch_drun(const uint32_t* dpair, uint32_t n, const uint32_t* pair_vox, const float* cum,
                        const float* stat, uint4* drun, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_drun<<<blocks(n, 256), 256, 0, s>>>(dpair, n, pair_vox, cum, stat, drun);
  return cudaGetLastError();
}

cudaError_t launch_static_pairs(const BpArrays& a, uint32_t p0, uint32_t p1, int jacobi,
                                cudaStream_t s) {
  if (p1 <= p0) return cudaSuccess;
  k_static_pairs<<<blocks(p1 - p0, 256), 256, 0, s>>>(p0, p1, a.pair_ndyn, a.pair_stat, a.pair_vox,
                                                      a.pair_m, a.pair_cum, a.L, a.pair_dm, jacobi);
  return cudaGetLastError();
}

cudaError_t launch_tile_first(const uint32_t* seg, uint32_t p0, uint32_t p1, uint32_t k0, uint32_t k1,
                              uint32_t* out, cudaStream_t s) {
  if (k1 <= k0) return cudaSuccess;
  uint32_t ntiles = (k1 - k0 + kTile - 1) / kTile;
  k_tile_first<<<blocks(ntiles, 256), 256, 0, s>>>(seg, p0, p1, k0, ntiles, out);
  return cudaGetLastError();
}

uint32_t pair_update_tiles(uint32_t n) { return (n + kTile - 1) / kTile; }

cudaError_t launch_voxel_apply(const uint32_t* vseg, const uint32_t* vpairs, const uint32_t* vvox,
                               uint32_t nvox, const float* pair_dm, float* L, cudaStream_t s) {
  if (!nvox) return cudaSuccess;
  k_voxel_apply<<<blocks(nvox, 256), 256, 0, s>>>(vseg, vpairs, vvox, nvox, pair_dm, L);
  return cudaGetLastError();
}

cudaError_t launch_active_voxels(const uint32_t* pair_vox, const float* cum, uint32_t np, uint8_t* flag,
                                 int64_t nvox, cudaStream_t s) {
  if (nvox <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(flag, 0, (size_t)nvox, s);
  if (e != cudaSuccess) return e;
  if (np) k_touch_pairs<<<blocks(np, 256), 256, 0, s>>>(pair_vox, cum, np, flag, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_mark_active(const uint32_t* pair_vox, const float* cum, uint32_t np, uint8_t* flag,
                               cudaStream_t s) {
  if (!np) return cudaSuccess;
  k_touch_pairs<<<blocks(np, 256), 256, 0, s>>>(pair_vox, cum, np, flag, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_belief_refresh(const float* L, const uint8_t* active, int64_t nvox, float* belief,
                                  cudaStream_t s) {
  if (nvox <= 0) return cudaSuccess;
  k_belief_refresh<<<(unsigned)std::min<int64_t>(blocks(nvox, 256), 8192), 256, 0, s>>>(L, active, nvox, belief);
  return cudaGetLastError();
}

cudaError_t launch_max_abs_diff(const float* a, const float* b, int64_t n, uint32_t* out,
                                cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, 4, s);
  if (e != cudaSuccess || n <= 0) return e;
  int64_t nb = std::min<int64_t>((n + 255) / 256, 4096);
  k_max_abs_diff<<<(unsigned)nb, 256, 0, s>>>(a, b, n, out);
  return cudaGetLastError();
}

cudaError_t launch_warm_split(const uint32_t* vseg, const uint32_t* vpairs, const uint32_t* vvox,
                              uint32_t nvox, const float* L_pred, float lp, const float* base, const float* cum,
                              const float* stat, const uint32_t* ndyn, float* m, cudaStream_t s) {
  if (!nvox) return cudaSuccess;
  k_warm_split<<<blocks(nvox, 256), 256, 0, s>>>(vseg, vpairs, vvox, nvox, L_pred, lp, base, cum, stat, ndyn, m);
  return cudaGetLastError();
}

cudaError_t launch_voxel_features(const uint32_t* vseg, const uint32_t* vpairs, const uint32_t* vvox,
                                  uint32_t nvox, const float* cum, const float* stat, const float* hit,
                                  const float* belief, int64_t n_slots_vox, float* feat, cudaStream_t s) {
  if (n_slots_vox <= 0) return cudaSuccess;
  k_feat_belief<<<blocks(n_slots_vox, 256), 256, 0, s>>>(belief, n_slots_vox, feat);
  if (nvox) k_voxel_features<<<blocks(nvox, 256), 256, 0, s>>>(vseg, vpairs, vvox, nvox, cum, stat, hit, feat);
  return cudaGetLastError();
}

cudaError_t launch_voxel_rebuild(const uint32_t* vseg, const uint32_t* vpairs, const uint32_t* vvox,
                                 uint32_t nvox, const float* m, const float* cum, float* L, float* belief,
                                 cudaStream_t s) {
  if (!nvox) return cudaSuccess;
  k_voxel_rebuild<<<blocks(nvox, 256), 256, 0, s>>>(vseg, vpairs, vvox, nvox, m, cum, L, belief);
  return cudaGetLastError();
}

cudaError_t launch_remove_messages(const BpArrays& a, uint32_t p0, uint32_t p1, cudaStream_t s) {
  if (p1 <= p0) return cudaSuccess;
  k_remove_messages<<<blocks(p1 - p0, 256), 256, 0, s>>>(a.pair_vox, a.pair_m, p0, p1, a.L, a.belief);
  return cudaGetLastError();
}

cudaError_t launch_fold_messages(const uint32_t* pair_vox, const float* pair_m, uint32_t n, float* base,
                                 cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_fold_messages<<<blocks(n, 256), 256, 0, s>>>(pair_vox, pair_m, n, base);
  return cudaGetLastError();
}

cudaError_t launch_remap_scatter(const uint32_t* pair_vox, const float* pair_m, uint32_t n,
                                 float* dense, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_remap_scatter<<<blocks(n, 256), 256, 0, s>>>(pair_vox, pair_m, n, dense);
  return cudaGetLastError();
}

cudaError_t launch_remap_gather(const uint32_t* pair_vox, float* pair_m, uint32_t n,
                                const float* dense, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_remap_gather<<<blocks(n, 256), 256, 0, s>>>(pair_vox, pair_m, n, dense);
  return cudaGetLastError();
}

__global__ void k_to_half(const float* __restrict__ in, int64_t n, __half* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __float2half_rn(in[i]);
}

cudaError_t launch_to_half(const float* in, int64_t n, __half* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_to_half<<<(unsigned)std::min<int64_t>(blocks(n, 256), 16384), 256, 0, s>>>(in, n, out);
  return cudaGetLastError();
}

cudaError_t launch_fill_u32(uint32_t* p, int64_t n, uint32_t v, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_fill_u32<<<blocks(n, 256), 256, 0, s>>>(p, n, v);
  return cudaGetLastError();
}

cudaError_t launch_fill_f32(float* p, int64_t n, float v, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_fill<<<blocks(n, 256), 256, 0, s>>>(p, n, v);
  return cudaGetLastError();
}

cudaError_t launch_vflag(const uint32_t* sk, uint32_t n, uint32_t* flag, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_vflag<<<blocks(n, 256), 256, 0, s>>>(sk, n, flag);
  return cudaGetLastError();
}

cudaError_t launch_vassign(const uint32_t* sk, const uint32_t* flag, const uint32_t* scan,
                           uint32_t n, uint32_t* vvox, uint32_t* vseg, cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_vassign<<<blocks(n, 256), 256, 0, s>>>(sk, flag, scan, n, vvox, vseg);
  return cudaGetLastError();
}

cudaError_t launch_touch_counts(const uint32_t* pair_vox, const float* cum, uint32_t np, uint8_t* flag,
                                int64_t nvox, unsigned long long* out2, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out2, 0, 16, s);
  if (e == cudaSuccess && nvox > 0) e = cudaMemsetAsync(flag, 0, (size_t)nvox, s);
  if (e != cudaSuccess) return e;
  if (np) k_touch_pairs<<<blocks(np, 256), 256, 0, s>>>(pair_vox, cum, np, flag, out2);
  if (nvox > 0)
    k_count_flags<<<(unsigned)std::min<int64_t>(blocks(nvox, 256), 4096), 256, 0, s>>>(flag, nvox, out2 + 1);
  return cudaGetLastError();
}

cudaError_t launch_sum_u32(const uint32_t* v, int64_t n, unsigned long long* out, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, 8, s);
  if (e != cudaSuccess || n <= 0) return e;
  k_sum_u32<<<(unsigned)std::min<int64_t>(blocks(n, 256), 4096), 256, 0, s>>>(v, n, out);
  return cudaGetLastError();
}

cudaError_t launch_ray_counters(const RayMeta* meta, int64_t n, unsigned long long* out, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, kRayCounters * sizeof(unsigned long long), s);
  if (e != cudaSuccess || n <= 0) return e;
  k_ray_counters<<<(unsigned)std::min<int64_t>(blocks(n, 256), 1024), 256, 0, s>>>(meta, n, out);
  return cudaGetLastError();
}

cudaError_t launch_scatter_const(const uint32_t* idx, uint32_t n, float v, float* dense,
                                 cudaStream_t s) {
  if (!n) return cudaSuccess;
  k_scatter_const<<<blocks(n, 256), 256, 0, s>>>(idx, n, v, dense);
  return cudaGetLastError();
}

}  // namespace mrf
