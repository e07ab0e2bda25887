// mrf_noalloc.cu -- likelihood entry point that allocates no device memory.
//
// Who needs it: callers that score depth images against a finished map
// from a loop that must not allocate -- e.g. a real-time localisation or
// pose-search loop on a robot, where cudaMalloc/cudaFree may synchronize the
// device and take unbounded time, or a host framework that owns all device
// memory through its own allocator and forbids other allocations.  The
// regular mrf_likelihood_device grows map-owned scratch (a cleaned copy of
// the depth image and the per-block partial sums) with cudaMalloc on first
// use; this variant cleans the depth on the fly and keeps its only scratch,
// the per-block partial sums, in a fixed file-scope device array.
//
// Limits and sharing:
//  * scratch: kNoAllocMaxBlocks FP64 partials (32 KiB, held by every GPU
//    that loads the library until the process exits), one per 128 pixels:
//    images up to kNoAllocMaxBlocks * 128 = 524,288 pixels (640x480 and
//    848x480 fit).  Larger images are rejected with MRF_ERR_INVALID.
//  * every call shares the array; each call overwrites the partials it uses
//    before reading them, so nothing has to start at zero.  Calls that
//    overlap on the GPU (two streams, or two maps on one device) race on the
//    array and must be serialized by the caller.
//  * the first call in each CUDA context (per device, and again after the
//    caller's process tears the context down and a new one is created, e.g.
//    after cudaDeviceReset) looks the array up with cudaGetSymbolAddress (the
//    host-side name of a __device__ array is not a device address); make
//    that first call before any stream capture.  The looked-up address is
//    kept per device together with the id of the context it belongs to, so an
//    address of a destroyed context is never reused.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/mrfmap_gb300.h"
#include "mrf_geometry.cuh"
#include "mrf_internal.h"
#include "mrf_like_pixel.cuh"

namespace mrf {

namespace {

constexpr int kNoAllocThreads = 128;
constexpr int kNoAllocMaxBlocks = 4096;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxBlocks];

// the array's device address per device, valid for the context whose id is
// stored with it
struct ScratchAddr {
  unsigned long long ctx_id = 0;
  double* ptr = nullptr;
};
std::mutex g_setup_mu;
ScratchAddr g_scratch[kMaxDevices];

// driver entry points for the current context's id, looked up through the
// runtime (the library does not link the driver library itself)
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// id of the calling thread's current context (0 on failure)
unsigned long long current_context_id() {
  if (!g_ctx_get_current || !g_ctx_get_id) {
    void* f0 = nullptr;
    void* f1 = nullptr;
    cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound, q1 = q0;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) !=
            cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1)
      return 0;
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f0);
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f1);
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  if (g_ctx_get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// raw depth in, cleaned on the fly by the same rule as the regular path's
// cleaned copy (clean_depth_value)
__global__ void __launch_bounds__(kNoAllocThreads)
    k_likelihood_noalloc(Geom g, Pose P, const float* __restrict__ depth,
                         const float* __restrict__ belief, float* __restrict__ out_img,
                         double* __restrict__ partials) {
  int pix = blockIdx.x * blockDim.x + threadIdx.x;
  float val = 0.0f;
  if (pix < g.rows * g.cols) {
    const float d = clean_depth_value(depth[pix], pix, g.rows, g.cols);
    if (d > 0.0f) val = likelihood_pixel(g, P, belief, pix, d);
    if (out_img) out_img[pix] = val;
  }
  double t = like_block_sum<kNoAllocThreads>((double)val);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

}  // namespace

}  // namespace mrf

extern "C" MRF_API mrf_status mrf_likelihood_device_noalloc(mrf_map* map, const float* pose,
                                                            const float* depth_dev,
                                                            float* out_img_dev, float* out_sum_dev) {
  using namespace mrf;
  Geom g;
  const float* belief = nullptr;
  cudaStream_t stream = nullptr;
  int device = 0;
  if (!pose || !depth_dev || !out_sum_dev) {
    mrf_internal_set_error("mrf_likelihood_device_noalloc: null argument");
    return MRF_ERR_INVALID;
  }
  mrf_status st = mrf_internal_like_inputs(map, &g, &belief, &stream, &device);
  if (st != MRF_OK) return st;
  int64_t npix = (int64_t)g.rows * g.cols;
  int64_t nblocks = (npix + kNoAllocThreads - 1) / kNoAllocThreads;
  if (nblocks > kNoAllocMaxBlocks) {
    mrf_internal_set_error(
        "mrf_likelihood_device_noalloc: image larger than 524288 pixels (fixed scratch limit)");
    return MRF_ERR_INVALID;
  }
  if (device < 0 || device >= kMaxDevices) {
    mrf_internal_set_error("mrf_likelihood_device_noalloc: device index out of range");
    return MRF_ERR_INVALID;
  }
  double* partials = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    const unsigned long long ctx = current_context_id();
    if (ctx == 0) {
      mrf_internal_set_error("mrf_likelihood_device_noalloc: no current CUDA context");
      return MRF_ERR_CUDA;
    }
    ScratchAddr& a = g_scratch[device];
    if (!a.ptr || a.ctx_id != ctx) {
      void* ptr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_partials);
      if (e != cudaSuccess || !ptr) {
        mrf_internal_set_error(std::string("mrf_likelihood_device_noalloc: cudaGetSymbolAddress: ") +
                               cudaGetErrorString(e));
        return MRF_ERR_CUDA;
      }
      a.ptr = static_cast<double*>(ptr);
      a.ctx_id = ctx;
    }
    partials = a.ptr;
  }
  // a map without active bricks has no belief field; every brick-table probe
  // then misses, so the kernel never reads through this (valid) pointer and
  // the result is the regular entry point's n * ln(LIKE_EPS)
  if (!belief) belief = reinterpret_cast<const float*>(partials);
  Pose P;
  for (int i = 0; i < 16; ++i) P.m[i] = pose[i];
  k_likelihood_noalloc<<<(unsigned)nblocks, kNoAllocThreads, 0, stream>>>(g, P, depth_dev, belief,
                                                                          out_img_dev, partials);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = launch_reduce_partials(partials, (int)nblocks, out_sum_dev, stream);
  if (e != cudaSuccess) {
    mrf_internal_set_error(std::string("mrf_likelihood_device_noalloc: ") + cudaGetErrorString(e));
    return MRF_ERR_CUDA;
  }
  return MRF_OK;
}
