// Allocation-free variant of the FP64 superblock matvec.
//
// hh_matvec keeps the stage-1 products T = opA(A) X (the first GEMM of every
// two-operator term) in a scratch buffer that hh_plan_create allocates with
// cudaMalloc.  Some callers cannot allocate device memory when they multiply:
// a Fortran code whose own memory pool already holds the GPU's memory, or a
// caller that reserves a fixed device budget up front and must not grow it.
// hh_matvec_noalloc runs the same two kernels with that scratch in a
// file-scope __device__ array instead, so the call itself allocates nothing
// (no cudaMalloc, cudaFree or allocating library routine).
//
// Limits and sharing:
//   * the array holds HH_NOALLOC_SCRATCH_BYTES (64 MiB); a plan whose stage-1
//     products need more is rejected with HH_ERR_INVALID and a message;
//   * every GPU that loads the library holds the array until the process exits;
//   * all calls on a device share the one array and it keeps the contents of
//     the last call: calls that overlap on the GPU (several streams or
//     contexts at once) race on it; stage 1 overwrites every scratch element it
//     later reads, so nothing needs clearing between calls;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) and caches it.
#include <mutex>

#include "hh_internal.h"

#define HH_NOALLOC_SCRATCH_BYTES (64ull << 20)

// The host-side name of this array is only a stand-in: host code must pass the
// address returned by cudaGetSymbolAddress to kernels, never the name itself.
static __device__ __align__(256) double2 g_noalloc_scratch[HH_NOALLOC_SCRATCH_BYTES / sizeof(double2)];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double2* g_scratch_ptr[kMaxDevices] = {nullptr};

int scratch_address(hh_ctx* ctx, double2** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return hh::cuda_check(ctx, e, "cudaGetDevice");
  if (dev != ctx->device)
    return hh::fail(ctx, HH_ERR_INVALID, "hh_matvec_noalloc: the context's device is not the current device");
  if (dev < 0 || dev >= kMaxDevices) return hh::fail(ctx, HH_ERR_INVALID, "device index out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return hh::cuda_check(ctx, e, "cudaGetSymbolAddress(static scratch)");
    g_scratch_ptr[dev] = static_cast<double2*>(p);
  }
  *out = g_scratch_ptr[dev];
  return HH_OK;
}
}  // namespace

extern "C" int hh_matvec_noalloc(hh_plan_t* p, const hh_wave_t* in, hh_wave_t* out) {
  if (!p || !in || !out) return HH_ERR_INVALID;
  hh_ctx* ctx = p->ctx;
  if (in->nelem != p->nelem || out->nelem != p->nelem || in == out)
    return hh::fail(ctx, HH_ERR_INVALID, "hh_matvec_noalloc: wave layout does not match the plan (or in == out)");
  const unsigned long long need = (unsigned long long)p->scratch_elems * sizeof(double2);
  if (need > HH_NOALLOC_SCRATCH_BYTES)
    return hh::fail(ctx, HH_ERR_INVALID,
                    "hh_matvec_noalloc: the plan needs " + std::to_string(need) +
                        " bytes of stage-1 scratch, the static buffer holds " +
                        std::to_string(HH_NOALLOC_SCRATCH_BYTES) + " bytes; use hh_matvec");
  double2* scr = nullptr;
  int st = scratch_address(ctx, &scr);
  if (st != HH_OK) return st;
  cudaError_t e = cudaMemsetAsync(out->d, 0, (size_t)p->nelem * sizeof(double2), ctx->stream);
  if (e == cudaSuccess) e = hh::launch_segment_gemm_fp64(p->stage1, in->d, scr, out->d, ctx->stream);
  if (e == cudaSuccess) e = hh::launch_segment_gemm_fp64(p->stage2, in->d, scr, out->d, ctx->stream);
  return hh::cuda_check(ctx, e, "hh_matvec_noalloc");
}
