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
//   * the array belongs to this file's module, which CUDA loads (lazily, by
//     default) when its address is first looked up.  hh_init does that lookup
//     for its device, with that device current, so the module and its 64 MiB
//     are loaded when the context is created, never inside a matvec; every GPU
//     that loads it holds the array until the process exits;
//   * the address belongs to the CUDA context that was current in hh_init (the
//     device's primary context for runtime-API callers), and it is kept in the
//     hh_ctx: calls must run with that same context current;
//   * all calls on a device share the one array and it keeps the contents of
//     the last call: calls that overlap on the GPU (several streams or
//     contexts at once) race on it; stage 1 overwrites every scratch element it
//     later reads, so nothing needs clearing between calls, and the vectors of
//     a batched wave run one after another in stream order on the same array.
#include "hh_internal.h"

#define HH_NOALLOC_SCRATCH_BYTES (64ull << 20)

// The host-side name of this array is only a stand-in: host code must pass the
// address returned by cudaGetSymbolAddress to kernels, never the name itself.
static __device__ __align__(256) double2 g_noalloc_scratch[HH_NOALLOC_SCRATCH_BYTES / sizeof(double2)];

namespace hh {

// Called by hh_init with ctx->device current.  It also loads the two FP64
// kernels the entry point launches, so that not even its first call makes
// CUDA load code.  A failed lookup does not fail hh_init: the context works
// without the allocation-free entry point, which then reports the failure.
void noalloc_setup(hh_ctx* ctx) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e == cudaSuccess) e = preload_segment_gemm_fp64();
  if (e != cudaSuccess) {
    cudaGetLastError();  // the failure is recorded here, not left to the next call
    ctx->noalloc_status = std::string("static scratch set-up failed: ") + cudaGetErrorString(e);
    ctx->noalloc_scratch = nullptr;
    return;
  }
  ctx->noalloc_scratch = p;
  ctx->noalloc_status.clear();
}

}  // namespace hh

extern "C" int hh_matvec_noalloc(hh_plan_t* p, const hh_wave_t* in, hh_wave_t* out) {
  if (!p || !in || !out) return HH_ERR_INVALID;
  hh_ctx* ctx = p->ctx;
  if (in->nelem != p->nelem || out->nelem != p->nelem || in == out || in->nbatch != out->nbatch)
    return hh::fail(ctx, HH_ERR_INVALID,
                    "hh_matvec_noalloc: wave layout does not match the plan (or in == out, or the two waves "
                    "hold different numbers of vectors)");
  const unsigned long long need = (unsigned long long)p->scratch_elems * sizeof(double2);
  if (need > HH_NOALLOC_SCRATCH_BYTES)
    return hh::fail(ctx, HH_ERR_INVALID,
                    "hh_matvec_noalloc: the plan needs " + std::to_string(need) +
                        " bytes of stage-1 scratch, the static buffer holds " +
                        std::to_string(HH_NOALLOC_SCRATCH_BYTES) + " bytes; use hh_matvec");
  if (!ctx->noalloc_scratch)
    return hh::fail(ctx, HH_ERR_CUDA, "hh_matvec_noalloc: " + ctx->noalloc_status);
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return hh::cuda_check(ctx, e, "cudaGetDevice");
  if (dev != ctx->device)
    return hh::fail(ctx, HH_ERR_INVALID, "hh_matvec_noalloc: the context's device is not the current device");
  double2* scr = static_cast<double2*>(ctx->noalloc_scratch);
  // one vector at a time: each stage 2 finishes reading the scratch before the
  // next stage 1 (same stream) overwrites it
  for (int b = 0; b < in->nbatch && e == cudaSuccess; ++b) {
    double2* x = in->d + (size_t)b * p->nelem;
    double2* y = out->d + (size_t)b * p->nelem;
    e = cudaMemsetAsync(y, 0, (size_t)p->nelem * sizeof(double2), ctx->stream);
    if (e == cudaSuccess) e = hh::launch_segment_gemm_fp64(p->stage1, x, scr, y, ctx->stream);
    if (e == cudaSuccess) e = hh::launch_segment_gemm_fp64(p->stage2, x, scr, y, ctx->stream);
  }
  return hh::cuda_check(ctx, e, "hh_matvec_noalloc");
}
