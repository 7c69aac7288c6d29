// Learned initial-guess corrector: a per-sector MLP (features -> 64 -> 64 -> 1,
// tanh hidden layers, FP32) with its own forward, backward and Adam kernels,
// and the two wave kernels the corrector needs (per-sector squared norms and
// per-sector rescaling).  There is no counterpart in the reference: it
// corrects the wave_trans_LR/RL guess (code/warm_up.f90:1855-2170) before
// lanczos_memo_new (code/lanczos.f90:4) runs.
//
// Parameter layout (nparams = 64 F + 64 + 64*64 + 64 + 64 + 1 floats):
//   W1[64][F] row-major, b1[64], W2[64][64] row-major (out, in), b2[64],
//   W3[64], b3.
// Loss: sum_s w_s (y_s - t_s)^2 / sum_s w_s.
//
// Reductions over samples go through per-block partial sums added in a fixed
// order, so that a training run gives the same parameters every time.
#include <algorithm>
#include <cmath>
#include <vector>

#include "hh_internal.h"

namespace {

constexpr int H = 64;          // hidden width
constexpr int kMaxFeat = 32;
constexpr int kMaxBlocks = 152;

__host__ __device__ int nparams_of(int F) { return H * F + H + H * H + H + H + 1; }

struct Off {
  int W1, b1, W2, b2, W3, b3, n;
  __host__ __device__ explicit Off(int F) {
    W1 = 0;
    b1 = W1 + H * F;
    W2 = b1 + H;
    b2 = W2 + H * H;
    W3 = b2 + H;
    b3 = W3 + H;
    n = b3 + 1;
  }
};

// One block of 64 threads per chunk of samples; thread j owns hidden unit j.
// Stores h1 and h2 for the backward pass.
__global__ void __launch_bounds__(H) mlp_forward_kernel(const float* __restrict__ P, int F,
                                                        const float* __restrict__ X, int n, int chunk,
                                                        float* __restrict__ h1s, float* __restrict__ h2s,
                                                        float* __restrict__ Y) {
  const Off o(F);
  const int j = threadIdx.x;
  __shared__ float sx[kMaxFeat];
  __shared__ float sh1[H];
  __shared__ float sred[H / 32];
  float w2[H];
#pragma unroll
  for (int k = 0; k < H; ++k) w2[k] = P[o.W2 + j * H + k];
  const float b1 = P[o.b1 + j], b2 = P[o.b2 + j], w3 = P[o.W3 + j], b3 = P[o.b3];
  const int s0 = blockIdx.x * chunk, s1 = min(n, s0 + chunk);
  for (int s = s0; s < s1; ++s) {
    if (j < F) sx[j] = X[(long long)s * F + j];
    __syncthreads();
    float z1 = b1;
    for (int f = 0; f < F; ++f) z1 = fmaf(P[o.W1 + j * F + f], sx[f], z1);
    const float a1 = tanhf(z1);
    sh1[j] = a1;
    __syncthreads();
    float z2 = b2;
#pragma unroll
    for (int k = 0; k < H; ++k) z2 = fmaf(w2[k], sh1[k], z2);
    const float a2 = tanhf(z2);
    h1s[(long long)s * H + j] = a1;
    h2s[(long long)s * H + j] = a2;
    float part = w3 * a2;
    for (int of = 16; of > 0; of >>= 1) part += __shfl_xor_sync(0xffffffffu, part, of);
    if ((j & 31) == 0) sred[j >> 5] = part;
    __syncthreads();
    if (j == 0) Y[s] = b3 + sred[0] + sred[1];
  }
}

// Per-block partial gradients (and weighted squared error) of a chunk of
// samples: part[block][0..nparams) and part[block][nparams] = sum w (y-t)^2,
// part[block][nparams+1] = sum w.
__global__ void __launch_bounds__(H) mlp_backward_kernel(const float* __restrict__ P, int F,
                                                         const float* __restrict__ X, const float* __restrict__ T,
                                                         const float* __restrict__ Wt, int n, int chunk,
                                                         const float* __restrict__ h1s,
                                                         const float* __restrict__ h2s,
                                                         const float* __restrict__ Y, const float* __restrict__ wsum,
                                                         float* __restrict__ part) {
  const Off o(F);
  const int j = threadIdx.x;
  __shared__ float sW2[H][H + 1];
  __shared__ float sdz2[H];
  __shared__ float sx[kMaxFeat];
  __shared__ float sh1[H];
  for (int k = 0; k < H; ++k) sW2[k][j] = P[o.W2 + k * H + j];
  float g2[H];
#pragma unroll
  for (int k = 0; k < H; ++k) g2[k] = 0.f;
  float g1[kMaxFeat];
#pragma unroll
  for (int f = 0; f < kMaxFeat; ++f) g1[f] = 0.f;
  float gb1 = 0.f, gb2 = 0.f, g3 = 0.f, gb3 = 0.f, sse = 0.f, sw = 0.f;
  const float w3 = P[o.W3 + j];
  const float inv = 1.0f / wsum[0];
  const int s0 = blockIdx.x * chunk, s1 = min(n, s0 + chunk);
  __syncthreads();
  for (int s = s0; s < s1; ++s) {
    if (j < F) sx[j] = X[(long long)s * F + j];
    const float a1 = h1s[(long long)s * H + j], a2 = h2s[(long long)s * H + j];
    sh1[j] = a1;
    const float r = Y[s] - T[s], wt = Wt[s];
    const float dy = 2.0f * wt * r * inv;
    if (j == 0) {
      sse = fmaf(wt * r, r, sse);
      sw += wt;
    }
    gb3 += dy;
    g3 = fmaf(dy, a2, g3);
    const float dz2 = dy * w3 * (1.0f - a2 * a2);
    sdz2[j] = dz2;
    gb2 += dz2;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < H; ++k) g2[k] = fmaf(dz2, sh1[k], g2[k]);
    float dh1 = 0.f;
#pragma unroll
    for (int k = 0; k < H; ++k) dh1 = fmaf(sW2[k][j], sdz2[k], dh1);
    const float dz1 = dh1 * (1.0f - a1 * a1);
    gb1 += dz1;
#pragma unroll
    for (int f = 0; f < kMaxFeat; ++f)
      if (f < F) g1[f] = fmaf(dz1, sx[f], g1[f]);
    __syncthreads();
  }
  const int np = o.n;
  float* out = part + (long long)blockIdx.x * (np + 2);
#pragma unroll
  for (int f = 0; f < kMaxFeat; ++f)
    if (f < F) out[o.W1 + j * F + f] = g1[f];
  out[o.b1 + j] = gb1;
#pragma unroll
  for (int k = 0; k < H; ++k) out[o.W2 + j * H + k] = g2[k];
  out[o.b2 + j] = gb2;
  out[o.W3 + j] = g3;
  // b3, the squared error and the weight sum: warp 0 lane 0 holds sse/sw,
  // every thread holds the same gb3
  if (j == 0) {
    out[o.b3] = gb3;
    out[np] = sse * inv;
    out[np + 1] = sw;
  }
}

// grad[i] = sum over blocks in order; loss = sum of the blocks' weighted
// squared errors.  With adam != 0 also takes one Adam step (Kingma & Ba,
// beta1 0.9, beta2 0.999, eps 1e-8); the step counter lives on the device so
// that the epoch can be replayed from a CUDA graph.
__global__ void mlp_reduce_adam_kernel(const float* __restrict__ part, int nblk, int np, float* __restrict__ grad,
                                       float* __restrict__ loss, float* __restrict__ P, float* __restrict__ m,
                                       float* __restrict__ v, int* __restrict__ step, float lr, int adam) {
  const int t = adam ? step[0] + 1 : 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np + 1; i += gridDim.x * blockDim.x) {
    const int col = i < np ? i : np;  // np: the loss column
    float g = 0.f;
    for (int b = 0; b < nblk; ++b) g += part[(long long)b * (np + 2) + col];
    if (i == np) {
      loss[0] = g;
      continue;
    }
    grad[i] = g;
    if (adam) {
      const float mi = 0.9f * m[i] + 0.1f * g;
      const float vi = 0.999f * v[i] + 0.001f * g * g;
      m[i] = mi;
      v[i] = vi;
      const float mh = mi / (1.0f - powf(0.9f, (float)t));
      const float vh = vi / (1.0f - powf(0.999f, (float)t));
      P[i] -= lr * mh / (sqrtf(vh) + 1e-8f);
    }
  }
}

__global__ void mlp_step_kernel(int* step) { step[0] += 1; }

__global__ void sum_weights_kernel(const float* __restrict__ w, int n, float* __restrict__ out) {
  __shared__ float sh[256];
  float s = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += w[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0] > 0.f ? sh[0] : 1.0f;
}

// ---------------------------------------------------------------- waves
struct SecRef {
  long long off, len;
};

__global__ void sector_norms_kernel(const double2* __restrict__ w, const SecRef* __restrict__ secs,
                                    double* __restrict__ out) {
  const SecRef sr = secs[blockIdx.x];
  __shared__ double sh[256];
  double s = 0.0;
  for (long long i = threadIdx.x; i < sr.len; i += blockDim.x) {
    const double2 z = w[sr.off + i];
    s = fma(z.x, z.x, fma(z.y, z.y, s));
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

__global__ void sector_scale_kernel(double2* __restrict__ w, const SecRef* __restrict__ secs,
                                    const double* __restrict__ scale) {
  const SecRef sr = secs[blockIdx.y];
  const double a = scale[blockIdx.y];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < sr.len;
       i += (long long)gridDim.x * blockDim.x) {
    double2 z = w[sr.off + i];
    z.x *= a;
    z.y *= a;
    w[sr.off + i] = z;
  }
}

}  // namespace

struct hh_mlp {
  hh_ctx* ctx = nullptr;
  int F = 0, np = 0;
  float* d_P = nullptr;  // parameters
  float* d_m = nullptr;  // Adam moments
  float* d_v = nullptr;
  int* d_step = nullptr;
  // per-call data (grown on demand)
  int cap = 0;
  float *d_X = nullptr, *d_T = nullptr, *d_W = nullptr, *d_Y = nullptr, *d_h1 = nullptr, *d_h2 = nullptr;
  float *d_part = nullptr, *d_grad = nullptr, *d_loss = nullptr, *d_wsum = nullptr;
};

using namespace hh;

static void mlp_release_data(hh_mlp* m) {
  for (float** p : {&m->d_X, &m->d_T, &m->d_W, &m->d_Y, &m->d_h1, &m->d_h2, &m->d_part}) {
    if (*p) cudaFree(*p);
    *p = nullptr;
  }
  m->cap = 0;
}

static int mlp_reserve(hh_mlp* m, int n) {
  if (n <= m->cap) return HH_OK;
  mlp_release_data(m);
  const size_t F = m->F;
  cudaError_t e = cudaMalloc(&m->d_X, (size_t)n * F * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_T, (size_t)n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_W, (size_t)n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_Y, (size_t)n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_h1, (size_t)n * H * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_h2, (size_t)n * H * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_part, (size_t)kMaxBlocks * (m->np + 2) * sizeof(float));
  if (e != cudaSuccess) {
    mlp_release_data(m);
    return cuda_check(m->ctx, e, "cudaMalloc(MLP data)");
  }
  m->cap = n;
  return HH_OK;
}

static void launch_shape(int n, int* nblk, int* chunk) {
  int b = (n + 15) / 16;
  if (b > kMaxBlocks) b = kMaxBlocks;
  if (b < 1) b = 1;
  *chunk = (n + b - 1) / b;
  *nblk = (n + *chunk - 1) / *chunk;
  if (*nblk < 1) *nblk = 1;
}

// One epoch: forward, backward, reduction (+ Adam).
static cudaError_t mlp_epoch(hh_mlp* m, int n, float lr, int adam, cudaStream_t s) {
  int nblk, chunk;
  launch_shape(n, &nblk, &chunk);
  mlp_forward_kernel<<<nblk, H, 0, s>>>(m->d_P, m->F, m->d_X, n, chunk, m->d_h1, m->d_h2, m->d_Y);
  mlp_backward_kernel<<<nblk, H, 0, s>>>(m->d_P, m->F, m->d_X, m->d_T, m->d_W, n, chunk, m->d_h1, m->d_h2, m->d_Y,
                                         m->d_wsum, m->d_part);
  mlp_reduce_adam_kernel<<<(m->np + 256) / 256, 256, 0, s>>>(m->d_part, nblk, m->np, m->d_grad, m->d_loss, m->d_P,
                                                             m->d_m, m->d_v, m->d_step, lr, adam);
  if (adam) mlp_step_kernel<<<1, 1, 0, s>>>(m->d_step);
  return cudaGetLastError();
}

static int mlp_upload(hh_mlp* m, const float* x, const float* t, const float* w, int n) {
  int st = mlp_reserve(m, n);
  if (st) return st;
  cudaStream_t s = m->ctx->stream;
  cudaError_t e = cudaMemcpyAsync(m->d_X, x, (size_t)n * m->F * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && t) e = cudaMemcpyAsync(m->d_T, t, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && t) {
    if (w) {
      e = cudaMemcpyAsync(m->d_W, w, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, s);
    } else {
      std::vector<float> ones(n, 1.0f);
      e = cudaMemcpyAsync(m->d_W, ones.data(), (size_t)n * sizeof(float), cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // ones goes out of scope
    }
    if (e == cudaSuccess) sum_weights_kernel<<<1, 256, 0, s>>>(m->d_W, n, m->d_wsum);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  return cuda_check(m->ctx, e, "MLP upload");
}

extern "C" {

int hh_mlp_create(hh_ctx_t* ctx, int nfeat, unsigned long long seed, hh_mlp_t** out) {
  if (!ctx || !out || nfeat < 1 || nfeat > kMaxFeat) return HH_ERR_INVALID;
  *out = nullptr;
  hh_mlp* m = new hh_mlp();
  m->ctx = ctx;
  m->F = nfeat;
  m->np = nparams_of(nfeat);
  // Glorot-uniform weights from a seeded splitmix64 stream, zero biases; the
  // last layer starts at zero so that the untrained network predicts no
  // correction.
  std::vector<float> p(m->np, 0.0f);
  const Off o(nfeat);
  unsigned long long z = seed;
  auto uni = [&]() {
    z += 0x9E3779B97F4A7C15ull;
    unsigned long long x = z;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    return (double)(x >> 11) * 0x1.0p-53 * 2.0 - 1.0;
  };
  const double a1 = std::sqrt(6.0 / (nfeat + H)), a2 = std::sqrt(6.0 / (2.0 * H));
  for (int i = 0; i < H * nfeat; ++i) p[o.W1 + i] = (float)(a1 * uni());
  for (int i = 0; i < H * H; ++i) p[o.W2 + i] = (float)(a2 * uni());
  cudaError_t e = cudaMalloc(&m->d_P, m->np * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_m, m->np * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_v, m->np * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_grad, m->np * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_loss, 2 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_wsum, sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_step, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(m->d_P, p.data(), m->np * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->d_m, 0, m->np * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(m->d_v, 0, m->np * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(m->d_step, 0, sizeof(int));
  if (e != cudaSuccess) {
    hh_mlp_free(m);
    return cuda_check(ctx, e, "MLP create");
  }
  *out = m;
  return HH_OK;
}

int hh_mlp_free(hh_mlp_t* m) {
  if (!m) return HH_ERR_INVALID;
  mlp_release_data(m);
  for (float* p : {m->d_P, m->d_m, m->d_v, m->d_grad, m->d_loss, m->d_wsum})
    if (p) cudaFree(p);
  if (m->d_step) cudaFree(m->d_step);
  delete m;
  return HH_OK;
}

int hh_mlp_nparams(const hh_mlp_t* m, int* n) {
  if (!m || !n) return HH_ERR_INVALID;
  *n = m->np;
  return HH_OK;
}

int hh_mlp_get_params(const hh_mlp_t* m, float* p) {
  if (!m || !p) return HH_ERR_INVALID;
  cudaError_t e = cudaMemcpyAsync(p, m->d_P, m->np * sizeof(float), cudaMemcpyDeviceToHost, m->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->ctx->stream);
  return cuda_check(m->ctx, e, "MLP get params");
}

int hh_mlp_set_params(hh_mlp_t* m, const float* p) {
  if (!m || !p) return HH_ERR_INVALID;
  cudaError_t e = cudaMemcpyAsync(m->d_P, p, m->np * sizeof(float), cudaMemcpyHostToDevice, m->ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->d_m, 0, m->np * sizeof(float), m->ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->d_v, 0, m->np * sizeof(float), m->ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->d_step, 0, sizeof(int), m->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->ctx->stream);
  return cuda_check(m->ctx, e, "MLP set params");
}

int hh_mlp_forward(hh_mlp_t* m, const float* x, int n, float* y) {
  if (!m || n < 0 || (n > 0 && (!x || !y))) return HH_ERR_INVALID;
  if (n == 0) return HH_OK;
  int st = mlp_upload(m, x, nullptr, nullptr, n);
  if (st) return st;
  int nblk, chunk;
  launch_shape(n, &nblk, &chunk);
  cudaStream_t s = m->ctx->stream;
  mlp_forward_kernel<<<nblk, H, 0, s>>>(m->d_P, m->F, m->d_X, n, chunk, m->d_h1, m->d_h2, m->d_Y);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(y, m->d_Y, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return cuda_check(m->ctx, e, "MLP forward");
}

int hh_mlp_loss_grad(hh_mlp_t* m, const float* x, const float* t, const float* w, int n, float* loss, float* grad) {
  if (!m || !x || !t || n < 1 || !loss) return HH_ERR_INVALID;
  int st = mlp_upload(m, x, t, w, n);
  if (st) return st;
  cudaStream_t s = m->ctx->stream;
  cudaError_t e = mlp_epoch(m, n, 0.0f, 0, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(loss, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && grad)
    e = cudaMemcpyAsync(grad, m->d_grad, m->np * sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return cuda_check(m->ctx, e, "MLP loss/gradient");
}

int hh_mlp_train(hh_mlp_t* m, const float* x, const float* t, const float* w, int n, int epochs, float lr,
                 float* final_loss) {
  if (!m || !x || !t || n < 1 || epochs < 0) return HH_ERR_INVALID;
  int st = mlp_upload(m, x, t, w, n);
  if (st) return st;
  cudaStream_t s = m->ctx->stream;
  // one epoch captured once, replayed epochs times
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t el = mlp_epoch(m, n, lr, 1, s);
    e = cudaStreamEndCapture(s, &g);
    if (e == cudaSuccess) e = el;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
  for (int i = 0; i < epochs && e == cudaSuccess; ++i) e = cudaGraphLaunch(ge, s);
  if (ge) cudaGraphExecDestroy(ge);
  if (g) cudaGraphDestroy(g);
  if (e == cudaSuccess && final_loss) {
    // loss at the trained parameters
    e = mlp_epoch(m, n, 0.0f, 0, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(final_loss, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return cuda_check(m->ctx, e, "MLP train");
}

static int sector_refs(const hh_wave* w, SecRef** d_refs) {
  std::vector<SecRef> r(w->secs.size());
  for (size_t k = 0; k < w->secs.size(); ++k)
    r[k] = SecRef{w->secs[k].off, (long long)w->secs[k].sdim * w->secs[k].edim};
  cudaError_t e = cudaMalloc(d_refs, std::max<size_t>(1, r.size()) * sizeof(SecRef));
  if (e == cudaSuccess && !r.empty())
    e = cudaMemcpyAsync(*d_refs, r.data(), r.size() * sizeof(SecRef), cudaMemcpyHostToDevice, w->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(w->ctx->stream);
  return cuda_check(w->ctx, e, "sector table");
}

int hh_wave_sector_norms(const hh_wave_t* w, double* norms2) {
  if (!w || !norms2) return HH_ERR_INVALID;
  const int ns = (int)w->secs.size();
  if (ns == 0) return HH_OK;
  SecRef* d_refs = nullptr;
  int st = sector_refs(w, &d_refs);
  if (st) return st;
  double* d_out = nullptr;
  cudaError_t e = cudaMalloc(&d_out, ns * sizeof(double));
  if (e == cudaSuccess) {
    sector_norms_kernel<<<ns, 256, 0, w->ctx->stream>>>(w->d, d_refs, d_out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(norms2, d_out, ns * sizeof(double), cudaMemcpyDeviceToHost, w->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(w->ctx->stream);
  cudaFree(d_refs);
  if (d_out) cudaFree(d_out);
  return cuda_check(w->ctx, e, "wave sector norms");
}

int hh_wave_scale_sectors(hh_wave_t* w, const double* scale) {
  if (!w || !scale) return HH_ERR_INVALID;
  const int ns = (int)w->secs.size();
  if (ns == 0) return HH_OK;
  for (int k = 0; k < ns; ++k)
    if (!std::isfinite(scale[k])) return fail(w->ctx, HH_ERR_INVALID, "non-finite sector scale");
  SecRef* d_refs = nullptr;
  int st = sector_refs(w, &d_refs);
  if (st) return st;
  double* d_s = nullptr;
  cudaError_t e = cudaMalloc(&d_s, ns * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_s, scale, ns * sizeof(double), cudaMemcpyHostToDevice, w->ctx->stream);
  if (e == cudaSuccess) {
    long long maxlen = 0;
    for (const auto& sc : w->secs) maxlen = std::max(maxlen, (long long)sc.sdim * sc.edim);
    const unsigned gx = (unsigned)std::min<long long>(64, std::max<long long>(1, (maxlen + 255) / 256));
    sector_scale_kernel<<<dim3(gx, ns), 256, 0, w->ctx->stream>>>(w->d, d_refs, d_s);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(w->ctx->stream);
  cudaFree(d_refs);
  if (d_s) cudaFree(d_s);
  return cuda_check(w->ctx, e, "wave sector scale");
}

}  // extern "C"
