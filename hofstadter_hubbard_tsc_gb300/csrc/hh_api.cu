// C ABI of the superblock step: context, operators, bases, waves, the
// model_wave plan, the matvec and the Lanczos driver.
#include <cstdio>
#include <cstring>
#include <cmath>
#include <algorithm>
#include <new>

#include "hh_internal.h"

namespace hh {

int fail(hh_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return code;
}

int cuda_check(hh_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return HH_OK;
  return fail(ctx, e == cudaErrorMemoryAllocation ? HH_ERR_NOMEM : HH_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

static int ensure_red(hh_ctx* ctx, size_t ndouble) {
  if (ctx->red_cap >= ndouble) return HH_OK;
  dev_free(ctx, ctx->d_red);
  ctx->d_red = nullptr;
  ctx->red_cap = 0;
  cudaError_t e = dev_alloc(ctx, (void**)&ctx->d_red, ndouble * sizeof(double));
  if (e != cudaSuccess) return cuda_check(ctx, e, "cudaMalloc(reduction)");
  ctx->red_cap = ndouble;
  return HH_OK;
}

static int ensure_hred(hh_ctx* ctx, size_t ndouble) {
  if (ctx->h_red_cap >= ndouble) return HH_OK;
  if (ctx->h_red) cudaFreeHost(ctx->h_red);
  ctx->h_red = nullptr;
  ctx->h_red_cap = 0;
  cudaError_t e = cudaMallocHost(&ctx->h_red, ndouble * sizeof(double));
  if (e != cudaSuccess) return cuda_check(ctx, e, "cudaMallocHost(reduction)");
  ctx->h_red_cap = ndouble;
  return HH_OK;
}

cudaError_t dev_alloc(hh_ctx* ctx, void** p, size_t bytes) {
  *p = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync(p, bytes ? bytes : 256, ctx->pool, ctx->stream);
  if (e == cudaSuccess && ((uintptr_t)*p & 255)) {
    cudaFreeAsync(*p, ctx->stream);
    *p = nullptr;
    e = cudaErrorMisalignedAddress;
  }
  return e;
}

void dev_free(hh_ctx* ctx, void* p) {
  if (p) cudaFreeAsync(p, ctx->stream);
}

}  // namespace hh

// Work list of the FP64 segment GEMM.  A GB300 SM retires about two FP64
// FMAs per clock, so one 64x64 tile advancing 16 k takes about 70 us on one
// SM: a list whose heavy tiles carry most of the k steps leaves most SMs idle.
// Tiles whose cost exceeds the target (total cost / (4 x SMs), at least two
// 16-k steps) are split: long segments into k ranges, then the segment list
// into contiguous parts of similar cost; each part stores a partial sum and
// hh_red items add the parts in slot order, so results do not depend on the
// split's timing.
void hh_gemm_list::upload(hh_ctx* ctx) {
  release();
  actx = ctx;
  const int sms = ctx->sm_count > 0 ? ctx->sm_count : 148;
  auto seg_cost = [](const hh_seg& s) { return s.kind == HH_SEG_COPY ? 1.0 : 1.0 + (s.K + 15) / 16; };
  double total = 0.0;
  for (const auto& t : tiles)
    for (int i = 0; i < t.nseg; ++i) total += seg_cost(segs[t.seg0 + i]);
  const double target = std::max(2.0, total / (4.0 * sms));
  std::vector<hh_seg> wsegs;
  std::vector<hh_tile> work;
  std::vector<hh_red> reds;
  int nparts = 0;
  const int kmax = (int)target * 16;  // longest k range of one piece
  auto shift = [](long long off, int base, long long elems) {
    return off + (base == HH_BASE_ABS ? elems * (long long)sizeof(double2) : elems);
  };
  for (const auto& t : tiles) {
    double cost = 0.0;
    for (int i = 0; i < t.nseg; ++i) cost += seg_cost(segs[t.seg0 + i]);
    if (cost <= 1.5 * target) {
      hh_tile w = t;
      w.seg0 = (int)wsegs.size();
      for (int i = 0; i < t.nseg; ++i) wsegs.push_back(segs[t.seg0 + i]);
      w.part = -1;
      work.push_back(w);
      continue;
    }
    // k-range pieces of this tile's segments
    std::vector<hh_seg> pieces;
    for (int i = 0; i < t.nseg; ++i) {
      const hh_seg& s = segs[t.seg0 + i];
      if (s.kind == HH_SEG_COPY || s.K <= kmax) {
        pieces.push_back(s);
        continue;
      }
      for (int k0 = 0; k0 < s.K; k0 += kmax) {
        hh_seg p = s;
        p.K = std::min(kmax, s.K - k0);
        p.poff = shift(s.poff, s.pbase, s.opP == HH_OP_N ? (long long)k0 * s.ldp : k0);
        p.qoff = shift(s.qoff, s.qbase, s.opQ == HH_OP_N ? (long long)k0 : (long long)k0 * s.ldq);
        pieces.push_back(p);
      }
    }
    // contiguous parts of about `target` cost
    hh_red r{t.ooff, t.obase, t.ldo, t.M, t.N, t.m0, t.n0, t.accumulate, nparts, 0};
    size_t i = 0;
    while (i < pieces.size()) {
      hh_tile w = t;
      w.seg0 = (int)wsegs.size();
      double c = 0.0;
      while (i < pieces.size() && (c == 0.0 || c + seg_cost(pieces[i]) <= target)) {
        c += seg_cost(pieces[i]);
        wsegs.push_back(pieces[i++]);
      }
      w.nseg = (int)wsegs.size() - w.seg0;
      w.part = nparts++;
      work.push_back(w);
      ++r.nparts;
    }
    reds.push_back(r);
  }
  n_work = (int)work.size();
  n_red = (int)reds.size();
  auto up = [&](void** dst, const void* src, size_t bytes) {
    if (bytes && hh::dev_alloc(ctx, dst, bytes) == cudaSuccess)
      cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
  };
  up((void**)&d_segs, wsegs.data(), wsegs.size() * sizeof(hh_seg));
  up((void**)&d_tiles, work.data(), work.size() * sizeof(hh_tile));
  up((void**)&d_reds, reds.data(), reds.size() * sizeof(hh_red));
  if (nparts > 0) hh::dev_alloc(ctx, (void**)&d_part, (size_t)nparts * 64 * 64 * sizeof(double2));
}

void hh_gemm_list::release() {
  if (actx) {
    hh::dev_free(actx, d_segs);
    hh::dev_free(actx, d_tiles);
    hh::dev_free(actx, d_reds);
    hh::dev_free(actx, d_part);
  }
  d_segs = nullptr;
  d_tiles = nullptr;
  d_reds = nullptr;
  d_part = nullptr;
  n_work = n_red = 0;
}

namespace hh {

// Lowest eigenpair of a symmetric tridiagonal matrix (diagonal alpha, off-
// diagonal beta[0..n-2]) by the implicit QL method with Wilkinson shifts
// (Bowdler, Martin, Reinsch and Wilkinson, "The QR and QL algorithms for
// symmetric matrices", Numer. Math. 11 (1968)); z receives the normalised
// eigenvector.  Replaces the DSTEV calls of code/lanczos.f90:99,118,142.
int tridiag_lowest(int n, const double* alpha, const double* beta, double* e0, double* z) {
  if (n <= 0) return HH_ERR_INVALID;
  std::vector<double> d(alpha, alpha + n), e(n, 0.0), Z((size_t)n * n, 0.0);
  for (int i = 0; i + 1 < n; ++i) e[i] = beta[i];
  for (int i = 0; i < n; ++i) Z[(size_t)i * n + i] = 1.0;
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    while (true) {
      int m = l;
      for (; m < n - 1; ++m) {
        double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= 1e-300 + 2.2204460492503131e-16 * dd) break;
      }
      if (m == l) break;
      if (++iter > 200) return HH_ERR_NUMERIC;
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + (g >= 0 ? std::fabs(r) : -std::fabs(r)));
      double s = 1.0, c = 1.0, p = 0.0;
      int i = m - 1;
      bool early = false;
      for (; i >= l; --i) {
        double f = s * e[i], b = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {
          d[i + 1] -= p;
          e[m] = 0.0;
          early = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        for (int k = 0; k < n; ++k) {
          double zf = Z[(size_t)(i + 1) * n + k];
          Z[(size_t)(i + 1) * n + k] = s * Z[(size_t)i * n + k] + c * zf;
          Z[(size_t)i * n + k] = c * Z[(size_t)i * n + k] - s * zf;
        }
      }
      if (early) continue;
      d[l] -= p;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  int imin = 0;
  for (int i = 1; i < n; ++i)
    if (d[i] < d[imin]) imin = i;
  *e0 = d[imin];
  if (z) {
    double nrm = 0.0;
    for (int k = 0; k < n; ++k) nrm += Z[(size_t)imin * n + k] * Z[(size_t)imin * n + k];
    nrm = std::sqrt(nrm);
    for (int k = 0; k < n; ++k) z[k] = Z[(size_t)imin * n + k] / nrm;
  }
  return HH_OK;
}

}  // namespace hh

using namespace hh;

void hh_block::build_index() {
  idx2.clear();
  idx3.clear();
  for (int j = int(subs.size()) - 1; j >= 0; --j) {
    idx2[key2(subs[j].up, subs[j].down)] = j;
    idx3[key3(subs[j].up, subs[j].down, subs[j].dd)] = j;
  }
}

extern "C" {

int hh_version(void) { return 100; }

const char* hh_status_string(int status) {
  switch (status) {
    case HH_OK: return "ok";
    case HH_ERR_INVALID: return "invalid argument";
    case HH_ERR_CUDA: return "CUDA error";
    case HH_ERR_NOMEM: return "out of memory";
    case HH_ERR_QN: return "quantum number mismatch";
    case HH_ERR_TIMEOUT: return "bounded device wait timed out";
    case HH_ERR_NUMERIC: return "numerical failure";
    case HH_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

int hh_init(int device, hh_ctx_t** out) {
  if (!out) return HH_ERR_INVALID;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return HH_ERR_CUDA;
  if (device < 0 || device >= n) return HH_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return HH_ERR_CUDA;
  hh_ctx* c = new (std::nothrow) hh_ctx();
  if (!c) return HH_ERR_NOMEM;
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return HH_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  if (cudaMemPoolCreate(&c->pool, &props) != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    delete c;
    return HH_ERR_CUDA;
  }
  uint64_t keep = UINT64_MAX;  // freed memory stays in the pool for the next step
  cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  noalloc_setup(c);
  *out = c;
  return HH_OK;
}

int hh_finalize(hh_ctx_t* ctx) {
  if (!ctx) return HH_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  dev_free(ctx, ctx->d_red);
  if (ctx->h_red) cudaFreeHost(ctx->h_red);
  release_step_resources(ctx);
  cudaStreamSynchronize(ctx->stream);
  // memory still held by live blocks, waves or plans returns with the pool
  cudaMemPoolDestroy(ctx->pool);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return HH_OK;
}

const char* hh_last_error(const hh_ctx_t* ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

int hh_ctx_stream(hh_ctx_t* ctx, void** stream) {
  if (!ctx || !stream) return HH_ERR_INVALID;
  *stream = (void*)ctx->stream;
  return HH_OK;
}

int hh_ctx_sync(hh_ctx_t* ctx) {
  if (!ctx) return HH_ERR_INVALID;
  return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
}

// ------------------------------------------------------------------ blocks
static int block_alloc(hh_ctx* ctx, int len, int up_dif, int down_dif, int nsub, const int* sub_qn,
                       hh_block** out) {
  if (!ctx || !out || nsub < 0 || (nsub > 0 && !sub_qn)) return HH_ERR_INVALID;
  hh_block* b = new (std::nothrow) hh_block();
  if (!b) return fail(ctx, HH_ERR_NOMEM, "host allocation");
  b->ctx = ctx;
  b->len = len;
  b->up_dif = up_dif;
  b->down_dif = down_dif;
  long long off = 0;
  b->subs.resize(nsub);
  for (int i = 0; i < nsub; ++i) {
    hh_sub_qn& s = b->subs[i];
    s.up = sub_qn[5 * i];
    s.down = sub_qn[5 * i + 1];
    s.dd = sub_qn[5 * i + 2];
    s.row = sub_qn[5 * i + 3];
    s.sdim = sub_qn[5 * i + 4];
    if (s.row < 0 || s.sdim < 0) {
      delete b;
      return fail(ctx, HH_ERR_INVALID, "negative sub-block dimension");
    }
    s.off = off;
    off += (long long)s.row * s.sdim;
  }
  b->nelem = off;
  b->build_index();
  if (off > 0) {
    cudaError_t e = dev_alloc(ctx, (void**)&b->d, off * sizeof(double2));
    if (e != cudaSuccess) {
      delete b;
      return cuda_check(ctx, e, "cudaMalloc(block)");
    }
  }
  *out = b;
  return HH_OK;
}

int hh_block_create(hh_ctx_t* ctx, int len, int up_dif, int down_dif, int nsub, const int* sub_qn,
                    const double* data, hh_block_t** out) {
  int st = block_alloc(ctx, len, up_dif, down_dif, nsub, sub_qn, out);
  if (st != HH_OK) return st;
  hh_block* b = *out;
  if (b->nelem > 0) {
    if (!data) {
      hh_block_free(b);
      *out = nullptr;
      return fail(ctx, HH_ERR_INVALID, "block data pointer is NULL");
    }
    cudaError_t e = cudaMemcpyAsync(b->d, data, b->nelem * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
      hh_block_free(b);
      *out = nullptr;
      return cuda_check(ctx, e, "upload block");
    }
  }
  b->scalar.assign(b->subs.size(), cplx(0, 0));
  for (size_t i = 0; i < b->subs.size(); ++i) {
    const auto& s = b->subs[i];
    if (s.row == 1 && s.sdim == 1) b->scalar[i] = cplx(data[2 * s.off], data[2 * s.off + 1]);
  }
  return HH_OK;
}

int hh_block_zeros(hh_ctx_t* ctx, int len, int up_dif, int down_dif, int nsub, const int* sub_qn,
                   hh_block_t** out) {
  int st = block_alloc(ctx, len, up_dif, down_dif, nsub, sub_qn, out);
  if (st != HH_OK) return st;
  hh_block* b = *out;
  if (b->nelem > 0) {
    cudaError_t e = cudaMemsetAsync(b->d, 0, b->nelem * sizeof(double2), ctx->stream);
    if (e != cudaSuccess) return cuda_check(ctx, e, "memset block");
  }
  b->scalar.assign(b->subs.size(), cplx(0, 0));
  return HH_OK;
}

int hh_block_info(const hh_block_t* b, int* len, int* up_dif, int* down_dif, int* nsub, long long* nelem) {
  if (!b) return HH_ERR_INVALID;
  if (len) *len = b->len;
  if (up_dif) *up_dif = b->up_dif;
  if (down_dif) *down_dif = b->down_dif;
  if (nsub) *nsub = (int)b->subs.size();
  if (nelem) *nelem = b->nelem;
  return HH_OK;
}

int hh_block_qn(const hh_block_t* b, int* q) {
  if (!b || !q) return HH_ERR_INVALID;
  for (size_t i = 0; i < b->subs.size(); ++i) {
    q[5 * i] = b->subs[i].up;
    q[5 * i + 1] = b->subs[i].down;
    q[5 * i + 2] = b->subs[i].dd;
    q[5 * i + 3] = b->subs[i].row;
    q[5 * i + 4] = b->subs[i].sdim;
  }
  return HH_OK;
}

int hh_block_download(const hh_block_t* b, double* data) {
  if (!b || (!data && b->nelem > 0)) return HH_ERR_INVALID;
  if (b->nelem == 0) return HH_OK;
  cudaError_t e = cudaMemcpyAsync(data, b->d, b->nelem * sizeof(double2), cudaMemcpyDeviceToHost, b->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->ctx->stream);
  return cuda_check(b->ctx, e, "download block");
}

int hh_block_free(hh_block_t* b) {
  if (!b) return HH_ERR_INVALID;
  dev_free(b->ctx, b->d);  // ordered after every queued use of the block
  delete b;
  return HH_OK;
}

namespace {
__global__ void caxpy_kernel(double2* y, const double2* x, double cr, double ci, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double2 v = x[i], o = y[i];
    o.x += cr * v.x - ci * v.y;
    o.y += cr * v.y + ci * v.x;
    y[i] = o;
  }
}
}  // namespace

int hh_block_add(hh_block_t* dst, const double* coef, const hh_block_t* src) {
  if (!dst || !src || !coef) return HH_ERR_INVALID;
  hh_ctx* ctx = dst->ctx;
  // forward scan of block_add_block_two (code/space_info.f90:176-214)
  size_t x1 = 0;
  for (size_t i = 0; i < dst->subs.size(); ++i) {
    const hh_sub_qn& ns = dst->subs[i];
    for (size_t x = x1; x < src->subs.size(); ++x) {
      const hh_sub_qn& s = src->subs[x];
      if (s.up == ns.up && s.down == ns.down && s.dd == ns.dd) {
        x1 = x + 1;
        if (s.row != ns.row || s.sdim != ns.sdim)
          return fail(ctx, HH_ERR_QN, "hh_block_add: sub-block shapes differ");
        long long n = (long long)s.row * s.sdim;
        if (n > 0) {
          int g = (int)std::min<long long>((n + 255) / 256, 4096);
          caxpy_kernel<<<g, 256, 0, ctx->stream>>>(dst->d + ns.off, src->d + s.off, coef[0], coef[1], n);
        }
        if (ns.row == 1 && ns.sdim == 1 && !src->scalar.empty() && !dst->scalar.empty())
          dst->scalar[i] += cplx(coef[0], coef[1]) * src->scalar[x];
        break;
      }
    }
  }
  return cuda_check(ctx, cudaGetLastError(), "hh_block_add");
}

// ------------------------------------------------------------------ bases
int hh_basis_create(hh_ctx_t* ctx, int len, int nsec, const int* sec, const int* subs, hh_basis_t** out) {
  if (!ctx || !out || nsec < 0 || (nsec > 0 && (!sec || !subs))) return HH_ERR_INVALID;
  hh_basis* b = new (std::nothrow) hh_basis();
  if (!b) return HH_ERR_NOMEM;
  b->ctx = ctx;
  b->len = len;
  b->secs.resize(nsec);
  int p = 0;
  for (int i = 0; i < nsec; ++i) {
    hh_bsec& s = b->secs[i];
    s.up = sec[3 * i];
    s.down = sec[3 * i + 1];
    int ns = sec[3 * i + 2];
    s.dim = 0;
    s.subs.resize(ns);
    for (int j = 0; j < ns; ++j, ++p) {
      hh_bsub& u = s.subs[j];
      u.spos = subs[6 * p];
      u.sdim = subs[6 * p + 1];
      u.bu = subs[6 * p + 2];
      u.bd = subs[6 * p + 3];
      u.su = subs[6 * p + 4];
      u.sd = subs[6 * p + 5];
      if (u.spos != s.dim || u.sdim < 0) {
        delete b;
        return fail(ctx, HH_ERR_INVALID, "basis sub-block offsets are not contiguous");
      }
      s.dim += u.sdim;
    }
    for (int j = ns - 1; j >= 0; --j) {
      const hh_bsub& u = s.subs[j];
      s.full[key4(u.bu, u.bd, u.su, u.sd)] = j;
      s.bl[key2(u.bu, u.bd)] = j;
    }
  }
  for (int i = nsec - 1; i >= 0; --i) b->idx[key2(b->secs[i].up, b->secs[i].down)] = i;
  *out = b;
  return HH_OK;
}

int hh_basis_free(hh_basis_t* b) {
  if (!b) return HH_ERR_INVALID;
  delete b;
  return HH_OK;
}

// ------------------------------------------------------------------- waves
int hh_wave_create(hh_ctx_t* ctx, int sys_len, int env_len, int nsec, const int* sec, int nbatch, hh_wave_t** out) {
  if (!ctx || !out || nsec < 0 || (nsec > 0 && !sec) || nbatch < 1) return HH_ERR_INVALID;
  hh_wave* w = new (std::nothrow) hh_wave();
  if (!w) return HH_ERR_NOMEM;
  w->ctx = ctx;
  w->sys_len = sys_len;
  w->env_len = env_len;
  w->nbatch = nbatch;
  w->secs.resize(nsec);
  long long off = 0;
  for (int i = 0; i < nsec; ++i) {
    hh_wsec& s = w->secs[i];
    s.su = sec[6 * i];
    s.sd = sec[6 * i + 1];
    s.eu = sec[6 * i + 2];
    s.ed = sec[6 * i + 3];
    s.sdim = sec[6 * i + 4];
    s.edim = sec[6 * i + 5];
    if (s.sdim < 0 || s.edim < 0) {
      delete w;
      return fail(ctx, HH_ERR_INVALID, "negative wave sector dimension");
    }
    s.off = off;
    off += (long long)s.sdim * s.edim;
  }
  for (int i = nsec - 1; i >= 0; --i)
    w->idx[key4(w->secs[i].su, w->secs[i].sd, w->secs[i].eu, w->secs[i].ed)] = i;
  w->nelem = off;
  if (off > 0) {
    cudaError_t e = dev_alloc(ctx, (void**)&w->d, (size_t)off * nbatch * sizeof(double2));
    if (e != cudaSuccess) {
      delete w;
      return cuda_check(ctx, e, "cudaMalloc(wave)");
    }
    cudaMemsetAsync(w->d, 0, (size_t)off * nbatch * sizeof(double2), ctx->stream);
  }
  *out = w;
  return HH_OK;
}

int hh_wave_info(const hh_wave_t* w, long long* nelem, int* nbatch) {
  if (!w) return HH_ERR_INVALID;
  if (nelem) *nelem = w->nelem;
  if (nbatch) *nbatch = w->nbatch;
  return HH_OK;
}

int hh_wave_upload(hh_wave_t* w, const double* data) {
  if (!w || (!data && w->nelem > 0)) return HH_ERR_INVALID;
  size_t bytes = (size_t)w->nelem * w->nbatch * sizeof(double2);
  if (!bytes) return HH_OK;
  cudaError_t e = cudaMemcpyAsync(w->d, data, bytes, cudaMemcpyHostToDevice, w->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(w->ctx->stream);
  return cuda_check(w->ctx, e, "upload wave");
}

int hh_wave_download(const hh_wave_t* w, double* data) {
  if (!w || (!data && w->nelem > 0)) return HH_ERR_INVALID;
  size_t bytes = (size_t)w->nelem * w->nbatch * sizeof(double2);
  if (!bytes) return HH_OK;
  cudaError_t e = cudaMemcpyAsync(data, w->d, bytes, cudaMemcpyDeviceToHost, w->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(w->ctx->stream);
  return cuda_check(w->ctx, e, "download wave");
}

int hh_wave_copy(hh_wave_t* dst, const hh_wave_t* src) {
  if (!dst || !src || dst->nelem * dst->nbatch != src->nelem * src->nbatch) return HH_ERR_INVALID;
  size_t bytes = (size_t)src->nelem * src->nbatch * sizeof(double2);
  if (!bytes) return HH_OK;
  return cuda_check(dst->ctx, cudaMemcpyAsync(dst->d, src->d, bytes, cudaMemcpyDeviceToDevice, dst->ctx->stream),
                    "copy wave");
}

int hh_wave_free(hh_wave_t* w) {
  if (!w) return HH_ERR_INVALID;
  dev_free(w->ctx, w->d);
  delete w;
  return HH_OK;
}

static int dot_dev(hh_ctx* ctx, const double2* a, const double2* b, long long n, double* out) {
  int st = ensure_red(ctx, 4096);
  if (st) return st;
  st = ensure_hred(ctx, 256);
  if (st) return st;
  cudaError_t e = wave_dot(a, b, n, ctx->d_red, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_red, ctx->d_red, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_check(ctx, e, "wave dot");
  *out = ctx->h_red[0];
  return HH_OK;
}

int hh_wave_dot(const hh_wave_t* a, const hh_wave_t* b, double* re) {
  if (!a || !b || !re || a->nelem != b->nelem) return HH_ERR_INVALID;
  return dot_dev(a->ctx, a->d, b->d, a->nelem, re);
}

int hh_wave_norm(const hh_wave_t* a, double* nrm) {
  if (!a || !nrm) return HH_ERR_INVALID;
  double s = 0.0;
  int st = dot_dev(a->ctx, a->d, a->d, a->nelem, &s);
  if (st) return st;
  *nrm = std::sqrt(s);
  return HH_OK;
}

int hh_wave_random(hh_wave_t* w, unsigned long long seed) {
  if (!w) return HH_ERR_INVALID;
  cudaError_t e = wave_fill_random(w->d, w->nelem * w->nbatch, seed, w->ctx->stream);
  if (e != cudaSuccess) return cuda_check(w->ctx, e, "wave random");
  return hh_wave_normalize(w);
}

int hh_wave_normalize(hh_wave_t* a) {
  if (!a) return HH_ERR_INVALID;
  double n = 0.0;
  int st = hh_wave_norm(a, &n);
  if (st) return st;
  if (!(n > 0.0) || !std::isfinite(n)) return fail(a->ctx, HH_ERR_NUMERIC, "wave norm is zero or not finite");
  return cuda_check(a->ctx, wave_scale(a->d, 1.0 / n, a->nelem, a->ctx->stream), "wave scale");
}

// ------------------------------------------------------------------- plans
int hh_plan_create(hh_ctx_t* ctx, const hh_basis_t* sys_bs, const hh_basis_t* env_bs, const hh_wave_t* layout,
                   int nterm, const hh_term_t* terms, hh_plan_t** out) {
  if (!ctx || !sys_bs || !env_bs || !layout || !out || nterm < 0 || (nterm > 0 && !terms)) return HH_ERR_INVALID;
  *out = nullptr;
  hh_plan* p = new (std::nothrow) hh_plan();
  if (!p) return HH_ERR_NOMEM;
  p->ctx = ctx;
  p->layout = layout;
  p->nelem = layout->nelem;
  int st = build_plan(ctx, sys_bs, env_bs, layout, nterm, terms, p);
  if (st != HH_OK) {
    delete p;
    return st;
  }
  if (p->scratch_elems > 0) {
    cudaError_t e = dev_alloc(ctx, (void**)&p->d_scratch, (size_t)p->scratch_elems * layout->nbatch * sizeof(double2));
    if (e != cudaSuccess) {
      delete p;
      return cuda_check(ctx, e, "cudaMalloc(plan scratch)");
    }
  }
  p->stage1.upload(ctx);
  p->stage2.upload(ctx);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    hh_plan_free(p);
    return cuda_check(ctx, e, "upload plan");
  }
  *out = p;
  return HH_OK;
}

int hh_plan_stats(const hh_plan_t* p, double* c) {
  if (!p || !c) return HH_ERR_INVALID;
  c[0] = p->ref_flops;
  c[1] = p->exec_flops;
  c[2] = (double)p->stage2.tiles.size() + (double)p->stage1.tiles.size();
  c[3] = (double)p->stage2.segs.size();
  c[4] = (double)p->stage1.segs.size();
  c[5] = (double)p->scratch_elems * 16.0;
  c[6] = p->op_bytes;
  c[7] = 2.0 * 16.0 * (double)p->nelem;
  c[8] = p->exec_flops_s1;
  c[9] = p->exec_flops_s2;
  c[10] = p->ref_flops_first;
  c[11] = p->ref_flops - p->ref_flops_first;
  c[12] = p->tc.mma_flops1;
  c[13] = p->tc.mma_flops2;
  c[14] = p->tc.bytes_op + p->tc.bytes_x + p->tc.bytes_t;
  c[15] = p->tc.ready ? 1.0 : 0.0;
  // kernels of one matvec: FP64 (two segment GEMMs and their reductions of
  // split tiles) and split precision (graph replay: set_io, wave images,
  // stage 1, zeroing when the stage-2 tiles do not cover the output, stage
  // 2, copy terms)
  c[16] = 2.0 + (p->stage1.n_red > 0) + (p->stage2.n_red > 0);
  c[17] = 2.0 + (p->tc.zero_out ? 1.0 : 0.0) + (p->tc.n_cseg > 0) + (p->tc.n_narrow1 > 0) +
          (p->tc.n_tiles1 > p->tc.n_narrow1) +
          (p->tc.n_narrow2 > 0) + (p->tc.n_tiles2 > p->tc.n_narrow2);
  c[18] = (double)(p->stage1.n_work + p->stage2.n_work);
  c[19] = p->tc.persistent1 ? 1.0 : 0.0;
  c[20] = (double)p->tc.n_tiles2;
  c[21] = (double)p->tc.n_stacked2;
  c[22] = p->tc.mma_cycles2;
  c[23] = (double)p->tc_shape;
  return HH_OK;
}

int hh_plan_free(hh_plan_t* p) {
  if (!p) return HH_ERR_INVALID;
  cudaStreamSynchronize(p->ctx->stream);
  p->stage1.release();
  p->stage2.release();
  release_tc_plan(p);
  dev_free(p->ctx, p->d_scratch);
  dev_free(p->ctx, p->d_krylov);
  dev_free(p->ctx, p->d_host_in);
  dev_free(p->ctx, p->d_host_out);
  delete p;
  return HH_OK;
}

static int matvec_dev(hh_plan* p, const double2* in, double2* out, int precision, bool check = true) {
  hh_ctx* ctx = p->ctx;
  const int arith = seg_arith_of(precision);
  if (arith < 0 && !split_of(precision)) return fail(ctx, HH_ERR_INVALID, "unknown precision");
  if (arith < 0) return matvec_tc(p, in, out, nullptr, check, split_of(precision));
  cudaError_t e = cudaMemsetAsync(out, 0, (size_t)p->nelem * sizeof(double2), ctx->stream);
  if (e == cudaSuccess)
    e = launch_segment_gemm_fp64(p->stage1, const_cast<double2*>(in), p->d_scratch, out, ctx->stream, arith);
  if (e == cudaSuccess)
    e = launch_segment_gemm_fp64(p->stage2, const_cast<double2*>(in), p->d_scratch, out, ctx->stream, arith);
  return cuda_check(ctx, e, "matvec");
}

// The vectors of a batch (waves of one layout holding nbatch vectors): in
// split precision one graph replay multiplies all of them (every stage one
// launch over the whole batch, matvec_tc_batch); in FP64 they are multiplied
// one after another on the same plan.  in and out must hold the same number
// of vectors.
static int matvec_batch(hh_plan* p, const hh_wave* in, hh_wave* out, int precision, bool check) {
  if (in->nelem != p->nelem || out->nelem != p->nelem || in == out || in->nbatch != out->nbatch)
    return fail(p->ctx, HH_ERR_INVALID, "matvec: wave layout does not match the plan (or in == out)");
  if (split_of(precision) && in->nbatch > 1)
    return matvec_tc_batch(p, in->d, out->d, in->nbatch, check, split_of(precision));
  for (int b = 0; b < in->nbatch; ++b) {
    const bool last = b + 1 == in->nbatch;
    const int st = matvec_dev(p, in->d + (size_t)b * p->nelem, out->d + (size_t)b * p->nelem, precision,
                              check && last);
    if (st != HH_OK) return st;
  }
  return HH_OK;
}

int hh_matvec(hh_plan_t* p, const hh_wave_t* in, hh_wave_t* out, int precision) {
  if (!p || !in || !out) return HH_ERR_INVALID;
  return matvec_batch(p, in, out, precision, true);
}

int hh_matvec_host(hh_plan_t* p, const double* in, double* out, int precision) {
  if (!p || !in || !out) return HH_ERR_INVALID;
  hh_ctx* ctx = p->ctx;
  size_t bytes = (size_t)p->nelem * sizeof(double2);
  cudaError_t e = cudaSuccess;
  if (!p->d_host_in) e = dev_alloc(ctx, (void**)&p->d_host_in, bytes);
  if (e == cudaSuccess && !p->d_host_out) e = dev_alloc(ctx, (void**)&p->d_host_out, bytes);
  if (e != cudaSuccess) return cuda_check(ctx, e, "cudaMalloc(matvec_host)");
  int st = ensure_hred(ctx, 16);
  if (st != HH_OK) return st;
  // one synchronisation: the tensor-core error flag comes back with the output
  e = cudaMemcpyAsync(p->d_host_in, in, bytes, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) st = matvec_dev(p, p->d_host_in, p->d_host_out, precision, false);
  int* h_err = reinterpret_cast<int*>(ctx->h_red + 8);
  *h_err = 0;
  const bool tc = split_of(precision) && p->tc.ready;
  if (e == cudaSuccess && st == HH_OK)
    e = cudaMemcpyAsync(out, p->d_host_out, bytes, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess && st == HH_OK && tc)
    e = cudaMemcpyAsync(h_err, p->tc.d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (st != HH_OK) return st;
  if (e != cudaSuccess) return cuda_check(ctx, e, "matvec_host");
  if (*h_err) {
    cudaMemsetAsync(p->tc.d_err, 0, sizeof(int), ctx->stream);
    return fail(ctx, HH_ERR_TIMEOUT, "tensor-core matvec: a bounded mbarrier wait ran out (code " +
                                         std::to_string(*h_err) + ")");
  }
  return HH_OK;
}

int hh_matvec_timed(hh_plan_t* p, const hh_wave_t* in, hh_wave_t* out, int precision, float* ms) {
  if (!p || !in || !out || !ms || in == out || in->nelem != p->nelem || out->nelem != p->nelem)
    return HH_ERR_INVALID;
  hh_ctx* ctx = p->ctx;
  const int arith = seg_arith_of(precision);
  if (arith < 0) {
    if (!split_of(precision)) return fail(ctx, HH_ERR_INVALID, "unknown precision");
    return matvec_tc(p, in->d, out->d, ms, true, split_of(precision));
  }
  cudaEvent_t ev[3];
  for (int i = 0; i < 3; ++i) cudaEventCreate(&ev[i]);
  cudaError_t e = cudaMemsetAsync(out->d, 0, (size_t)p->nelem * sizeof(double2), ctx->stream);
  cudaEventRecord(ev[0], ctx->stream);
  if (e == cudaSuccess) e = launch_segment_gemm_fp64(p->stage1, in->d, p->d_scratch, out->d, ctx->stream, arith);
  cudaEventRecord(ev[1], ctx->stream);
  if (e == cudaSuccess) e = launch_segment_gemm_fp64(p->stage2, in->d, p->d_scratch, out->d, ctx->stream, arith);
  cudaEventRecord(ev[2], ctx->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(ev[2]);
  if (e == cudaSuccess) {
    cudaEventElapsedTime(&ms[0], ev[0], ev[2]);
    cudaEventElapsedTime(&ms[1], ev[0], ev[1]);
    cudaEventElapsedTime(&ms[2], ev[1], ev[2]);
    ms[3] = 0.f;
  }
  for (int i = 0; i < 3; ++i) cudaEventDestroy(ev[i]);
  return cuda_check(ctx, e, "matvec_timed");
}

int hh_matvec_async(hh_plan_t* p, const hh_wave_t* in, hh_wave_t* out, int precision) {
  if (!p || !in || !out) return HH_ERR_INVALID;
  return matvec_batch(p, in, out, precision, false);
}

int hh_plan_check(hh_plan_t* p) {
  if (!p) return HH_ERR_INVALID;
  hh_ctx* ctx = p->ctx;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_check(ctx, e, "plan check");
  for (hh_tc_plan* t : {&p->tc, &p->tcb}) {  // the single-vector and the batch schedules
    if (!t->ready) continue;
    int herr = 0;
    e = cudaMemcpy(&herr, t->d_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_check(ctx, e, "plan check");
    if (herr) {
      cudaMemset(t->d_err, 0, sizeof(int));
      return fail(ctx, HH_ERR_TIMEOUT, "tensor-core matvec: a bounded mbarrier wait ran out (code " +
                                           std::to_string(herr) + ")");
    }
  }
  return HH_OK;
}

int hh_plan_tune(hh_plan_t* p, int precision, int reps, double* ms, int* choice) {
  if (!p || reps < 1) return HH_ERR_INVALID;
  if (seg_arith_of(precision) >= 0) {  // one launch shape: nothing to choose
    if (choice) *choice = 0;
    return HH_OK;
  }
  if (!split_of(precision)) return fail(p->ctx, HH_ERR_INVALID, "unknown precision");
  int st = tune_tc_plan(p, reps, ms, split_of(precision));
  if (st == HH_OK && choice) *choice = 4 * p->tc_shape + 2 * (int)p->tc.persistent1 + (int)p->tc.persistent2;
  return st;
}

int hh_plan_set_tiles(hh_plan_t* p, int shape) {
  if (!p || shape < 0 || shape >= HH_TILE_SHAPES) return HH_ERR_INVALID;
  if (shape == p->tc_shape) return HH_OK;
  cudaError_t e = cudaStreamSynchronize(p->ctx->stream);  // no replay of the old schedule in flight
  if (e != cudaSuccess) return cuda_check(p->ctx, e, "hh_plan_set_tiles");
  release_tc_plan(p);
  p->tc_shape = shape;
  return HH_OK;
}

int hh_host_alloc(long long bytes, void** ptr) {
  if (!ptr || bytes < 0) return HH_ERR_INVALID;
  *ptr = nullptr;
  if (bytes == 0) return HH_OK;
  return cudaMallocHost(ptr, (size_t)bytes) == cudaSuccess ? HH_OK : HH_ERR_NOMEM;
}

int hh_host_free(void* ptr) {
  if (!ptr) return HH_OK;
  return cudaFreeHost(ptr) == cudaSuccess ? HH_OK : HH_ERR_CUDA;
}

// ----------------------------------------------------------------- Lanczos
static int lanczos_core(hh_plan* p, hh_wave* psi, double lanzero, int maxit, int first_precision, int precision,
                        double* energy, int* iterations);

int hh_lanczos(hh_plan_t* p, hh_wave_t* psi, double lanzero, int maxit, int precision, double* energy,
               int* iterations) {
  if (!p || !psi || !energy || psi->nelem != p->nelem || maxit < 1) return HH_ERR_INVALID;
  if (seg_arith_of(precision) >= 0)
    return lanczos_core(p, psi, lanzero, maxit, precision, precision, energy, iterations);
  if (!split_of(precision)) return fail(p->ctx, HH_ERR_INVALID, "unknown precision");
  // Split precision, two passes.  (1) Lanczos on the tensor-core matvec down
  // to its noise floor: Ritz value change <= max(lanzero, 1e-8).  (2) Lanczos
  // restarted from that vector psi_m whose first product H psi_m is
  // FP64-class (double-float by default, ctx->restart_precision) and whose
  // later ones are split precision.  The accurate residual H psi_m - a0 psi_m
  // starts the correction space and the Gram-Schmidt step keeps every later
  // vector orthogonal to psi_m and to it, so the tridiagonal's first row is
  // accurate to the product's ~1e-14; the split-precision entries enter the
  // Ritz value weighted by the squares of the correction coefficients (about
  // the vector error of psi_m, 1e-4), which takes the energy to FP64
  // accuracy at the cost of one FP64-class matvec.
  double e_mixed = 0.0;
  int it1 = 0, it2 = 0;
  int st = lanczos_core(p, psi, std::max(lanzero, 1e-8), maxit, precision, precision, &e_mixed, &it1);
  if (st) return st;
  st = lanczos_core(p, psi, lanzero, maxit, p->ctx->restart_precision, precision, energy, &it2);
  if (st) return st;
  if (iterations) *iterations = it1 + it2;
  return HH_OK;
}

// alpha, beta^2, the Krylov norms <v_j|v_j> and the Gram-Schmidt
// coefficients stay on the device; one synchronisation per iteration brings
// alpha_j and beta_j^2 (and the tensor-core error flag) to the host for the
// breakdown test, the tridiagonal solve and the convergence test.
static int lanczos_core(hh_plan* p, hh_wave* psi, double lanzero, int maxit, int first_precision, int precision,
                        double* energy, int* iterations) {
  hh_ctx* ctx = p->ctx;
  if (maxit > 100) maxit = 100;  // loop_in (code/lanczos.f90:14)
  const long long n = p->nelem;
  const int slots = maxit + 1;
  // The split first pass (its products split precision from the start) keeps
  // its Krylov basis in FP32, half the bytes of the Gram-Schmidt passes: its
  // products carry ~1e-5 relative error and it stops at a 1e-8 Ritz change,
  // and the restart pass (FP64 basis) fixes the energy.  The three newest
  // vectors stay FP64 (the recurrence and the products use them), at the
  // start of the same buffer.
  const bool f32 = split_of(first_precision) && ctx->krylov_f32;
  const int cap = std::max(slots, 3 + (slots + 1) / 2);  // in FP64 vectors
  if (p->krylov_cap < cap) {
    dev_free(ctx, p->d_krylov);
    p->d_krylov = nullptr;
    p->krylov_cap = 0;
    cudaError_t e = dev_alloc(ctx, (void**)&p->d_krylov, (size_t)cap * n * sizeof(double2));
    if (e != cudaSuccess) return cuda_check(ctx, e, "cudaMalloc(Krylov basis)");
    p->krylov_cap = cap;
  }
  // d_red: [0, KRY) Gram-Schmidt coefficients and partials, then the scalars
  constexpr size_t KRY = 128 + 600 * 128;
  int st = ensure_red(ctx, KRY + 4 * 128 + 8 + 1024);
  if (st) return st;
  st = ensure_hred(ctx, 256);
  if (st) return st;
  double* d_alpha = ctx->d_red + KRY;
  double* d_beta2 = d_alpha + 128;
  double* d_beta = d_beta2 + 128;
  double* d_vv = d_beta + 128;
  double* d_w2 = d_vv + 128;
  double* d_part = d_w2 + 8;
  const bool uses_tc = split_of(precision) || split_of(first_precision);
  double2* V = p->d_krylov;
  cudaStream_t s = ctx->stream;
  auto slot = [&](int j) { return V + (size_t)j * n; };
  auto dot_into = [&](const double2* a, const double2* b, double* r) { return wave_dot_into(a, b, n, r, d_part, s); };
  // fetch a few device scalars (and the tensor-core error flag) with one sync
  int* h_err = reinterpret_cast<int*>(ctx->h_red + 8);
  auto fetch = [&](std::initializer_list<const double*> src) -> int {
    int i = 0;
    cudaError_t e = cudaSuccess;
    for (const double* q : src) {
      if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_red + i, q, sizeof(double), cudaMemcpyDeviceToHost, s);
      ++i;
    }
    *h_err = 0;
    int* d_tcerr = uses_tc && p->tc.ready ? p->tc.d_err : nullptr;  // the plan is built by the first product
    if (e == cudaSuccess && d_tcerr) e = cudaMemcpyAsync(h_err, d_tcerr, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_check(ctx, e, "Lanczos");
    if (*h_err) {
      cudaMemsetAsync(d_tcerr, 0, sizeof(int), s);
      return fail(ctx, HH_ERR_TIMEOUT, "tensor-core matvec: a bounded mbarrier wait ran out (code " +
                                           std::to_string(*h_err) + ")");
    }
    return HH_OK;
  };
  std::vector<double> alpha, beta;
  // cur = v_{last-1}, prev = v_{last-2}, w = the product, then the next
  // vector: basis slots (FP64 basis), or three rotating FP64 vectors beside
  // the FP32 basis V32
  float2* V32 = reinterpret_cast<float2*>(V + 3 * n);
  double2* cur = f32 ? V : slot(0);
  double2* prev = f32 ? V + 2 * n : nullptr;
  double2* w = f32 ? V + n : slot(1);
  // <v_j|v_j> of a new basis vector (and its FP32 copy)
  auto store = [&](const double2* v, int j) {
    return f32 ? krylov_store_f32(v, V32 + (size_t)j * n, n, d_vv + j, d_part, s) : dot_into(v, v, d_vv + j);
  };
  cudaError_t e = cudaMemcpyAsync(cur, psi->d, n * sizeof(double2), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = dot_into(cur, cur, d_w2);
  if (e != cudaSuccess) return cuda_check(ctx, e, "Lanczos start");
  if ((st = fetch({d_w2}))) return st;
  if (!(ctx->h_red[0] > 0.0)) return fail(ctx, HH_ERR_NUMERIC, "Lanczos start vector is zero");
  e = wave_scale_rsqrt_dev(cur, d_w2, nullptr, n, s);
  if (e == cudaSuccess) e = store(cur, 0);
  if (e != cudaSuccess) return cuda_check(ctx, e, "Lanczos start");
  int last = 1;
  if ((st = matvec_dev(p, cur, w, first_precision, false))) return st;
  if ((e = dot_into(cur, w, d_alpha + 0)) != cudaSuccess) return cuda_check(ctx, e, "Lanczos alpha");
  if ((st = fetch({d_alpha}))) return st;
  alpha.push_back(ctx->h_red[0]);
  double ritz = alpha[0];
  while (last < maxit) {
    // three-term recurrence (code/lanczos.f90:65-75)
    e = wave_axpy_dev(w, cur, d_alpha + (last - 1), -1.0, n, s);
    if (e == cudaSuccess && last >= 2) e = wave_axpy_dev(w, prev, d_beta + (last - 2), -1.0, n, s);
    // beta = ||w||, w /= beta
    if (e == cudaSuccess) e = dot_into(w, w, d_beta2 + (last - 1));
    if (e == cudaSuccess) e = wave_scale_rsqrt_dev(w, d_beta2 + (last - 1), d_beta + (last - 1), n, s);
    // Gram-Schmidt against all previous vectors, real inner product
    // (Gram_Schmidt_process, code/space_info.f90:1176-1214)
    if (e == cudaSuccess) e = f32 ? krylov_dots(V32, last, n, w, n, ctx->d_red, s) : krylov_dots(V, last, n, w, n, ctx->d_red, s);
    if (e == cudaSuccess) e = divide_dev(ctx->d_red, d_vv, last, s);
    if (e == cudaSuccess)
      e = f32 ? krylov_update(V32, last, n, w, n, ctx->d_red, s) : krylov_update(V, last, n, w, n, ctx->d_red, s);
    if (e == cudaSuccess) e = dot_into(w, w, d_w2);
    if (e == cudaSuccess) e = wave_scale_rsqrt_dev(w, d_w2, nullptr, n, s);
    if (e == cudaSuccess) e = store(w, last);
    if (e != cudaSuccess) return cuda_check(ctx, e, "Lanczos recurrence");
    ++last;
    if (f32) {
      double2* t = prev;
      prev = cur;
      cur = w;
      w = t;
    } else {
      prev = cur;
      cur = w;
      w = slot(last);
    }
    if ((st = matvec_dev(p, cur, w, precision, false))) return st;
    if ((e = dot_into(cur, w, d_alpha + (last - 1))) != cudaSuccess)
      return cuda_check(ctx, e, "Lanczos alpha");
    if ((st = fetch({d_beta2 + (last - 2), d_alpha + (last - 1)}))) return st;
    const double b = std::sqrt(ctx->h_red[0]);
    beta.push_back(b);
    if (!std::isfinite(b)) return fail(ctx, HH_ERR_NUMERIC, "Lanczos: non-finite beta");
    if (std::fabs(b) <= lanzero) {  // breakdown (code/lanczos.f90:78): the new vector is not kept
      --last;
      break;
    }
    alpha.push_back(ctx->h_red[1]);
    double d0 = 0.0;
    if ((st = tridiag_lowest(last, alpha.data(), beta.data(), &d0, nullptr)))
      return fail(ctx, st, "tridiagonal eigensolver did not converge");
    if (std::fabs(d0 - ritz) <= lanzero || last == maxit) {  // code/lanczos.f90:102
      ritz = d0;
      break;
    }
    ritz = d0;
  }
  std::vector<double> z(last);
  double e0 = 0.0;
  if ((st = tridiag_lowest(last, alpha.data(), beta.data(), &e0, z.data())))
    return fail(ctx, st, "tridiagonal eigensolver did not converge");
  e = cudaMemcpyAsync(ctx->d_red, z.data(), last * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = f32 ? krylov_combine(V32, last, n, psi->d, n, ctx->d_red, s) : krylov_combine(V, last, n, psi->d, n, ctx->d_red, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_check(ctx, e, "Lanczos final combination");
  if ((st = hh_wave_normalize(psi))) return st;
  *energy = e0;
  if (iterations) *iterations = last;
  return HH_OK;
}

}  // extern "C"
