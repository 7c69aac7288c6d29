// Batched Hermitian eigensolver for the sectors of a reduced density matrix:
// the per-sector ZHEEV('V','U') of code/get_den.f90:242, eigenvalues
// ascending.
//
// Default path (eig_values, then eig_vectors once the host has chosen the
// kept states): sectors of up to kJacobiOwnMaxN states are solved completely by
// the Jacobi kernel below; larger ones go through the tridiagonal pipeline of
// eig_tri.cu (cluster Householder reduction, bisection for every eigenvalue,
// inverse iteration and back-transformation for the kept eigenvectors only).
// Everything is FP64 and the library's own code.
//
// Comparison path (eig_hermitian_sectors, HH_EIG_CUSOLVER): every eigenpair,
// sectors above kJacobiMaxN through cuSOLVER zheevd.
//
// Sectors of up to kJacobiMaxN states are solved together in ONE launch, one
// CTA per sector: cyclic two-sided Jacobi with the round-robin parallel
// ordering, the sector held in shared memory and its eigenvectors accumulated
// in an L2-resident scratch matrix.  Jacobi costs about 150 n^3 FP64 flops
// against zheevd's 22 n^3, and a GB300 SM retires about two FP64 FMAs per
// clock, so it only pays where zheevd's per-call latency (0.4 ms at n = 8,
// 1.2 ms at n = 32, 3.7 ms at n = 64, measured) dominates: n <= 32.  In the
// comparison path, larger sectors go to cuSOLVER zheevd; most of a small
// zheevd's time is host-side work between its kernels, so the large sectors
// are shared out over kPool host threads, each with its own solver handle and
// stream, concurrently with the Jacobi launch.  A canonical phase (largest-
// modulus component real positive) is applied to every eigenvector.
#include <cusolverDn.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>
#include <vector>

#include "eig_tri.h"
#include "hh_internal.h"

namespace hh {
namespace {

constexpr int kJacobiMaxN = 32;  // 32^2 complex doubles = 16 KiB of shared memory
// The own path hands sectors above 16 states to the tridiagonal pipeline: the
// Jacobi kernel's per-round rotation parameters (a square root and divisions
// in FP64) make a 32-state sector cost ~1.9 ms, against ~0.4 ms for the
// cluster reduction (measured on the 2x16 ladder sweep at m = 256).
constexpr int kJacobiOwnMaxN = 16;
constexpr int kJacobiThreads = 256;
constexpr int kJacobiMaxSweeps = 30;
constexpr int kPool = 8;  // zheevd host threads, each with a stream and a solver handle
constexpr int kBigCluster = 32;  // degenerate clusters this large go through Cholesky QR

struct EigItem {
  long long off;   // n x n sector (column-major, ld n) in the density block
  long long voff;  // n x n eigenvector scratch of a Jacobi sector
  long long woff;  // first eigenvalue of the sector in the global list
  int n;
  int jacobi;      // 1: Jacobi kernel, 0: zheevd
};

// What eig_values leaves for eig_vectors.
struct TriRun {
  bool valid = false;
  double2* A = nullptr;                // the sectors (reflectors of the reduced ones)
  std::vector<long long> offs;
  std::vector<int> dims;
  std::vector<long long> woff;         // first eigenvalue of each sector
  std::vector<int> tri_pos;            // sector -> index in secs, -1 when the Jacobi kernel solved it
  std::vector<tri::Sector> secs;       // reduced sectors, largest first
  std::vector<double> w;               // every eigenvalue (host copy)
  tri::Sector* d_secs = nullptr;
  double* d_d = nullptr;
  double* d_e = nullptr;
  double* d_w = nullptr;
  double2* d_tau = nullptr;
};

struct EigState {
  bool pool_ready = false;             // zheevd streams and handles (comparison path only)
  cusolverDnHandle_t solver[kPool] = {};
  cudaStream_t stream[kPool] = {};
  cudaEvent_t fork = nullptr, join[kPool] = {};
  void* d_buf = nullptr;               // eig_hermitian_sectors
  size_t cap = 0;
  void* d_buf2 = nullptr;              // eig_values (kept until eig_vectors)
  size_t cap2 = 0;
  void* d_buf3 = nullptr;              // eig_vectors
  size_t cap3 = 0;
  bool smem_set = false;
  cudaStream_t side = nullptr;         // the larger sectors' reduction beside the smaller ones'
  cudaEvent_t side_fork = nullptr, side_join = nullptr;
  TriRun run;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Two-sided cyclic Jacobi for one Hermitian sector per CTA.  Each round
// rotates n/2 disjoint index pairs (p, q): the pair's 2x2 block
// [[a, c], [conj(c), b]], c = r e^{i phi}, is diagonalised by
//   G = diag(1, e^{-i phi}) [[cs, sn], [-sn, cs]],
// the real rotation of Golub & Van Loan (symmetric Schur decomposition):
//   tau = (b - a) / (2 r), t = sign(tau) / (|tau| + sqrt(1 + tau^2)),
//   cs = 1 / sqrt(1 + t^2), sn = t cs.
// A <- G^H A G is applied as all row rotations, then all column rotations,
// and V <- V G; the rotated pair's off-diagonal entries are then set to zero.
// A pair is rotated while r > 1e-15 sqrt(|a b|) (relative accuracy for the
// small eigenvalues of a density matrix) and r > 1e-16 of the sector's
// Frobenius norm (below that only rounding noise is left, e.g. in the null
// space of a rank-deficient sector); a sweep without rotations ends the
// iteration.
// status[item] = sweeps used, or -1 when kJacobiMaxSweeps did not converge.
__global__ void __launch_bounds__(kJacobiThreads)
    jacobi_herm_kernel(double2* __restrict__ den, double2* __restrict__ vscr, double* __restrict__ w,
                       const EigItem* __restrict__ items, int* __restrict__ status) {
  const EigItem it = items[blockIdx.x];
  if (!it.jacobi || it.n <= 0) return;
  extern __shared__ double2 sA[];
  __shared__ double s_cs[kJacobiMaxN / 2], s_sn[kJacobiMaxN / 2];
  __shared__ double2 s_ph[kJacobiMaxN / 2];
  __shared__ int s_p[kJacobiMaxN / 2], s_q[kJacobiMaxN / 2], s_rank[kJacobiMaxN];
  __shared__ double s_red[kJacobiThreads / 32];
  __shared__ int s_rot;
  const int n = it.n, np = n + (n & 1), npair = np / 2, tid = threadIdx.x;
  double2* Ag = den + it.off;
  double2* V = vscr + it.voff;
  double fro2 = 0.0;
  for (int i = tid; i < n * n; i += kJacobiThreads) {
    const double2 a = Ag[i];
    sA[i] = a;
    fro2 += a.x * a.x + a.y * a.y;
    V[i] = make_double2((i % n) == (i / n) ? 1.0 : 0.0, 0.0);
  }
  for (int o = 16; o > 0; o >>= 1) fro2 += __shfl_xor_sync(0xffffffffu, fro2, o);
  if ((tid & 31) == 0) s_red[tid >> 5] = fro2;
  __syncthreads();
  fro2 = 0.0;
  for (int i = 0; i < kJacobiThreads / 32; ++i) fro2 += s_red[i];
  const double floor_abs = 1e-16 * sqrt(fro2);
  int sweep = 0;
  for (; sweep < kJacobiMaxSweeps; ++sweep) {
    __syncthreads();  // every thread has read s_rot of the previous sweep
    if (tid == 0) s_rot = 0;
    for (int round = 0; round < np - 1; ++round) {
      __syncthreads();  // previous column update (and s_rot reset) visible
      if (tid < npair) {
        const int a = tid == 0 ? 0 : 1 + (tid - 1 + round) % (np - 1);
        const int b = 1 + (np - 2 - tid + round) % (np - 1);
        const int p = min(a, b), q = max(a, b);
        double cs = 1.0, sn = 0.0;
        double2 ph = make_double2(1.0, 0.0);
        if (q < n) {
          const double app = sA[p + p * n].x, aqq = sA[q + q * n].x;
          const double2 c = sA[p + q * n];  // row p, column q
          const double r = hypot(c.x, c.y);
          if (r > floor_abs && r > 1e-15 * sqrt(fabs(app * aqq))) {
            ph = make_double2(c.x / r, c.y / r);
            const double tau = (aqq - app) / (2.0 * r);
            const double t = copysign(1.0, tau) / (fabs(tau) + sqrt(1.0 + tau * tau));
            cs = 1.0 / sqrt(1.0 + t * t);
            sn = t * cs;
            s_rot = 1;
          }
        }
        s_p[tid] = p;
        s_q[tid] = q < n ? q : -1;
        s_cs[tid] = cs;
        s_sn[tid] = sn;
        s_ph[tid] = ph;
      }
      __syncthreads();
      // rows: A[p][k] <- cs A[p][k] - sn e^{i phi} A[q][k];  A[q][k] <- sn A[p][k] + cs e^{i phi} A[q][k]
      for (int x = tid; x < npair * n; x += kJacobiThreads) {
        const int i = x % npair, k = x / npair;
        const int q = s_q[i];
        if (q < 0 || s_sn[i] == 0.0) continue;
        const int p = s_p[i];
        const double cs = s_cs[i], sn = s_sn[i];
        const double2 ph = s_ph[i];
        const double2 ap = sA[p + k * n], aq = cmul(ph, sA[q + k * n]);
        sA[p + k * n] = make_double2(cs * ap.x - sn * aq.x, cs * ap.y - sn * aq.y);
        sA[q + k * n] = make_double2(sn * ap.x + cs * aq.x, sn * ap.y + cs * aq.y);
      }
      __syncthreads();
      // columns of A and V: X[k][p] <- cs X[k][p] - sn e^{-i phi} X[k][q];
      //                     X[k][q] <- sn X[k][p] + cs e^{-i phi} X[k][q]
      for (int x = tid; x < npair * n; x += kJacobiThreads) {
        const int k = x % n, i = x / n;
        const int q = s_q[i];
        if (q < 0 || s_sn[i] == 0.0) continue;
        const int p = s_p[i];
        const double cs = s_cs[i], sn = s_sn[i];
        const double2 phc = make_double2(s_ph[i].x, -s_ph[i].y);
        double2 ap = sA[k + p * n], aq = cmul(phc, sA[k + q * n]);
        sA[k + p * n] = k == q ? make_double2(0.0, 0.0) : make_double2(cs * ap.x - sn * aq.x, cs * ap.y - sn * aq.y);
        sA[k + q * n] = k == p ? make_double2(0.0, 0.0) : make_double2(sn * ap.x + cs * aq.x, sn * ap.y + cs * aq.y);
        ap = V[k + (long long)p * n];
        aq = cmul(phc, V[k + (long long)q * n]);
        V[k + (long long)p * n] = make_double2(cs * ap.x - sn * aq.x, cs * ap.y - sn * aq.y);
        V[k + (long long)q * n] = make_double2(sn * ap.x + cs * aq.x, sn * ap.y + cs * aq.y);
      }
    }
    __syncthreads();
    const int rotated = s_rot;  // same value in every thread: no write until the next barrier
    if (rotated == 0) break;
  }
  __syncthreads();
  // ascending order (ties by index), eigenvectors into the sector
  for (int j = tid; j < n; j += kJacobiThreads) {
    const double wj = sA[j + j * n].x;
    int r = 0;
    for (int i = 0; i < n; ++i) {
      const double wi = sA[i + i * n].x;
      r += (wi < wj) || (wi == wj && i < j);
    }
    s_rank[j] = r;
    w[it.woff + r] = wj;
  }
  __syncthreads();
  for (int x = tid; x < n * n; x += kJacobiThreads) {
    const int j = x / n, r = x % n;
    Ag[r + (long long)s_rank[j] * n] = V[x];
  }
  if (tid == 0) status[blockIdx.x] = sweep < kJacobiMaxSweeps ? sweep + 1 : -1;
}

// Rotates every eigenvector so that its largest-modulus component (first one
// on ties) is real and positive: one fixed phase convention for the oracle
// and this library, where LAPACK implementations differ.  One block per
// column of every sector.
__global__ void canonical_phase_kernel(double2* den, const EigItem* __restrict__ items) {
  const EigItem it = items[blockIdx.y];
  const int col = blockIdx.x;
  if (col >= it.n) return;
  double2* v = den + it.off + (long long)col * it.n;
  __shared__ double best[256];
  __shared__ int bidx[256];
  double m = -1.0;
  int mi = 0;
  for (int i = threadIdx.x; i < it.n; i += blockDim.x) {
    const double a = v[i].x * v[i].x + v[i].y * v[i].y;
    if (a > m) {
      m = a;
      mi = i;
    }
  }
  best[threadIdx.x] = m;
  bidx[threadIdx.x] = mi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const double o = best[threadIdx.x + s];
      const int oi = bidx[threadIdx.x + s];
      if (o > best[threadIdx.x] || (o == best[threadIdx.x] && oi < bidx[threadIdx.x])) {
        best[threadIdx.x] = o;
        bidx[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  const double2 p = v[bidx[0]];
  const double a = sqrt(p.x * p.x + p.y * p.y);
  if (a == 0.0) return;
  const double2 ph = make_double2(p.x / a, -p.y / a);  // conj(p)/|p|
  for (int i = threadIdx.x; i < it.n; i += blockDim.x) v[i] = cmul(v[i], ph);
}

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

int get_state(hh_ctx* ctx, EigState** out) {
  if (!ctx->eig) ctx->eig = new EigState();  // released by release_step_resources
  *out = (EigState*)ctx->eig;
  return HH_OK;
}

// zheevd host threads, streams and handles, created on the first use of the
// comparison path
int ensure_pool(hh_ctx* ctx, EigState* s) {
  if (s->pool_ready) return HH_OK;
  for (int i = 0; i < kPool; ++i) {
    if (cudaStreamCreateWithFlags(&s->stream[i], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->join[i], cudaEventDisableTiming) != cudaSuccess)
      return fail(ctx, HH_ERR_CUDA, "eigensolver stream pool");
    if (cusolverDnCreate(&s->solver[i]) != CUSOLVER_STATUS_SUCCESS)
      return fail(ctx, HH_ERR_CUDA, "cusolverDnCreate failed");
    cusolverDnSetStream(s->solver[i], s->stream[i]);
  }
  if (cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming) != cudaSuccess)
    return fail(ctx, HH_ERR_CUDA, "eigensolver event");
  s->pool_ready = true;
  return HH_OK;
}

// grow-only device buffer from the context's pool
int reserve(hh_ctx* ctx, void** buf, size_t* cap, size_t need, const char* what) {
  if (*cap >= need) return HH_OK;
  dev_free(ctx, *buf);
  *buf = nullptr;
  *cap = 0;
  cudaError_t e = dev_alloc(ctx, buf, need);
  if (e != cudaSuccess) return cuda_check(ctx, e, what);
  *cap = need;
  return HH_OK;
}

// bump allocation inside one buffer (256-byte aligned pieces)
struct Carve {
  char* base = nullptr;
  size_t off = 0;
  template <class T>
  T* take(size_t n) {
    T* p = reinterpret_cast<T*>(base + off);
    off += (std::max<size_t>(1, n) * sizeof(T) + 255) / 256 * 256;
    return p;
  }
};

}  // namespace

void release_step_resources(hh_ctx* ctx) {
  EigState* s = (EigState*)ctx->eig;
  if (!s) return;
  for (int i = 0; i < kPool; ++i) {
    if (s->solver[i]) cusolverDnDestroy(s->solver[i]);
    if (s->stream[i]) cudaStreamDestroy(s->stream[i]);
    if (s->join[i]) cudaEventDestroy(s->join[i]);
  }
  if (s->fork) cudaEventDestroy(s->fork);
  if (s->side) cudaStreamDestroy(s->side);
  if (s->side_fork) cudaEventDestroy(s->side_fork);
  if (s->side_join) cudaEventDestroy(s->side_join);
  dev_free(ctx, s->d_buf);
  dev_free(ctx, s->d_buf2);
  dev_free(ctx, s->d_buf3);
  delete s;
  ctx->eig = nullptr;
}

int eig_hermitian_sectors(hh_ctx* ctx, double2* A, const std::vector<long long>& offs,
                          const std::vector<int>& dims, double** d_w_out) {
  EigState* S = nullptr;
  int st = get_state(ctx, &S);
  if (st) return st;
  if ((st = ensure_pool(ctx, S))) return st;
  S->run.valid = false;
  const size_t ns = dims.size();
  std::vector<EigItem> items(ns);
  long long nev = 0, vtot = 0;
  int maxn = 0, maxj = 0, lwork = 0;
  std::vector<int> big;
  for (size_t k = 0; k < ns; ++k) {
    const int n = dims[k];
    items[k] = EigItem{offs[k], 0, nev, n, n <= kJacobiMaxN ? 1 : 0};
    nev += n;
    maxn = std::max(maxn, n);
    if (n <= 0) continue;
    if (items[k].jacobi) {
      items[k].voff = vtot;
      vtot += (long long)n * n;
      maxj = std::max(maxj, n);
    } else {
      int lw = 0;
      if (cusolverDnZheevd_bufferSize(S->solver[0], CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n,
                                      reinterpret_cast<cuDoubleComplex*>(A + offs[k]), n,
                                      reinterpret_cast<double*>(A), &lw) != CUSOLVER_STATUS_SUCCESS)
        return fail(ctx, HH_ERR_NUMERIC, "cusolverDnZheevd_bufferSize failed");
      lwork = std::max(lwork, lw);
      big.push_back((int)k);
    }
  }
  const size_t b_items = align256(std::max<size_t>(1, ns) * sizeof(EigItem));
  const size_t b_w = align256(std::max<long long>(1, nev) * sizeof(double));
  const size_t b_v = align256(std::max<long long>(1, vtot) * sizeof(double2));
  const size_t b_status = align256((ns + 1) * sizeof(int));
  const size_t b_work = align256(std::max<size_t>(16, (size_t)lwork * sizeof(cuDoubleComplex)));
  const size_t need = b_items + b_w + b_v + b_status + kPool * b_work;
  if (S->cap < need) {
    dev_free(ctx, S->d_buf);
    S->d_buf = nullptr;
    S->cap = 0;
    cudaError_t e = dev_alloc(ctx, &S->d_buf, need);
    if (e != cudaSuccess) return cuda_check(ctx, e, "allocate eigensolver workspace");
    S->cap = need;
  }
  char* base = (char*)S->d_buf;
  EigItem* d_items = (EigItem*)base;
  double* d_w = (double*)(base + b_items);
  double2* d_v = (double2*)(base + b_items + b_w);
  int* d_status = (int*)(base + b_items + b_w + b_v);
  char* d_work = base + b_items + b_w + b_v + b_status;
  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaSuccess;
  if (ns > 0) e = cudaMemcpyAsync(d_items, items.data(), ns * sizeof(EigItem), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_status, 0, b_status, s);
  if (e != cudaSuccess) return cuda_check(ctx, e, "eigensolver set-up");
  // large sectors: zheevd on the pool streams (after everything queued so
  // far), largest first, handed out to the host threads through a counter
  std::vector<std::thread> workers;
  std::atomic<int> next{0}, solver_failed{0};
  if (!big.empty()) {
    e = cudaEventRecord(S->fork, s);
    for (int i = 0; i < kPool && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(S->stream[i], S->fork, 0);
    if (e != cudaSuccess) return cuda_check(ctx, e, "eigensolver fork");
  }
  // small sectors: one Jacobi launch on the context stream, concurrent with the pool
  if (maxj > 0) {
    const size_t smem = (size_t)maxj * maxj * sizeof(double2);
    if (!S->smem_set) {
      e = cudaFuncSetAttribute(jacobi_herm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               kJacobiMaxN * kJacobiMaxN * (int)sizeof(double2));
      if (e != cudaSuccess) return cuda_check(ctx, e, "Jacobi shared memory");
      S->smem_set = true;
    }
    jacobi_herm_kernel<<<(unsigned)ns, kJacobiThreads, smem, s>>>(A, d_v, d_w, d_items, d_status);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_check(ctx, e, "Jacobi eigensolver launch");
  }
  if (!big.empty()) {
    std::stable_sort(big.begin(), big.end(), [&](int a, int b) { return items[a].n > items[b].n; });
    const int nthreads = std::min<int>(kPool, (int)big.size());
    const int device = ctx->device;
    auto work = [&, device](int slot) {
      cudaSetDevice(device);
      for (int b = next.fetch_add(1); b < (int)big.size(); b = next.fetch_add(1)) {
        const int k = big[b];
        const int n = items[k].n;
        if (cusolverDnZheevd(S->solver[slot], CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n,
                             reinterpret_cast<cuDoubleComplex*>(A + items[k].off), n, d_w + items[k].woff,
                             reinterpret_cast<cuDoubleComplex*>(d_work + slot * b_work), lwork,
                             d_status + k) != CUSOLVER_STATUS_SUCCESS)
          solver_failed = 1;
      }
    };
    for (int i = 1; i < nthreads; ++i) workers.emplace_back(work, i);
    if (nthreads > 0) work(0);  // this thread takes slot 0
  }
  for (auto& w : workers) w.join();
  if (solver_failed) return fail(ctx, HH_ERR_NUMERIC, "cusolverDnZheevd failed");
  if (!big.empty()) {
    for (int i = 0; i < kPool && e == cudaSuccess; ++i) {
      e = cudaEventRecord(S->join[i], S->stream[i]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s, S->join[i], 0);
    }
    if (e != cudaSuccess) return cuda_check(ctx, e, "eigensolver join");
  }
  if (maxn > 0) canonical_phase_kernel<<<dim3(maxn, (unsigned)ns), 256, 0, s>>>(A, d_items);
  e = cudaGetLastError();
  std::vector<int> status(ns + 1, 0);
  if (e == cudaSuccess && ns > 0)
    e = cudaMemcpyAsync(status.data(), d_status, ns * sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_check(ctx, e, "density eigensolve");
  for (size_t k = 0; k < ns; ++k) {
    if (items[k].n <= 0) continue;
    if (items[k].jacobi ? status[k] < 0 : status[k] != 0)
      return fail(ctx, HH_ERR_NUMERIC,
                  std::string(items[k].jacobi ? "Jacobi" : "zheevd") + " eigensolver did not converge in sector " +
                      std::to_string(k));
  }
  *d_w_out = d_w;
  return HH_OK;
}

int eig_values(hh_ctx* ctx, double2* A, const std::vector<long long>& offs, const std::vector<int>& dims,
               bool force_tri, std::vector<double>& w_host) {
  EigState* S = nullptr;
  int st = get_state(ctx, &S);
  if (st) return st;
  TriRun& R = S->run;
  R = TriRun();
  R.A = A;
  R.offs = offs;
  R.dims = dims;
  const size_t ns = dims.size();
  std::vector<EigItem> items(ns);
  R.woff.resize(ns);
  R.tri_pos.assign(ns, -1);
  long long nev = 0, vtot = 0, ttot = 0;
  int maxj = 0, maxn = 0;
  std::vector<int> tri;
  for (size_t k = 0; k < ns; ++k) {
    const int n = dims[k];
    const bool jac = n > 0 && n <= kJacobiOwnMaxN && !force_tri;
    items[k] = EigItem{offs[k], 0, nev, n, jac ? 1 : 0};
    R.woff[k] = nev;
    nev += n;
    if (jac) {
      items[k].voff = vtot;
      vtot += (long long)n * n;
      maxj = std::max(maxj, n);
    } else if (n > 0) {
      tri.push_back((int)k);
      maxn = std::max(maxn, n);
    }
  }
  if (maxn > tri::kMaxN)
    return fail(ctx, HH_ERR_UNSUPPORTED, "density sector of " + std::to_string(maxn) +
                                             " states: the eigensolver takes at most " +
                                             std::to_string(tri::kMaxN));
  // largest sectors first: their clusters start first
  std::stable_sort(tri.begin(), tri.end(), [&](int a, int b) { return dims[a] > dims[b]; });
  for (size_t q = 0; q < tri.size(); ++q) {
    const int k = tri[q];
    R.secs.push_back(tri::Sector{offs[k], ttot, R.woff[k], dims[k], 0});
    R.tri_pos[k] = (int)q;
    ttot += dims[k];
  }
  const int ntri = (int)R.secs.size();
  // workspace
  size_t need = 0;
  {
    Carve c;
    c.take<EigItem>(ns);
    c.take<int>(ns + 1);
    c.take<double>(nev);
    c.take<double2>(vtot);
    c.take<tri::Sector>(ntri);
    c.take<double>(ttot);
    c.take<double>(ttot);
    c.take<double2>(ttot);
    c.take<double2>(ttot);
    c.take<double2>((size_t)ntri * tri::kCluster);
    need = c.off;
  }
  if ((st = reserve(ctx, &S->d_buf2, &S->cap2, need, "allocate eigensolver workspace"))) return st;
  Carve c;
  c.base = (char*)S->d_buf2;
  EigItem* d_items = c.take<EigItem>(ns);
  int* d_status = c.take<int>(ns + 1);
  R.d_w = c.take<double>(nev);
  double2* d_v = c.take<double2>(vtot);
  R.d_secs = c.take<tri::Sector>(ntri);
  R.d_d = c.take<double>(ttot);
  R.d_e = c.take<double>(ttot);
  R.d_tau = c.take<double2>(ttot);
  double2* d_p = c.take<double2>(ttot);
  double2* d_dots = c.take<double2>((size_t)ntri * tri::kCluster);
  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaSuccess;
  if (ns > 0) e = cudaMemcpyAsync(d_items, items.data(), ns * sizeof(EigItem), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && ntri > 0)
    e = cudaMemcpyAsync(R.d_secs, R.secs.data(), ntri * sizeof(tri::Sector), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_status, 0, (ns + 1) * sizeof(int), s);
  if (e != cudaSuccess) return cuda_check(ctx, e, "eigensolver set-up");
  if (maxj > 0) {
    if (!S->smem_set) {
      e = cudaFuncSetAttribute(jacobi_herm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               kJacobiMaxN * kJacobiMaxN * (int)sizeof(double2));
      if (e != cudaSuccess) return cuda_check(ctx, e, "Jacobi shared memory");
      S->smem_set = true;
    }
    jacobi_herm_kernel<<<(unsigned)ns, kJacobiThreads, (size_t)maxj * maxj * sizeof(double2), s>>>(A, d_v, R.d_w,
                                                                                                  d_items, d_status);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_check(ctx, e, "Jacobi eigensolver launch");
  }
  // three groups of sectors, largest first in the list: beyond the cluster
  // kernel's vector slots (the row-split kernel, rare), lower columns in place
  // in global memory, lower columns in the cluster's shared memory.  The
  // larger groups run on a side stream beside the shared-memory group.
  const int max_g = tri::ds_max_n(true), max_s = tri::ds_max_n(false);
  int n_old = 0, n_glob = 0;
  while (n_old < ntri && R.secs[n_old].n > max_g) ++n_old;
  while (n_old + n_glob < ntri && R.secs[n_old + n_glob].n > max_s) ++n_glob;
  const int n_smem = ntri - n_old - n_glob;
  const bool fork = n_smem > 0 && n_old + n_glob > 0;
  cudaStream_t big = s;
  if (fork) {
    if (!S->side) {
      if (cudaStreamCreateWithFlags(&S->side, cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&S->side_fork, cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&S->side_join, cudaEventDisableTiming) != cudaSuccess)
        return fail(ctx, HH_ERR_CUDA, "eigensolver side stream");
    }
    big = S->side;
    e = cudaEventRecord(S->side_fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(big, S->side_fork, 0);
  }
  if (e == cudaSuccess && n_old > 0)
    e = tri::reduce(R.d_secs, n_old, maxn, A, R.d_d, R.d_e, R.d_tau, d_p, d_dots, big);
  if (e == cudaSuccess && n_glob > 0)
    e = tri::reduce_ds(R.d_secs + n_old, n_glob, R.secs[n_old].n, true, A, R.d_d, R.d_e, R.d_tau, big);
  if (e == cudaSuccess && fork) e = cudaEventRecord(S->side_join, big);
  if (e == cudaSuccess && n_smem > 0)
    e = tri::reduce_ds(R.d_secs + n_old + n_glob, n_smem, R.secs[n_old + n_glob].n, false, A, R.d_d, R.d_e,
                       R.d_tau, s);
  if (e == cudaSuccess && fork) e = cudaStreamWaitEvent(s, S->side_join, 0);
  if (e != cudaSuccess) return cuda_check(ctx, e, "tridiagonal reduction");
  e = tri::bisect(R.d_secs, ntri, maxn, R.d_d, R.d_e, R.d_w, s);
  if (e != cudaSuccess) return cuda_check(ctx, e, "bisection");
  w_host.assign((size_t)std::max<long long>(1, nev), 0.0);
  std::vector<int> status(ns + 1, 0);
  if (nev > 0) e = cudaMemcpyAsync(w_host.data(), R.d_w, nev * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && ns > 0)
    e = cudaMemcpyAsync(status.data(), d_status, ns * sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_check(ctx, e, "density eigenvalues");
  for (size_t k = 0; k < ns; ++k)
    if (items[k].jacobi && status[k] < 0)
      return fail(ctx, HH_ERR_NUMERIC, "Jacobi eigensolver did not converge in sector " + std::to_string(k));
  for (long long i = 0; i < nev; ++i)
    if (!std::isfinite(w_host[i])) return fail(ctx, HH_ERR_NUMERIC, "non-finite density eigenvalue");
  R.w.assign(w_host.begin(), w_host.begin() + nev);
  R.valid = true;
  return HH_OK;
}

int eig_vectors(hh_ctx* ctx, const std::vector<int>& ncol, double2* X, const std::vector<long long>& xoff) {
  EigState* S = (EigState*)ctx->eig;
  if (!S || !S->run.valid) return fail(ctx, HH_ERR_INVALID, "eig_vectors without eig_values");
  TriRun& R = S->run;
  const size_t ns = R.dims.size();
  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaSuccess;
  std::vector<tri::InvItem> inv;
  std::vector<tri::CgsBlock> cgs, cgs_low;
  std::vector<int2> clusters;
  // clusters of at least kBigCluster columns (the null space of a
  // rank-deficient sector, kept when kept_max exceeds its rank): the columns
  // are projected off the later columns and orthonormalised by Cholesky QR,
  // twice each, with the FP64 GEMM kernel; scratch W, G, R^{-1} at xoff
  struct BigCl { long long zoff; int n, k, c0, c1; long long woff, goff, roff; };
  std::vector<BigCl> bigs;
  long long xtot = 0;
  std::vector<tri::BtItem> bt;
  std::vector<tri::PhaseItem> ph;
  struct Blk { long long zoff, goff; int n, k; };
  std::vector<Blk> blks;
  long long zt = 0, gt = 0;
  int maxn = 0, maxk = 0, maxcols = 0;
  for (size_t k = 0; k < ns; ++k) {
    const int n = R.dims[k], nc = ncol[k];
    if (n <= 0 || nc <= 0) continue;
    ph.push_back(tri::PhaseItem{xoff[k], n, nc});
    maxcols = std::max(maxcols, nc);
    if (R.tri_pos[k] < 0) {  // Jacobi sector: its top nc eigenvectors, ascending
      e = cudaMemcpyAsync(X + xoff[k], R.A + R.offs[k] + (long long)(n - nc) * n, (size_t)n * nc * sizeof(double2),
                          cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return cuda_check(ctx, e, "kept eigenvectors");
      continue;
    }
    const int q = R.tri_pos[k];
    for (int col = 0; col < nc; ++col) inv.push_back(tri::InvItem{q, n - nc + col, col, nc, zt});
    // clusters of numerically degenerate kept eigenvalues (consecutive gaps
    // below 1e-13 ||T||): Gram-Schmidt within each before Newton-Schulz
    const double* wk = R.w.data() + R.woff[k];
    const double tn = std::max(std::fabs(wk[0]), std::fabs(wk[n - 1]));
    // clusters above the sector's large cluster (or all, without one) go
    // through Gram-Schmidt before the large cluster's Cholesky QR, the ones
    // below it after, so that every column a cluster is projected against
    // is final
    std::vector<int2> upper, lower;
    bool big_here = false;
    for (int j1 = n; j1 > n - nc;) {  // from the top down
      int j0 = j1 - 1;
      while (j0 > n - nc && wk[j0] - wk[j0 - 1] <= 1e-13 * tn) --j0;
      const int c0 = j0 - (n - nc), c1 = j1 - (n - nc), cw = c1 - c0;
      // Cholesky QR (multi-SM GEMMs) instead of Gram-Schmidt for the topmost
      // large cluster of a sector (a lower one would read columns that the
      // same launches rewrite)
      if (cw >= kBigCluster && !big_here) {
        big_here = true;
        BigCl b{zt, n, nc, c0, c1, 0, 0, 0};
        b.woff = xtot;
        xtot += (long long)(nc - c1) * cw;
        b.goff = xtot;
        xtot += (long long)cw * cw;
        b.roff = xtot;
        xtot += (long long)cw * cw;
        bigs.push_back(b);
      } else if (cw > 1) {
        (big_here ? lower : upper).push_back(make_int2(c0, c1));
      }
      j1 = j0;
    }
    if (!upper.empty()) {
      cgs.push_back(tri::CgsBlock{zt, n, nc, (int)clusters.size(), (int)upper.size()});
      clusters.insert(clusters.end(), upper.begin(), upper.end());
    }
    if (!lower.empty()) {
      cgs_low.push_back(tri::CgsBlock{zt, n, nc, (int)clusters.size(), (int)lower.size()});
      clusters.insert(clusters.end(), lower.begin(), lower.end());
    }
    for (int c0 = 0; c0 < nc; c0 += tri::kBtCols)
      bt.push_back(tri::BtItem{q, c0, std::min(tri::kBtCols, nc - c0), nc, zt, xoff[k]});
    blks.push_back(Blk{zt, gt, n, nc});
    zt += (long long)n * nc;
    gt += (long long)nc * nc;
    maxn = std::max(maxn, n);
    maxk = std::max(maxk, nc);
  }
  // Newton-Schulz: three steps Z -> Z1 -> Z -> Z1, each G = Z^T Z then
  // Z' = 1.5 Z - 0.5 Z G (buffer: Z at 0, Z1 at zt, G at 2 zt)
  constexpr int kSteps = 3;
  std::vector<tri::GemmItem> gi[2 * kSteps];
  int ntiles[2 * kSteps] = {};
  for (int stp = 0; stp < kSteps; ++stp) {
    const long long zin = (stp % 2 == 0) ? 0 : zt, zout = (stp % 2 == 0) ? zt : 0, g0 = 2 * zt;
    for (size_t bi = 0; bi < blks.size(); ++bi) {
      const Blk& b = blks[bi];
      tri::GemmItem G{};
      G.a = zin + b.zoff; G.b = zin + b.zoff; G.c = g0 + b.goff; G.c0 = G.c;
      G.M = b.k; G.N = b.k; G.K = b.n;
      G.a_r = 1; G.a_c = b.k; G.b_r = b.k; G.b_c = 1; G.c_r = b.k; G.c_c = 1;
      G.alpha = 1.0; G.beta = 0.0;
      G.tiles_n = (b.k + 63) / 64;
      G.tile0 = ntiles[2 * stp];
      G.gate = (int)bi + 1;
      G.step = stp;
      ntiles[2 * stp] += ((b.k + 63) / 64) * G.tiles_n;
      gi[2 * stp].push_back(G);
      tri::GemmItem H{};
      H.a = zin + b.zoff; H.b = g0 + b.goff; H.c = zout + b.zoff; H.c0 = zin + b.zoff;
      H.M = b.n; H.N = b.k; H.K = b.k;
      H.a_r = b.k; H.a_c = 1; H.b_r = b.k; H.b_c = 1; H.c_r = b.k; H.c_c = 1;
      H.alpha = -0.5; H.beta = 1.5;
      H.tiles_n = (b.k + 63) / 64;
      H.tile0 = ntiles[2 * stp + 1];
      H.gate = (int)bi + 1;
      H.step = stp;
      ntiles[2 * stp + 1] += ((b.n + 63) / 64) * H.tiles_n;
      gi[2 * stp + 1].push_back(H);
    }
  }
  const long long final_z = (kSteps % 2 == 1) ? zt : 0;
  // after the first step's Gram matrices: the steps each block needs (a
  // skipped step copies its Z, so the result stays at final_z)
  std::vector<tri::NsBlock> nsb;
  for (const Blk& b : blks) nsb.push_back(tri::NsBlock{2 * zt + b.goff, b.k, 0});
  // Cholesky QR of the large clusters: item lists of its launches.  Z blocks
  // are row-major (element (i, j) of a block at zoff + i k + j); T, the
  // first pass's result, sits in the Newton-Schulz buffer's second half.
  const long long xbase = 2 * zt + gt, tbase = zt;
  std::vector<tri::GemmItem> projA, projB, gram1, app1, gram2, app2;
  std::vector<tri::CholItem> chol;
  int nt_projA = 0, nt_projB = 0, nt_gram1 = 0, nt_app1 = 0, nt_gram2 = 0, nt_app2 = 0;
  auto item = [](std::vector<tri::GemmItem>& v, int& ntile, long long a, int a_r, int a_c, long long b, int b_r,
                 int b_c, long long c, int c_r, int c_c, long long c0, int M, int N, int K, double alpha,
                 double beta) {
    if (M <= 0 || N <= 0 || K <= 0) return;
    tri::GemmItem g{};
    g.a = a; g.b = b; g.c = c; g.c0 = c0;
    g.M = M; g.N = N; g.K = K;
    g.a_r = a_r; g.a_c = a_c; g.b_r = b_r; g.b_c = b_c; g.c_r = c_r; g.c_c = c_c;
    g.alpha = alpha; g.beta = beta;
    g.tiles_n = (N + 63) / 64;
    g.tile0 = ntile;
    ntile += ((M + 63) / 64) * g.tiles_n;
    v.push_back(g);
  };
  for (const BigCl& b : bigs) {
    const int cw = b.c1 - b.c0, L = b.k - b.c1, k = b.k;
    const long long zc = b.zoff + b.c0, zl = b.zoff + b.c1, w = xbase + b.woff, g = xbase + b.goff,
                    r = xbase + b.roff, t = tbase + b.zoff + (long long)b.n * b.c0;
    // W = Z_L^T Z_c, then Z_c -= Z_L W
    item(projA, nt_projA, zl, 1, k, zc, k, 1, w, cw, 1, w, L, cw, b.n, 1.0, 0.0);
    item(projB, nt_projB, zl, k, 1, w, cw, 1, zc, k, 1, zc, b.n, cw, L, -1.0, 1.0);
    // G = Z_c^T Z_c, T = Z_c R^{-1}; G = T^T T, Z_c = T R^{-1}
    item(gram1, nt_gram1, zc, 1, k, zc, k, 1, g, cw, 1, g, cw, cw, b.n, 1.0, 0.0);
    item(app1, nt_app1, zc, k, 1, r, cw, 1, t, cw, 1, t, b.n, cw, cw, 1.0, 0.0);
    item(gram2, nt_gram2, t, 1, cw, t, cw, 1, g, cw, 1, g, cw, cw, b.n, 1.0, 0.0);
    item(app2, nt_app2, t, cw, 1, r, cw, 1, zc, k, 1, zc, b.n, cw, cw, 1.0, 0.0);
    chol.push_back(tri::CholItem{g, r, cw, 0});
  }
  const int nitems = (int)inv.size();
  size_t need = 0;
  {
    Carve c;
    c.take<tri::InvItem>(inv.size());
    c.take<double>((size_t)5 * maxn * std::max(1, nitems));
    c.take<double>((size_t)(2 * zt + gt + xtot));
    for (auto& v : gi) c.take<tri::GemmItem>(v.size());
    for (auto* v : {&projA, &projB, &gram1, &app1, &gram2, &app2}) c.take<tri::GemmItem>(v->size());
    c.take<tri::CholItem>(chol.size());
    c.take<tri::BtItem>(bt.size());
    c.take<tri::PhaseItem>(ph.size());
    c.take<tri::CgsBlock>(cgs.size());
    c.take<tri::CgsBlock>(cgs_low.size());
    c.take<int2>(clusters.size());
    c.take<tri::NsBlock>(nsb.size());
    c.take<int>(nsb.size());
    need = c.off;
  }
  int st = reserve(ctx, &S->d_buf3, &S->cap3, need, "allocate eigenvector workspace");
  if (st) return st;
  Carve c;
  c.base = (char*)S->d_buf3;
  tri::InvItem* d_inv = c.take<tri::InvItem>(inv.size());
  double* d_lu = c.take<double>((size_t)5 * maxn * std::max(1, nitems));
  double* d_z = c.take<double>((size_t)(2 * zt + gt + xtot));
  tri::GemmItem* d_gi[2 * kSteps];
  for (int q = 0; q < 2 * kSteps; ++q) d_gi[q] = c.take<tri::GemmItem>(gi[q].size());
  std::vector<tri::GemmItem>* qr_lists[6] = {&projA, &projB, &gram1, &app1, &gram2, &app2};
  tri::GemmItem* d_qr[6];
  for (int q = 0; q < 6; ++q) d_qr[q] = c.take<tri::GemmItem>(qr_lists[q]->size());
  tri::CholItem* d_chol = c.take<tri::CholItem>(chol.size());
  tri::BtItem* d_bt = c.take<tri::BtItem>(bt.size());
  tri::PhaseItem* d_ph = c.take<tri::PhaseItem>(ph.size());
  tri::CgsBlock* d_cgs = c.take<tri::CgsBlock>(cgs.size());
  tri::CgsBlock* d_cgs_low = c.take<tri::CgsBlock>(cgs_low.size());
  int2* d_clusters = c.take<int2>(clusters.size());
  tri::NsBlock* d_nsb = c.take<tri::NsBlock>(nsb.size());
  int* d_need = c.take<int>(nsb.size());
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess && bytes > 0) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
  };
  up(d_inv, inv.data(), inv.size() * sizeof(tri::InvItem));
  for (int q = 0; q < 2 * kSteps; ++q) up(d_gi[q], gi[q].data(), gi[q].size() * sizeof(tri::GemmItem));
  for (int q = 0; q < 6; ++q) up(d_qr[q], qr_lists[q]->data(), qr_lists[q]->size() * sizeof(tri::GemmItem));
  up(d_chol, chol.data(), chol.size() * sizeof(tri::CholItem));
  up(d_bt, bt.data(), bt.size() * sizeof(tri::BtItem));
  up(d_ph, ph.data(), ph.size() * sizeof(tri::PhaseItem));
  up(d_cgs, cgs.data(), cgs.size() * sizeof(tri::CgsBlock));
  up(d_cgs_low, cgs_low.data(), cgs_low.size() * sizeof(tri::CgsBlock));
  up(d_clusters, clusters.data(), clusters.size() * sizeof(int2));
  up(d_nsb, nsb.data(), nsb.size() * sizeof(tri::NsBlock));
  if (e != cudaSuccess) return cuda_check(ctx, e, "eigenvector work lists");
  if (nitems > 0) {
    e = tri::inverse_iteration(R.d_secs, d_inv, nitems, maxn, R.d_d, R.d_e, R.d_w, d_z, d_lu, s);
    if (e == cudaSuccess) e = tri::cgs2(d_cgs, (int)cgs.size(), d_clusters, maxk, d_z, s);
    if (!bigs.empty()) {
      for (int pass = 0; pass < 2 && e == cudaSuccess; ++pass) {
        e = tri::gemm(d_qr[0], (int)projA.size(), nt_projA, d_z, s);
        if (e == cudaSuccess) e = tri::gemm(d_qr[1], (int)projB.size(), nt_projB, d_z, s);
      }
      if (e == cudaSuccess) e = tri::gemm(d_qr[2], (int)gram1.size(), nt_gram1, d_z, s);
      if (e == cudaSuccess) e = tri::chol_inv(d_chol, (int)chol.size(), d_z, s);
      if (e == cudaSuccess) e = tri::gemm(d_qr[3], (int)app1.size(), nt_app1, d_z, s);
      if (e == cudaSuccess) e = tri::gemm(d_qr[4], (int)gram2.size(), nt_gram2, d_z, s);
      if (e == cudaSuccess) e = tri::chol_inv(d_chol, (int)chol.size(), d_z, s);
      if (e == cudaSuccess) e = tri::gemm(d_qr[5], (int)app2.size(), nt_app2, d_z, s);
    }
    if (e == cudaSuccess) e = tri::cgs2(d_cgs_low, (int)cgs_low.size(), d_clusters, maxk, d_z, s);
    for (int q = 0; q < 2 * kSteps && e == cudaSuccess; ++q) {
      e = tri::gemm(d_gi[q], (int)gi[q].size(), ntiles[q], d_z, s, q == 0 ? nullptr : d_need);
      if (q == 0 && e == cudaSuccess) e = tri::ns_gate(d_nsb, (int)nsb.size(), d_z, d_need, s);
    }
    if (e == cudaSuccess) e = tri::backtransform(R.d_secs, d_bt, (int)bt.size(), R.A, R.d_tau, d_z + final_z, X, s);
    if (e != cudaSuccess) return cuda_check(ctx, e, "kept eigenvectors (inverse iteration)");
  }
  e = tri::phase_columns(d_ph, (int)ph.size(), maxcols, X, s);
  if (e != cudaSuccess) return cuda_check(ctx, e, "canonical phase");
  R.valid = false;
  return HH_OK;
}

}  // namespace hh
