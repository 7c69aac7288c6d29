// FP64 batched Hermitian eigensolver for the density-matrix sectors of more
// than 32 states: the per-sector ZHEEV('V','U') of code/get_den.f90:242,
// restated as the reduction / bisection / inverse-iteration pipeline of
// LAPACK's expert driver (zhetrd, dstebz, dstein, zunmtr), every step written
// for many SMs at once:
//
//   1. reduce: Householder reduction of each sector to a real symmetric
//      tridiagonal T = Q^H A Q (the unblocked lower-triangle algorithm of
//      zhetd2).  One thread-block cluster per sector: sectors of up to about
//      600 states are held in the cluster's distributed shared memory
//      (reduce_ds_kernel, 16 CTAs where the device allows, else 8); larger
//      ones stay in global memory (reduce_kernel, L2-resident, rows of the
//      trailing block split over the CTAs);
//   2. bisect: every eigenvalue of every T by bisection on Sturm counts, one
//      thread per eigenvalue: first in FP32 on a scaled copy of T, which
//      brackets the eigenvalue to a few FP32 eps ||T|| at a sixty-fourth of
//      the FP64 cost on GB300, then (bracket confirmed by FP64 counts) in
//      FP64 to an absolute accuracy of a few eps ||T||;
//   (the host sorts all eigenvalues and selects the kept states)
//   3. inverse_iteration: each kept eigenvector of T from three steps of
//      inverse iteration (Gaussian elimination with partial pivoting of
//      T - lambda I), one thread per vector; then Newton-Schulz steps
//      Z <- Z (3 I - Z^T Z) / 2 (gemm) make the kept vectors of a sector
//      orthonormal, after classical Gram-Schmidt twice (cgs2) where kept
//      eigenvalues are numerically degenerate;
//   4. backtransform: X = Q Z, one reflector at a time, one warp per column.
//
// A GB300 SM retires about two FP64 FMAs per clock, so the O(n^3) steps
// (reduction, back-transformation, orthonormalisation) are spread over many
// SMs per sector rather than run one sector per SM.
#include "eig_tri.h"

#include <cfloat>
#include <cmath>
#include <cstdint>

namespace hh {
namespace tri {
namespace {

constexpr int kRows = 32;                        // rows per pass of a reduction CTA (one warp's lanes)
constexpr int kGroups = kReduceThreads / kRows;  // column groups per pass

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
// c + a b
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
// c + conj(a) b
__device__ __forceinline__ double2 cfmac(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, fma(a.y, b.y, c.x)), fma(a.x, b.y, fma(-a.y, b.x, c.y)));
}

// b - v_i conj(w_j) - w_i conj(v_j) as eight FMAs
__device__ __forceinline__ double2 rank2(double2 b, double2 vi, double2 wi, double2 vj, double2 wj) {
  double re = fma(-vi.x, wj.x, b.x);
  re = fma(-vi.y, wj.y, re);
  re = fma(-wi.x, vj.x, re);
  re = fma(-wi.y, vj.y, re);
  double im = fma(-vi.y, wj.x, b.y);
  im = fma(vi.x, wj.y, im);
  im = fma(-wi.y, vj.x, im);
  im = fma(wi.x, vj.y, im);
  return make_double2(re, im);
}

// Sum over the CTA; every thread receives it.  scratch holds >= 32 entries.
__device__ double block_sum(double v, double* scratch) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) scratch[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < nw; ++i) s += scratch[i];
  return s;
}

__device__ double2 block_sum2(double2 v, double2* scratch) {
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) scratch[w] = v;
  __syncthreads();
  double2 s = make_double2(0.0, 0.0);
  for (int i = 0; i < nw; ++i) s = cadd(s, scratch[i]);
  return s;
}

// Release/acquire barrier over the CTAs of the cluster: global- and shared-
// memory writes before it are visible to every CTA of the cluster after it.
// Every thread of every CTA calls it the same number of times (no
// CTA-dependent branches around it).
__device__ __forceinline__ void cluster_barrier() {
  __threadfence();
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// ---------------------------------------------------------------- reduce
// Column k (k = 0 .. n-2) of the lower-triangle Householder reduction:
//   x = A[k+1:n, k], alpha = x_0, beta = -sign(Re alpha) sqrt(|alpha|^2 + |x_1:|^2),
//   tau = (beta - alpha) / beta, v = (1, x_1: / (alpha - beta)),
//   H = I - tau v v^H with H^H x = beta e_1 (zlarfg);
//   p = tau B v on the trailing block B = A[k+1:n, k+1:n],
//   w = p - (tau / 2) (p^H v) v,  B <- B - v w^H - w v^H  (= H^H B H),
//   d_k = Re A[k, k], e_k = beta, and v stored in place of column k.
// Both triangles of B are kept (full rank-2 update), so the matrix-vector
// product reads whole rows and every CTA owns a contiguous range of rows.
__global__ void __launch_bounds__(kReduceThreads)
    reduce_kernel(double2* __restrict__ den, const Sector* __restrict__ secs, double* __restrict__ dvec,
                  double* __restrict__ evec, double2* __restrict__ tauv, double2* __restrict__ pbuf,
                  double2* __restrict__ dotbuf) {
  const int sec = blockIdx.x / kCluster;
  const int rank = blockIdx.x % kCluster;  // rank inside the (1-D) cluster
  const Sector S = secs[sec];
  const int n = S.n;
  double2* A = den + S.aoff;
  double* d = dvec + S.toff;
  double* e = evec + S.toff;
  double2* tau_out = tauv + S.toff;
  double2* P = pbuf + S.toff;
  double2* dots = dotbuf + (long long)sec * kCluster;
  extern __shared__ double2 sm[];
  double2* v = sm;      // n
  double2* w = sm + n;  // n
  __shared__ double2 red[kReduceThreads];
  __shared__ double red_d[32];
  __shared__ double2 red_c[32];
  __shared__ double2 s_tau, s_scale, s_a2;
  const int t = threadIdx.x;
  const int lr = t % kRows, g = t / kRows;

  for (int k = 0; k + 1 < n; ++k) {
    const int m = n - k - 1;
    const double2* colk = A + (long long)k * n + (k + 1);
    // (a) Householder vector, computed by every CTA from column k
    double xn = 0.0;
    for (int i = t; i < m; i += kReduceThreads) {
      const double2 x = colk[i];
      v[i] = x;
      if (i > 0) xn += x.x * x.x + x.y * x.y;
    }
    xn = block_sum(xn, red_d);  // ends with a barrier: v is complete
    if (t == 0) {
      const double2 alpha = v[0];
      double2 tau = make_double2(0.0, 0.0), scale = make_double2(0.0, 0.0);
      double beta = alpha.x;
      if (xn > 0.0 || alpha.y != 0.0) {
        beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn), alpha.x);
        tau = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
        const double2 den_ = make_double2(alpha.x - beta, alpha.y);  // 1 / (alpha - beta)
        const double r2 = den_.x * den_.x + den_.y * den_.y;
        scale = make_double2(den_.x / r2, -den_.y / r2);
      }
      s_tau = tau;
      s_scale = scale;
      if (rank == 0) {
        d[k] = A[(long long)k * n + k].x;
        e[k] = beta;
        tau_out[k] = tau;
      }
    }
    __syncthreads();
    const double2 tau = s_tau, scale = s_scale;
    for (int i = t; i < m; i += kReduceThreads) v[i] = i == 0 ? make_double2(1.0, 0.0) : cmul(v[i], scale);
    __syncthreads();
    // (b) p = tau B v on this CTA's rows [r0, r1) of the trailing block
    const int chunk = (m + kCluster - 1) / kCluster;
    const int r0 = min(m, rank * chunk), r1 = min(m, r0 + chunk);
    double2* B = A + (long long)(k + 1) * n + (k + 1);  // B(i, j) = B[i + j n]
    double2 dotp = make_double2(0.0, 0.0);
    for (int rt = r0; rt < r1; rt += kRows) {
      const int i = rt + lr;
      double2 acc = make_double2(0.0, 0.0);
      if (i < r1)
        for (int j = g; j < m; j += kGroups) acc = cfma(B[i + (long long)j * n], v[j], acc);
      red[t] = acc;
      __syncthreads();
      if (g == 0 && i < r1) {
        double2 s = red[lr];
        for (int q = 1; q < kGroups; ++q) s = cadd(s, red[q * kRows + lr]);
        const double2 p = cmul(tau, s);
        P[k + 1 + i] = p;
        dotp = cfmac(p, v[i], dotp);  // conj(p_i) v_i
      }
      __syncthreads();
    }
    dotp = block_sum2(dotp, red_c);
    if (t == 0) dots[rank] = dotp;
    cluster_barrier();  // p and the partial dots of every CTA are visible
    // (c) w = p + a2 v with a2 = -(tau / 2) (p^H v); rank-2 update of this CTA's rows
    if (t == 0) {
      double2 s = make_double2(0.0, 0.0);
      for (int r = 0; r < kCluster; ++r) s = cadd(s, dots[r]);
      s_a2 = cmul(make_double2(-0.5 * tau.x, -0.5 * tau.y), s);
    }
    __syncthreads();
    const double2 a2 = s_a2;
    for (int j = t; j < m; j += kReduceThreads) w[j] = cfma(a2, v[j], P[k + 1 + j]);
    __syncthreads();
    for (int rt = r0; rt < r1; rt += kRows) {
      const int i = rt + lr;
      if (i < r1) {
        const double2 vi = v[i], wi = w[i];
        for (int j = g; j < m; j += kGroups) {
          const long long o = i + (long long)j * n;
          // B(i,j) -= v_i conj(w_j) + w_i conj(v_j)
          const double2 upd = cadd(cmul(vi, cconj(w[j])), cmul(wi, cconj(v[j])));
          B[o] = csub(B[o], upd);
        }
      }
    }
    for (int i = r0 + t; i < r1; i += kReduceThreads) A[(long long)k * n + (k + 1) + i] = v[i];
    cluster_barrier();  // the trailing block and column k are complete
  }
  if (rank == 0 && t == 0) {
    d[n - 1] = A[(long long)(n - 1) * n + (n - 1)].x;
    e[n - 1] = 0.0;
    tau_out[n - 1] = make_double2(0.0, 0.0);
  }
}

// ------------------------------------------------------- reduce (DSMEM)
// The same reduction with the sector held in the cluster's distributed
// shared memory.  CTA r of the C-CTA cluster owns the columns j = r, r + C,
// r + 2C, ... (cyclic, so the shrinking trailing block stays balanced) and
// keeps only their lower parts, rows j .. n-1, packed one after another;
// B(i, j) for i < j is conj(B(j, i)).  Column k, three cluster barriers:
//   (B) every CTA copies v_k and tau_k from the column's owner and forms its
//       partial B v from its own columns: rows i >= j of column j (row part)
//       and the column's conjugate dot with v (column part);     barrier
//   (C) reduce-scatter: CTA r sums the C partials of the rows i = r (mod C),
//       scales them by tau and forms its share of p^H v;          barrier
//   (D) every CTA gathers p, forms w = p - (tau/2)(p^H v) v and applies
//       B <- B - v w^H - w v^H to its own lower columns.  The owner of column
//       k + 1 updates that column first and forms the next reflector
//       (zlarfg: d, e, tau, v; v also to global memory for the back-
//       transformation) while the other CTAs are still updating;   barrier
// GB300's FP64 pipe issues one warp instruction per SM sub-partition every
// 64 cycles or so, so the scalar chain between barriers (reductions, the
// reflector's square root and divisions) is kept short: shuffle trees, two
// divisions per reflector, and the next reflector overlapped with the
// update.  The vector slots sit at the front of the dynamic allocation, so at
// the same offsets in every CTA, and are read remotely through mapa
// addresses; v and tau are double-buffered by column parity.
__host__ __device__ __forceinline__ long long ds_col_off(int q, int n, int C, int r) {
  // packed offset of owned column q (column q C + r): sum over q' < q of n - (q' C + r)
  return (long long)q * (n - r) - (long long)C * q * (q - 1) / 2;
}

// shared::cluster address of the same shared-memory object in CTA `rank`
__device__ __forceinline__ uint32_t ds_map(const void* p, int rank) {
  const uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(p));
  uint32_t ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
  return ra;
}

__device__ __forceinline__ double2 ds_ld2(uint32_t addr) {
  double2 v;
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(addr) : "memory");
  return v;
}

__device__ __forceinline__ int cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return (int)r;
}

__device__ __forceinline__ int cluster_nctas() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return (int)r;
}

// Cluster barrier of the distributed-shared-memory kernel: its shared-memory
// writes before it are visible to the whole cluster after it.  The global
// writes (d, e, tau, reflectors) are read only by later kernels, so no
// GPU-scope fence.
__device__ __forceinline__ void ds_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double2 warp_sum2(double2 v) {
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}

// Sum over a kDsThreads CTA, received by every thread: two shuffle trees.
__device__ __forceinline__ double ds_block_sum(double v, double* scratch) {
  static_assert(kDsThreads / 32 <= 32, "one warp sums the warp partials");
  v = warp_sum(v);
  __syncthreads();  // scratch is free
  if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = v;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  return warp_sum(lane < kDsThreads / 32 ? scratch[lane] : 0.0);
}

// Reflector of column k (zlarfg) from x[i - k] = B(i, k), i >= k, by the
// owning CTA: H = I - tau v v^H with H^H x = beta e_1, v_{k+1} = 1.  Only
// warps holding elements take part in the norm's first tree and warp 0 alone
// forms the scalars (square root, two divisions): an FP64 warp instruction
// costs GB300 the same whatever the number of active lanes, so redundant
// copies in idle warps would cost as much as real work.  sc holds the scale
// for the other warps.
__device__ __forceinline__ void ds_reflector(int k, int n, const double2* x, double2* vb, double2* tau_slot,
                                             double2* sc, double* scratch, double2* A, const Sector& S,
                                             double* dvec, double* evec, double2* tauv) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  double xn = 0.0;
  if (warp * 32 < n - (k + 2)) {  // warps holding elements of x_2: (uniform per warp)
    for (int i = k + 2 + t; i < n; i += kDsThreads) {
      const double2 xi = x[i - k];
      xn = fma(xi.x, xi.x, fma(xi.y, xi.y, xn));
    }
    xn = warp_sum(xn);
  }
  if (lane == 0) scratch[warp] = xn;
  __syncthreads();
  if (warp == 0) {
    xn = warp_sum(lane < kDsThreads / 32 ? scratch[lane] : 0.0);
    const double2 alpha = x[1];
    double2 tau = make_double2(0.0, 0.0), scale = make_double2(0.0, 0.0);
    double beta = alpha.x;
    if (xn > 0.0 || alpha.y != 0.0) {
      beta = -copysign(sqrt(fma(alpha.x, alpha.x, fma(alpha.y, alpha.y, xn))), alpha.x);
      const double ib = 1.0 / beta;
      tau = make_double2((beta - alpha.x) * ib, -alpha.y * ib);
      const double dr = alpha.x - beta, di = alpha.y;  // scale = 1 / (alpha - beta)
      const double ir2 = 1.0 / fma(dr, dr, di * di);
      scale = make_double2(dr * ir2, -di * ir2);
    }
    if (lane == 0) {
      dvec[S.toff + k] = x[0].x;
      evec[S.toff + k] = beta;
      tauv[S.toff + k] = tau;
      *tau_slot = tau;
      *sc = scale;
    }
  }
  __syncthreads();
  const double2 scale = *sc;
  double2* Ak = A + (long long)k * n;
  for (int i = k + 1 + t; i < n; i += kDsThreads) {
    const double2 vi = i == k + 1 ? make_double2(1.0, 0.0) : cmul(x[i - k], scale);
    vb[i] = vi;
    Ak[i] = vi;
  }
}

// kGlobal: the owned lower columns stay in place in global memory (L2)
// instead of the CTA's shared memory, for sectors too large for the cluster's
// shared memory; the O(n) vector slots stay in shared memory either way.
template <bool kGlobal>
__global__ void __launch_bounds__(kDsThreads, 1)
    reduce_ds_kernel(double2* __restrict__ den, const Sector* __restrict__ secs, double* __restrict__ dvec,
                     double* __restrict__ evec, double2* __restrict__ tauv) {
  constexpr int kWarps = kDsThreads / 32;
  const int C = cluster_nctas();
  const int r = cluster_rank();
  const Sector S = secs[blockIdx.x / C];
  const int n = S.n;
  double2* A = den + S.aoff;
  extern __shared__ double2 sm[];
  double2* vbuf = sm;         // 2 n: v of the even / odd columns, indexed by row
  double2* wb = sm + 2 * n;   // p, then w
  double2* pp = sm + 3 * n;   // this CTA's partial B v
  double2* ps = sm + 4 * n;   // tau (B v) of the rows i = r (mod C), summed over the cluster
  double2* col = sm + 5 * n;  // the owned lower columns (packed; unused when kGlobal)
  // element (i, j), i >= j, of an owned column whose packed offset is o
  auto el = [&](long long o, int j, int i) -> double2& { return kGlobal ? A[(long long)j * n + i] : col[o + (i - j)]; };
  __shared__ double2 s_tau[2], s_dot, s_a2, s_scale;
  __shared__ double red_d[kWarps];
  __shared__ double2 red_c[kWarps];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int nq = n > r ? (n - r + C - 1) / C : 0;
  if (!kGlobal) {
    for (int q = 0; q < nq; ++q) {
      const int j = q * C + r;
      const long long o = ds_col_off(q, n, C, r);
      for (int i = j + t; i < n; i += kDsThreads) col[o + (i - j)] = A[(long long)j * n + i];
    }
  }
  __syncthreads();
  if (r == 0) {  // column 0
    if (n > 1) {
      ds_reflector(0, n, &el(0, 0, 0), vbuf, &s_tau[0], &s_scale, red_d, A, S, dvec, evec, tauv);
    } else if (t == 0) {
      dvec[S.toff] = el(0, 0, 0).x;
      evec[S.toff] = 0.0;
      tauv[S.toff] = make_double2(0.0, 0.0);
    }
  }
  ds_sync();
  for (int k = 0; k + 1 < n; ++k) {
    const int owner = k % C;
    double2* vb = vbuf + (k & 1) * n;
    // ---- (B) v and tau from the owner, then this CTA's partial B v
    double2 tau;
    if (owner != r) {
      const uint32_t rv = ds_map(vb, owner);
      for (int i = k + 1 + t; i < n; i += kDsThreads) vb[i] = ds_ld2(rv + (uint32_t)(i * sizeof(double2)));
      tau = ds_ld2(ds_map(&s_tau[k & 1], owner));
    } else {
      tau = s_tau[k & 1];
    }
    __syncthreads();
    const int qlo = k + 1 > r ? (k + 1 - r + C - 1) / C : 0;  // first owned column > k
    const long long olo = ds_col_off(qlo, n, C, r);
    // row part: pp[i] = sum over owned j in (k, i] of B(i, j) v_j
    for (int i = k + 1 + t; i < n; i += kDsThreads) {
      double2 acc = make_double2(0.0, 0.0);
      long long o = olo;
      for (int j = qlo * C + r; j <= i; j += C) {
        acc = cfma(el(o, j, i), vb[j], acc);
        o += n - j;
      }
      pp[i] = acc;
    }
    __syncthreads();
    // column part: pp[j] += sum over i > j of conj(B(i, j)) v_i, one warp per owned column
    for (int q = qlo + warp, j = (qlo + warp) * C + r; j < n; q += kWarps, j += kWarps * C) {
      const long long o = ds_col_off(q, n, C, r);
      double2 sum = make_double2(0.0, 0.0);
      for (int i = j + 1 + lane; i < n; i += 32) sum = cfmac(el(o, j, i), vb[i], sum);
      sum = warp_sum2(sum);
      if (lane == 0) pp[j] = cadd(pp[j], sum);
    }
    ds_sync();  // every CTA's partial is complete
    // ---- (C) reduce-scatter of the rows i = r (mod C) and this CTA's share of p^H v
    {
      const int i0 = k + 1 + ((r - (k + 1)) % C + C) % C;  // first row > k with i = r (mod C)
      const int nr = i0 < n ? (n - 1 - i0) / C + 1 : 0;
      const int src = t % C, slot = t / C, per = kDsThreads / C;
      const uint32_t rp = ds_map(pp, src);
      double2 dot = make_double2(0.0, 0.0);
      for (int base = 0; base < nr; base += per) {  // the same trip count in every thread
        if (base + (warp * 32) / C >= nr) continue;  // this warp has no rows in this pass (uniform per warp)
        const int ri = base + slot, i = i0 + ri * C;
        // every lane of a C-lane group takes part in its shuffles
        double2 val = ri < nr ? ds_ld2(rp + (uint32_t)(i * sizeof(double2))) : make_double2(0.0, 0.0);
        for (int sh = C >> 1; sh > 0; sh >>= 1) {
          val.x += __shfl_xor_sync(0xffffffffu, val.x, sh);
          val.y += __shfl_xor_sync(0xffffffffu, val.y, sh);
        }
        if (src == 0 && ri < nr) {
          const double2 p = cmul(tau, val);
          ps[i] = p;
          dot = cfmac(p, vb[i], dot);  // conj(p_i) v_i
        }
      }
      if ((warp * 32) / C < nr) dot = warp_sum2(dot);  // warps that held rows
      if (lane == 0) red_c[warp] = dot;
      __syncthreads();
      if (warp == 0) {
        const double2 sd = warp_sum2(lane < kWarps ? red_c[lane] : make_double2(0.0, 0.0));
        if (lane == 0) s_dot = sd;
      }
    }
    ds_sync();  // p and the partial dots are complete
    // ---- (D) w = p + a2 v with a2 = -(tau/2) (p^H v); rank-2 update; next reflector
    if (warp == 0) {
      const double2 sd = warp_sum2(lane < C ? ds_ld2(ds_map(&s_dot, lane)) : make_double2(0.0, 0.0));
      if (lane == 0) s_a2 = cmul(make_double2(-0.5 * tau.x, -0.5 * tau.y), sd);
    }
    for (int i = k + 1 + t; i < n; i += kDsThreads) wb[i] = ds_ld2(ds_map(ps + i, i % C));
    __syncthreads();
    {
      const double2 a2 = s_a2;
      for (int i = k + 1 + t; i < n; i += kDsThreads) wb[i] = cfma(a2, vb[i], wb[i]);
    }
    __syncthreads();
    const int nx = k + 1;  // the next column
    const bool own_next = nx % C == r;
    if (own_next) {
      // column nx first (rows nx .. n-1), then its reflector or, for the last
      // column, its diagonal
      const long long o = ds_col_off(nx / C, n, C, r);
      const double2 vj = vb[nx], wj = wb[nx];
      for (int i = nx + t; i < n; i += kDsThreads) el(o, nx, i) = rank2(el(o, nx, i), vb[i], wb[i], vj, wj);
      __syncthreads();
      if (nx + 1 < n) {
        ds_reflector(nx, n, &el(o, nx, nx), vbuf + (nx & 1) * n, &s_tau[nx & 1], &s_scale, red_d, A, S, dvec, evec,
                     tauv);
      } else if (t == 0) {
        dvec[S.toff + nx] = el(o, nx, nx).x;
        evec[S.toff + nx] = 0.0;
        tauv[S.toff + nx] = make_double2(0.0, 0.0);
      }
    }
    for (int i = k + 1 + t; i < n; i += kDsThreads) {
      const double2 vi = vb[i], wi = wb[i];
      long long o = olo;
      for (int j = qlo * C + r; j <= i; j += C) {
        if (j != nx || !own_next) el(o, j, i) = rank2(el(o, j, i), vi, wi, vb[j], wb[j]);
        o += n - j;
      }
    }
    ds_sync();  // the next v is posted and every column is updated
  }
}

// ---------------------------------------------------------------- bisect
// Number of eigenvalues of T (d, e) below x: the negative pivots q_i of the
// LDL^T factorisation of T - x I (the Sturm count of dstebz).  The FP64 count
// runs on the leading principal minors p_{i+1} = (d_i - x) p_i - e_{i-1}^2
// p_{i-1} (q_i = p_{i+1} / p_i: a negative pivot is a sign change), three
// FP64 operations per step and no division; signs, exponents and the
// rescaling of the pair by powers of two are integer operations on the bit
// patterns, so they stay off GB300's slow FP64 pipe.  A pivot below 2^-200 in
// magnitude counts as -2^-200 (dstebz uses -pivmin; either way the next pivot
// is huge and positive and the count is the same).  e2 holds e^2; the minors
// stay in [2^-600, 2^500] between rescalings.
__device__ __forceinline__ int sturm_count(const double* d, const double* e2, int n, double x) {
  constexpr long long kSign = (long long)0x8000000000000000ull;
  double pm = 1.0, p = d[0] - x;
  long long bp = __double_as_longlong(p);
  int ep = (int)((bp >> 52) & 0x7ff);
  if (ep < 1023 - 200) {  // |p| < 2^-200 (zero included): the pivot -2^-200
    p = -0x1p-200;
    bp = __double_as_longlong(p);
    ep = 1023 - 200;
  }
  int c = (int)((unsigned long long)bp >> 63);
  for (int i = 1; i < n; ++i) {
    double pn = fma(d[i] - x, p, -e2[i - 1] * pm);
    long long bn = __double_as_longlong(pn);
    int en = (int)((bn >> 52) & 0x7ff);
    if (en + 200 < ep) {  // tiny pivot: -sign(p) 2^(exp(p) - 200)
      bn = ((bp ^ kSign) & kSign) | ((long long)(ep - 200) << 52);
      pn = __longlong_as_double(bn);
      en = ep - 200;
    }
    c += (int)((unsigned long long)(bn ^ bp) >> 63);
    pm = p;
    p = pn;
    bp = bn;
    ep = en;
    if (ep > 1023 + 400 || ep < 1023 - 400) {  // rescale the pair by 2^-(ep - 1023): |p| into [1, 2)
      const double f = __longlong_as_double((long long)(2046 - ep) << 52);
      p *= f;
      pm *= f;
      bp = __double_as_longlong(p);
      ep = 1023;
    }
  }
  return c;
}

// The pivot count in FP32 on T scaled by a power of two (d32 = s d, e32 =
// (s e)^2, s ||T|| in [1/2, 1)), pivots below 16 FLT_MIN counted as negative.
__device__ __forceinline__ int sturm_count32(const float* d, const float* e2, int n, float x) {
  constexpr float kPiv = 16.0f * FLT_MIN;
  float q = d[0] - x;
  if (fabsf(q) < kPiv) q = -kPiv;
  int c = q < 0.0f;
  for (int i = 1; i < n; ++i) {
    q = (d[i] - x) - e2[i - 1] / q;
    if (fabsf(q) < kPiv) q = -kPiv;
    c += q < 0.0f;
  }
  return c;
}

constexpr int kBisectWarps = 4;  // eigenvalues per CTA, one warp each

// Every eigenvalue of every T, ascending: one warp per eigenvalue j, whose 32
// lanes count at 32 interior points of the current bracket at once (a
// 33-section: five bits per round).  T is staged in shared memory in FP64
// and, scaled by a power of two, in FP32.  The FP32 rounds bracket lambda_j
// to a few FP32 eps ||T||; the bracket, widened by 16 FP32 eps ||T|| (beyond
// the FP32 count's backward error), is kept when two FP64 counts confirm it,
// else the Gershgorin interval is used; FP64 rounds then close it to
// 2 eps ||T|| + 4 DBL_MIN.
__global__ void __launch_bounds__(kBisectWarps * 32)
    bisect_kernel(const Sector* __restrict__ secs, const double* __restrict__ dvec,
                  const double* __restrict__ evec, double* __restrict__ w) {
  const Sector S = secs[blockIdx.y];
  const int n = S.n;
  if ((int)blockIdx.x * kBisectWarps >= n) return;  // the whole CTA is beyond this sector
  extern __shared__ double sh[];
  double* d = sh;                                      // n
  double* e2 = sh + n;                                 // n: e_i^2
  float* d32 = reinterpret_cast<float*>(sh + 2 * n);   // n
  float* e32 = d32 + n;                                // n: (s e_i)^2
  __shared__ double s_red[3][kBisectWarps];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  double lo = 1e300, hi = -1e300, emax2 = 0.0;
  for (int i = t; i < n; i += kBisectWarps * 32) {
    const double di = dvec[S.toff + i];
    const double ei = i + 1 < n ? evec[S.toff + i] : 0.0;
    const double em = i > 0 ? evec[S.toff + i - 1] : 0.0;
    const double rr = fabs(ei) + fabs(em);
    d[i] = di;
    e2[i] = ei * ei;
    emax2 = fmax(emax2, ei * ei);
    lo = fmin(lo, di - rr);
    hi = fmax(hi, di + rr);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    emax2 = fmax(emax2, __shfl_xor_sync(0xffffffffu, emax2, o));
  }
  if (lane == 0) {
    s_red[0][warp] = lo;
    s_red[1][warp] = hi;
    s_red[2][warp] = emax2;
  }
  __syncthreads();
  for (int q = 0; q < kBisectWarps; ++q) {
    lo = fmin(lo, s_red[0][q]);
    hi = fmax(hi, s_red[1][q]);
  }
  const double tnorm = fmax(fabs(lo), fabs(hi));
  const double tol = 2.0 * DBL_EPSILON * tnorm + 4.0 * DBL_MIN;
  int ex = 0;
  frexp(tnorm > 0.0 ? tnorm : 1.0, &ex);
  const double sc = ldexp(1.0, -ex);  // s ||T|| in [1/2, 1)
  for (int i = t; i < n; i += kBisectWarps * 32) {
    d32[i] = (float)(sc * d[i]);
    const double es = sc * sqrt(e2[i]);
    e32[i] = (float)(es * es);
  }
  __syncthreads();
  const int j = blockIdx.x * kBisectWarps + warp;
  if (j >= n) return;  // whole warps only
  lo -= tol;
  hi += tol;
  // FP32 rounds on the scaled matrix
  float l32 = (float)(sc * lo), h32 = (float)(sc * hi);
  for (int it = 0; it < 12 && h32 - l32 > 4.0f * FLT_EPSILON; ++it) {
    const float x = l32 + (h32 - l32) * (float)(lane + 1) * (1.0f / 33.0f);
    const unsigned above = __ballot_sync(0xffffffffu, x > l32 && x < h32 && sturm_count32(d32, e32, n, x) > j);
    // the first point above lambda_j bounds it from above, the point before from below
    float nl = l32, nh = h32;
    if (above) {
      const int f = __ffs(above) - 1;
      nh = __shfl_sync(0xffffffffu, x, f);
      if (f > 0) nl = __shfl_sync(0xffffffffu, x, f - 1);
    } else {
      nl = __shfl_sync(0xffffffffu, x, 31);
    }
    if (nl == l32 && nh == h32) break;
    l32 = nl;
    h32 = nh;
  }
  {
    const double widen = 16.0 * FLT_EPSILON;
    const double blo = fmax(lo, ((double)l32 - widen) / sc), bhi = fmin(hi, ((double)h32 + widen) / sc);
    // lanes 0 and 1 confirm the bracket with FP64 counts
    const int cnt = lane < 2 && blo < bhi ? sturm_count(d, e2, n, lane == 0 ? blo : bhi) : 0;
    const int c0 = __shfl_sync(0xffffffffu, cnt, 0), c1 = __shfl_sync(0xffffffffu, cnt, 1);
    if (blo < bhi && c0 <= j && c1 > j) {
      lo = blo;
      hi = bhi;
    }
  }
  // FP64 rounds: count(x) > j  <=>  lambda_j < x
  for (int it = 0; it < 24 && hi - lo > tol; ++it) {
    const double x = lo + (hi - lo) * (double)(lane + 1) * (1.0 / 33.0);
    const unsigned above = __ballot_sync(0xffffffffu, x > lo && x < hi && sturm_count(d, e2, n, x) > j);
    double nl = lo, nh = hi;
    if (above) {
      const int f = __ffs(above) - 1;
      nh = __shfl_sync(0xffffffffu, x, f);
      if (f > 0) nl = __shfl_sync(0xffffffffu, x, f - 1);
    } else {
      nl = __shfl_sync(0xffffffffu, x, 31);
    }
    if (nl == lo && nh == hi) break;
    lo = nl;
    hi = nh;
  }
  if (lane == 0) w[S.woff + j] = 0.5 * (lo + hi);
}

// ------------------------------------------------------ inverse iteration
__device__ __forceinline__ double start_value(unsigned long long a, unsigned long long b) {
  unsigned long long z = a * 0x9E3779B97F4A7C15ull + b * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;  // [-1, 1)
}

// Eigenvector of T for lambda_j: Gaussian elimination with partial pivoting
// of M = T - lambda I (row i of M has e_{i-1}, d_i - lambda, e_i), kept as
// the rows (1 / u0, u1, u2) of U (the pivot's reciprocal, so that the solves
// multiply: an FP64 division costs GB300 several FP64-pipe operations), the
// multipliers and the row swaps; then three
// solves M x_{t+1} = x_t from a pseudo-random x_0, normalised each time.
// Pivots below eps ||T|| are raised to eps ||T|| (the exact-eigenvalue case).
__global__ void inverse_iteration_kernel(const Sector* __restrict__ secs, const InvItem* __restrict__ items,
                                         int nitems, int maxn, const double* __restrict__ dvec,
                                         const double* __restrict__ evec, const double* __restrict__ w,
                                         double* __restrict__ Z, double* __restrict__ lu) {
  const int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= nitems) return;
  const InvItem I = items[it];
  const Sector S = secs[I.sec];
  const int n = S.n;
  const double* d = dvec + S.toff;
  const double* e = evec + S.toff;
  const double lam = w[S.woff + I.j];
  const long long stride = nitems;
  double* U0 = lu + (0ll * maxn) * stride + it;
  double* U1 = lu + (1ll * maxn) * stride + it;
  double* U2 = lu + (2ll * maxn) * stride + it;
  double* ML = lu + (3ll * maxn) * stride + it;
  double* SW = lu + (4ll * maxn) * stride + it;
  double* x = Z + I.zoff + I.col;
  const long long ldz = I.ldz;
  double tnorm = 0.0;
  for (int i = 0; i < n; ++i)
    tnorm = fmax(tnorm, fabs(d[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < n ? fabs(e[i]) : 0.0));
  const double pivtol = fmax(DBL_EPSILON * tnorm, DBL_MIN);
  auto guard = [pivtol](double u) { return fabs(u) < pivtol ? (u < 0.0 ? -pivtol : pivtol) : u; };
  // factorisation
  double u0 = d[0] - lam, u1 = n > 1 ? e[0] : 0.0;
  for (int i = 0; i + 1 < n; ++i) {
    const double s = e[i], tt = d[i + 1] - lam, r = i + 2 < n ? e[i + 1] : 0.0;
    if (fabs(u0) >= fabs(s)) {  // keep row i as the pivot row
      u0 = guard(u0);
      const double inv = 1.0 / u0;
      const double mult = s * inv;
      U0[i * stride] = inv;
      U1[i * stride] = u1;
      U2[i * stride] = 0.0;
      ML[i * stride] = mult;
      SW[i * stride] = 0.0;
      u0 = tt - mult * u1;
      u1 = r;
    } else {  // row i + 1 is the pivot row
      const double inv = 1.0 / s;
      const double mult = u0 * inv;
      U0[i * stride] = inv;
      U1[i * stride] = tt;
      U2[i * stride] = r;
      ML[i * stride] = mult;
      SW[i * stride] = 1.0;
      const double nu0 = u1 - mult * tt;
      u1 = -mult * r;
      u0 = nu0;
    }
  }
  U0[(long long)(n - 1) * stride] = 1.0 / guard(u0);
  U1[(long long)(n - 1) * stride] = 0.0;
  U2[(long long)(n - 1) * stride] = 0.0;
  for (int i = 0; i < n; ++i) x[i * ldz] = start_value(((unsigned long long)I.sec << 32) + (unsigned)I.j, i);
  for (int step = 0; step < 3; ++step) {
    // forward: apply the row operations
    double cur = x[0];
    for (int i = 0; i + 1 < n; ++i) {
      const double nxt = x[(i + 1) * ldz];
      const double mult = ML[i * stride];
      if (SW[i * stride] == 0.0) {
        x[i * ldz] = cur;
        cur = nxt - mult * cur;
      } else {
        x[i * ldz] = nxt;
        cur = cur - mult * nxt;
      }
    }
    x[(n - 1) * ldz] = cur;
    // back substitution with U
    double x1 = 0.0, x2 = 0.0, nrm = 0.0;  // x_{i+1}, x_{i+2}
    for (int i = n - 1; i >= 0; --i) {
      const double xi = (x[i * ldz] - U1[i * stride] * x1 - U2[i * stride] * x2) * U0[i * stride];
      x[i * ldz] = xi;
      x2 = x1;
      x1 = xi;
      nrm = fmax(nrm, fabs(xi));
    }
    // normalise (max-norm first, then the 2-norm, against overflow)
    const double inv = nrm > 0.0 ? 1.0 / nrm : 1.0;
    double s2 = 0.0;
    for (int i = 0; i < n; ++i) {
      const double xi = x[i * ldz] * inv;
      x[i * ldz] = xi;
      s2 += xi * xi;
    }
    const double r = s2 > 0.0 ? 1.0 / sqrt(s2) : 1.0;
    for (int i = 0; i < n; ++i) x[i * ldz] *= r;
  }
}

// ------------------------------------------------------------------- cgs2
// One CTA per sector block with clusters of numerically degenerate kept
// eigenvalues: each column of each cluster, from the last (largest
// eigenvalue) to the first, is orthogonalised against every column after it
// in the block (the rest of its cluster and the larger eigenvalues'
// columns), twice, and normalised; the block's clusters are taken from the
// top down so that every column it projects against is final.  Inverse
// iteration leaves the vectors of a degenerate cluster as independent but
// non-orthogonal combinations of its eigenspace; vectors of eigenvalues
// further apart (relative gap above 1e-13) are orthogonal to about
// eps / gap, which the Newton-Schulz steps that follow remove.  Only the
// clusters' columns are processed (the whole block, column by column, cost
// tens of milliseconds per sector).
__global__ void cgs2_kernel(const CgsBlock* __restrict__ blocks, const int2* __restrict__ clusters,
                            double* __restrict__ Z) {
  const CgsBlock b = blocks[blockIdx.x];
  double* Zb = Z + b.zoff;
  const int n = b.n, k = b.ldz;
  extern __shared__ double coef[];  // k
  __shared__ double scratch[32];
  for (int cl = 0; cl < b.ncl; ++cl) {
  const int2 range = clusters[b.cl0 + cl];
  for (int c = range.y - 1; c >= range.x; --c) {
    for (int pass = 0; pass < 2; ++pass) {
      // coefficients against the columns c+1 .. k-1, one per thread (rows of
      // the row-major block are contiguous over q)
      for (int q = c + 1 + threadIdx.x; q < k; q += blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < n; ++i) s = fma(Zb[(long long)i * k + q], Zb[(long long)i * k + c], s);
        coef[q] = s;
      }
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double s = Zb[(long long)i * k + c];
        for (int q = c + 1; q < k; ++q) s = fma(-coef[q], Zb[(long long)i * k + q], s);
        Zb[(long long)i * k + c] = s;
      }
      __syncthreads();
    }
    double s2 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double z = Zb[(long long)i * k + c];
      s2 = fma(z, z, s2);
    }
    s2 = block_sum(s2, scratch);
    const double r = s2 > 0.0 ? 1.0 / sqrt(s2) : 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) Zb[(long long)i * k + c] *= r;
    __syncthreads();
  }
  }
}

// --------------------------------------------------------------- chol_inv
// One CTA per item: the upper Cholesky factor R of G + s I (in place in G's
// upper triangle; s = 1e-14 trace(G) / c keeps a nearly singular Gram matrix
// factorisable, the second Cholesky QR pass removes its effect), then
// R^{-1} column by column (thread q solves R x = e_q backwards, four
// independent partial sums against the FP64 latency).  Used by the Cholesky
// QR of large clusters of degenerate kept eigenvalues (null spaces of
// rank-deficient density matrices), where column-by-column Gram-Schmidt on
// one CTA costs tens of milliseconds.
__global__ void __launch_bounds__(512) chol_inv_kernel(const CholItem* __restrict__ items, double* __restrict__ buf) {
  const CholItem it = items[blockIdx.x];
  double* G = buf + it.g;
  double* Ri = buf + it.r;
  const int c = it.c;
  __shared__ double s_shift, s_piv;
  __shared__ double red[32];
  double tr = 0.0;
  for (int i = threadIdx.x; i < c; i += blockDim.x) tr += G[(long long)i * c + i];
  tr = block_sum(tr, red);
  if (threadIdx.x == 0) s_shift = 1e-14 * tr / (c > 0 ? c : 1) + DBL_MIN;
  __syncthreads();
  for (int i = threadIdx.x; i < c; i += blockDim.x) G[(long long)i * c + i] += s_shift;
  __syncthreads();
  for (int j = 0; j < c; ++j) {
    if (threadIdx.x == 0) {
      const double d = G[(long long)j * c + j];
      s_piv = sqrt(d > s_shift ? d : s_shift);
    }
    __syncthreads();
    const double rjj = s_piv, inv = 1.0 / rjj;
    for (int q = j + threadIdx.x; q < c; q += blockDim.x)
      G[(long long)j * c + q] = q == j ? rjj : G[(long long)j * c + q] * inv;
    __syncthreads();
    // trailing update of the upper triangle: rows p over the warps, columns
    // q >= p over the lanes (coalesced, no index division, no lower half)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    for (int p = j + 1 + warp; p < c; p += nwarp) {
      const double gjp = G[(long long)j * c + p];
      for (int q = p + lane; q < c; q += 32)
        G[(long long)p * c + q] = fma(-gjp, G[(long long)j * c + q], G[(long long)p * c + q]);
    }
    __syncthreads();
  }
  for (int q = threadIdx.x; q < c; q += blockDim.x) {
    for (int p = c - 1; p > q; --p) Ri[(long long)p * c + q] = 0.0;
    Ri[(long long)q * c + q] = 1.0 / G[(long long)q * c + q];
    for (int p = q - 1; p >= 0; --p) {
      double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
      int t = p + 1;
      for (; t + 3 <= q; t += 4) {
        a0 = fma(G[(long long)p * c + t], Ri[(long long)t * c + q], a0);
        a1 = fma(G[(long long)p * c + t + 1], Ri[(long long)(t + 1) * c + q], a1);
        a2 = fma(G[(long long)p * c + t + 2], Ri[(long long)(t + 2) * c + q], a2);
        a3 = fma(G[(long long)p * c + t + 3], Ri[(long long)(t + 3) * c + q], a3);
      }
      for (; t <= q; ++t) a0 = fma(G[(long long)p * c + t], Ri[(long long)t * c + q], a0);
      Ri[(long long)p * c + q] = -((a0 + a1) + (a2 + a3)) / G[(long long)p * c + p];
    }
  }
}

// ------------------------------------------------------------------- gemm
constexpr int kTile = 64, kKc = 16, kGemmThreads = 256;

__global__ void __launch_bounds__(kGemmThreads)
    gemm_kernel(const GemmItem* __restrict__ items, int nitems, double* __restrict__ buf,
                const int* __restrict__ need) {
  // the item owning this tile (items sorted by tile0)
  int lo = 0, hi = nitems - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (items[mid].tile0 <= (int)blockIdx.x)
      lo = mid;
    else
      hi = mid - 1;
  }
  const GemmItem G = items[lo];
  const int tile = blockIdx.x - G.tile0;
  const int m0 = (tile / G.tiles_n) * kTile, n0 = (tile % G.tiles_n) * kTile;
  if (need && G.gate > 0 && G.step >= need[G.gate - 1]) {  // a Newton-Schulz step this block skips
    if (G.beta != 0.0)
      for (int x = threadIdx.x; x < kTile * kTile; x += kGemmThreads) {
        const int gi = m0 + x / kTile, gj = n0 + x % kTile;
        if (gi < G.M && gj < G.N)
          buf[G.c + (long long)gi * G.c_r + (long long)gj * G.c_c] =
              buf[G.c0 + (long long)gi * G.c_r + (long long)gj * G.c_c];
      }
    return;
  }
  __shared__ double As[kKc][kTile + 1];
  __shared__ double Bs[kKc][kTile + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // 4 x 4 outputs per thread
  double acc[4][4] = {};
  const double* A = buf + G.a;
  const double* B = buf + G.b;
  for (int k0 = 0; k0 < G.K; k0 += kKc) {
    for (int x = threadIdx.x; x < kKc * kTile; x += kGemmThreads) {
      const int kk = x / kTile, r = x % kTile;
      const int gi = m0 + r, gk = k0 + kk, gj = n0 + r;
      As[kk][r] = (gi < G.M && gk < G.K) ? A[(long long)gi * G.a_r + (long long)gk * G.a_c] : 0.0;
      Bs[kk][r] = (gj < G.N && gk < G.K) ? B[(long long)gk * G.b_r + (long long)gj * G.b_c] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kKc; ++kk) {
      double a[4], bb[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[kk][ty * 4 + q];
        bb[q] = Bs[kk][tx * 4 + q];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = fma(a[p], bb[q], acc[p][q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int gi = m0 + ty * 4 + p, gj = n0 + tx * 4 + q;
      if (gi < G.M && gj < G.N) {
        double v = G.alpha * acc[p][q];
        if (G.beta != 0.0) v = fma(G.beta, buf[G.c0 + (long long)gi * G.c_r + (long long)gj * G.c_c], v);
        buf[G.c + (long long)gi * G.c_r + (long long)gj * G.c_c] = v;
      }
    }
}

// need[b] from delta = max |G_b - I| (one CTA per block; NaN counts as large)
__global__ void __launch_bounds__(256) ns_gate_kernel(const NsBlock* __restrict__ blocks, const double* __restrict__ buf,
                                                      int* __restrict__ need) {
  const NsBlock B = blocks[blockIdx.x];
  const double* G = buf + B.goff;
  double d = 0.0;
  const long long kk = (long long)B.k * B.k;
  for (long long x = threadIdx.x; x < kk; x += blockDim.x) {
    const double v = fabs(G[x] - ((x / B.k == x % B.k) ? 1.0 : 0.0));
    d = (v > d || v != v) ? v : d;  // a NaN propagates
  }
  __shared__ double sh[8];
  for (int o = 16; o > 0; o >>= 1) {
    const double w = __shfl_xor_sync(0xffffffffu, d, o);
    d = (w > d || w != w) ? w : d;
  }
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = d;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int q = 0; q < 8; ++q) m = (sh[q] > m || sh[q] != sh[q]) ? sh[q] : m;
    need[blockIdx.x] = (m <= 1e-8) ? 1 : (m <= 1e-4) ? 2 : 3;
  }
}

// ---------------------------------------------------------- backtransform
// X = H_0 H_1 ... H_{n-2} Z: the reflectors are applied from the last to the
// first, X[j+1:, c] -= tau_j v_j (v_j^H X[j+1:, c]); one warp per column, so
// the columns need no barrier between reflectors.
__global__ void __launch_bounds__(kBtCols * 32)
    backtransform_kernel(const Sector* __restrict__ secs, const BtItem* __restrict__ items,
                         const double2* __restrict__ den, const double2* __restrict__ tauv,
                         const double* __restrict__ Z, double2* __restrict__ X) {
  const BtItem I = items[blockIdx.x];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (wid >= I.nc) return;
  const Sector S = secs[I.sec];
  const int n = S.n;
  const int c = I.c0 + wid;
  const double2* V = den + S.aoff;
  double2* x = X + I.xoff + (long long)c * n;
  for (int i = lane; i < n; i += 32) x[i] = make_double2(Z[I.zoff + (long long)i * I.ldz + c], 0.0);
  __syncwarp();
  for (int j = n - 2; j >= 0; --j) {
    const double2 tau = tauv[S.toff + j];
    if (tau.x == 0.0 && tau.y == 0.0) continue;
    const double2* v = V + (long long)j * n;  // v_j in rows j+1 .. n-1
    double2 s = make_double2(0.0, 0.0);
    for (int i = j + 1 + lane; i < n; i += 32) s = cfmac(v[i], x[i], s);
    for (int o = 16; o > 0; o >>= 1) {
      s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    const double2 f = cmul(tau, s);
    for (int i = j + 1 + lane; i < n; i += 32) x[i] = csub(x[i], cmul(v[i], f));
    __syncwarp();
  }
}

// ----------------------------------------------------------- phase_columns
// One block per column: the largest-modulus component (first on ties) is
// made real and positive.
__global__ void phase_columns_kernel(const PhaseItem* __restrict__ items, double2* __restrict__ X) {
  const PhaseItem it = items[blockIdx.y];
  const int col = blockIdx.x;
  if (col >= it.cols) return;
  double2* v = X + it.off + (long long)col * it.rows;
  __shared__ double best[256];
  __shared__ int bidx[256];
  double m = -1.0;
  int mi = 0;
  for (int i = threadIdx.x; i < it.rows; i += blockDim.x) {
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
  const double2 ph = make_double2(p.x / a, -p.y / a);
  for (int i = threadIdx.x; i < it.rows; i += blockDim.x) v[i] = cmul(v[i], ph);
}

}  // namespace

cudaError_t reduce(const Sector* d_secs, int nsec, int maxn, double2* den, double* d, double* e, double2* tau,
                   double2* p, double2* dots, cudaStream_t s) {
  if (nsec <= 0) return cudaSuccess;
  if (maxn > kMaxN) return cudaErrorInvalidValue;
  const size_t smem = (size_t)2 * maxn * sizeof(double2);
  cudaError_t e0 = cudaFuncSetAttribute(reduce_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e0 != cudaSuccess) return e0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nsec * kCluster), 1, 1);
  cfg.blockDim = dim3(kReduceThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kCluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, reduce_kernel, den, d_secs, d, e, tau, p, dots);
}

namespace {

// dynamic shared memory of reduce_ds_kernel for sectors of at most n states:
// the five vector slots and, in shared memory, the packed lower columns of
// cluster rank 0 (the most of any rank)
size_t ds_smem_bytes(int n, int C, bool global_cols) {
  const int nq = (n + C - 1) / C;
  return (size_t)(5LL * n + (global_cols ? 0 : ds_col_off(nq, n, C, 0))) * sizeof(double2);
}

template <bool kGlobal>
size_t ds_smem_limit() {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, reduce_ds_kernel<kGlobal>) != cudaSuccess) return 0;
  return optin > (int)fa.sharedSizeBytes ? (size_t)optin - fa.sharedSizeBytes : 0;
}

template <bool kGlobal>
cudaError_t launch_ds(const Sector* d_secs, int nsec, size_t smem, int C, double2* den, double* d, double* e,
                      double2* tau, cudaStream_t s) {
  cudaError_t e0 = cudaFuncSetAttribute(reduce_ds_kernel<kGlobal>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem);
  if (e0 == cudaSuccess && C > 8)
    e0 = cudaFuncSetAttribute(reduce_ds_kernel<kGlobal>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e0 != cudaSuccess) return e0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nsec * C), 1, 1);
  cfg.blockDim = dim3(kDsThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, reduce_ds_kernel<kGlobal>, den, d_secs, d, e, tau);
}

}  // namespace

int ds_cluster_size() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 8;
  static int cached[64] = {0};
  if (dev >= 0 && dev < 64 && cached[dev]) return cached[dev];
  // 16 CTAs per cluster is beyond the portable size: used where the device
  // can place such a cluster with the kernel's largest shared-memory use
  int size = 8;
  const size_t smem = ds_smem_limit<false>();
  if (smem > 0 &&
      cudaFuncSetAttribute(reduce_ds_kernel<false>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
          cudaSuccess &&
      cudaFuncSetAttribute(reduce_ds_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
          cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kClusterMax, 1, 1);
    cfg.blockDim = dim3(kDsThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kClusterMax;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, reduce_ds_kernel<false>, &cfg) == cudaSuccess && nclusters >= 1)
      size = kClusterMax;
  }
  cudaGetLastError();  // a refused query leaves no error behind
  if (dev >= 0 && dev < 64) cached[dev] = size;
  return size;
}

int ds_max_n(bool global_cols) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  static int cached[2][64] = {};
  if (dev >= 0 && dev < 64 && cached[global_cols][dev]) return cached[global_cols][dev];
  const int C = ds_cluster_size();
  const size_t lim = global_cols ? ds_smem_limit<true>() : ds_smem_limit<false>();
  int n = 0;
  while (n < kMaxN && ds_smem_bytes(n + 1, C, global_cols) <= lim) ++n;
  cudaGetLastError();
  if (dev >= 0 && dev < 64) cached[global_cols][dev] = n;
  return n;
}

cudaError_t reduce_ds(const Sector* d_secs, int nsec, int maxn, bool global_cols, double2* den, double* d, double* e,
                      double2* tau, cudaStream_t s) {
  if (nsec <= 0) return cudaSuccess;
  if (maxn > ds_max_n(global_cols)) return cudaErrorInvalidValue;
  const int C = ds_cluster_size();
  const size_t smem = ds_smem_bytes(maxn, C, global_cols);
  return global_cols ? launch_ds<true>(d_secs, nsec, smem, C, den, d, e, tau, s)
                     : launch_ds<false>(d_secs, nsec, smem, C, den, d, e, tau, s);
}

cudaError_t bisect(const Sector* d_secs, int nsec, int maxn, const double* d, const double* e, double* w,
                   cudaStream_t s) {
  if (nsec <= 0) return cudaSuccess;
  const size_t smem = (size_t)maxn * (2 * sizeof(double) + 2 * sizeof(float));
  cudaError_t e0 = cudaFuncSetAttribute(bisect_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e0 != cudaSuccess) return e0;
  bisect_kernel<<<dim3((unsigned)((maxn + kBisectWarps - 1) / kBisectWarps), (unsigned)nsec), kBisectWarps * 32,
                  smem, s>>>(d_secs, d, e, w);
  return cudaGetLastError();
}

cudaError_t inverse_iteration(const Sector* d_secs, const InvItem* d_items, int nitems, int maxn, const double* d,
                              const double* e, const double* w, double* Z, double* lu, cudaStream_t s) {
  if (nitems <= 0) return cudaSuccess;
  constexpr int kT = 32;
  inverse_iteration_kernel<<<(unsigned)((nitems + kT - 1) / kT), kT, 0, s>>>(d_secs, d_items, nitems, maxn, d, e,
                                                                            w, Z, lu);
  return cudaGetLastError();
}

cudaError_t cgs2(const CgsBlock* d_blocks, int nblocks, const int2* d_clusters, int maxk, double* Z,
                 cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  cgs2_kernel<<<(unsigned)nblocks, 256, (size_t)maxk * sizeof(double), s>>>(d_blocks, d_clusters, Z);
  return cudaGetLastError();
}

cudaError_t chol_inv(const CholItem* d_items, int nitems, double* buf, cudaStream_t s) {
  if (nitems <= 0) return cudaSuccess;
  chol_inv_kernel<<<(unsigned)nitems, 512, 0, s>>>(d_items, buf);
  return cudaGetLastError();
}

cudaError_t gemm(const GemmItem* d_items, int nitems, int ntiles, double* buf, cudaStream_t s, const int* need) {
  if (nitems <= 0 || ntiles <= 0) return cudaSuccess;
  gemm_kernel<<<(unsigned)ntiles, kGemmThreads, 0, s>>>(d_items, nitems, buf, need);
  return cudaGetLastError();
}

cudaError_t ns_gate(const NsBlock* d_blocks, int nblocks, const double* buf, int* need, cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  ns_gate_kernel<<<(unsigned)nblocks, 256, 0, s>>>(d_blocks, buf, need);
  return cudaGetLastError();
}

cudaError_t backtransform(const Sector* d_secs, const BtItem* d_items, int nitems, const double2* den,
                          const double2* tau, const double* Z, double2* X, cudaStream_t s) {
  if (nitems <= 0) return cudaSuccess;
  backtransform_kernel<<<(unsigned)nitems, kBtCols * 32, 0, s>>>(d_secs, d_items, den, tau, Z, X);
  return cudaGetLastError();
}

cudaError_t phase_columns(const PhaseItem* d_items, int nitems, int maxcols, double2* X, cudaStream_t s) {
  if (nitems <= 0 || maxcols <= 0) return cudaSuccess;
  phase_columns_kernel<<<dim3((unsigned)maxcols, (unsigned)nitems), 256, 0, s>>>(d_items, X);
  return cudaGetLastError();
}

}  // namespace tri
}  // namespace hh
