// FP64 batched Hermitian eigensolver for the density-matrix sectors of more
// than 32 states: the per-sector ZHEEV('V','U') of code/get_den.f90:242,
// restated as the reduction / bisection / inverse-iteration pipeline of
// LAPACK's expert driver (zhetrd, dstebz, dstein, zunmtr), every step written
// for many SMs at once:
//
//   1. reduce: Householder reduction of each sector to a real symmetric
//      tridiagonal T = Q^H A Q (the unblocked lower-triangle algorithm of
//      zhetd2).  One thread-block cluster of kCluster CTAs per sector: the
//      sector stays in global memory (L2-resident), the rows of the trailing
//      block are split over the CTAs, and two cluster barriers per column
//      order the matrix-vector product and the rank-2 update;
//   2. bisect: every eigenvalue of every T by bisection on Sturm counts, one
//      thread per eigenvalue, to an absolute accuracy of a few eps ||T||;
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

// Release/acquire barrier over the CTAs of the cluster: global-memory writes
// before it are visible to every CTA of the cluster after it.  Every thread of
// every CTA calls it the same number of times (no CTA-dependent branches
// around it).
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

// ---------------------------------------------------------------- bisect
// Number of eigenvalues of T (d, e) below x: negative pivots of the LDL^T
// factorisation of T - x I, q_i = (d_i - x) - e_{i-1}^2 / q_{i-1}, a pivot
// smaller than pivmin replaced by -pivmin (Sturm sequence, as dstebz counts).
__device__ __forceinline__ int sturm_count(const double* d, const double* e, int n, double x, double pivmin) {
  double q = d[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  int c = q < 0.0;
  for (int i = 1; i < n; ++i) {
    const double ei = e[i - 1];
    q = (d[i] - x) - ei * ei / q;
    if (fabs(q) < pivmin) q = -pivmin;
    c += q < 0.0;
  }
  return c;
}

__global__ void bisect_kernel(const Sector* __restrict__ secs, const double* __restrict__ dvec,
                              const double* __restrict__ evec, double* __restrict__ w) {
  const Sector S = secs[blockIdx.y];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= S.n) return;
  const int n = S.n;
  const double* d = dvec + S.toff;
  const double* e = evec + S.toff;
  // Gershgorin interval and the scale of T
  double lo = 0.0, hi = 0.0, emax2 = 0.0;
  for (int i = 0; i < n; ++i) {
    const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < n ? fabs(e[i]) : 0.0);
    if (i + 1 < n) emax2 = fmax(emax2, e[i] * e[i]);
    lo = i == 0 ? d[i] - r : fmin(lo, d[i] - r);
    hi = i == 0 ? d[i] + r : fmax(hi, d[i] + r);
  }
  const double tnorm = fmax(fabs(lo), fabs(hi));
  const double pivmin = DBL_MIN * fmax(1.0, emax2);
  const double tol = 2.0 * DBL_EPSILON * tnorm + 4.0 * pivmin;
  lo -= tol;
  hi += tol;
  // j-th smallest eigenvalue: count(x) > j  <=>  lambda_j < x
  for (int it = 0; it < 128 && hi - lo > tol; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (sturm_count(d, e, n, mid, pivmin) > j)
      hi = mid;
    else
      lo = mid;
  }
  w[S.woff + j] = 0.5 * (lo + hi);
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
// the rows (u0, u1, u2) of U, the multipliers and the row swaps; then three
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
      const double mult = s / u0;
      U0[i * stride] = u0;
      U1[i * stride] = u1;
      U2[i * stride] = 0.0;
      ML[i * stride] = mult;
      SW[i * stride] = 0.0;
      u0 = tt - mult * u1;
      u1 = r;
    } else {  // row i + 1 is the pivot row
      const double mult = u0 / s;
      U0[i * stride] = s;
      U1[i * stride] = tt;
      U2[i * stride] = r;
      ML[i * stride] = mult;
      SW[i * stride] = 1.0;
      const double nu0 = u1 - mult * tt;
      u1 = -mult * r;
      u0 = nu0;
    }
  }
  U0[(long long)(n - 1) * stride] = guard(u0);
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
      const double xi = (x[i * ldz] - U1[i * stride] * x1 - U2[i * stride] * x2) / U0[i * stride];
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
// One CTA per block: each column, from the last (largest eigenvalue) to the
// first, is orthogonalised against the ones already done, twice, and
// normalised.
__global__ void cgs2_kernel(const CgsBlock* __restrict__ blocks, double* __restrict__ Z) {
  const CgsBlock b = blocks[blockIdx.x];
  double* Zb = Z + b.zoff;
  const int n = b.n, k = b.ldz;
  extern __shared__ double coef[];  // k
  __shared__ double scratch[32];
  for (int c = k - 1; c >= 0; --c) {
    for (int pass = 0; pass < 2; ++pass) {
      // coefficients against the finished columns c+1 .. k-1
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
      s2 += z * z;
    }
    s2 = block_sum(s2, scratch);
    const double r = s2 > 0.0 ? 1.0 / sqrt(s2) : 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) Zb[(long long)i * k + c] *= r;
    __syncthreads();
  }
}

// ------------------------------------------------------------------- gemm
constexpr int kTile = 64, kKc = 16, kGemmThreads = 256;

__global__ void __launch_bounds__(kGemmThreads)
    gemm_kernel(const GemmItem* __restrict__ items, int nitems, double* __restrict__ buf) {
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

cudaError_t bisect(const Sector* d_secs, int nsec, int maxn, const double* d, const double* e, double* w,
                   cudaStream_t s) {
  if (nsec <= 0) return cudaSuccess;
  constexpr int kT = 64;
  bisect_kernel<<<dim3((unsigned)((maxn + kT - 1) / kT), (unsigned)nsec), kT, 0, s>>>(d_secs, d, e, w);
  return cudaGetLastError();
}

cudaError_t inverse_iteration(const Sector* d_secs, const InvItem* d_items, int nitems, int maxn, const double* d,
                              const double* e, const double* w, double* Z, double* lu, cudaStream_t s) {
  if (nitems <= 0) return cudaSuccess;
  constexpr int kT = 64;
  inverse_iteration_kernel<<<(unsigned)((nitems + kT - 1) / kT), kT, 0, s>>>(d_secs, d_items, nitems, maxn, d, e,
                                                                            w, Z, lu);
  return cudaGetLastError();
}

cudaError_t cgs2(const CgsBlock* d_blocks, int nblocks, int maxk, double* Z, cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  cgs2_kernel<<<(unsigned)nblocks, 256, (size_t)maxk * sizeof(double), s>>>(d_blocks, Z);
  return cudaGetLastError();
}

cudaError_t gemm(const GemmItem* d_items, int nitems, int ntiles, double* buf, cudaStream_t s) {
  if (nitems <= 0 || ntiles <= 0) return cudaSuccess;
  gemm_kernel<<<(unsigned)ntiles, kGemmThreads, 0, s>>>(d_items, nitems, buf);
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
