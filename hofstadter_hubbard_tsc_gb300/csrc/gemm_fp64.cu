// Grouped segment GEMM in complex FP64 and the wave-vector kernels.
//
// One CTA owns one 64x64 output tile (or one part of a tile split for
// balance, see hh_gemm_list::upload) and accumulates every segment of it
// (c_s * opP(P_s) * opQ(Q_s), or c_s * P_s for copies) in registers before a
// single store: the sum over terms that the reference performs with
// successive ZGEMM(beta=1) calls on the same output sub-block is done here
// without atomics and in a fixed order; the parts of a split tile are added
// in slot order by seg_reduce_kernel.
#include "hh_internal.h"

#include <type_traits>

namespace hh {

namespace {

constexpr int TM = 64, TN = 64, TK = 16, NT = 256;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ const double2* resolve(long long off, int base, const double2* bin,
                                                  const double2* bscr, const double2* bout) {
  switch (base) {
    case HH_BASE_IN: return bin + off;
    case HH_BASE_SCR: return bscr + off;
    case HH_BASE_OUT: return bout + off;
    default: return reinterpret_cast<const double2*>(off);
  }
}

// One complex number as two double-float parts: re = rh + rl, im = ih + il
// (hi = the FP64 value rounded to FP32, lo = the FP32 rounding of the rest;
// 48 significand bits).
struct alignas(16) df2 {
  float rh, rl, ih, il;
};

// x = h + l to 2^-47: h is x's leading 24 significand bits (truncated), l
// the remaining 29 rounded to a float.  Built from the bit pattern on the
// integer and FP32 pipes (GB300 converts FP64 on its FP64 pipe, at 1/64 of
// the FP32 rate) wherever both parts are normal floats, |x| in [2^-74,
// 2^127], and for zero; elsewhere (tiny or huge values) by FP64 conversions.
__device__ __forceinline__ void split_f64(double x, float& h, float& l) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((u >> 52) & 0x7FF);
  if (e >= 949 && e <= 1150) {
    const unsigned sign = (unsigned)(u >> 63) << 31;
    const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
    h = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | (unsigned)(m >> 29));
    const float r = __fmul_rn(__uint2float_rn((unsigned)(m & 0x1FFFFFFFu)), __uint_as_float((unsigned)(e - 948) << 23));
    l = __uint_as_float(__float_as_uint(r) | sign);
  } else if (e == 0) {  // zero (the padding of partial tiles) or an FP64 subnormal, below every float
    h = 0.f;
    l = 0.f;
  } else {
    h = __double2float_rn(x);
    l = __double2float_rn(x - (double)h);
  }
}

__device__ __forceinline__ df2 to_df(double2 v) {
  df2 r;
  split_f64(v.x, r.rh, r.rl);
  split_f64(v.y, r.ih, r.il);
  return r;
}

// (sh, sl) += (xh + xl)(yh + yl) in double-float: the leading product with
// its exact rounding error (FMA residual, Dekker's TwoProduct), its addition
// to sh with the exact rounding error (Knuth's TwoSum), the cross products
// into sl; xl yl (2^-48 relative) is dropped.  The _rn intrinsics keep the
// compiler from fusing or reordering the error-free steps.
__device__ __forceinline__ void df_mac(float& sh, float& sl, float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh);
  const float pe = __fmaf_rn(xh, yh, -p);
  const float s = __fadd_rn(sh, p);
  const float bv = __fsub_rn(s, sh);
  const float se = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bv)), __fsub_rn(p, bv));
  sl = __fadd_rn(sl, __fadd_rn(se, pe));
  sl = __fmaf_rn(xh, yl, sl);
  sl = __fmaf_rn(xl, yh, sl);
  sh = s;
}

// (sh, sl) <- the same value with |sl| <= ulp(sh) / 2 (TwoSum of the two):
// keeps the rounding errors of the low accumulator at 2^-48 of the sum
__device__ __forceinline__ void df_renorm(float& sh, float& sl) {
  const float s = __fadd_rn(sh, sl);
  const float bv = __fsub_rn(s, sh);
  sl = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bv)), __fsub_rn(sl, bv));
  sh = s;
}

// c v for double-float complex numbers (the segment coefficient on a staged
// operand), renormalised
__device__ __forceinline__ df2 df_cmul(const df2& c, const df2& v) {
  df2 r{0.f, 0.f, 0.f, 0.f};
  df_mac(r.rh, r.rl, c.rh, c.rl, v.rh, v.rl);
  df_mac(r.rh, r.rl, -c.ih, -c.il, v.ih, v.il);
  df_mac(r.ih, r.il, c.rh, c.rl, v.ih, v.il);
  df_mac(r.ih, r.il, c.ih, c.il, v.rh, v.rl);
  df_renorm(r.rh, r.rl);
  df_renorm(r.ih, r.il);
  return r;
}

// (sh, sl) += x for an FP64 x (copy terms)
__device__ __forceinline__ void df_add(float& sh, float& sl, double x) {
  const float xh = __double2float_rn(x);
  const float xl = __double2float_rn(x - (double)xh);
  const float s = __fadd_rn(sh, xh);
  const float bv = __fsub_rn(s, sh);
  const float se = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bv)), __fsub_rn(xh, bv));
  sl = __fadd_rn(sl, __fadd_rn(se, xl));
  sh = s;
}

// Arithmetic of the segment GEMM (ARITH):
//  kArithFp64: FP64, as the reference;
//  kArithFp32: inputs rounded to FP32 as they are staged, FP32 products and
//    sums, outputs widened to FP64: for results that only start an iteration,
//    where GB300's FP32 pipe (64 times the FP64 rate) is worth the 2^-24
//    rounding;
//  kArithDf: double-float (df2 operands, df_mac): about 2^-47 relative per
//    operation, FP64-class products on the FP32 pipe (48 FP32 operations per
//    complex multiply-add, against four FP64 FMAs at 1/64 of the rate).
template <int ARITH>
__global__ void __launch_bounds__(NT, ARITH == kArithDf ? 2 : 0) seg_gemm_fp64_kernel(const hh_tile* __restrict__ tiles,
                                                          const hh_seg* __restrict__ segs,
                                                          const double2* __restrict__ bin,
                                                          double2* __restrict__ bscr,
                                                          double2* __restrict__ bout,
                                                          double2* __restrict__ part,
                                                          long long sin, long long sscr, long long sout) {
  constexpr bool F32 = ARITH == kArithFp32, DF = ARITH == kArithDf;
  using V = typename std::conditional<DF, df2, typename std::conditional<F32, float2, double2>::type>::type;
  using R = typename std::conditional<F32, float, double>::type;
  auto narrow = [](double2 v) {
    V r;
    if constexpr (DF) {
      r = to_df(v);
    } else {
      r.x = (R)v.x;
      r.y = (R)v.y;
    }
    return r;
  };
  __shared__ V Ps[TK][TM + 1];
  __shared__ V Qs[TK][TN + 1];
  const hh_tile t = tiles[blockIdx.x];
  const int b = blockIdx.y;
  const double2* in = bin + (long long)b * sin;
  double2* scr = bscr + (long long)b * sscr;
  double2* out = bout + (long long)b * sout;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int mrem = min(TM, t.M - t.m0), nrem = min(TN, t.N - t.n0);
  V acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if constexpr (DF)
        acc[i][j] = df2{0.f, 0.f, 0.f, 0.f};
      else
        acc[i][j].x = acc[i][j].y = (R)0;
    }

  for (int si = 0; si < t.nseg; ++si) {
    const hh_seg s = segs[t.seg0 + si];
    const double2 c = make_double2(s.cre, s.cim);
    const double2* P = resolve(s.poff, s.pbase, in, scr, out);
    if (s.kind == HH_SEG_COPY) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          int r = ty * 4 + i, q = tx * 4 + j;
          if (r < mrem && q < nrem) {
            double2 v = P[(long long)(t.m0 + r) + (long long)(t.n0 + q) * s.ldp];
            double2 cv = cmul(c, v);
            if constexpr (DF) {
              df_add(acc[i][j].rh, acc[i][j].rl, cv.x);
              df_add(acc[i][j].ih, acc[i][j].il, cv.y);
            } else {
              acc[i][j].x += (R)cv.x;
              acc[i][j].y += (R)cv.y;
            }
          }
        }
      continue;
    }
    const double2* Q = resolve(s.qoff, s.qbase, in, scr, out);
    // double-float: the coefficient applied after the split (FP32 pipe)
    const bool c_one = s.cre == 1.0 && s.cim == 0.0;
    df2 c_df{0.f, 0.f, 0.f, 0.f};
    if constexpr (DF) c_df = to_df(c);
    for (int k0 = 0; k0 < s.K; k0 += TK) {
      const int krem = min(TK, s.K - k0);
      // stage the P tile (TM x TK), scaled by the segment coefficient
#pragma unroll
      for (int r = 0; r < (TM * TK) / NT; ++r) {
        int e = tid + r * NT;
        int m, kk;
        if (s.opP == HH_OP_N) { m = e % TM; kk = e / TM; } else { kk = e % TK; m = e / TK; }
        double2 v = make_double2(0.0, 0.0);
        if (m < mrem && kk < krem) {
          if (s.opP == HH_OP_N) {
            v = P[(long long)(t.m0 + m) + (long long)(k0 + kk) * s.ldp];
          } else {
            v = P[(long long)(k0 + kk) + (long long)(t.m0 + m) * s.ldp];
            if (s.opP == HH_OP_C) v.y = -v.y;
          }
          if constexpr (!DF) v = cmul(c, v);
        }
        if constexpr (DF)
          Ps[kk][m] = c_one ? to_df(v) : df_cmul(c_df, to_df(v));
        else
          Ps[kk][m] = narrow(v);
      }
#pragma unroll
      for (int r = 0; r < (TN * TK) / NT; ++r) {
        int e = tid + r * NT;
        int n, kk;
        if (s.opQ == HH_OP_N) { kk = e % TK; n = e / TK; } else { n = e % TN; kk = e / TN; }
        double2 v = make_double2(0.0, 0.0);
        if (n < nrem && kk < krem) {
          if (s.opQ == HH_OP_N) {
            v = Q[(long long)(k0 + kk) + (long long)(t.n0 + n) * s.ldq];
          } else {
            v = Q[(long long)(t.n0 + n) + (long long)(k0 + kk) * s.ldq];
            if (s.opQ == HH_OP_C) v.y = -v.y;
          }
        }
        Qs[kk][n] = narrow(v);
      }
      __syncthreads();
      if constexpr (DF) {
        // B operands one at a time, no unrolling over k: the accumulators
        // fill the registers of two CTAs per SM
#pragma unroll 1
        for (int kk = 0; kk < TK; ++kk) {
          df2 a[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) a[i] = Ps[kk][ty * 4 + i];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const df2 q = Qs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              df2& z = acc[i][j];
              df_mac(z.rh, z.rl, a[i].rh, a[i].rl, q.rh, q.rl);
              df_mac(z.rh, z.rl, -a[i].ih, -a[i].il, q.ih, q.il);
              df_mac(z.ih, z.il, a[i].rh, a[i].rl, q.ih, q.il);
              df_mac(z.ih, z.il, a[i].ih, a[i].il, q.rh, q.rl);
            }
          }
        }
      }
#pragma unroll 4
      for (int kk = 0; kk < (DF ? 0 : TK); ++kk) {
        V a[4], bb[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = Ps[kk][ty * 4 + i];
#pragma unroll
        for (int j = 0; j < 4; ++j) bb[j] = Qs[kk][tx * 4 + j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            if constexpr (!DF) {
              acc[i][j].x = fma(a[i].x, bb[j].x, acc[i][j].x);
              acc[i][j].x = fma(-a[i].y, bb[j].y, acc[i][j].x);
              acc[i][j].y = fma(a[i].x, bb[j].y, acc[i][j].y);
              acc[i][j].y = fma(a[i].y, bb[j].x, acc[i][j].y);
            }
          }
      }
      if constexpr (DF) {  // once per 16 k: the low parts stay small
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            df_renorm(acc[i][j].rh, acc[i][j].rl);
            df_renorm(acc[i][j].ih, acc[i][j].il);
          }
      }
      __syncthreads();
    }
  }
  // the accumulator as FP64
  auto wide = [](const V& z) {
    if constexpr (DF)
      return make_double2((double)z.rh + (double)z.rl, (double)z.ih + (double)z.il);
    else
      return make_double2((double)z.x, (double)z.y);
  };
  if (t.part >= 0) {
    // partial sum of a split tile: the whole 64x64 slot, column-major
    double2* S = part + (long long)t.part * (TM * TN);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) S[(ty * 4 + i) + (tx * 4 + j) * TM] = wide(acc[i][j]);
    return;
  }
  double2* O = (t.obase == HH_BASE_SCR) ? scr : out;
  O += t.ooff;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int r = ty * 4 + i, q = tx * 4 + j;
      if (r < mrem && q < nrem) {
        long long idx = (long long)(t.m0 + r) + (long long)(t.n0 + q) * t.ldo;
        const double2 v = wide(acc[i][j]);
        if (t.accumulate) {
          double2 o = O[idx];
          o.x += v.x;
          o.y += v.y;
          O[idx] = o;
        } else {
          O[idx] = v;
        }
      }
    }
}

// out (+)= sum over the parts of a split tile, in slot order
__global__ void __launch_bounds__(NT) seg_reduce_kernel(const hh_red* __restrict__ reds,
                                                        const double2* __restrict__ part,
                                                        double2* __restrict__ bscr, double2* __restrict__ bout) {
  const hh_red r = reds[blockIdx.x];
  const int mrem = min(TM, r.M - r.m0), nrem = min(TN, r.N - r.n0);
  double2* O = ((r.obase == HH_BASE_SCR) ? bscr : bout) + r.ooff;
  for (int e = threadIdx.x; e < TM * TN; e += NT) {
    const int m = e % TM, n = e / TM;
    if (m >= mrem || n >= nrem) continue;
    double2 v = make_double2(0.0, 0.0);
    for (int p = 0; p < r.nparts; ++p) {
      const double2 x = part[(long long)(r.part0 + p) * (TM * TN) + e];
      v.x += x.x;
      v.y += x.y;
    }
    const long long idx = (long long)(r.m0 + m) + (long long)(r.n0 + n) * r.ldo;
    if (r.accumulate) {
      double2 o = O[idx];
      o.x += v.x;
      o.y += v.y;
      O[idx] = o;
    } else {
      O[idx] = v;
    }
  }
}

// ----------------------------------------------------------- wave vectors
constexpr int RB = 256;

__global__ void dot_partial_kernel(const double2* a, const double2* b, long long n, double* part) {
  __shared__ double sh[RB / 32];
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)RB + threadIdx.x; i < n; i += (long long)gridDim.x * RB) {
    double2 x = a[i], y = b[i];
    s = fma(x.x, y.x, s);
    s = fma(x.y, y.y, s);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < RB / 32 ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
  }
}

__global__ void sum_kernel(const double* part, int n, double* out) {
  __shared__ double sh[RB / 32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += RB) s += part[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < RB / 32 ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[0] = s;
  }
}

__global__ void axpy_kernel(double2* y, const double2* x, double a, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double2 v = y[i], u = x[i];
    v.x = fma(a, u.x, v.x);
    v.y = fma(a, u.y, v.y);
    y[i] = v;
  }
}

__global__ void axpy_dev_kernel(double2* y, const double2* x, const double* sc, double sign, long long n) {
  const double a = sign * sc[0];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double2 v = y[i], u = x[i];
    v.x = fma(a, u.x, v.x);
    v.y = fma(a, u.y, v.y);
    y[i] = v;
  }
}

__global__ void scale_rsqrt_kernel(double2* y, const double* sc, double* root, long long n) {
  const double r = sqrt(sc[0]);
  const double a = 1.0 / r;
  if (root && blockIdx.x == 0 && threadIdx.x == 0) root[0] = r;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double2 v = y[i];
    v.x *= a;
    v.y *= a;
    y[i] = v;
  }
}

__global__ void divide_kernel(double* c, const double* d, int k) {
  for (int j = threadIdx.x; j < k; j += blockDim.x) c[j] /= d[j];
}

__global__ void scale_kernel(double2* y, double a, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double2 v = y[i];
    v.x *= a;
    v.y *= a;
    y[i] = v;
  }
}

// Re<V_j, w> for j < k: one pass over w; partial sums per CTA, k <= 128.
constexpr int KMAX = 128;
// V holds double2 vectors, or float2 ones (the split Lanczos's first pass
// keeps its Krylov basis in FP32).  With float2 vectors the products run in
// double-float on the FP32 pipe (df_mac; the FP64 operand split once per
// element by split_f64): an FP64 FMA costs GB300 as much issue as some 80
// FP32 operations, and these kernels make two per element and vector.
template <class VT>
__global__ void krylov_dots_kernel(const VT* V, int k, long long ld, const double2* w, long long n,
                                   double* part) {
  constexpr bool F32V = std::is_same<VT, float2>::value;
  __shared__ double sh[KMAX][RB / 32 + 1];
  double acc[8];
  float dh[8], dl[8];
  for (int j0 = 0; j0 < k; j0 += 8) {
    int jn = min(8, k - j0);
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] = 0.0, dh[j] = dl[j] = 0.f;
    for (long long i = blockIdx.x * (long long)RB + threadIdx.x; i < n; i += (long long)gridDim.x * RB) {
      double2 x = w[i];
      if constexpr (F32V) {
        float xh, xl, yh, yl;
        split_f64(x.x, xh, xl);
        split_f64(x.y, yh, yl);
#pragma unroll
        for (int j = 0; j < 8; ++j)
          if (j < jn) {
            const float2 v = reinterpret_cast<const float2*>(V)[(long long)(j0 + j) * ld + i];
            df_mac(dh[j], dl[j], v.x, 0.f, xh, xl);
            df_mac(dh[j], dl[j], v.y, 0.f, yh, yl);
          }
      } else {
#pragma unroll
        for (int j = 0; j < 8; ++j)
          if (j < jn) {
            const double2 v = reinterpret_cast<const double2*>(V)[(long long)(j0 + j) * ld + i];
            acc[j] = fma(v.x, x.x, acc[j]);
            acc[j] = fma(v.y, x.y, acc[j]);
          }
      }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      double s = F32V ? (double)dh[j] + (double)dl[j] : acc[j];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if ((threadIdx.x & 31) == 0 && j < jn) sh[j0 + j][threadIdx.x >> 5] = s;
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < k; j += RB) {
    double s = 0.0;
    for (int q = 0; q < RB / 32; ++q) s += sh[j][q];
    part[(long long)blockIdx.x * KMAX + j] = s;
  }
}

__global__ void krylov_reduce_kernel(const double* part, int nblk, int k, double* out) {
  int j = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += part[(long long)b * KMAX + j];
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[j] = s;
  }
}

// w -= sum_j c_j V_j  (sign = -1) or out = sum_j c_j V_j (sign = 0)
template <class VT>
__global__ void krylov_axpy_kernel(const VT* V, int k, long long ld, double2* w, long long n,
                                   const double* coef, int overwrite) {
  constexpr bool F32V = std::is_same<VT, float2>::value;
  __shared__ double c[KMAX];
  __shared__ float ch[KMAX], cl[KMAX];  // float2 vectors: the coefficients split once
  for (int j = threadIdx.x; j < k; j += blockDim.x) {
    c[j] = coef[j];
    if constexpr (F32V) split_f64(coef[j], ch[j], cl[j]);
  }
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double2 s = make_double2(0.0, 0.0);
    if constexpr (F32V) {
      float xh = 0.f, xl = 0.f, yh = 0.f, yl = 0.f;
      for (int j = 0; j < k; ++j) {
        const float2 v = reinterpret_cast<const float2*>(V)[(long long)j * ld + i];
        df_mac(xh, xl, ch[j], cl[j], v.x, 0.f);
        df_mac(yh, yl, ch[j], cl[j], v.y, 0.f);
      }
      s = make_double2((double)xh + (double)xl, (double)yh + (double)yl);
    } else {
      for (int j = 0; j < k; ++j) {
        const double2 v = reinterpret_cast<const double2*>(V)[(long long)j * ld + i];
        s.x = fma(c[j], v.x, s.x);
        s.y = fma(c[j], v.y, s.y);
      }
    }
    if (overwrite) {
      w[i] = s;
    } else {
      double2 o = w[i];
      o.x -= s.x;
      o.y -= s.y;
      w[i] = o;
    }
  }
}

// v = FP32 rounding of w, and the partial sums of <v|v> per CTA (sum_kernel
// finishes them): a new Krylov vector stored in FP32 with the norm of what
// was stored
__global__ void store_f32_kernel(const double2* __restrict__ w, float2* __restrict__ v, long long n,
                                 double* __restrict__ part) {
  __shared__ double sh[RB / 32];
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)RB + threadIdx.x; i < n; i += (long long)gridDim.x * RB) {
    const double2 x = w[i];
    const float2 f = make_float2(__double2float_rn(x.x), __double2float_rn(x.y));
    v[i] = f;
    s = fma((double)f.x, (double)f.x, s);
    s = fma((double)f.y, (double)f.y, s);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < RB / 32 ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
  }
}

int grid_for(long long n, int threads) {
  long long g = (n + threads - 1) / threads;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long cap = (long long)sms * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace

namespace {
// counter-based generator (splitmix64) so that a seed gives the same wave on every GPU
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__global__ void random_kernel(double2* w, long long n, unsigned long long seed) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    unsigned long long a = mix64(seed ^ (2ull * i)), b = mix64(seed ^ (2ull * i + 1));
    w[i] = make_double2((double)(a >> 11) * 0x1.0p-53, (double)(b >> 11) * 0x1.0p-53);
  }
}
}  // namespace

cudaError_t wave_fill_random(double2* w, long long n, unsigned long long seed, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  random_kernel<<<grid_for(n, 256), 256, 0, s>>>(w, n, seed);
  return cudaGetLastError();
}

cudaError_t launch_segment_gemm_fp64(const hh_gemm_list& L, double2* base_in, double2* base_scr,
                                     double2* base_out, cudaStream_t s, int arith) {
  if (L.n_work == 0) return cudaSuccess;
  // grid.x = work tiles; the 65535 limit applies to grid.y only
  dim3 grid((unsigned)L.n_work, 1);
  if (arith == kArithFp32)
    seg_gemm_fp64_kernel<kArithFp32><<<grid, NT, 0, s>>>(L.d_tiles, L.d_segs, base_in, base_scr, base_out, L.d_part,
                                                         0, 0, 0);
  else if (arith == kArithDf)
    seg_gemm_fp64_kernel<kArithDf><<<grid, NT, 0, s>>>(L.d_tiles, L.d_segs, base_in, base_scr, base_out, L.d_part,
                                                       0, 0, 0);
  else
    seg_gemm_fp64_kernel<kArithFp64><<<grid, NT, 0, s>>>(L.d_tiles, L.d_segs, base_in, base_scr, base_out, L.d_part,
                                                         0, 0, 0);
  if (L.n_red > 0) seg_reduce_kernel<<<(unsigned)L.n_red, NT, 0, s>>>(L.d_reds, L.d_part, base_scr, base_out);
  return cudaGetLastError();
}

// Loads the two kernels above into the current context now (CUDA loads
// modules and functions lazily, at first launch, by default), so that a later
// launch reserves no device memory for their code.
cudaError_t preload_segment_gemm_fp64() {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, seg_gemm_fp64_kernel<kArithFp64>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, seg_reduce_kernel);
  return e;
}

cudaError_t wave_dot(const double2* a, const double2* b, long long n, double* d_out, cudaStream_t s) {
  // d_out must hold >= 1 + nblocks doubles: [0] result, [1..] partials
  int g = grid_for(n, RB);
  if (g > 1024) g = 1024;
  dot_partial_kernel<<<g, RB, 0, s>>>(a, b, n, d_out + 1);
  sum_kernel<<<1, RB, 0, s>>>(d_out + 1, g, d_out);
  return cudaGetLastError();
}

cudaError_t wave_dot_into(const double2* a, const double2* b, long long n, double* result, double* part,
                          cudaStream_t s) {
  int g = grid_for(n, RB);
  if (g > 1024) g = 1024;
  dot_partial_kernel<<<g, RB, 0, s>>>(a, b, n, part);
  sum_kernel<<<1, RB, 0, s>>>(part, g, result);
  return cudaGetLastError();
}

cudaError_t wave_axpy_dev(double2* y, const double2* x, const double* sc, double sign, long long n, cudaStream_t s) {
  axpy_dev_kernel<<<grid_for(n, 256), 256, 0, s>>>(y, x, sc, sign, n);
  return cudaGetLastError();
}

cudaError_t wave_scale_rsqrt_dev(double2* y, const double* sc, double* root, long long n, cudaStream_t s) {
  scale_rsqrt_kernel<<<grid_for(n, 256), 256, 0, s>>>(y, sc, root, n);
  return cudaGetLastError();
}

cudaError_t divide_dev(double* c, const double* d, int k, cudaStream_t s) {
  if (k > 0) divide_kernel<<<1, 128, 0, s>>>(c, d, k);
  return cudaGetLastError();
}

cudaError_t wave_axpy(double2* y, const double2* x, double a, long long n, cudaStream_t s) {
  axpy_kernel<<<grid_for(n, 256), 256, 0, s>>>(y, x, a, n);
  return cudaGetLastError();
}

cudaError_t wave_scale(double2* y, double a, long long n, cudaStream_t s) {
  scale_kernel<<<grid_for(n, 256), 256, 0, s>>>(y, a, n);
  return cudaGetLastError();
}

template <class VT>
cudaError_t krylov_dots(const VT* V, int k, long long ld, const double2* w, long long n, double* d_out,
                        cudaStream_t s) {
  // d_out: [0, KMAX) results, then nblk*KMAX partials
  if (k > KMAX) return cudaErrorInvalidValue;
  int g = grid_for(n, RB);
  if (g > 512) g = 512;
  krylov_dots_kernel<VT><<<g, RB, 0, s>>>(V, k, ld, w, n, d_out + KMAX);
  krylov_reduce_kernel<<<k, 256, 0, s>>>(d_out + KMAX, g, k, d_out);
  return cudaGetLastError();
}

template <class VT>
cudaError_t krylov_update(const VT* V, int k, long long ld, double2* w, long long n, const double* d_coef,
                          cudaStream_t s) {
  if (k > KMAX) return cudaErrorInvalidValue;
  krylov_axpy_kernel<VT><<<grid_for(n, 256), 256, 0, s>>>(V, k, ld, w, n, d_coef, 0);
  return cudaGetLastError();
}

template <class VT>
cudaError_t krylov_combine(const VT* V, int k, long long ld, double2* out, long long n, const double* d_coef,
                           cudaStream_t s) {
  if (k > KMAX) return cudaErrorInvalidValue;
  krylov_axpy_kernel<VT><<<grid_for(n, 256), 256, 0, s>>>(V, k, ld, out, n, d_coef, 1);
  return cudaGetLastError();
}

template cudaError_t krylov_dots<double2>(const double2*, int, long long, const double2*, long long, double*,
                                          cudaStream_t);
template cudaError_t krylov_dots<float2>(const float2*, int, long long, const double2*, long long, double*,
                                         cudaStream_t);
template cudaError_t krylov_update<double2>(const double2*, int, long long, double2*, long long, const double*,
                                            cudaStream_t);
template cudaError_t krylov_update<float2>(const float2*, int, long long, double2*, long long, const double*,
                                           cudaStream_t);
template cudaError_t krylov_combine<double2>(const double2*, int, long long, double2*, long long, const double*,
                                             cudaStream_t);
template cudaError_t krylov_combine<float2>(const float2*, int, long long, double2*, long long, const double*,
                                            cudaStream_t);

cudaError_t krylov_store_f32(const double2* w, float2* v, long long n, double* vv, double* part, cudaStream_t s) {
  int g = grid_for(n, RB);
  if (g > 1024) g = 1024;
  store_f32_kernel<<<g, RB, 0, s>>>(w, v, n, part);
  sum_kernel<<<1, RB, 0, s>>>(part, g, vv);
  return cudaGetLastError();
}

}  // namespace hh
