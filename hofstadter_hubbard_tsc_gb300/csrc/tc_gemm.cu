// Split-precision tensor-core path of the block-sparse matvec (sm_103a).
//
// Every complex FP64 operand is carried as six BF16 planes: re0 im0 re1 im1
// re2 im2 with x = x0 + x1 + x2 (x0 = bf16(x), x1 = bf16(x - x0), ...), i.e.
// 24 significand bits.  The kernels use the first SPLIT parts of each:
//   SPLIT = 3 (BF16x6): the six split products with i + j <= 2 for each of
//     the four real products (re.re, im.im, re.im, im.re), 24 tcgen05.mma
//     (M=128, K=16, FP32 accumulate in TMEM) per 16 complex k; the dropped
//     products are below 2^-24 relative;
//   SPLIT = 2 (BF16x3): x0 y0 + x0 y1 + x1 y0, 12 MMAs per 16 complex k and
//     two thirds of the operand bytes; dropped terms about 2^-16 relative.
// Both read the same images (their first 2 SPLIT planes).  The tensor core rounds
// every accumulation toward zero, so the leading products x0 y0 and the five
// correction products go to separate accumulators (main: TMEM columns
// [0,2NT), correction: [2NT,4NT), re then im): the correction terms, 2^-8 of
// the main ones, then cost no accumulator precision, and the bias of the main
// accumulator grows with 2 instead of 4 (SPLIT 2) or 12 (SPLIT 3)
// accumulations per 16 complex k.  The
// epilogue adds the two in FP64.  The -im.im product uses the negate-A bit of
// the instruction descriptor.
//
// Stacked tiles (at most 64 rows): the M = 128 MMA costs the same at 64 rows,
// and a K = 16 MMA costs about max(45, N/2) SM cycles whatever its M
// (measured: 45 at N <= 64, 64 at N = 128, 128 at N = 256).  So for a tile
// of at most 64 rows the re and im parts of A share one operand (re rows
// from 0, im rows from row h <= 64) and B's re and im parts are adjacent rows
// of one 2N-row operand: ONE MMA of width 2N per part pair gives all four
// real products,
//   D[r][c] = Ar Br, D[r][N+c] = Ar Bi, D[h+r][c] = Ai Br, D[h+r][N+c] = Ai Bi,
// in place of four MMAs of width N (2x to 4x fewer MMA cycles).  The epilogue
// combines re = Ar Br - Ai Bi and im = Ar Bi + Ai Br across the lanes
// through a 4 KB shared-memory exchange.  Same main / correction
// accumulators, operand bytes and TMEM columns.
//
// Operand "images": a complex matrix used as an MMA operand with R rows and
// Kc complex k is stored as BF16 in the canonical K-major no-swizzle UMMA
// layout, padded to Rpad = roundup(R,16) rows and K16 = roundup(Kc,16):
//   byte offset of core matrix (chunk kc, plane p, row group g, k half h) =
//     ((kc * 6 + p) * (Rpad / 8) + g) * 256 + h * 128
//   inside it, row r%8 occupies 16 bytes holding k%8 = 0..7; LBO = 128 B
//   (next 8 k), SBO = 256 B (next 8 rows).
// The rows of one plane and one 16-wide k chunk are contiguous, and so are
// the planes of one chunk: a tile that spans its operand's whole (padded)
// height loads the first 2 SPLIT planes of a chunk with ONE cp.async.bulk
// ("packed"; a bulk copy costs about 30 ns of the SM's copy engine below
// 1 KB, so eight small copies per chunk limited the kernel); other tiles
// load one copy per plane.  In shared memory, A plane q sits at
// (q / 2) * a_pair + (q % 2) * a_im (packed: the image's own plane stride;
// per plane: 128-row slots, or 64-row halves when stacked) and B plane q at
// q * ntile rows (packed B needs planes exactly ntile rows high).
#include <cuda_bf16.h>
#include <cstdint>
#include <vector>

#include "hh_internal.h"
#include "tc.h"

namespace hh {
namespace tc {

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Attempts per bounded mbarrier wait.  One try_wait attempt (it may suspend
// the thread) plus the back-off costs about 5 us on GB300 (measured by the
// held-tile check: 2^12 attempts in ~20 ms), so a wait gives up after about
// 5 s: far beyond any legitimate wait here (a tile's MMAs take at most
// milliseconds) and short enough to report instead of appearing hung.
constexpr uint32_t kWaitLimit = 1u << 20;

// bounded wait on an mbarrier phase (at most `limit` try_wait attempts);
// returns false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = kWaitLimit) {
  const uint32_t addr = smem_u32(bar);
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
    if (i > 64) __nanosleep(32);
  }
  return false;
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  // start address >> 4 (bits 0-13), LBO = 128 B (bits 16-29), SBO = 256 B
  // (bits 32-45), version 1 (bits 46-47), no swizzle (bits 61-63 = 0)
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((128u >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((256u >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

__host__ __device__ constexpr uint32_t idesc_bf16(int n, bool neg_a) {
  // D f32 (bits 4-5 = 1), A bf16 (7-9 = 1), B bf16 (10-12 = 1), negate A
  // (bit 13), K-major A and B (bits 15, 16 = 0), N >> 3 (17-22), M >> 4 (24-28)
  return (1u << 4) | (1u << 7) | (1u << 10) | (neg_a ? (1u << 13) : 0u) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ------------------------------------------------------------------ splitting
__device__ __forceinline__ void split3d(double x, __nv_bfloat16* o) {
  __nv_bfloat16 a = __double2bfloat16(x);
  double r = x - (double)__bfloat162float(a);
  __nv_bfloat16 b = __double2bfloat16(r);
  r = r - (double)__bfloat162float(b);
  o[0] = a;
  o[1] = b;
  o[2] = __double2bfloat16(r);
}

__device__ __forceinline__ void split3f(float x, __nv_bfloat16* o) {
  __nv_bfloat16 a = __float2bfloat16_rn(x);
  float r = x - __bfloat162float(a);
  __nv_bfloat16 b = __float2bfloat16_rn(r);
  r = r - __bfloat162float(b);
  o[0] = a;
  o[1] = b;
  o[2] = __float2bfloat16_rn(r);
}

__device__ __forceinline__ uint4 pack8(const __nv_bfloat16* v) {
  uint32_t w[4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
    w[i] = (uint32_t)__bfloat16_as_ushort(v[2 * i]) | ((uint32_t)__bfloat16_as_ushort(v[2 * i + 1]) << 16);
  return make_uint4(w[0], w[1], w[2], w[3]);
}

__device__ __forceinline__ size_t img_off(int rpad, int r, int k) {
  // byte offset of the 16-byte row chunk (row r, k rounded down to 8) in plane 0
  return ((size_t)((k >> 4) * 6) * (rpad >> 3) + (r >> 3)) * 256 + ((k >> 3) & 1) * 128 + (r & 7) * 16;
}

// ------------------------------------------------------------------ image build
// One CTA per task: value(r,k) = coef * (conj?) src[trans ? k + r*ld : r + k*ld]
// for r < rows, k < kc, zero in the padding; the first SPLIT BF16 parts of
// re and im are written (planes 2p and 2p + 1).  The value is rounded to FP32
// first and scaled and split in FP32: three BF16 parts hold FP32's 24
// significand bits, and GB300 retires FP32 at 64 times its FP64 rate.
// Operator images (built once per plan, all three parts) keep the FP64 split.
// With a block list (blocks != nullptr), block b converts row groups
// [blocks[b].y, blocks[b].y + kImgGroupsPerBlock) of task blocks[b].x, so
// that large and small images spread evenly over the SMs; without one, block
// b converts all of task b.
constexpr int kImgGroupsPerBlock = 256;

template <bool kFp32, int SPLIT>
__global__ void __launch_bounds__(256) build_images_kernel(const ImgTask* __restrict__ tasks,
                                                           const int2* __restrict__ blocks,
                                                           const double2* __restrict__ base_in,
                                                           const IoPtrs* __restrict__ io) {
  if (io) base_in = io->in;
  const int2 bw = blocks ? blocks[blockIdx.x] : make_int2((int)blockIdx.x, 0);
  const ImgTask t = tasks[bw.x];
  const double2* src = t.sbase == HH_BASE_IN ? base_in + t.src : reinterpret_cast<const double2*>(t.src);
  uint8_t* dst = reinterpret_cast<uint8_t*>(t.dst);
  const int rpad = t.rpad, k16 = t.k16, prow = t.prow;
  const size_t plane = (size_t)(rpad >> 3) * 256;
  const int ngroups = prow * (k16 >> 3);
  const int g_end = blocks ? min(ngroups, bw.y + kImgGroupsPerBlock) : ngroups;
  const float fre = (float)t.cre, fim = (float)t.cim;
  for (int idx = bw.y + threadIdx.x; idx < g_end; idx += blockDim.x) {
    const int r = idx % prow, k0 = (idx / prow) * 8;  // r: row of this task's operator
    __nv_bfloat16 re[3][8], im[3][8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int k = k0 + j;
      __nv_bfloat16 s[3];
      if (kFp32) {
        float2 v = make_float2(0.f, 0.f);
        if (r < t.rows && k < t.kc) {
          const double2 d = t.trans ? src[(long long)k + (long long)r * t.ld] : src[(long long)r + (long long)k * t.ld];
          v = make_float2((float)d.x, t.conj ? -(float)d.y : (float)d.y);
          v = make_float2(fre * v.x - fim * v.y, fre * v.y + fim * v.x);
        }
        split3f(v.x, s);
        re[0][j] = s[0]; re[1][j] = s[1]; re[2][j] = s[2];
        split3f(v.y, s);
        im[0][j] = s[0]; im[1][j] = s[1]; im[2][j] = s[2];
      } else {
        double2 v = make_double2(0.0, 0.0);
        if (r < t.rows && k < t.kc) {
          v = t.trans ? src[(long long)k + (long long)r * t.ld] : src[(long long)r + (long long)k * t.ld];
          if (t.conj) v.y = -v.y;
          v = make_double2(t.cre * v.x - t.cim * v.y, t.cre * v.y + t.cim * v.x);
        }
        split3d(v.x, s);
        re[0][j] = s[0]; re[1][j] = s[1]; re[2][j] = s[2];
        split3d(v.y, s);
        im[0][j] = s[0]; im[1][j] = s[1]; im[2][j] = s[2];
      }
    }
    const size_t o = img_off(rpad, t.row0 + r, k0);
#pragma unroll
    for (int p = 0; p < SPLIT; ++p) {
      *reinterpret_cast<uint4*>(dst + o + (size_t)(2 * p) * plane) = pack8(re[p]);
      *reinterpret_cast<uint4*>(dst + o + (size_t)(2 * p + 1) * plane) = pack8(im[p]);
    }
  }
}

// ------------------------------------------------------------------ tile GEMM
constexpr int kPlaneA = 128 * 32;            // 128 rows x 16 bf16
constexpr int kThreads = 192;                // producer, MMA, 4 epilogue warps

// one pipeline stage: 2*SPLIT planes of A (128 rows) and of B (NT rows)
__host__ __device__ constexpr int stage_bytes_of(int nt, int split) { return 2 * split * (kPlaneA + nt * 32); }

__device__ __forceinline__ void flag_error(int* err, int code) {
  if (err) atomicCAS(err, 0, code);
}

// Copies of chunk kc of segment sg into one stage (A planes from sa, B planes
// from sa + a_region), completing on bar: planes 0 .. 2 SPLIT - 1 (re and im
// of the first SPLIT parts), as one copy per operand when the tile is
// packed, else one per plane.
template <int SPLIT>
__device__ __forceinline__ void load_chunk(uint8_t* sa, int a_region, const Tile& t, const Seg& sg, int kc,
                                           uint64_t* bar) {
  uint8_t* sb = sa + a_region;
  mbar_expect_tx(bar, 2u * SPLIT * (sg.a_bytes + sg.b_bytes));
  const uint8_t* ga = reinterpret_cast<const uint8_t*>(sg.a) + (size_t)kc * 6 * sg.a_plane;
  const uint8_t* gb = reinterpret_cast<const uint8_t*>(sg.b) + (size_t)kc * 6 * sg.b_plane;
  if (t.pack & 1) {
    bulk_g2s(sa, ga, 2u * SPLIT * sg.a_bytes, bar);
  } else {
#pragma unroll
    for (int q = 0; q < 2 * SPLIT; ++q)
      bulk_g2s(sa + (q >> 1) * t.a_pair + (q & 1) * t.a_im, ga + (size_t)q * sg.a_plane, sg.a_bytes, bar);
  }
  if (t.pack & 2) {
    bulk_g2s(sb, gb, 2u * SPLIT * sg.b_bytes, bar);
  } else {
#pragma unroll
    for (int q = 0; q < 2 * SPLIT; ++q)
      bulk_g2s(sb + q * (t.ntile * 32), gb + (size_t)q * sg.b_plane, sg.b_bytes, bar);
  }
}

// The split products of one staged chunk: parts i + j < SPLIT of the four
// real products; x0 y0 into the main accumulators (columns [0, 2NT)), the
// others into the correction accumulators ([2NT, 4NT)).  acc / acc_c: 0 for
// the first chunk of a tile (overwrite), then 1.
template <int SPLIT, int NT>
__device__ __forceinline__ void mma_chunk(uint32_t sa, int a_region, const Tile& t, uint32_t tmem, uint32_t& acc,
                                          uint32_t& acc_c) {
  const uint32_t sb = sa + a_region;
  const int ntile = t.ntile;
  const uint32_t d_re = tmem, d_im = tmem + NT, c_re = tmem + 2 * NT, c_im = tmem + 3 * NT;
  if (t.stack) {
    // main: columns [0, 2 ntile), correction: [2 NT, 2 NT + 2 ntile)
    const uint32_t id2 = idesc_bf16(2 * ntile, false);
#pragma unroll
    for (int i = 0; i < SPLIT; ++i) {
#pragma unroll
      for (int j = 0; j < SPLIT - i; ++j) {
        const uint64_t a = smem_desc(sa + i * t.a_pair), b = smem_desc(sb + 2 * j * ntile * 32);
        if (i + j == 0) {
          mma_bf16(d_re, a, b, id2, acc);
          acc = 1u;
        } else {
          mma_bf16(c_re, a, b, id2, acc_c);
          acc_c = 1u;
        }
      }
    }
    return;
  }
  const uint32_t id_pos = idesc_bf16(ntile, false), id_neg = idesc_bf16(ntile, true);
#pragma unroll
  for (int i = 0; i < SPLIT; ++i) {
#pragma unroll
    for (int j = 0; j < SPLIT - i; ++j) {
      const uint64_t are = smem_desc(sa + i * t.a_pair), aim = smem_desc(sa + i * t.a_pair + t.a_im);
      const uint64_t bre = smem_desc(sb + 2 * j * ntile * 32), bim = smem_desc(sb + (2 * j + 1) * ntile * 32);
      if (i + j == 0) {
        mma_bf16(d_re, are, bre, id_pos, acc);
        mma_bf16(d_re, aim, bim, id_neg, 1u);
        mma_bf16(d_im, are, bim, id_pos, acc);
        mma_bf16(d_im, aim, bre, id_pos, 1u);
        acc = 1u;
      } else {
        mma_bf16(c_re, are, bre, id_pos, acc_c);
        mma_bf16(c_re, aim, bim, id_neg, 1u);
        mma_bf16(c_im, are, bim, id_pos, acc_c);
        mma_bf16(c_im, aim, bre, id_pos, 1u);
        acc_c = 1u;
      }
    }
  }
}

// Epilogue of accumulator columns [c0, c0 + 16) for one row of the tile:
// main + correction summed in FP32 (one rounding at 2^-24), then either
// stored to the output wave (mode 0; the FP64 copy terms follow in
// copy_terms_kernel) or split into the T image (mode 1: rows of T, k = T
// columns, zero outside the valid rectangle, the SPLIT parts the next stage
// reads).
template <int SPLIT>
__device__ __forceinline__ void epilogue16(const Tile& t, int row, int c0, const float* re, const float* im,
                                           const float* cr, const float* cm, double2* base_out,
                                           const TPiece* __restrict__ pieces) {
  if (t.mode == 0) {
    if (row < t.mrem) {
      double2* O = base_out + t.out;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int col = c0 + j;
        if (col < t.nrem) O[(long long)row + (long long)col * t.ldo] = make_double2(re[j] + cr[j], im[j] + cm[j]);
      }
    }
    return;
  }
  int r = t.m0 + row;        // row of the T image
  bool vrow = row < t.mrem;  // a row of the product (else zero padding)
  uint8_t* img = reinterpret_cast<uint8_t*>(t.out);
  int trp = t.t_rpad;
  if (t.npiece > 0) {  // row-packed tile: this row's product and its T image
    int k = 0;
    while (k < t.npiece && row >= pieces[t.piece0 + k].row0 + pieces[t.piece0 + k].t_rpad) ++k;
    if (k == t.npiece) return;
    const TPiece pc = pieces[t.piece0 + k];
    r = row - pc.row0;
    vrow = r < pc.rows;
    img = reinterpret_cast<uint8_t*>(pc.out);
    trp = pc.t_rpad;
  }
  if (r < 0 || r >= trp) return;
  const size_t plane = (size_t)(trp >> 3) * 256;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    __nv_bfloat16 pr[3][8], pi[3][8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int cc = c0 + h * 8 + j;
      const bool valid = vrow && cc < t.nrem;
      __nv_bfloat16 s3[3];
      split3f(valid ? re[h * 8 + j] + cr[h * 8 + j] : 0.f, s3);
      pr[0][j] = s3[0]; pr[1][j] = s3[1]; pr[2][j] = s3[2];
      split3f(valid ? im[h * 8 + j] + cm[h * 8 + j] : 0.f, s3);
      pi[0][j] = s3[0]; pi[1][j] = s3[1]; pi[2][j] = s3[2];
    }
    const size_t o = img_off(trp, r, t.n0 + c0 + h * 8);
#pragma unroll
    for (int p = 0; p < SPLIT; ++p) {
      *reinterpret_cast<uint4*>(img + o + (size_t)(2 * p) * plane) = pack8(pr[p]);
      *reinterpret_cast<uint4*>(img + o + (size_t)(2 * p + 1) * plane) = pack8(pi[p]);
    }
  }
}

// Named barriers of the four epilogue warps (128 threads; barrier 0 is the
// CTA-wide one): 1 for the stacked exchange, 2 for the per-tile abort vote.
__device__ __forceinline__ void epi_sync() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

__device__ __forceinline__ bool epi_any(bool p) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred pi, po;\n setp.ne.u32 pi, %1, 0;\n bar.red.or.pred po, 2, 128, pi;\n selp.u32 %0, 1, 0, po;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)p)
      : "memory");
  return r != 0;
}

constexpr int kXbufBytes = 16 * 64 * 4;  // stacked exchange: 64 rows x (8 + 8) floats
constexpr int kMaxStages = 16;           // barriers of the per-tile kernel's variable pipeline

// Epilogue of one tile by epilogue warp q (TMEM lanes 32q .. 32q + 31).  All
// four epilogue warps call it for every tile with the same tile, so the
// stacked exchange's barriers always see all of them.  Plain tiles: main
// (re, im) and correction (re, im) blocks at columns 0, NT, 2NT, 3NT.
// Stacked tiles (im rows from h = a_im / 32 <= 64): the main block
// [Ar Br | Ar Bi] on lanes 0 .. h-1 and [Ai Br | Ai Bi] on lanes h .. 2h-1,
// columns 0 and ntile (correction at 2NT + the same); lanes h + r hand
// Ai Br and Ai Bi (main + correction) of row r to lane r through xbuf,
// eight columns at a time, and lanes r < h form re = Ar Br - Ai Bi,
// im = Ar Bi + Ai Br.
template <int SPLIT, int NT>
__device__ __forceinline__ void epilogue_tile(const Tile& t, int q, int lane, uint32_t lane_base, bool have,
                                              double2* base_out, float* xbuf, const TPiece* __restrict__ pieces) {
  const int row = q * 32 + lane;
  const uint32_t o2 = t.stack ? (uint32_t)t.ntile : (uint32_t)NT;
  const int h = t.a_im >> 5;
  float zero[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) zero[j] = 0.f;
  for (int c0 = 0; c0 < t.ntile; c0 += 16) {
    float x1[16], x2[16], y1[16], y2[16];
    if (have) {
      tmem_ld16(lane_base + c0, x1);
      tmem_ld16(lane_base + o2 + c0, x2);
      tmem_ld16(lane_base + 2 * NT + c0, y1);
      tmem_ld16(lane_base + 2 * NT + o2 + c0, y2);
    } else {
#pragma unroll
      for (int j = 0; j < 16; ++j) x1[j] = x2[j] = y1[j] = y2[j] = 0.f;
    }
    if (!t.stack) {
      epilogue16<SPLIT>(t, row, c0, x1, x2, y1, y2, base_out, pieces);
      continue;
    }
    float re[16], im[16];
    const bool reader = row < h, writer = row >= h && row < 2 * h;
    const int xr = writer ? row - h : row;  // the output row (< h <= 64) of these values
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      if (writer) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          xbuf[j * 64 + xr] = x1[hh * 8 + j] + y1[hh * 8 + j];        // Ai Br
          xbuf[(8 + j) * 64 + xr] = x2[hh * 8 + j] + y2[hh * 8 + j];  // Ai Bi
        }
      }
      epi_sync();
      if (reader) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          re[hh * 8 + j] = (x1[hh * 8 + j] + y1[hh * 8 + j]) - xbuf[(8 + j) * 64 + xr];
          im[hh * 8 + j] = (x2[hh * 8 + j] + y2[hh * 8 + j]) + xbuf[j * 64 + xr];
        }
      }
      epi_sync();
    }
    if (reader) epilogue16<SPLIT>(t, row, c0, re, im, zero, zero, base_out, pieces);
  }
}

// One CTA per tile (grid = number of tiles; the hardware hands tiles to SMs
// as they free up).  Same roles, layout and epilogue as the persistent kernel
// below, without its tile loop: used for stage 2, whose few hundred long,
// uneven tiles run faster this way than under the persistent kernel (0.50
// against 0.54-0.62 ms on the m = 2000 workload, measured).  Every wait is
// bounded and reports through *err.
template <int STAGES, int NT, int SPLIT>
__global__ void __launch_bounds__(kThreads, NT == 64 ? 2 : 1) tc_tile_once_kernel(const Tile* __restrict__ tiles,
                                                                  const Seg* __restrict__ segs,
                                                                  double2* __restrict__ base_out, int* err,
                                                                  const IoPtrs* __restrict__ io,
                                                                  const TPiece* __restrict__ pieces) {
  if (io) base_out = io->out;
  extern __shared__ __align__(1024) uint8_t smem[];
  const Tile t = tiles[blockIdx.x];
  constexpr int budget = STAGES * stage_bytes_of(NT, SPLIT);
  constexpr uint32_t kCols = 4 * NT;  // main re, im, correction re, im
  // fixed stages (sizing them to the tile, up to 16 in flight, measured
  // slower: 0.298 against 0.270 ms for stage 2 at m = 2000)
  constexpr int a_region = 2 * SPLIT * kPlaneA;
  constexpr int stage_bytes = stage_bytes_of(NT, SPLIT);
  constexpr int nst = STAGES;
  float* xbuf = reinterpret_cast<float*>(smem + budget);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + budget + kXbufBytes);
  uint64_t* empty = full + kMaxStages;
  uint64_t* accf = empty + kMaxStages;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(accf + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < nst; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accf, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "n"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t lim = t.hold ? (1u << 12) : kWaitLimit;  // attempts per bounded wait

  if (warp == 0) {
    if (lane == 0) {
      int it = 0;
      bool ok = true;
      for (int si = 0; si < t.nseg && ok; ++si) {
        const Seg sg = segs[t.seg0 + si];
        for (int kc = 0; kc < sg.nkc; ++kc, ++it) {
          const int s = it % nst;
          if (it >= nst && !mbar_wait(&empty[s], ((it / nst) + 1) & 1, lim)) {
            flag_error(err, 1);
            ok = false;
            break;
          }
          if (t.hold && it == 0)  // failure-detection test: bytes announced, never sent
            mbar_expect_tx(&full[s], 2u * SPLIT * (sg.a_bytes + sg.b_bytes));
          else
            load_chunk<SPLIT>(smem + s * stage_bytes, a_region, t, sg, kc, &full[s]);
        }
      }
      // copies still in flight land before the CTA leaves (already done
      // unless a wait gave up)
      for (int j = it > nst ? it - nst : 0; j < it; ++j)
        if (!mbar_wait(&full[j % nst], (j / nst) & 1, lim)) flag_error(err, 5);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int it = 0;
      uint32_t acc = 0, acc_c = 0;
      bool ok = true;
      for (int si = 0; si < t.nseg && ok; ++si) {
        const Seg sg = segs[t.seg0 + si];
        for (int kc = 0; kc < sg.nkc; ++kc, ++it) {
          const int s = it % nst;
          if (!mbar_wait(&full[s], (it / nst) & 1, lim)) {
            flag_error(err, 2);
            ok = false;
            break;
          }
          fence_after();
          mma_chunk<SPLIT, NT>(smem_u32(smem + s * stage_bytes), a_region, t, tmem, acc, acc_c);
          mma_commit(&empty[s]);
        }
      }
      if (it > 0) mma_commit(accf);
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32*(w%4) .. +31, one output row per thread
    const int q = warp & 3;
    int total = 0;
    for (int si = 0; si < t.nseg; ++si) total += segs[t.seg0 + si].nkc;
    bool have = total > 0;
    if (have) {
      if (!mbar_wait(accf, 0, lim)) {
        flag_error(err, 3);
        have = false;
      }
      fence_after();
    }
    have = __all_sync(0xffffffffu, have);  // tcgen05.ld below is warp-collective
    const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
    epilogue_tile<SPLIT, NT>(t, q, lane, lane_base, have, base_out, xbuf, pieces);
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kCols) : "memory");
  }
}


__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Persistent: CTA b of G handles tiles b, b + G, b + 2G, ... (the plan orders
// them so that the CTAs' shares balance); TMEM (512 columns) and the barriers
// are set up once per CTA.  Used for stage 1, thousands of short tiles whose
// set-up cost it amortises.  The producer runs up to STAGES chunks ahead
// across tile boundaries, so the next tile's operands stream in while the
// epilogue drains the accumulators.  Barriers: full/empty per stage
// (producer <-> MMA), accf (MMA -> epilogue) and tfree (epilogue -> MMA, four
// warp arrivals), one phase each per tile that has MMAs; tiles without MMAs
// (copy terms only) never touch TMEM and skip both, so neither side runs more
// than one phase ahead of the other.  Every wait is bounded; a wait that runs
// out sets *err and an abort flag in shared memory that every role checks
// between chunks, so the CTA winds down without another full-length wait per
// remaining tile.  On the way out the producer waits (bounded) for the copies
// it issued and the MMA warp for its MMAs (mdone) before TMEM is freed.
template <int STAGES, int NT, int SPLIT>
__global__ void __launch_bounds__(kThreads, NT == 64 ? 2 : 1) tc_tile_kernel(const Tile* __restrict__ tiles, int ntile,
                                                             const Seg* __restrict__ segs,
                                                             double2* __restrict__ base_out, int* err,
                                                             const IoPtrs* __restrict__ io,
                                                             const TPiece* __restrict__ pieces) {
  if (io) base_out = io->out;
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr int stage_bytes = stage_bytes_of(NT, SPLIT);
  constexpr uint32_t kCols = 4 * NT;  // main re, im, correction re, im
  float* xbuf = reinterpret_cast<float*>(smem + STAGES * stage_bytes);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * stage_bytes + kXbufBytes);
  uint64_t* empty = full + STAGES;
  uint64_t* accf = empty + STAGES;
  uint64_t* tfree = accf + 1;
  uint64_t* mdone = tfree + 1;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mdone + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accf, 1);
    mbar_init(tfree, 4);
    mbar_init(mdone, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "n"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tslot;
  auto give_up = [&](int code) {
    flag_error(err, code);
    *abort_flag = 1;
  };

  if (warp == 0) {
    if (lane == 0) {
      int it = 0;
      for (int ti = blockIdx.x; ti < ntile && !*abort_flag; ti += gridDim.x) {
        const Tile t = tiles[ti];
        Seg nxt;
        if (t.nseg > 0) nxt = segs[t.seg0];
        for (int si = 0; si < t.nseg && !*abort_flag; ++si) {
          const Seg sg = nxt;
          if (si + 1 < t.nseg) nxt = segs[t.seg0 + si + 1];  // in flight while this one's copies go out
          for (int kc = 0; kc < sg.nkc; ++kc, ++it) {
            const int s = it % STAGES;
            if (*abort_flag) break;
            if (it >= STAGES && !mbar_wait(&empty[s], ((it / STAGES) + 1) & 1)) {
              give_up(1);
              break;
            }
            load_chunk<SPLIT>(smem + s * stage_bytes, 2 * SPLIT * kPlaneA, t, sg, kc, &full[s]);
          }
        }
      }
      // copies still in flight land before the CTA leaves (already done
      // unless a wait gave up)
      for (int j = it > STAGES ? it - STAGES : 0; j < it; ++j)
        if (!mbar_wait(&full[j % STAGES], (j / STAGES) & 1)) flag_error(err, 5);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int it = 0, n = 0;  // n: tiles with MMAs so far
      bool issued = false;
      for (int ti = blockIdx.x; ti < ntile && !*abort_flag; ti += gridDim.x) {
        const Tile t = tiles[ti];
        if (t.nchunk == 0) continue;
        // the epilogue has read the previous tile's accumulators
        if (n > 0 && !mbar_wait(tfree, (n - 1) & 1)) {
          give_up(4);
          break;
        }
        ++n;
        fence_after();
        uint32_t acc = 0, acc_c = 0;
        int chunks = 0;
        int nkc_next = t.nseg > 0 ? segs[t.seg0].nkc : 0;
        for (int si = 0; si < t.nseg && !*abort_flag; ++si) {
          const int nkc = nkc_next;
          if (si + 1 < t.nseg) nkc_next = segs[t.seg0 + si + 1].nkc;
          for (int kc = 0; kc < nkc; ++kc, ++it, ++chunks) {
            const int s = it % STAGES;
            if (*abort_flag) break;
            if (!mbar_wait(&full[s], (it / STAGES) & 1)) {
              give_up(2);
              break;
            }
            fence_after();
            mma_chunk<SPLIT, NT>(smem_u32(smem + s * stage_bytes), 2 * SPLIT * kPlaneA, t, tmem, acc, acc_c);
            mma_commit(&empty[s]);
            issued = true;
          }
        }
        if (chunks > 0) mma_commit(accf);
      }
      // every MMA issued here has completed before TMEM is freed
      if (issued) {
        mma_commit(mdone);
        if (!mbar_wait(mdone, 0)) flag_error(err, 6);
      }
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32*(w%4) .. +31, one output row per thread
    const int q = warp & 3;
    const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
    int nacc = 0;
    for (int ti = blockIdx.x; ti < ntile; ti += gridDim.x) {
      // one decision for all four epilogue warps (they share named barriers)
      if (epi_any(*abort_flag != 0)) break;
      const Tile t = tiles[ti];
      const bool mmas = t.nchunk > 0;
      bool have = mmas;
      if (have) {
        if (!mbar_wait(accf, nacc & 1)) {
          give_up(3);
          have = false;
        }
        ++nacc;
        fence_after();
      }
      have = __all_sync(0xffffffffu, have);  // tcgen05.ld below is warp-collective
      epilogue_tile<SPLIT, NT>(t, q, lane, lane_base, have, base_out, xbuf, pieces);
      // accumulators read: release them to the MMA warp
      if (mmas) {
        fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(tfree);
      }
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kCols) : "memory");
  }
}

// out[rect] += sum_c coef_c * in[region_c] for the copy terms (site-diagonal
// terms) of the stage-2 tiles, element by element after the tiles; block b
// handles elements [blocks[b].y, + kCopyElemsPerBlock) of tile blocks[b].x
// (only tiles with copy terms are listed).  Coalesced along the
// column-major rows.  The products are summed in FP32 (GB300 retires FP32
// at 64 times its FP64 rate; 2^-24 relative on these terms, far below the
// split products' error) and added to the FP64 output in FP64.
constexpr int kCopyElemsPerBlock = 512;

__global__ void __launch_bounds__(256) copy_terms_kernel(const Tile* __restrict__ tiles,
                                                         const int2* __restrict__ blocks,
                                                         const hh_seg* __restrict__ csegs,
                                                         const double2* __restrict__ base_in,
                                                         double2* __restrict__ base_out,
                                                         const IoPtrs* __restrict__ io) {
  if (io) {
    base_in = io->in;
    base_out = io->out;
  }
  const int2 bw = blocks[blockIdx.x];
  const Tile t = tiles[bw.x];
  double2* O = base_out + t.out;
  const int n = min(t.mrem * t.nrem, bw.y + kCopyElemsPerBlock);
  for (int idx = bw.y + threadIdx.x; idx < n; idx += blockDim.x) {
    const int row = idx % t.mrem, col = idx / t.mrem;
    float ar = 0.f, ai = 0.f;
    for (int ci = 0; ci < t.ncseg; ++ci) {
      const hh_seg cs = csegs[t.cseg0 + ci];
      const double2 x = base_in[cs.poff + (long long)(t.m0 + row) + (long long)(t.n0 + col) * cs.ldp];
      const float xr = (float)x.x, xi = (float)x.y, cr = (float)cs.cre, cim = (float)cs.cim;
      ar = fmaf(cr, xr, fmaf(-cim, xi, ar));
      ai = fmaf(cr, xi, fmaf(cim, xr, ai));
    }
    double2* o = O + (long long)row + (long long)col * t.ldo;
    double2 v = *o;
    v.x += (double)ar;
    v.y += (double)ai;
    *o = v;
  }
}

__global__ void set_io_kernel(IoPtrs* io, const double2* in, double2* out) {
  io->in = in;
  io->out = out;
}

__global__ void zero_out_kernel(double2* out, long long n, const IoPtrs* __restrict__ io) {
  if (io) out = io->out;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = make_double2(0.0, 0.0);
}

// Pipeline depth: 128-wide tiles (one CTA per SM) fill 192 KB of shared
// memory, 4 x 48 KB (SPLIT 3) or 6 x 32 KB (SPLIT 2); 64-wide tiles (256 TMEM
// columns, two CTAs per SM) about 100 KB each, 3 x 36 KB or 4 x 24 KB.
__host__ __device__ constexpr int stages_of(int nt, int split) {
  return nt == 64 ? (split == 3 ? 3 : 4) : (split == 3 ? 4 : 6);
}

size_t tile_smem_bytes(int nt, int split) {
  const int st = stages_of(nt, split);
  return (size_t)st * stage_bytes_of(nt, split) + kXbufBytes + 8 * (2 * kMaxStages + 4) + 64;
}

}  // namespace tc

cudaError_t tc_build_images(const tc::ImgTask* d_tasks, int ntask, const double2* base_in, bool fp32,
                            cudaStream_t s, const tc::IoPtrs* io, int split, const int2* d_blocks, int nblocks) {
  if (ntask <= 0) return cudaSuccess;
  const int grid = d_blocks ? nblocks : ntask;
  if (grid <= 0) return cudaSuccess;
  if (!fp32)
    tc::build_images_kernel<false, 3><<<grid, 256, 0, s>>>(d_tasks, d_blocks, base_in, io);
  else if (split == 2)
    tc::build_images_kernel<true, 2><<<grid, 256, 0, s>>>(d_tasks, d_blocks, base_in, io);
  else
    tc::build_images_kernel<true, 3><<<grid, 256, 0, s>>>(d_tasks, d_blocks, base_in, io);
  return cudaGetLastError();
}

int tc_image_blocks(const tc::ImgTask* tasks, int ntask, std::vector<int2>& out) {
  out.clear();
  for (int i = 0; i < ntask; ++i) {
    const int ngroups = tasks[i].prow * (tasks[i].k16 >> 3);
    for (int g = 0; g < ngroups; g += tc::kImgGroupsPerBlock) out.push_back(make_int2(i, g));
  }
  return (int)out.size();
}

cudaError_t tc_copy_terms(const tc::Tile* d_tiles, const int2* d_blocks, int nblocks, const hh_seg* d_csegs,
                          const double2* base_in, double2* base_out, cudaStream_t s, const tc::IoPtrs* io) {
  if (nblocks <= 0) return cudaSuccess;
  tc::copy_terms_kernel<<<nblocks, 256, 0, s>>>(d_tiles, d_blocks, d_csegs, base_in, base_out, io);
  return cudaGetLastError();
}

int tc_copy_blocks(const tc::Tile* tiles, int ntile, std::vector<int2>& out) {
  out.clear();
  for (int i = 0; i < ntile; ++i) {
    if (tiles[i].mode != 0 || tiles[i].ncseg == 0) continue;
    const int n = tiles[i].mrem * tiles[i].nrem;
    for (int e = 0; e < n; e += tc::kCopyElemsPerBlock) out.push_back(make_int2(i, e));
  }
  return (int)out.size();
}

cudaError_t tc_set_io(tc::IoPtrs* d_io, const double2* in, double2* out, cudaStream_t s) {
  tc::set_io_kernel<<<1, 1, 0, s>>>(d_io, in, out);
  return cudaGetLastError();
}

cudaError_t tc_zero_out(double2* out, long long n, cudaStream_t s, const tc::IoPtrs* io) {
  if (n <= 0) return cudaSuccess;
  long long g = (n + 255) / 256;
  if (g > 4096) g = 4096;
  tc::zero_out_kernel<<<(unsigned)g, 256, 0, s>>>(out, n, io);
  return cudaGetLastError();
}

template <int NT, int SPLIT>
static cudaError_t launch_tiles(const tc::Tile* d_tiles, int ntile, const tc::Seg* d_segs, double2* base_out,
                                int* d_err, bool persistent, cudaStream_t s, const tc::IoPtrs* io,
                                const tc::TPiece* d_pieces) {
  constexpr int ST = tc::stages_of(NT, SPLIT);
  constexpr int per_sm = NT == 64 ? 2 : 1;  // shared memory and TMEM columns of one SM
  const size_t smem = tc::tile_smem_bytes(NT, SPLIT);
  static int sms = 0;
  if (!sms) {
    cudaError_t e = cudaFuncSetAttribute(tc::tc_tile_kernel<ST, NT, SPLIT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(tc::tc_tile_once_kernel<ST, NT, SPLIT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
    int dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  const int resident = per_sm * sms;
  if (persistent && ntile > resident)
    tc::tc_tile_kernel<ST, NT, SPLIT>
        <<<resident, tc::kThreads, smem, s>>>(d_tiles, ntile, d_segs, base_out, d_err, io, d_pieces);
  else
    tc::tc_tile_once_kernel<ST, NT, SPLIT>
        <<<ntile, tc::kThreads, smem, s>>>(d_tiles, d_segs, base_out, d_err, io, d_pieces);
  return cudaGetLastError();
}

cudaError_t tc_run_tiles(const tc::Tile* d_tiles, int ntile, const tc::Seg* d_segs, double2* base_out, int* d_err,
                         bool persistent, cudaStream_t s, const tc::IoPtrs* io, int nt, int split,
                         const tc::TPiece* d_pieces) {
  if (ntile <= 0) return cudaSuccess;
  if (split == 2) {
    if (nt == 64) return launch_tiles<64, 2>(d_tiles, ntile, d_segs, base_out, d_err, persistent, s, io, d_pieces);
    return launch_tiles<128, 2>(d_tiles, ntile, d_segs, base_out, d_err, persistent, s, io, d_pieces);
  }
  if (nt == 64) return launch_tiles<64, 3>(d_tiles, ntile, d_segs, base_out, d_err, persistent, s, io, d_pieces);
  return launch_tiles<128, 3>(d_tiles, ntile, d_segs, base_out, d_err, persistent, s, io, d_pieces);
}

}  // namespace hh
