// Task formats of the split-precision tensor-core path (see tc_gemm.cu).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

struct hh_seg;

namespace hh {
namespace tc {

// builds one operand image: value(r,k) = coef * (conj?) src[trans ? k + r*ld : r + k*ld]
struct ImgTask {
  long long src;   // absolute address (HH_BASE_ABS) or element offset into the input wave
  int sbase;
  int ld;
  int rows, kc;    // logical extent (complex)
  int rpad, k16;   // padded extent of the image (rows to a multiple of 16, k to 16)
  int trans, conj;
  int row0, prow;  // image rows [row0, row0 + prow) are this task's (several operators can
                   // share one image, stacked in rows); one-operator images: 0, rpad
  double cre, cim;
  long long dst;   // absolute address of the image (256-byte aligned)
};

// one GEMM segment of a tile: 6 planes of A rows [m0, m0+128) and of B rows
// [n0, n0+ntile) for nkc chunks of 16 complex k
struct Seg {
  long long a, b;        // address of plane 0, chunk 0 at the tile's first row
  long long a_plane, b_plane;  // bytes between planes (= Rpad/8 * 256 of the image)
  int a_bytes, b_bytes;  // bytes per plane copy (rows * 32)
  int nkc;
  int pad;
};

struct Tile {
  int seg0, nseg;        // GEMM segments
  int cseg0, ncseg;      // FP64 copy segments (copy_terms_kernel)
  int mode;              // 0: FP64 output rectangle, 1: T image
  int ntile;             // MMA N (multiple of 16, <= 128)
  int mrem, nrem;        // valid rows / columns of the tile
  long long out;         // mode 0: element offset of (m0, n0) in the output wave; mode 1: image address
  int ldo;
  int t_rpad;            // mode 1: padded rows of the T image
  int m0, n0;            // tile origin inside its rectangle
  int nchunk;            // sum of the segments' nkc (MMA chunks of the tile)
  int stack;             // 1: at most 64 rows (every segment's A copy too): re and im parts of A
                         // stacked in one 128-row operand, one MMA per part pair (tc_gemm.cu)
  int pack;              // bit 0: every segment's A copy is its whole image height (one copy
                         // of all planes per chunk); bit 1: the same for B with planes ntile rows
  int a_pair, a_im;      // shared memory of A plane q: (q / 2) * a_pair + (q % 2) * a_im bytes
  int hold;              // failure-detection test only (0 in every plan): the producer posts the first
                         // chunk's bytes without issuing its copies, so the bounded waits run out
                         // (each after 2^12 attempts instead of 2^20) and the CTA reports and unwinds
  int piece0, npiece;    // mode 1, row-packed tiles: rows of several products, routed by the pieces
                         // [piece0, piece0 + npiece) to their own T images (npiece 0: one product)
};

// One product's rows inside a row-packed stage-1 tile: tile rows [row0, row0
// + t_rpad) are rows [0, t_rpad) of the T image at `out` (rows >= `rows` are
// its zero padding).
struct TPiece {
  long long out;
  int row0, rows, t_rpad, pad;
};

// Fills a finished tile's nchunk, stack, pack, a_pair and a_im from its
// segments (tc_plan.cpp).
void finish_tile(Tile& t, const Seg* segs);

// Input and output waves of a matvec, read by the kernels from device memory
// when a captured graph replays the matvec for new vectors (io != nullptr);
// the explicit pointer arguments serve the eager launches.
struct IoPtrs {
  const double2* in;
  double2* out;
};

// dynamic shared memory of the tile kernels for tiles at most nt (64 or 128)
// wide using split (2 or 3) BF16 parts per operand
size_t tile_smem_bytes(int nt, int split);

}  // namespace tc

// fp32: scale and split in FP32 (wave images, the first `split` parts)
// instead of FP64 (operator images, all three parts); d_blocks (from
// tc_image_blocks) spreads the tasks' row groups evenly over the CTAs,
// without it one CTA converts one task
cudaError_t tc_build_images(const tc::ImgTask* d_tasks, int ntask, const double2* base_in, bool fp32,
                            cudaStream_t s, const tc::IoPtrs* io = nullptr, int split = 3,
                            const int2* d_blocks = nullptr, int nblocks = 0);
// block list of tc_build_images for host tasks: (task, first row group) per CTA
int tc_image_blocks(const tc::ImgTask* tasks, int ntask, std::vector<int2>& out);
// adds the copy terms of the stage-2 tiles to their output rectangles, over
// the block list of tc_copy_blocks (tile, first element) built on the same
// tile array
cudaError_t tc_copy_terms(const tc::Tile* d_tiles, const int2* d_blocks, int nblocks, const hh_seg* d_csegs,
                          const double2* base_in, double2* base_out, cudaStream_t s,
                          const tc::IoPtrs* io = nullptr);
int tc_copy_blocks(const tc::Tile* tiles, int ntile, std::vector<int2>& out);
// writes the vectors of the next graph replay (one thread; arguments by value)
cudaError_t tc_set_io(tc::IoPtrs* d_io, const double2* in, double2* out, cudaStream_t s);
// zeroes n complex elements of io->out (graph replays) or of out
cudaError_t tc_zero_out(double2* out, long long n, cudaStream_t s, const tc::IoPtrs* io = nullptr);
// tile GEMM over ntile tiles: persistent (one CTA per SM, CTA b takes tiles
// b, b + G, ...: the list must be ordered for balance) or one CTA per tile
// nt: the list's widest tile (<= 64: the 64-wide kernels, two CTAs per SM);
// split: BF16 parts per operand, 3 (six products) or 2 (three products)
// d_pieces: the row-packed tiles' pieces (stage 1)
cudaError_t tc_run_tiles(const tc::Tile* d_tiles, int ntile, const tc::Seg* d_segs, double2* base_out, int* d_err,
                         bool persistent, cudaStream_t s, const tc::IoPtrs* io = nullptr, int nt = 128,
                         int split = 3, const tc::TPiece* d_pieces = nullptr);

}  // namespace hh
