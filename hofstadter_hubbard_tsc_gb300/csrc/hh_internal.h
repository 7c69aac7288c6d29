// Internal types of the GB300 superblock-step library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>
#include <unordered_map>
#include <complex>

#include "../../include/hh_dmrg.h"

namespace hh {

using cplx = std::complex<double>;

// ---------------------------------------------------------------------------
// Hash of small integer tuples used for the quantum-number lookups.
static inline uint64_t key2(int a, int b) {
  return (uint64_t(uint32_t(a)) << 32) | uint32_t(b);
}
static inline uint64_t key3(int a, int b, int c) {
  return (uint64_t(uint32_t(a) & 0xFFFFF) << 40) | (uint64_t(uint32_t(b) & 0xFFFFF) << 20) |
         uint64_t(uint32_t(c) & 0xFFFFF);
}
static inline uint64_t key4(int a, int b, int c, int d) {
  return (uint64_t(uint16_t(a)) << 48) | (uint64_t(uint16_t(b)) << 32) |
         (uint64_t(uint16_t(c)) << 16) | uint64_t(uint16_t(d));
}

}  // namespace hh

struct hh_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  int sm_count = 0;
  // stream-ordered memory pool of this context (memory stays cached in the
  // pool for reuse; allocation and release never synchronise the device)
  cudaMemPool_t pool = nullptr;
  // scratch reused by reductions (device)
  double* d_red = nullptr;
  size_t red_cap = 0;
  double* h_red = nullptr;  // pinned
  size_t h_red_cap = 0;
  // density-matrix eigensolver state (streams, solver handles, workspace),
  // created on first use (eig.cu), and the eigensolver in use
  // (HH_EIG_OWN or HH_EIG_CUSOLVER)
  void* eig = nullptr;
  int eig_solver = 0;
  // arithmetic of hh_wave_transform's products: HH_PREC_FP64 (default) or
  // HH_PREC_FP32 (the transformed wave only starts Lanczos)
  int transform_precision = 0;
  int restart_precision = HH_PREC_FP32X2;  // the split Lanczos's energy-setting product
  int renorm_precision = 0;                // hh_renormalize's products (FP64 or FP32X2)
  bool krylov_f32 = true;                  // FP32 Krylov basis in the split Lanczos's first pass
  // device address of the static scratch array of hh_matvec_noalloc, looked
  // up by hh_init in this context (noalloc.cu); null with a reason if that
  // lookup failed
  void* noalloc_scratch = nullptr;
  std::string noalloc_status;
};

struct hh_sub_qn {
  int up, down, dd, row, sdim;
  long long off;  // element offset (complex) of the sub matrix in the block data
};

struct hh_block {
  hh_ctx* ctx = nullptr;
  int len = 0, up_dif = 0, down_dif = 0;
  std::vector<hh_sub_qn> subs;
  long long nelem = 0;
  double2* d = nullptr;
  // host copy of the 1x1 entries (site operators are used as scalars)
  std::vector<hh::cplx> scalar;
  std::unordered_map<uint64_t, int> idx2, idx3;
  void build_index();
  int find2(int up, int down) const {
    auto it = idx2.find(hh::key2(up, down));
    return it == idx2.end() ? -1 : it->second;
  }
  int find3(int up, int down, int dd) const {
    auto it = idx3.find(hh::key3(up, down, dd));
    return it == idx3.end() ? -1 : it->second;
  }
};

struct hh_bsub { int spos, sdim, bu, bd, su, sd; };
struct hh_bsec {
  int up, down, dim;
  std::vector<hh_bsub> subs;
  std::unordered_map<uint64_t, int> full, bl;
};

struct hh_basis {
  hh_ctx* ctx = nullptr;
  int len = 0;
  std::vector<hh_bsec> secs;
  std::unordered_map<uint64_t, int> idx;
  int find(int up, int down) const {
    auto it = idx.find(hh::key2(up, down));
    return it == idx.end() ? -1 : it->second;
  }
};

struct hh_wsec { int su, sd, eu, ed, sdim, edim; long long off; };

struct hh_wave {
  hh_ctx* ctx = nullptr;
  int sys_len = 0, env_len = 0, nbatch = 1;
  std::vector<hh_wsec> secs;
  long long nelem = 0;  // per vector
  double2* d = nullptr; // nbatch * nelem
  std::unordered_map<uint64_t, int> idx;
  int find(int su, int sd, int eu, int ed) const {
    auto it = idx.find(hh::key4(su, sd, eu, ed));
    return it == idx.end() ? -1 : it->second;
  }
};

// ---------------------------------------------------------------------------
// Device task list of the grouped segment GEMM.
//
// A tile owns a rectangle of an output matrix (one elementary output
// sub-block of a wave sector, an intermediate product, a density matrix ...)
// and accumulates  sum_s coef_s * opP(P_s) * opQ(Q_s)  over its segments; a
// copy segment adds coef_s * P_s.  Operand addresses are either absolute
// (operators) or offsets into one of the per-launch bases.
enum : int { HH_BASE_ABS = 0, HH_BASE_IN = 1, HH_BASE_SCR = 2, HH_BASE_OUT = 3 };
enum : int { HH_OP_N = 0, HH_OP_C = 1, HH_OP_T = 2 };
enum : int { HH_SEG_GEMM = 0, HH_SEG_COPY = 1 };

struct hh_seg {
  long long poff, qoff;   // element offsets (complex) or absolute addresses
  int pbase, qbase;
  int ldp, ldq;
  int opP, opQ;
  int K;
  int kind;
  double cre, cim;
};

struct hh_tile {
  long long ooff;  // element offset of the rectangle origin in the output base
  int obase;
  int ldo;
  int M, N;        // rectangle extent
  int m0, n0;      // tile origin inside the rectangle
  int seg0, nseg;
  int accumulate;  // 1: out += acc, 0: out = acc
  int part;        // -1: store to the output; >= 0: store the partial sum to slot `part`
};

// Sum, in slot order, of the partial sums of one split output tile.
struct hh_red {
  long long ooff;
  int obase, ldo, M, N, m0, n0, accumulate;
  int part0, nparts;
};

struct hh_gemm_list {
  std::vector<hh_seg> segs;     // as built: one tile per output tile
  std::vector<hh_tile> tiles;
  // device copy (upload): the work list, where tiles heavier than the
  // balance target are split by segment and k ranges into parts of similar
  // cost, the reductions of the split tiles and their partial-sum slots
  hh_seg* d_segs = nullptr;
  hh_tile* d_tiles = nullptr;
  hh_red* d_reds = nullptr;
  double2* d_part = nullptr;
  int n_work = 0, n_red = 0;
  double flops = 0.0;
  hh_ctx* actx = nullptr;  // context whose pool holds the device copy
  void upload(hh_ctx* ctx);
  void release();
};

// One contribution out_k[rect] += c * opA(A) * X_i[region] * opB(B) of the
// model_wave term loops (see plan.cpp); the schedules of both precisions are
// built from this list.
struct hh_mat_ref {
  long long off = 0;  // absolute address for operators
  int base = 0;
  int ld = 1;
  int op = 0;         // HH_OP_N or HH_OP_C
};

struct hh_contrib {
  int k_out, orow, ocol, M, N;
  int i_in, irow, icol, Ka, Kb;
  bool hasA, hasB;
  hh_mat_ref A, B;
  double cre, cim;
};

namespace hh { namespace tc { struct ImgTask; struct Seg; struct Tile; struct IoPtrs; struct TPiece; } }

struct hh_tc_plan {
  bool ready = false;
  void* d_op_img = nullptr;    // operator images (built once)
  void* d_x_img = nullptr;     // images of the input wave (built every matvec)
  void* d_t_img = nullptr;     // stage-1 products
  hh::tc::ImgTask* d_op_tasks = nullptr;
  hh::tc::ImgTask* d_x_tasks = nullptr;
  int n_op_tasks = 0, n_x_tasks = 0;
  hh::tc::Tile* d_tiles1 = nullptr;
  hh::tc::Tile* d_tiles2 = nullptr;   // stage 2, longest first (one CTA per tile)
  hh::tc::Tile* d_tiles2b = nullptr;  // the same tiles ordered for the persistent kernel
  hh::tc::TPiece* d_pieces = nullptr; // pieces of the row-packed stage-1 tiles
  int2* d_x_blocks = nullptr;         // wave-image block list (tc_image_blocks)
  int n_x_blocks = 0;
  int2* d_c_blocks = nullptr;         // copy-term block list over d_tiles2 (tc_copy_blocks)
  int n_c_blocks = 0;
  bool zero_out = true;               // stage-2 tiles do not cover the whole output
  int n_tiles1 = 0, n_tiles2 = 0, n_cseg = 0;
  int n_narrow1 = 0, n_narrow2 = 0;  // leading tiles at most 64 wide (64-wide kernels)
  hh::tc::Seg* d_segs = nullptr;
  hh_seg* d_csegs = nullptr;
  int* d_err = nullptr;
  // the matvec captured as a CUDA graph (after the first, eager call); the
  // graph's kernels read the vectors from d_io, set before each replay
  hh::tc::IoPtrs* d_io = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int calls = 0;
  int graph_split = 0;  // BF16 parts per operand of the captured graph
  // launch choices (hh_plan_tune): stage 1 / stage 2 on the persistent kernel
  bool persistent1 = true, persistent2 = false;
  double bytes_op = 0, bytes_x = 0, bytes_t = 0;
  double mma_flops1 = 0, mma_flops2 = 0;  // tensor FLOPs issued (bf16), padding included
  int n_stacked2 = 0;                     // stage-2 tiles of at most 64 rows (stacked MMAs)
  double mma_cycles2 = 0;                 // stage-2 MMA cycles at BF16x3 (summed over tiles)
};

struct hh_plan {
  hh_ctx* ctx = nullptr;
  std::vector<hh_contrib> contribs;
  hh_tc_plan tc;
  hh_tc_plan tcb;  // the schedule of a batch of tcb_nb vectors (hh_matvec on a wave of several vectors)
  int tcb_nb = 0;
  int tc_shape = 0;  // row split of the stage-2 tiles (tc_plan.cpp; chosen by hh_plan_tune)
  const hh_wave* layout = nullptr;
  long long nelem = 0;
  hh_gemm_list stage1, stage2;
  long long scratch_elems = 0;
  double2* d_scratch = nullptr;
  double ref_flops = 0.0, exec_flops = 0.0;
  double ref_flops_first = 0.0, exec_flops_s1 = 0.0, exec_flops_s2 = 0.0;
  double2* d_host_in = nullptr;   // device buffers of hh_matvec_host
  double2* d_host_out = nullptr;
  double op_bytes = 0.0;
  std::vector<const hh_block*> ops;
  // Lanczos workspace
  double2* d_krylov = nullptr;
  int krylov_cap = 0;
};

namespace hh {
int fail(hh_ctx* ctx, int code, const std::string& msg);
// device memory from the context's pool, ordered on its stream (256-byte
// aligned; a misaligned pointer is returned as an error)
cudaError_t dev_alloc(hh_ctx* ctx, void** p, size_t bytes);
void dev_free(hh_ctx* ctx, void* p);
int cuda_check(hh_ctx* ctx, cudaError_t e, const char* what);
// looks up the static scratch of hh_matvec_noalloc for ctx->device (noalloc.cu)
void noalloc_setup(hh_ctx* ctx);
// grouped segment GEMM; bases[4] = {abs(unused), in, scr, out}; arithmetic
// FP64, FP32 or double-float (gemm_fp64.cu)
enum { kArithFp64 = 0, kArithFp32 = 1, kArithDf = 2 };
cudaError_t launch_segment_gemm_fp64(const hh_gemm_list& L, double2* base_in, double2* base_scr,
                                     double2* base_out, cudaStream_t s, int arith = kArithFp64);
// loads the segment GEMM kernels into the current context (gemm_fp64.cu)
cudaError_t preload_segment_gemm_fp64();
// wave vector kernels
cudaError_t wave_dot(const double2* a, const double2* b, long long n, double* d_out, cudaStream_t s);
// device-resident scalars (Lanczos): *result = Re<a|b> (part: >= 1024 partials),
// y += sign * s[0] * x, y *= 1/sqrt(s[0]) (and root[0] = sqrt(s[0]) when
// root != nullptr), c[j] /= d[j] for j < k
cudaError_t wave_dot_into(const double2* a, const double2* b, long long n, double* result, double* part,
                          cudaStream_t s);
cudaError_t wave_axpy_dev(double2* y, const double2* x, const double* sc, double sign, long long n, cudaStream_t s);
cudaError_t wave_scale_rsqrt_dev(double2* y, const double* sc, double* root, long long n, cudaStream_t s);
cudaError_t divide_dev(double* c, const double* d, int k, cudaStream_t s);
cudaError_t wave_axpy(double2* y, const double2* x, double a, long long n, cudaStream_t s);
cudaError_t wave_scale(double2* y, double a, long long n, cudaStream_t s);
cudaError_t wave_fill_random(double2* w, long long n, unsigned long long seed, cudaStream_t s);
// Krylov bases of double2 (FP64) or float2 (the split Lanczos's first pass)
// vectors; products and sums in FP64
template <class VT>
cudaError_t krylov_dots(const VT* V, int k, long long ld, const double2* w, long long n,
                        double* d_out, cudaStream_t s);
template <class VT>
cudaError_t krylov_update(const VT* V, int k, long long ld, double2* w, long long n,
                          const double* d_coef, cudaStream_t s);
template <class VT>
cudaError_t krylov_combine(const VT* V, int k, long long ld, double2* out, long long n,
                           const double* d_coef, cudaStream_t s);
// v = FP32 rounding of w, *vv = <v|v> (part: >= 1024 partials)
cudaError_t krylov_store_f32(const double2* w, float2* v, long long n, double* vv, double* part, cudaStream_t s);
int build_plan(hh_ctx* ctx, const hh_basis* sb, const hh_basis* eb, const hh_wave* layout,
               int nterm, const hh_term_t* terms, hh_plan* plan);
int build_tc_plan(hh_plan* plan);
void release_tc_plan(hh_plan* plan);
// check = false: queue only; a bounded wait that ran out is left in the
// plan's error flag (p->tc.d_err) for the caller to read
// split: BF16 parts per operand (3: BF16x6, 2: BF16x3)
int matvec_tc(hh_plan* p, const double2* in, double2* out, float* ms, bool check = true, int split = 3);
// nb vectors one after another in in / out, one launch per stage for all of
// them (the batch schedule is built on first use and kept for that nb)
int matvec_tc_batch(hh_plan* p, const double2* in, double2* out, int nb, bool check, int split);
int tune_tc_plan(hh_plan* p, int reps, double* ms, int split);
// BF16 parts per operand of a split precision, 0 for FP64 or an unknown code
inline int split_of(int precision) {
  return precision == HH_PREC_BF16X6 ? 3 : precision == HH_PREC_BF16X3 ? 2 : 0;
}
// the segment-GEMM arithmetic of an FP64-class matvec precision (FP64 or
// double-float), -1 for the split precisions and unknown codes
inline int seg_arith_of(int precision) {
  return precision == HH_PREC_FP64 ? kArithFp64 : precision == HH_PREC_FP32X2 ? kArithDf : -1;
}
double w6j(int j1, int j2, int j3, int l1, int l2, int l3);
double w3j(int j1, int j2, int j3, int m1, int m2, int m3);
int tridiag_lowest(int n, const double* alpha, const double* beta, double* e0, double* z);
// Eigenvalues (ascending, into *d_w: sector k's at the sum of the earlier
// dims) and eigenvectors (in place) of the Hermitian sectors A + offs[k] of
// size dims[k]; *d_w is context-owned scratch valid until the next call.
int eig_hermitian_sectors(hh_ctx* ctx, double2* A, const std::vector<long long>& offs,
                          const std::vector<int>& dims, double** d_w);
// The library's own two-phase eigensolver of the same sectors (eig.cu):
// eig_values returns every eigenvalue (ascending per sector, sectors in
// order) on the host and leaves the reduced sectors in A; eig_vectors then
// writes the eigenvectors of the ncol[k] largest eigenvalues of sector k,
// ascending, in the canonical phase, to X + xoff[k] (column-major, ld dims[k])
// on the context stream.  force_tri sends every sector through the
// tridiagonal pipeline (tests), otherwise sectors of up to 32 states are
// solved by the Jacobi kernel.
int eig_values(hh_ctx* ctx, double2* A, const std::vector<long long>& offs, const std::vector<int>& dims,
               bool force_tri, std::vector<double>& w_host);
int eig_vectors(hh_ctx* ctx, const std::vector<int>& ncol, double2* X, const std::vector<long long>& xoff);
// frees the eigensolver state held by the context
void release_step_resources(hh_ctx* ctx);
}  // namespace hh
