// Work items of the tridiagonal eigensolver (eig_tri.cu) shared with its host
// orchestration (eig.cu).
#pragma once

#include <cuda_runtime.h>

namespace hh {
namespace tri {

constexpr int kCluster = 8;        // CTAs of the global-memory reduction's cluster (sectors above ds_max_n())
constexpr int kReduceThreads = 256;
constexpr int kClusterMax = 16;    // CTAs of the distributed-shared-memory reduction's cluster (at most)
constexpr int kDsThreads = 512;    // threads of one CTA of that reduction
constexpr int kMaxN = 4096;        // largest sector (shared memory holds two n-vectors)
constexpr int kBtCols = 8;         // columns per CTA of the back-transformation (one warp each)

// One sector reduced to tridiagonal form.
struct Sector {
  long long aoff;  // n x n sector in the density block (column-major, ld n); reflectors on exit
  long long toff;  // first of its n entries in the d, e, tau and p arrays
  long long woff;  // first of its n eigenvalues in the global (ascending per sector) list
  int n;
  int pad;
};

// One kept eigenvector of a reduced sector, computed by inverse iteration.
struct InvItem {
  int sec;         // index into the Sector array
  int j;           // eigenvalue index within the sector (ascending)
  int col;         // column of the sector's Z block
  int ldz;         // columns of the Z block (kept states of the sector)
  long long zoff;  // Z block (n x ldz, row-major) in the Z buffer
};

// C = alpha A B + beta C0 on strided FP64 views (Newton-Schulz steps).
struct GemmItem {
  long long a, b, c, c0;
  int M, N, K;
  int a_r, a_c, b_r, b_c, c_r, c_c;  // element (i, k) of A at a + i a_r + k a_c, etc.
  double alpha, beta;
  int tiles_n;     // tiles along N
  int tile0;       // first tile of this item in the launch
  int gate;        // Newton-Schulz items: 1 + their block (0: always run)
  int step;        // ... and their step: skipped when step >= need[gate - 1]; a
                   // skipped item with beta != 0 copies C0 to C instead
};

// The Gram matrix of one Newton-Schulz block (k x k at goff) after its first
// step's G = Z^T Z.
struct NsBlock {
  long long goff;
  int k, pad;
};

// Back-transformation X = Q Z of kBtCols columns of one sector.
struct BtItem {
  int sec;
  int c0, nc;      // columns [c0, c0 + nc) of the sector
  int ldz;
  long long zoff;  // Z block (row-major n x ldz)
  long long xoff;  // output: column-major n x ldz block (ld n), absolute element offset
};

// The Z block of a sector with clusters of numerically degenerate kept
// eigenvalues: the column ranges [c0, c1) in clusters[cl0, cl0 + ncl), last
// (largest eigenvalues) first, go through Gram-Schmidt against every later
// column of the block.
struct CgsBlock {
  long long zoff;  // row-major n x ldz
  int n, ldz;
  int cl0, ncl;
};

// One large cluster's Cholesky factor: G (c x c, row-major, symmetric) at g
// becomes the upper factor R of G + s I (s = 1e-14 trace(G) / c); R^{-1} is
// written at r (c x c, row-major).
struct CholItem {
  long long g, r;
  int c, pad;
};

// A column range to put in the canonical phase.
struct PhaseItem {
  long long off;   // first element of the first column
  int rows, cols;
};

// density sectors -> tridiagonal T = Q^H A Q (d, e), reflectors in place,
// tau; p (n per sector) and dots (kCluster per sector) are scratch
cudaError_t reduce(const Sector* d_secs, int nsec, int maxn, double2* den, double* d, double* e, double2* tau,
                   double2* p, double2* dots, cudaStream_t s);
// the same reduction on a cluster of ds_cluster_size() CTAs (16 where the
// device can place such a cluster, else 8) with its vectors in distributed
// shared memory and each sector's lower columns in the CTAs' shared memory
// (global_cols false: sectors of at most ds_max_n(false) states) or in place
// in global memory (global_cols true: at most ds_max_n(true)); maxn is the
// largest sector of the launch
int ds_cluster_size();
int ds_max_n(bool global_cols);
cudaError_t reduce_ds(const Sector* d_secs, int nsec, int maxn, bool global_cols, double2* den, double* d, double* e,
                      double2* tau, cudaStream_t s);
// all eigenvalues of every T, ascending, by bisection
cudaError_t bisect(const Sector* d_secs, int nsec, int maxn, const double* d, const double* e, double* w,
                   cudaStream_t s);
// kept eigenvectors of T by inverse iteration (lu: 5 * maxn * nitems doubles)
cudaError_t inverse_iteration(const Sector* d_secs, const InvItem* d_items, int nitems, int maxn, const double* d,
                              const double* e, const double* w, double* Z, double* lu, cudaStream_t s);
// classical Gram-Schmidt twice of the clusters' columns (numerically
// degenerate kept eigenvalues) against the later columns of their block, one
// CTA per block; clusters holds (c0, c1) column ranges
cudaError_t cgs2(const CgsBlock* d_blocks, int nblocks, const int2* d_clusters, int maxk, double* Z,
                 cudaStream_t s);
// R^{-1} of the Cholesky factor of each item's Gram matrix, one CTA per item
// (orthonormalisation of large degenerate clusters by Cholesky QR)
cudaError_t chol_inv(const CholItem* d_items, int nitems, double* buf, cudaStream_t s);
// batched strided FP64 GEMMs, ntiles = total 64 x 64 tiles of the items;
// need (may be null) gates the Newton-Schulz items
cudaError_t gemm(const GemmItem* d_items, int nitems, int ntiles, double* buf, cudaStream_t s,
                 const int* need = nullptr);
// Newton-Schulz steps each block needs, from delta = max |G - I| of its first
// Gram matrix: the error after a step is about (3/4) delta^2, so 1 step for
// delta <= 1e-8, 2 for delta <= 1e-4, else 3
cudaError_t ns_gate(const NsBlock* d_blocks, int nblocks, const double* buf, int* need, cudaStream_t s);
// X = Q Z into the truncation operator
cudaError_t backtransform(const Sector* d_secs, const BtItem* d_items, int nitems, const double2* den,
                          const double2* tau, const double* Z, double2* X, cudaStream_t s);
// largest-modulus component of every column real positive
cudaError_t phase_columns(const PhaseItem* d_items, int nitems, int maxcols, double2* X, cudaStream_t s);

}  // namespace tri
}  // namespace hh
