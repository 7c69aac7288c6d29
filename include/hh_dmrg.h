/*
 * hh_dmrg.h -- C ABI of the GB300 superblock step of the SU(2) block DMRG.
 *
 * The entry points replace the hot-path subroutines of the Fortran code in
 * cfengno1/Hofstadter_Hubbard_TSC (paths below are inside that project).  A
 * Fortran caller binds them with ISO_C_BINDING; every argument is a plain
 * pointer, an int or a double.  Complex data are interleaved (re, im) doubles,
 * sub-blocks column-major exactly as the Fortran arrays are laid out, so the
 * caller passes its own buffers without reshuffling.
 *
 * Conventions
 *   - every call returns an int status: HH_OK (0) or a negative HH_ERR_* code;
 *     hh_last_error() returns a message for the last failure in a context;
 *   - the library owns device memory; the caller owns host buffers;
 *   - all work of a context runs on one CUDA stream (hh_ctx_stream), calls on
 *     one context must not overlap from several host threads;
 *   - quantum numbers follow the reference: num_up = electron number N,
 *     num_down = 2S, down_dif = change of 2S, up_dif = change of N.
 */
#ifndef HH_DMRG_H
#define HH_DMRG_H

#ifdef __cplusplus
extern "C" {
#endif

#define HH_OK 0
#define HH_ERR_INVALID (-1)   /* bad argument or handle                          */
#define HH_ERR_CUDA (-2)      /* CUDA runtime / library failure                  */
#define HH_ERR_NOMEM (-3)     /* device or host allocation failed                */
#define HH_ERR_QN (-4)        /* quantum-number mismatch (the reference stops)   */
#define HH_ERR_TIMEOUT (-5)   /* a bounded device wait ran out                   */
#define HH_ERR_NUMERIC (-6)   /* eigensolver failure or non-finite result        */
#define HH_ERR_UNSUPPORTED (-7)

/* precision of the superblock matvec */
#define HH_PREC_FP64 0        /* complex FP64 on the CUDA cores                   */
#define HH_PREC_BF16X6 1      /* three BF16 parts, six products per real product,
                                 FP32 accumulate (tcgen05): ~2^-24 per product    */
#define HH_PREC_BF16X3 2      /* two BF16 parts, three products (x0y0 + x0y1 +
                                 x1y0), FP32 accumulate: ~2^-16 per product       */
#define HH_PREC_FP32 3        /* complex FP32 on the CUDA cores (the wave
                                 transform's guess only, hh_ctx_set_transform_
                                 precision)                                       */
#define HH_PREC_FP32X2 4      /* double-float on the FP32 pipe: every operand as
                                 a sum of two floats (48 bits), exact products
                                 by FMA residuals, sums by TwoSum: ~2^-47 per
                                 operation, FP64-class (the split Lanczos's
                                 restart product by default)                      */

typedef struct hh_ctx hh_ctx_t;
typedef struct hh_block hh_block_t;
typedef struct hh_basis hh_basis_t;
typedef struct hh_wave hh_wave_t;
typedef struct hh_plan hh_plan_t;
typedef struct hh_mlp hh_mlp_t;

/* ---------------------------------------------------------------- context */
int hh_init(int device, hh_ctx_t** ctx);
int hh_finalize(hh_ctx_t* ctx);
const char* hh_last_error(const hh_ctx_t* ctx);
const char* hh_status_string(int status);
int hh_ctx_stream(hh_ctx_t* ctx, void** stream);   /* cudaStream_t of the context */
int hh_ctx_sync(hh_ctx_t* ctx);
int hh_version(void);

/* Eigensolver of the density-matrix sectors (hh_density_truncate), all FP64:
 * HH_EIG_OWN (default): the library's own kernels -- sectors of up to 16
 *   states by one-CTA Jacobi, larger ones by Householder reduction to a real
 *   tridiagonal on a thread-block cluster, bisection for every eigenvalue,
 *   and inverse iteration plus back-transformation for the kept
 *   eigenvectors only;
 * HH_EIG_CUSOLVER: every eigenpair, sectors above 32 states by cuSOLVER
 *   zheevd (kept for comparison).                                          */
#define HH_EIG_OWN 0
#define HH_EIG_CUSOLVER 1
int hh_ctx_set_eigensolver(hh_ctx_t* ctx, int solver);
/* Arithmetic of hh_wave_transform's products: HH_PREC_FP64 (default, the
 * reference's ZGEMM) or HH_PREC_FP32 (inputs rounded to FP32, FP32
 * accumulation, FP64 result).  The transformed wave only starts the next
 * Lanczos, so a split-precision sweep can take the 2^-24 rounding for
 * GB300's FP32 rate (64x its FP64 rate).  No counterpart in the reference. */
int hh_ctx_set_transform_precision(hh_ctx_t* ctx, int precision);
/* Arithmetic of the one product of the split-precision hh_lanczos that sets
 * the energy to FP64 accuracy (the restart product, below): HH_PREC_FP32X2
 * (default; double-float on the FP32 pipe, which GB300 runs at 64 times its
 * FP64 rate) or HH_PREC_FP64.  No counterpart in the reference.           */
int hh_ctx_set_restart_precision(hh_ctx_t* ctx, int precision);
/* Arithmetic of hh_renormalize's products T^H O T: HH_PREC_FP64 (default,
 * the reference's ZGEMM pair) or HH_PREC_FP32X2 (double-float on the FP32
 * pipe, ~2^-47 per operation: the block operators of a split-precision sweep
 * stay FP64-class at about a third of the FP64 time).  No counterpart in the
 * reference.                                                              */
int hh_ctx_set_renormalize_precision(hh_ctx_t* ctx, int precision);
/* Storage of the Krylov basis in the first pass of the split-precision
 * hh_lanczos: HH_PREC_FP32 (default; half the bytes of its Gram-Schmidt
 * passes, far below the split products' own error) or HH_PREC_FP64.  The
 * restart pass keeps an FP64 basis.  No counterpart in the reference.     */
int hh_ctx_set_krylov_storage(hh_ctx_t* ctx, int precision);
/* Diagnostic: every eigenpair of one dense Hermitian matrix A (n x n,
 * column-major, interleaved complex) through the tridiagonal pipeline of
 * HH_EIG_OWN (whatever n): w ascending (n doubles), V the eigenvectors
 * (n x n interleaved complex, canonical phase: the largest-modulus component
 * of each column real positive).                                          */
int hh_eig_selftest(hh_ctx_t* ctx, int n, const double* A, double* w, double* V);

/* ----------------------------------------------- Total_Block (operators)
 * Replaces the in-memory Total_Block of code/pubdata.f90:141-149 with a
 * device-resident copy.  sub_qn holds 5 ints per sub: num_up, num_down,
 * down_dif, row_dim, sdim.  data holds the sub matrices back to back, each
 * row_dim x sdim column-major, interleaved complex.                        */
int hh_block_create(hh_ctx_t* ctx, int len, int up_dif, int down_dif, int nsub,
                    const int* sub_qn, const double* data, hh_block_t** out);
int hh_block_zeros(hh_ctx_t* ctx, int len, int up_dif, int down_dif, int nsub,
                   const int* sub_qn, hh_block_t** out);
int hh_block_info(const hh_block_t* b, int* len, int* up_dif, int* down_dif,
                  int* nsub, long long* nelem);
int hh_block_qn(const hh_block_t* b, int* sub_qn);
int hh_block_download(const hh_block_t* b, double* data);
int hh_block_free(hh_block_t* b);
/* dst += coef * src sub by sub, matching (num_up, num_down, down_dif) with the
 * forward scan of block_add_block_two (code/space_info.f90:176-214); hmerge
 * (code/mat_vec.f90:3623-3852) is a sequence of these calls. coef = {re, im}. */
int hh_block_add(hh_block_t* dst, const double* coef, const hh_block_t* src);

/* --------------------------------------------- Total_Basis (enlarged blocks)
 * Replaces Total_Basis (code/pubdata.f90:91-108) as produced by Get_basis
 * (code/update.f90:11-112).  sec: 3 ints per sector (new_num_up, new_num_down,
 * number of sub-blocks); subs: 6 ints per sub-block (spos, sdim, bl_num_up,
 * bl_num_down, st_num_up, st_num_down), sector after sector.               */
int hh_basis_create(hh_ctx_t* ctx, int len, int nsec, const int* sec,
                    const int* subs, hh_basis_t** out);
int hh_basis_free(hh_basis_t* b);

/* ---------------------------------------- Wavefunction (super basis layout)
 * Replaces Wavefunction / Super_Basis (code/pubdata.f90:114-136).  sec: 6 ints
 * per sector (sys_num_up, sys_num_down, env_num_up, env_num_down, sys_dim,
 * env_dim).  nbatch independent vectors share the layout (batched matvec). */
int hh_wave_create(hh_ctx_t* ctx, int sys_len, int env_len, int nsec,
                   const int* sec, int nbatch, hh_wave_t** out);
int hh_wave_info(const hh_wave_t* w, long long* nelem, int* nbatch);
int hh_wave_upload(hh_wave_t* w, const double* data);     /* nbatch*nelem complex */
int hh_wave_download(const hh_wave_t* w, double* data);
int hh_wave_copy(hh_wave_t* dst, const hh_wave_t* src);
int hh_wave_free(hh_wave_t* w);
/* wave_product (Re<a|b>), wave_norm, wave_normalize (code/space_info.f90:1018-1075) */
int hh_wave_dot(const hh_wave_t* a, const hh_wave_t* b, double* re);
int hh_wave_norm(const hh_wave_t* a, double* nrm);
int hh_wave_normalize(hh_wave_t* a);

/* ------------------------------------------------------------- model_wave
 * One term of model_wave (code/mat_vec.f90:3476-3620).  kind selects the term
 * kernel it replaces; op0/op1 are the (sys-side, env-side) operators in the
 * argument order of that kernel; trans0/trans1 = 1 means the operand is passed
 * through block_transfer_trans (code/space_info.f90:32-63) first; flag0/flag1
 * are 'F' (fermion) or 'B' (boson) as in the reference.                    */
enum hh_term_kind {
  HH_BLOCK_VEC_DIA = 1,        /* code/mat_vec.f90:165  (op0 = sys block)            */
  HH_VEC_BLOCK_DIA = 2,        /* code/mat_vec.f90:218  (op0 = env block)            */
  HH_SITE_VEC_SITE_DIA = 3,    /* code/mat_vec.f90:540  (op0 sys site, op1 env site) */
  HH_SITE_VEC_SITE_NDIA = 4,   /* code/mat_vec.f90:3101                              */
  HH_BLOCK_SITE_VEC_NDIA = 5,  /* code/mat_vec.f90:960  (sys block, sys site)        */
  HH_VEC_BLOCK_SITE_NDIA = 6,  /* code/mat_vec.f90:1219 (env block, env site)        */
  HH_BLOCK_VEC_SITE_NDIA = 7,  /* code/mat_vec.f90:2324 (sys block, env site)        */
  HH_SITE_VEC_BLOCK_NDIA = 8,  /* code/mat_vec.f90:2695 (sys site, env block)        */
  HH_BLOCK_VEC_BLOCK_NDIA = 9, /* code/mat_vec.f90:1505 (sys block, env block)       */
  HH_BLOCK_SITE_VEC_DIA = 10,  /* code/mat_vec.f90:388                               */
  HH_VEC_BLOCK_SITE_DIA = 11,  /* code/mat_vec.f90:463                               */
  HH_BLOCK_VEC_SITE_DIA = 12,  /* code/mat_vec.f90:640                               */
  HH_SITE_VEC_BLOCK_DIA = 13,  /* code/mat_vec.f90:743                               */
  HH_BLOCK_VEC_BLOCK_DIA = 14  /* code/mat_vec.f90:846                               */
};

typedef struct {
  int kind;
  int flag0, flag1;            /* 'F' or 'B' (ignored for the _DIA kinds)  */
  int trans0, trans1;
  const hh_block_t* op0;
  const hh_block_t* op1;       /* NULL for the one-operator kinds          */
  double coef_re, coef_im;
} hh_term_t;

/* Builds the task list of model_wave for one superblock (the loop nests of the
 * term kernels, their 6j coefficients, phases and fermion signs), resolved
 * once and reused by every matvec of a Lanczos call.                       */
int hh_plan_create(hh_ctx_t* ctx, const hh_basis_t* sys_bs, const hh_basis_t* env_bs,
                   const hh_wave_t* layout, int nterm, const hh_term_t* terms,
                   hh_plan_t** out);
/* counts (HH_PLAN_STATS doubles): [0] reference FLOPs per matvec (8MNK over the
 * reference's ZGEMM calls + 8 per element of the axpy terms), [1] FLOPs this
 * plan executes, [2] output tiles, [3] segments, [4] stage-1 products,
 * [5] scratch bytes, [6] operator bytes, [7] wave bytes (in + out),
 * [8] executed FLOPs of stage 1, [9] of stage 2, [10] reference FLOPs of the
 * first GEMM of the two-GEMM terms, [11] the remaining reference FLOPs,
 * [12], [13] BF16 tensor FLOPs issued by the split-precision stages 1 and 2
 * at HH_PREC_BF16X6 (padding included; HH_PREC_BF16X3 issues half),
 * [14] bytes of its operand images, [15] 1 once the split-precision
 * schedule has been built (first split-precision matvec), [16] kernel
 * launches of one FP64 matvec, [17] of one split-precision matvec (graph
 * replay included), [18] FP64 work tiles after balancing, [19] 1 when stage
 * 1 of the split-precision matvec runs on the persistent kernel, [20]
 * stage-2 tiles of the split-precision schedule, [21] those of at most 64
 * rows (stacked MMAs), [22] the stage's MMA cycles at HH_PREC_BF16X3 summed
 * over its tiles (a K = 16 MMA costs max(45, width / 2) SM cycles), [23] its
 * tile shape (hh_plan_tune).  counts holds HH_PLAN_STATS = 24 doubles.      */
#define HH_PLAN_STATS 24
int hh_plan_stats(const hh_plan_t* p, double* counts);
int hh_plan_free(hh_plan_t* p);

/* model_wave (code/mat_vec.f90:3476): out = H in, device-resident waves;
 * waves holding nbatch vectors (hh_wave_create; in and out must hold the
 * same number): in split precision all of them in one batched replay (every
 * stage one launch over the batch; the batch schedule is built on the first
 * call for that nbatch and kept), in FP64 vector by vector.               */
int hh_matvec(hh_plan_t* p, const hh_wave_t* in, hh_wave_t* out, int precision);
/* model_wave with host buffers: copies in, multiplies, copies out (device
 * buffers of the plan are reused between calls).                          */
int hh_matvec_host(hh_plan_t* p, const double* in, double* out, int precision);
/* hh_matvec with CUDA events on the context stream around each stage;
 * ms[0] = whole matvec, ms[1] = stage 1 (left products), ms[2] = stage 2
 * (its tile kernel; the site-diagonal copy terms that follow are the rest of
 * ms[0]), ms[3] = BF16 split of the input wave (split-precision path
 * only).                                                                  */
int hh_matvec_timed(hh_plan_t* p, const hh_wave_t* in, hh_wave_t* out, int precision, float* ms);

/* hh_matvec (FP64) that allocates nothing during the call.  No counterpart
 * in the reference: it exists for callers that cannot call cudaMalloc when
 * they multiply (their own pool already holds the GPU's memory, or a fixed
 * device budget is reserved up front).  The stage-1 scratch is a static
 * device array of 64 MiB that every GPU loading the library holds until exit;
 * larger plans are rejected with HH_ERR_INVALID.  All calls on a device share
 * the array: calls that overlap on the GPU race.  hh_init looks up the
 * array's address (cudaGetSymbolAddress) with its device current, which loads
 * the array's module and reserves its 64 MiB when the context is created, not
 * in a matvec; calls must run with the CUDA context that was current in
 * hh_init (the device's primary context for runtime-API callers).  Waves of
 * nbatch vectors are multiplied vector by vector, in and out holding the same
 * number.                                                                  */
int hh_matvec_noalloc(hh_plan_t* p, const hh_wave_t* in, hh_wave_t* out);

/* pinned host memory for the caller's wave buffers (fast H2D/D2H copies)   */
int hh_host_alloc(long long bytes, void** ptr);
int hh_host_free(void* ptr);

/* hh_matvec without the wait: queued on the context stream (the tensor-core
 * path as one CUDA-graph replay after its first call); a bounded wait that
 * ran out is reported by the next hh_plan_check, which waits for the stream. */
int hh_matvec_async(hh_plan_t* plan, const hh_wave_t* in, hh_wave_t* out, int precision);
int hh_plan_check(hh_plan_t* plan);
/* Autotuner of the split-precision schedule: for each of the HH_TILE_SHAPES
 * shapes of the stage-2 output tiles (0: 128 rows x 64 columns; 1: every
 * output rectangle in near-equal tiles of at most 64 rows x 64 columns; 2:
 * 128 x 64, remainders of 65-127 rows in two tiles of at most 64; 3: 128 x
 * 128) it times the
 * four launch variants of the tile GEMM (stage 1 / stage 2 on the persistent
 * kernel or one CTA per tile) on this plan at the given split precision, reps
 * runs each after a warm-up, and keeps the fastest shape and variant for the
 * plan's later matvecs.  ms (may be NULL) receives HH_TUNE_VARIANTS mean
 * times in ms, index 4 * shape + 2 * stage1_persistent + stage2_persistent;
 * *choice (may be NULL) the kept index.  FP64 plans have nothing to tune
 * (choice 0).  hh_plan_set_tiles fixes the shape without timing (the
 * split-precision schedule is rebuilt at the next split matvec).          */
#define HH_TILE_SHAPES 4
#define HH_TUNE_VARIANTS 16
int hh_plan_tune(hh_plan_t* plan, int precision, int reps, double* ms, int* choice);
int hh_plan_set_tiles(hh_plan_t* plan, int shape);
/* lanczos_memo_new (code/lanczos.f90:4-177), levels = 1.  psi is the start
 * vector on entry and the ground state on exit; lanzero is the breakdown and
 * convergence threshold; maxit <= 100 is loop_in.  With a split precision
 * (HH_PREC_BF16X6, HH_PREC_BF16X3) the
 * Krylov recurrence first runs on the split-precision matvec until the Ritz
 * value moves by <= max(lanzero, 1e-8); a second Lanczos restarted from that
 * vector takes its first product in FP64-class arithmetic (double-float or
 * FP64, hh_ctx_set_restart_precision) and the rest in split precision and
 * converges to lanzero (one such product per call); *iterations counts the
 * Krylov vectors of both passes.  HH_PREC_FP32X2 runs every product in
 * double-float.                                                           */
int hh_lanczos(hh_plan_t* p, hh_wave_t* psi, double lanzero, int maxit,
               int precision, double* energy, int* iterations);
/* Fills a wave with uniform [0,1) real and imaginary parts from a seeded
 * generator and normalises it (wave_initialize, code/space_info.f90:1079).  */
int hh_wave_random(hh_wave_t* w, unsigned long long seed);

/* ------------------------------------------- density matrix and truncation
 * Get_density_matrix_sys/env + Get_truncation_operator (code/get_den.f90:4-99,
 * 184-428): rho = psi psi^H (side 0, sys) or psi^H psi (side 1, env) per
 * sector, per-sector Hermitian eigensolve (ascending, eigenvector phases fixed
 * so that the largest-modulus component is real positive), global descending
 * sort (the reference's quicksort), normalisation to trace 1, selection from
 * kept_min until the discarded weight is <= trun_err or kept_max states are
 * kept.  *trun receives the truncation operator (enlarged x kept per sector,
 * device resident); spectrum (may be NULL) receives the sorted normalised
 * eigenvalues (total dimension of the side).                             */
int hh_density_truncate(hh_ctx_t* ctx, const hh_wave_t* psi, int side, int kept_min, int kept_max,
                        double trun_err, hh_block_t** trun, int* num_state, double* discarded,
                        double* entropy, double* spectrum);
/* update_trun_dia (dia = 1) / update_trun_ndia (dia = 0), code/update.f90:
 * 1387-1605: *out = T^H O T sector pair by sector pair.                    */
int hh_renormalize(hh_ctx_t* ctx, const hh_block_t* op, const hh_block_t* trun, int dia, hh_block_t** out);
/* wave_trans_LR (dir 0) / wave_trans_RL (dir 1), code/warm_up.f90:1855-2170:
 * the initial Lanczos vector of the next superblock from the last ground
 * state; sys_bs/env_bs are the bases the reference passes (the new sys basis
 * and the old env basis for LR, the old sys basis and the new env basis for
 * RL); new_wave is overwritten and normalised.                            */
int hh_wave_transform(hh_ctx_t* ctx, int dir, const hh_basis_t* sys_bs, const hh_basis_t* env_bs,
                      const hh_block_t* sys_trun, const hh_block_t* env_trun, const hh_wave_t* old_wave,
                      hh_wave_t* new_wave);

/* ------------------------------------------------------- block enlargement
 * Embeds an operator in the enlarged basis B (block + site), returning a new
 * block: mode 0 update_block_dia, 1 update_site_dia, 2 update_block_ndia_sys/
 * env, 3 update_site_ndia_sys/env (code/update.f90:419-1381); flag 'F'/'B',
 * side 0 sys / 1 env (fermion sign conventions of the two sides).          */
int hh_enlarge_operator(hh_ctx_t* ctx, int mode, const hh_block_t* op, const hh_basis_t* B, int flag, int side,
                        hh_block_t** out);
/* Get_hamiltonian_ndia (code/get_ham.f90:954-1152): ham += coef [O_block .
 * O_site]^0 + h.c.; site_trans = 1 passes the site operator through
 * block_transfer_trans; flags 'S' (sys) or 'E' (env).                     */
int hh_ham_add_bond(hh_ctx_t* ctx, hh_block_t* ham, const hh_block_t* block, const hh_block_t* site,
                    int site_trans, const hh_basis_t* B, const double* coef, int flag_sign, int flags);
/* Get_hamiltonian_dia (code/get_ham.f90:852-941): ham += coef/sqrt(2S+1) O1 O2 */
int hh_ham_add_product(hh_ctx_t* ctx, hh_block_t* ham, const hh_block_t* o1, const hh_block_t* o2,
                       const double* coef);
/* block_mul_block_ndia, flags 'N' 'N' (code/space_info.f90:373-631):
 * *out = coef (o1 o2)^K, the product of two operators of one block coupled
 * to rank K = down_dif / 2, laid out over the sectors of the basis B.      */
int hh_block_product(hh_ctx_t* ctx, const hh_block_t* o1, const hh_block_t* o2, int down_dif,
                     const hh_basis_t* B, const double* coef, hh_block_t** out);
/* block_transfer (code/space_info.f90:100-129): device copy of a block     */
int hh_block_copy(hh_ctx_t* ctx, const hh_block_t* src, hh_block_t** out);

/* --------------------------------------- learned initial-guess corrector
 * No counterpart in the reference: a per-sector MLP that corrects the
 * wave_trans_LR/RL guess (code/warm_up.f90:1855-2170) before
 * lanczos_memo_new (code/lanczos.f90:4).  Network: nfeat inputs -> 64 -> 64
 * -> 1, tanh hidden layers, FP32, trained full batch with Adam on the
 * weighted mean squared error sum_s w_s (y_s - t_s)^2 / sum_s w_s.
 * Parameters (hh_mlp_nparams floats): W1[64][nfeat] row-major, b1[64],
 * W2[64][64] (out, in) row-major, b2[64], W3[64], b3.  x is n x nfeat
 * row-major; all buffers are host memory; w may be NULL (unit weights).  */
int hh_mlp_create(hh_ctx_t* ctx, int nfeat, unsigned long long seed, hh_mlp_t** mlp);
int hh_mlp_free(hh_mlp_t* mlp);
int hh_mlp_nparams(const hh_mlp_t* mlp, int* n);
int hh_mlp_get_params(const hh_mlp_t* mlp, float* params);
/* also resets the Adam state                                              */
int hh_mlp_set_params(hh_mlp_t* mlp, const float* params);
int hh_mlp_forward(hh_mlp_t* mlp, const float* x, int n, float* y);
/* loss and its gradient with respect to the parameters (grad may be NULL) */
int hh_mlp_loss_grad(hh_mlp_t* mlp, const float* x, const float* t, const float* w, int n, float* loss,
                     float* grad);
/* epochs full-batch Adam steps (beta 0.9/0.999, eps 1e-8, learning rate lr),
 * one epoch captured as a CUDA graph; *final_loss (may be NULL) is the loss
 * at the trained parameters.                                              */
int hh_mlp_train(hh_mlp_t* mlp, const float* x, const float* t, const float* w, int n, int epochs, float lr,
                 float* final_loss);
/* Squared norm of every sector of a wave (host array, one per sector, in the
 * wave's sector order).                                                   */
int hh_wave_sector_norms(const hh_wave_t* w, double* norms2);
/* Multiplies sector k of a wave by scale[k] (host array).                 */
int hh_wave_scale_sectors(hh_wave_t* w, const double* scale);

/* Diagnostic: C = A B for dense complex column-major A (M x K), B (K x N)
 * through the split-precision tensor-core tile kernel (host buffers) at a
 * split precision (HH_PREC_BF16X6 or HH_PREC_BF16X3).                     */
int hh_tc_selftest(hh_ctx_t* ctx, int M, int N, int K, const double* A, const double* B, double* C,
                   int precision);
/* Failure-detection check of the tensor-core kernels: one tile whose first
 * chunk is announced to its copy barrier but never sent, so the kernel's
 * bounded waits run out (short limit) and it unwinds (TMEM freed, no copy in
 * flight).  Returns HH_ERR_TIMEOUT (hh_last_error names the wait that gave
 * up); the context stays usable.                                          */
int hh_tc_selftest_hold(hh_ctx_t* ctx, int precision);

#ifdef __cplusplus
}
#endif
#endif /* HH_DMRG_H */
