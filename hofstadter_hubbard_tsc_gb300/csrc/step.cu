// The rest of the superblock step on the GPU: reduced density matrix and
// per-sector truncation (code/get_den.f90), operator renormalisation
// (update_trun_dia/ndia, code/update.f90:1387-1605) and the wavefunction
// transformations (wave_trans_LR/RL, code/warm_up.f90:1855-2170).
//
// Products run on the FP64 grouped segment GEMM; the per-sector Hermitian
// eigensolves (ascending eigenvalues like the ZHEEV call of
// code/get_den.f90:242) are eig.cu's batched solver.  The global sort and the
// selection of kept states are host work on the eigenvalues only.
#include <algorithm>
#include <cmath>
#include <map>
#include <tuple>
#include <vector>

#include "hh_internal.h"

namespace hh {
namespace {

constexpr int TM = 64, TN = 64;

// Device-side task lists used once per call.
struct GemmRun {
  hh_gemm_list L;
  // queued on the context stream; the task list returns to the pool in
  // stream order, so nothing here waits for the device
  int run(hh_ctx* ctx, double2* base_in, double2* base_scr, double2* base_out, int arith = kArithFp64) {
    L.upload(ctx);
    cudaError_t e = launch_segment_gemm_fp64(L, base_in, base_scr, base_out, ctx->stream, arith);
    L.release();
    return cuda_check(ctx, e, "step GEMM");
  }
  void add_rect(long long ooff, int obase, int ldo, int M, int N, const std::vector<hh_seg>& segs, int accumulate) {
    int seg0 = (int)L.segs.size();
    for (const auto& s : segs) L.segs.push_back(s);
    for (int m0 = 0; m0 < M; m0 += TM)
      for (int n0 = 0; n0 < N; n0 += TN) {
        hh_tile t{};
        t.ooff = ooff;
        t.obase = obase;
        t.ldo = ldo;
        t.M = M;
        t.N = N;
        t.m0 = m0;
        t.n0 = n0;
        t.seg0 = seg0;
        t.nseg = (int)segs.size();
        t.accumulate = accumulate;
        L.tiles.push_back(t);
      }
  }
};

hh_seg gemm_seg(long long poff, int pbase, int ldp, int opP, long long qoff, int qbase, int ldq, int opQ, int K,
                double cre = 1.0, double cim = 0.0) {
  hh_seg s{};
  s.poff = poff;
  s.pbase = pbase;
  s.ldp = ldp;
  s.opP = opP;
  s.qoff = qoff;
  s.qbase = qbase;
  s.ldq = ldq;
  s.opQ = opQ;
  s.K = K;
  s.kind = HH_SEG_GEMM;
  s.cre = cre;
  s.cim = cim;
  return s;
}

long long addr(const hh_block* b, int j) { return (long long)(uintptr_t)(b->d + b->subs[j].off); }

// QuickSort_Double of the reference (code/update.f90:322-368): descending,
// middle pivot, Hoare partition, index array carried along.  Restated exactly
// so that ties among eigenvalues of different sectors are resolved in the
// reference's order.
void quicksort_double(std::vector<double>& a, std::vector<int>& idx, int lower, int upper) {
  std::vector<std::pair<int, int>> stack{{lower, upper}};
  while (!stack.empty()) {
    auto [lo, hi] = stack.back();
    stack.pop_back();
    int i = lo, j = hi;
    const double pivot = a[(lo + hi + 2) / 2 - 1];
    while (i <= j) {
      while (a[i] > pivot) ++i;
      while (a[j] < pivot) --j;
      if (i <= j) {
        std::swap(a[i], a[j]);
        std::swap(idx[i], idx[j]);
        ++i;
        --j;
      }
    }
    if (i < hi) stack.push_back({i, hi});
    if (lo < j) stack.push_back({lo, j});
  }
}

int make_block(hh_ctx* ctx, int len, int up_dif, int down_dif, const std::vector<int>& qn, hh_block** out) {
  return hh_block_zeros(ctx, len, up_dif, down_dif, (int)(qn.size() / 5), qn.empty() ? nullptr : qn.data(), out);
}

}  // namespace
}  // namespace hh

using namespace hh;


extern "C" int hh_density_truncate(hh_ctx_t* ctx, const hh_wave_t* psi, int side, int kept_min, int kept_max,
                                   double trun_err, hh_block_t** trun_out, int* num_state_out, double* discarded,
                                   double* entropy, double* spectrum) {
  if (!ctx || !psi || !trun_out || (side != 0 && side != 1) || kept_min < 0 || kept_max < 0) return HH_ERR_INVALID;
  *trun_out = nullptr;
  // ---- density matrices, one sub per wave sector (code/get_den.f90:4-99)
  std::vector<int> qn;
  for (const auto& w : psi->secs) {
    const int d = side == 0 ? w.sdim : w.edim;
    qn.insert(qn.end(), {side == 0 ? w.su : w.eu, side == 0 ? w.sd : w.ed, 0, d, d});
  }
  hh_block* den = nullptr;
  int st = make_block(ctx, side == 0 ? psi->sys_len : psi->env_len, 0, 0, qn, &den);
  if (st) return st;
  GemmRun G;
  for (size_t k = 0; k < psi->secs.size(); ++k) {
    const hh_wsec& w = psi->secs[k];
    if (w.sdim == 0 || w.edim == 0) continue;
    std::vector<hh_seg> s;
    if (side == 0)  // rho_s = psi psi^H
      s.push_back(gemm_seg(w.off, HH_BASE_IN, w.sdim, HH_OP_N, w.off, HH_BASE_IN, w.sdim, HH_OP_C, w.edim));
    else  // rho_e = psi^H psi
      s.push_back(gemm_seg(w.off, HH_BASE_IN, w.sdim, HH_OP_C, w.off, HH_BASE_IN, w.sdim, HH_OP_N, w.sdim));
    const int d = side == 0 ? w.sdim : w.edim;
    G.add_rect(den->subs[k].off, HH_BASE_OUT, d, d, d, s, 0);
  }
  if ((st = G.run(ctx, psi->d, nullptr, den->d))) {
    hh_block_free(den);
    return st;
  }
  // ---- per-sector eigensolve (ZHEEV 'V','U', ascending; code/get_den.f90:242):
  // every eigenvalue now, the eigenvectors of the kept states once they are known
  long long nev = 0;
  std::vector<long long> offs;
  std::vector<int> dims;
  for (const auto& sq : den->subs) {
    offs.push_back(sq.off);
    dims.push_back(sq.sdim);
    nev += sq.sdim;
  }
  const bool own = ctx->eig_solver == HH_EIG_OWN;
  std::vector<double> w(std::max<long long>(1, nev));
  cudaError_t e = cudaSuccess;
  if (own) {
    st = eig_values(ctx, den->d, offs, dims, false, w);
  } else {
    double* d_w = nullptr;
    st = eig_hermitian_sectors(ctx, den->d, offs, dims, &d_w);
    if (!st) {
      e = cudaMemcpy(w.data(), d_w, nev * sizeof(double), cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) st = cuda_check(ctx, e, "density eigenvalues");
    }
  }
  if (st) {
    hh_block_free(den);
    return st;
  }
  // ---- global sort, renormalisation, selection (code/get_den.f90:268-311)
  std::vector<double> arr(w.begin(), w.begin() + nev);
  std::vector<int> idx(nev);
  for (long long i = 0; i < nev; ++i) idx[i] = (int)i + 1;
  if (nev > 0) quicksort_double(arr, idx, 0, (int)nev - 1);
  double tot = 0.0;
  for (double a : arr) tot += a;
  for (double& a : arr) a /= tot;
  long long num_state;
  double err = 0.0;
  if (nev <= kept_min) {
    num_state = nev;
  } else {
    for (long long i = kept_min; i < nev; ++i) err += arr[i];
    num_state = kept_min;
    while (err > trun_err) {
      ++num_state;
      err -= arr[num_state - 1];
      if (err <= trun_err || num_state >= kept_max) break;
    }
  }
  double ent = 0.0;  // code/get_den.f90:317-326
  for (double a : arr)
    if (a >= 1.0e-15) ent -= a * std::log(a);
  std::vector<char> kept(nev + 1, 0);
  for (long long i = 0; i < num_state; ++i) kept[idx[i]] = 1;
  // ---- truncation operator: top columns of every sector (code/get_den.f90:362-412)
  std::vector<int> tqn;
  std::vector<std::pair<int, int>> tcols;  // (sector, ncol)
  long long gid = 1;
  for (size_t k = 0; k < den->subs.size(); ++k) {
    const int n = den->subs[k].sdim;
    int ncol = 0;
    for (int i = 0; i < n; ++i, ++gid) ncol += kept[gid];
    if (ncol > 0) {
      tqn.insert(tqn.end(), {den->subs[k].up, den->subs[k].down, 0, n, ncol});
      tcols.push_back({(int)k, ncol});
    }
  }
  hh_block* trun = nullptr;
  if ((st = make_block(ctx, den->len, 0, 0, tqn, &trun))) {
    hh_block_free(den);
    return st;
  }
  if (own) {
    std::vector<int> ncolv(den->subs.size(), 0);
    std::vector<long long> xoff(den->subs.size(), 0);
    for (size_t t = 0; t < tcols.size(); ++t) {
      ncolv[tcols[t].first] = tcols[t].second;
      xoff[tcols[t].first] = trun->subs[t].off;
    }
    st = eig_vectors(ctx, ncolv, trun->d, xoff);
    if (st) {
      hh_block_free(den);
      hh_block_free(trun);
      return st;
    }
  } else {
    for (size_t t = 0; t < tcols.size(); ++t) {
      const auto& ds = den->subs[tcols[t].first];
      const int n = ds.sdim, ncol = tcols[t].second;
      e = cudaMemcpyAsync(trun->d + trun->subs[t].off, den->d + ds.off + (long long)(n - ncol) * n,
                          (size_t)n * ncol * sizeof(double2), cudaMemcpyDeviceToDevice, ctx->stream);
      if (e != cudaSuccess) break;
    }
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  hh_block_free(den);
  if (e != cudaSuccess) {
    hh_block_free(trun);
    return cuda_check(ctx, e, "truncation operator");
  }
  *trun_out = trun;
  if (num_state_out) *num_state_out = (int)num_state;
  if (discarded) *discarded = err;
  if (entropy) *entropy = ent;
  if (spectrum)
    for (long long i = 0; i < nev; ++i) spectrum[i] = arr[i];
  return HH_OK;
}

extern "C" int hh_ctx_set_eigensolver(hh_ctx_t* ctx, int solver) {
  if (!ctx || (solver != HH_EIG_OWN && solver != HH_EIG_CUSOLVER)) return HH_ERR_INVALID;
  ctx->eig_solver = solver;
  return HH_OK;
}

extern "C" int hh_ctx_set_transform_precision(hh_ctx_t* ctx, int precision) {
  if (!ctx || (precision != HH_PREC_FP64 && precision != HH_PREC_FP32)) return HH_ERR_INVALID;
  ctx->transform_precision = precision;
  return HH_OK;
}

extern "C" int hh_ctx_set_renormalize_precision(hh_ctx_t* ctx, int precision) {
  if (!ctx || (precision != HH_PREC_FP64 && precision != HH_PREC_FP32X2)) return HH_ERR_INVALID;
  ctx->renorm_precision = precision;
  return HH_OK;
}

extern "C" int hh_ctx_set_krylov_storage(hh_ctx_t* ctx, int precision) {
  if (!ctx || (precision != HH_PREC_FP64 && precision != HH_PREC_FP32)) return HH_ERR_INVALID;
  ctx->krylov_f32 = precision == HH_PREC_FP32;
  return HH_OK;
}

extern "C" int hh_ctx_set_restart_precision(hh_ctx_t* ctx, int precision) {
  if (!ctx || (precision != HH_PREC_FP64 && precision != HH_PREC_FP32X2)) return HH_ERR_INVALID;
  ctx->restart_precision = precision;
  return HH_OK;
}

extern "C" int hh_eig_selftest(hh_ctx_t* ctx, int n, const double* A, double* w, double* V) {
  if (!ctx || n <= 0 || !A || !w || !V) return HH_ERR_INVALID;
  const size_t bytes = (size_t)n * n * sizeof(double2);
  double2 *dA = nullptr, *dX = nullptr;
  cudaError_t e = dev_alloc(ctx, (void**)&dA, bytes);
  if (e == cudaSuccess) e = dev_alloc(ctx, (void**)&dX, bytes);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dA, A, bytes, cudaMemcpyHostToDevice, ctx->stream);
  int st = e == cudaSuccess ? HH_OK : cuda_check(ctx, e, "eig selftest set-up");
  std::vector<double> wh;
  if (!st) st = eig_values(ctx, dA, {0}, {n}, true, wh);
  if (!st) st = eig_vectors(ctx, {n}, dX, {0});
  if (!st) {
    e = cudaMemcpyAsync(V, dX, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) st = cuda_check(ctx, e, "eig selftest");
    for (int i = 0; i < n && !st; ++i) w[i] = wh[i];
  }
  dev_free(ctx, dA);
  dev_free(ctx, dX);
  return st;
}

extern "C" int hh_renormalize(hh_ctx_t* ctx, const hh_block_t* ori, const hh_block_t* trun, int dia,
                              hh_block_t** out) {
  if (!ctx || !ori || !trun || !out) return HH_ERR_INVALID;
  *out = nullptr;
  const int k = ori->down_dif, up_dif = ori->up_dif;
  std::map<std::pair<int, int>, int> tidx;
  for (int j = (int)trun->subs.size() - 1; j >= 0; --j) tidx[{trun->subs[j].up, trun->subs[j].down}] = j;
  auto tfind = [&](int up, int down) {
    auto it = tidx.find({up, down});
    return it == tidx.end() ? -1 : it->second;
  };
  // layout (code/update.f90:1404-1423 dia, 1478-1532 ndia)
  std::vector<int> qn;
  std::vector<std::tuple<int, int, int>> pieces;  // (eff index, lhs trun, rhs trun)
  if (dia) {
    for (size_t x = 0; x < trun->subs.size(); ++x) {
      qn.insert(qn.end(), {trun->subs[x].up, trun->subs[x].down, 0, trun->subs[x].sdim, trun->subs[x].sdim});
      pieces.emplace_back((int)x, (int)x, (int)x);
    }
  } else {
    for (size_t x = 0; x < trun->subs.size(); ++x)
      for (int dd = -k; dd <= k; dd += 2) {
        int l = tfind(trun->subs[x].up + up_dif, trun->subs[x].down + dd);
        if (l >= 0) {
          pieces.emplace_back((int)(qn.size() / 5), l, (int)x);
          qn.insert(qn.end(), {trun->subs[x].up, trun->subs[x].down, dd, trun->subs[l].sdim, trun->subs[x].sdim});
        }
      }
  }
  hh_block* eff = nullptr;
  int st = make_block(ctx, ori->len, up_dif, ori->down_dif, qn, &eff);
  if (st) return st;
  GemmRun G1, G2;
  long long scr = 0;
  for (const auto& pc : pieces) {
    const int ei = std::get<0>(pc), li = std::get<1>(pc), ri = std::get<2>(pc);
    const hh_sub_qn& es = eff->subs[ei];
    int oi = dia ? ori->find2(es.up, es.down) : ori->find3(es.up, es.down, es.dd);
    if (oi < 0) continue;
    const hh_sub_qn& os = ori->subs[oi];
    const hh_sub_qn& tr = trun->subs[ri];
    const hh_sub_qn& tl = trun->subs[li];
    if (os.sdim != tr.row || os.row != tl.row) {
      hh_block_free(eff);
      return fail(ctx, HH_ERR_QN, "hh_renormalize: operator and truncation dimensions differ");
    }
    if (os.row == 0 || tr.sdim == 0 || tl.sdim == 0) continue;
    // mid = O T_rhs (ori_row x rhs_dim), eff = T_lhs^H mid
    std::vector<hh_seg> s1{gemm_seg(addr(ori, oi), HH_BASE_ABS, os.row, HH_OP_N, addr(trun, ri), HH_BASE_ABS,
                                    tr.row, HH_OP_N, os.sdim)};
    G1.add_rect(scr, HH_BASE_SCR, os.row, os.row, tr.sdim, s1, 0);
    std::vector<hh_seg> s2{gemm_seg(addr(trun, li), HH_BASE_ABS, tl.row, HH_OP_C, scr, HH_BASE_SCR, os.row,
                                    HH_OP_N, os.row)};
    G2.add_rect(es.off, HH_BASE_OUT, es.row, es.row, es.sdim, s2, 0);
    scr += (long long)os.row * tr.sdim;
  }
  double2* d_scr = nullptr;
  cudaError_t e = dev_alloc(ctx, (void**)&d_scr, std::max<long long>(1, scr) * sizeof(double2));
  if (e != cudaSuccess) {
    hh_block_free(eff);
    return cuda_check(ctx, e, "renormalise scratch");
  }
  const int arith = ctx->renorm_precision == HH_PREC_FP32X2 ? kArithDf : kArithFp64;
  st = G1.run(ctx, nullptr, d_scr, eff->d, arith);
  if (!st) st = G2.run(ctx, nullptr, d_scr, eff->d, arith);
  dev_free(ctx, d_scr);
  if (st) {
    hh_block_free(eff);
    return st;
  }
  *out = eff;
  return HH_OK;
}

// wave_trans_LR (dir 0, code/warm_up.f90:1855-2012) and wave_trans_RL (dir 1,
// code/warm_up.f90:2016-2170): new_wave = sum of coef * T_sys^(H) psi T_env^(H)
// pieces re-blocked into the next superblock, then normalised.
extern "C" int hh_wave_transform(hh_ctx_t* ctx, int dir, const hh_basis_t* sys_bs, const hh_basis_t* env_bs,
                                 const hh_block_t* sys_trun, const hh_block_t* env_trun, const hh_wave_t* old_wave,
                                 hh_wave_t* new_wave) {
  if (!ctx || !sys_bs || !env_bs || !sys_trun || !env_trun || !old_wave || !new_wave || (dir != 0 && dir != 1))
    return HH_ERR_INVALID;
  if (old_wave->d == new_wave->d) return HH_ERR_INVALID;
  struct Piece {
    int k, i;
    int orow, ocol, M, N;       // output rect in new sector k
    int irow, icol, Ka, Kb;     // input region in old sector i
    long long a, b;             // operator sub addresses
    int lda, ldb, opa, opb;
    double c;
  };
  std::vector<Piece> P;
  auto psign = [](int n) { return ((n / 2) % 2) ? -1.0 : 1.0; };
  for (size_t ii = 0; ii < old_wave->secs.size(); ++ii) {
    const hh_wsec& ow = old_wave->secs[ii];
    if (dir == 0) {
      int st_id = sys_trun->find2(ow.su, ow.sd);
      if (st_id < 0) continue;
      int es = env_bs->find(ow.eu, ow.ed);
      if (es < 0) continue;
      for (const auto& x : env_bs->secs[es].subs) {
        const int su = x.su, sd = x.sd, neu = x.bu, ned = x.bd;
        int et_id = env_trun->find2(neu, ned);
        for (int nsd = std::abs(ow.sd - sd); nsd <= ow.sd + sd; nsd += 2) {
          int nsu = ow.su + su;
          int ss = sys_bs->find(nsu, nsd);
          if (ss < 0 || et_id < 0) continue;
          auto it = sys_bs->secs[ss].full.find(key4(ow.su, ow.sd, su, sd));
          if (it == sys_bs->secs[ss].full.end()) continue;
          const hh_bsub& y = sys_bs->secs[ss].subs[it->second];
          int k = new_wave->find(nsu, nsd, neu, ned);
          if (k < 0) continue;
          const int j12 = ow.sd, j3 = sd, j4 = ned, j123 = nsd, j34 = ow.ed;
          double c = psign(j12 + j3 + j123) / std::sqrt((1.0 + j12) * (1.0 + j123));
          c *= std::sqrt((1.0 + j123) * (j34 + 1.0));
          if (((j12 + j3 + j4) / 2) % 2) c = -c;
          if (((j3 + j4 - j34) / 2) % 2) c = -c;
          const hh_sub_qn& T = sys_trun->subs[st_id];
          const hh_sub_qn& E = env_trun->subs[et_id];
          const hh_wsec& nw = new_wave->secs[k];
          if (T.row != ow.sdim || T.sdim != y.sdim || E.sdim != x.sdim || E.row != nw.edim)
            return fail(ctx, HH_ERR_QN, "hh_wave_transform: truncation and basis dimensions differ");
          // new[y rows, :] += c T^H old[:, x cols] E^H
          P.push_back({k, (int)ii, y.spos, 0, y.sdim, nw.edim, 0, x.spos, ow.sdim, x.sdim,
                       addr(sys_trun, st_id), addr(env_trun, et_id), T.row, E.row, HH_OP_C, HH_OP_C, c});
        }
      }
    } else {
      int et_id = env_trun->find2(ow.eu, ow.ed);
      if (et_id < 0) continue;
      int ss = sys_bs->find(ow.su, ow.sd);
      if (ss < 0) continue;
      for (const auto& x : sys_bs->secs[ss].subs) {
        const int sd = x.sd, su = x.su, nsu = x.bu, nsd = x.bd;
        for (int ned = std::abs(ow.ed - sd); ned <= ow.ed + sd; ned += 2) {
          int neu = ow.eu + su;
          int st_id = sys_trun->find2(nsu, nsd);
          int es = env_bs->find(neu, ned);
          if (st_id < 0 || es < 0) continue;
          auto it = env_bs->secs[es].full.find(key4(ow.eu, ow.ed, su, sd));
          if (it == env_bs->secs[es].full.end()) continue;
          const hh_bsub& y = env_bs->secs[es].subs[it->second];
          int k = new_wave->find(nsu, nsd, neu, ned);
          if (k < 0) continue;
          const int j12 = ow.ed, j3 = sd, j4 = nsd, j123 = ned, j34 = ow.sd;
          double c = psign(j34 + j4 + j3) / std::sqrt((1.0 + j12) * (1.0 + j4));
          c *= std::sqrt((1.0 + j123) * (j34 + 1.0));
          if (((j4 + j3 + j12) / 2) % 2) c = -c;
          if (((j12 + j3 - j123) / 2) % 2) c = -c;
          const hh_sub_qn& T = sys_trun->subs[st_id];
          const hh_sub_qn& E = env_trun->subs[et_id];
          const hh_wsec& nw = new_wave->secs[k];
          if (T.sdim != x.sdim || T.row != nw.sdim || E.row != ow.edim || E.sdim != y.sdim)
            return fail(ctx, HH_ERR_QN, "hh_wave_transform: truncation and basis dimensions differ");
          // new[:, y cols] += c T old[x rows, :] E
          P.push_back({k, (int)ii, 0, y.spos, nw.sdim, y.sdim, x.spos, 0, x.sdim, ow.edim,
                       addr(sys_trun, st_id), addr(env_trun, et_id), T.row, E.row, HH_OP_N, HH_OP_N, c});
        }
      }
    }
  }
  // stage 1: S = opA(A) old_region (M x Kb) per distinct (old sector, region,
  // operator): the pieces that differ only in the new sector's spin (the
  // nsd / ned loops above) share it; stage 2: grouped by output rect
  GemmRun G1, G2;
  long long scr = 0;
  std::map<std::tuple<int, int, int, int, int, long long, int>, long long> s1_done;
  std::map<std::tuple<int, int, int, int, int>, std::vector<hh_seg>> rects;
  std::vector<std::tuple<int, int, int, int, int>> order;
  for (const Piece& q : P) {
    const hh_wsec& ow = old_wave->secs[q.i];
    const auto s1key = std::make_tuple(q.i, q.irow, q.icol, q.Ka, q.Kb, q.a, q.M);
    long long soff;
    auto found = s1_done.find(s1key);
    if (found != s1_done.end()) {
      soff = found->second;
    } else {
      std::vector<hh_seg> s1{gemm_seg(q.a, HH_BASE_ABS, q.lda, q.opa,
                                      ow.off + (long long)q.icol * ow.sdim + q.irow, HH_BASE_IN, ow.sdim, HH_OP_N,
                                      q.Ka)};
      G1.add_rect(scr, HH_BASE_SCR, q.M, q.M, q.Kb, s1, 0);
      soff = scr;
      s1_done.emplace(s1key, soff);
      scr += (long long)q.M * q.Kb;
    }
    auto key = std::make_tuple(q.k, q.orow, q.ocol, q.M, q.N);
    if (!rects.count(key)) order.push_back(key);
    rects[key].push_back(gemm_seg(soff, HH_BASE_SCR, q.M, HH_OP_N, q.b, HH_BASE_ABS, q.ldb, q.opb, q.Kb, q.c, 0.0));
  }
  for (const auto& key : order) {
    const auto& [k, orow, ocol, M, N] = key;
    const hh_wsec& nw = new_wave->secs[k];
    G2.add_rect(nw.off + (long long)ocol * nw.sdim + orow, HH_BASE_OUT, nw.sdim, M, N, rects[key], 0);
  }
  double2* d_scr = nullptr;
  cudaError_t e = dev_alloc(ctx, (void**)&d_scr, std::max<long long>(1, scr) * sizeof(double2));
  if (e == cudaSuccess) e = cudaMemsetAsync(new_wave->d, 0, (size_t)new_wave->nelem * sizeof(double2), ctx->stream);
  if (e != cudaSuccess) {
    dev_free(ctx, d_scr);
    return cuda_check(ctx, e, "wave transform scratch");
  }
  const int arith = ctx->transform_precision == HH_PREC_FP32 ? kArithFp32 : kArithFp64;
  int st = G1.run(ctx, old_wave->d, d_scr, new_wave->d, arith);
  if (!st) st = G2.run(ctx, old_wave->d, d_scr, new_wave->d, arith);
  dev_free(ctx, d_scr);
  if (st) return st;
  return hh_wave_normalize(new_wave);
}
