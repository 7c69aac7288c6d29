// Block enlargement on the GPU (code/update.f90:419-1381, code/get_ham.f90:
// 852-1152): embedding block and site operators in the enlarged basis and
// adding the block-site bonds to the enlarged Hamiltonian.  Every one of these
// routines is a set of scaled sub-block placements
//     dst_sub[r0:r0+R, c0:c0+C] += coef * op(src_sub)      (or coef * identity)
// whose positions and coefficients (6j symbols, phases, fermion signs) come
// from the same loop nests as the reference; the host builds the placement
// list, one kernel applies it.
#include <algorithm>
#include <cmath>
#include <map>
#include <vector>

#include "hh_internal.h"

namespace hh {
namespace {

constexpr int SU = 2;

struct Place {
  long long dst;   // absolute address of the destination origin
  long long src;   // absolute address of the source origin (0: identity)
  int ldd, lds;
  int rows, cols;
  int herm;        // 1: place src^H (rows x cols of the result)
  int pad;
  double cre, cim;
};

__global__ void place_kernel(const Place* __restrict__ P) {
  const Place p = P[blockIdx.x];
  double2* d = reinterpret_cast<double2*>(p.dst);
  const double2* s = reinterpret_cast<const double2*>(p.src);
  const long long n = (long long)p.rows * p.cols;
  for (long long e = threadIdx.x; e < n; e += blockDim.x) {
    const int r = (int)(e % p.rows), c = (int)(e / p.rows);
    double2 v;
    if (!s) {
      if (r != c) continue;
      v = make_double2(1.0, 0.0);
    } else if (p.herm) {
      v = s[(long long)c + (long long)r * p.lds];
      v.y = -v.y;
    } else {
      v = s[(long long)r + (long long)c * p.lds];
    }
    double2& o = d[(long long)r + (long long)c * p.ldd];
    o.x += p.cre * v.x - p.cim * v.y;
    o.y += p.cre * v.y + p.cim * v.x;
  }
}

inline double psign(int n) { return ((n / 2) & 1) ? -1.0 : 1.0; }
long long addr_of(const hh_block* b, int j) { return (long long)(uintptr_t)(b->d + b->subs[j].off); }

// Queued on the context stream: the placement list (copied from pageable
// host memory, so the vector may go at once) returns to the pool in stream
// order after the kernel; nothing waits for the device.
int run_places(hh_ctx* ctx, const std::vector<Place>& P) {
  if (P.empty()) return HH_OK;
  Place* d = nullptr;
  cudaError_t e = dev_alloc(ctx, (void**)&d, P.size() * sizeof(Place));
  if (e == cudaSuccess) e = cudaMemcpyAsync(d, P.data(), P.size() * sizeof(Place), cudaMemcpyHostToDevice, ctx->stream);
  // placements into one destination sub-block never overlap in the
  // reference's loops except for accumulations of the same element, which are
  // serialised by launching in chunks that touch disjoint destinations
  if (e == cudaSuccess) place_kernel<<<(unsigned)P.size(), 256, 0, ctx->stream>>>(d);
  if (e == cudaSuccess) e = cudaGetLastError();
  dev_free(ctx, d);
  return cuda_check(ctx, e, "placement");
}

// Placements that add into the same destination elements must not run in the
// same launch (no atomics): split the list into rounds where every destination
// rectangle is touched at most once.
int run_places_safe(hh_ctx* ctx, const std::vector<Place>& P) {
  std::vector<std::vector<Place>> rounds;
  std::vector<std::map<long long, int>> seen;  // dst -> count per round (same origin means same rectangle)
  for (const auto& p : P) {
    size_t r = 0;
    for (; r < rounds.size(); ++r)
      if (!seen[r].count(p.dst)) break;
    if (r == rounds.size()) {
      rounds.emplace_back();
      seen.emplace_back();
    }
    rounds[r].push_back(p);
    seen[r][p.dst] = 1;
  }
  for (const auto& R : rounds) {
    int st = run_places(ctx, R);
    if (st) return st;
  }
  return HH_OK;
}

int new_block(hh_ctx* ctx, int len, int up, int down, const std::vector<int>& qn, hh_block** out) {
  return hh_block_zeros(ctx, len, up, down, (int)(qn.size() / 5), qn.empty() ? nullptr : qn.data(), out);
}

// sub layout of update_*_ndia_* (code/update.f90:572-633)
void ndia_layout(const hh_basis* B, int up_dif, int k, std::vector<int>& qn) {
  for (const auto& sec : B->secs)
    for (int dd = -k; dd <= k; dd += SU) {
      int l = B->find(sec.up + up_dif, sec.down + dd);
      if (l >= 0) qn.insert(qn.end(), {sec.up, sec.down, dd, B->secs[l].dim, sec.dim});
    }
}

}  // namespace
}  // namespace hh

using namespace hh;

// mode: 0 update_block_dia, 1 update_site_dia, 2 update_block_ndia, 3 update_site_ndia
// side: 0 sys, 1 env; flag: 'F' or 'B'
extern "C" int hh_enlarge_operator(hh_ctx_t* ctx, int mode, const hh_block_t* op, const hh_basis_t* B, int flag,
                                   int side, hh_block_t** out) {
  if (!ctx || !op || !B || !out || mode < 0 || mode > 3) return HH_ERR_INVALID;
  *out = nullptr;
  std::vector<int> qn;
  std::vector<Place> P;
  hh_block* nb = nullptr;
  int st;
  if (mode <= 1) {
    for (const auto& sec : B->secs) qn.insert(qn.end(), {sec.up, sec.down, 0, sec.dim, sec.dim});
    if ((st = new_block(ctx, B->len, 0, 0, qn, &nb))) return st;
    for (size_t k = 0; k < B->secs.size(); ++k) {
      const auto& sec = B->secs[k];
      const long long base = addr_of(nb, (int)k);
      for (const auto& x : sec.subs) {
        int i = mode == 0 ? op->find2(x.bu, x.bd) : op->find2(x.su, x.sd);
        if (i < 0) continue;
        const auto& s = op->subs[i];
        const double c = std::sqrt((1.0 + sec.down) / (1.0 + s.down));
        Place p{};
        p.dst = base + (long long)16 * ((long long)x.spos * sec.dim + x.spos);
        p.ldd = sec.dim;
        p.rows = p.cols = x.sdim;
        if (mode == 0) {  // code/update.f90:450-460
          if (s.row < x.sdim || s.sdim < x.sdim) {
            hh_block_free(nb);
            return fail(ctx, HH_ERR_QN, "update_block_dia: block smaller than the basis sub-block");
          }
          p.src = addr_of(op, i);
          p.lds = s.row;
          p.cre = c;
        } else {  // code/update.f90:513-524: identity times the site element
          p.src = 0;
          p.lds = 1;
          const cplx v = op->scalar.empty() ? cplx(0, 0) : op->scalar[i];
          p.cre = c * v.real();
          p.cim = c * v.imag();
        }
        P.push_back(p);
      }
    }
  } else {
    const int k = op->down_dif, up_dif = op->up_dif;
    ndia_layout(B, up_dif, k, qn);
    if ((st = new_block(ctx, B->len, up_dif, k, qn, &nb))) return st;
    for (size_t i = 0; i < nb->subs.size(); ++i) {
      const auto& s = nb->subs[i];
      int rhs = B->find(s.up, s.down), lhs = B->find(s.up + up_dif, s.down + s.dd);
      if (rhs < 0 || lhs < 0) continue;
      const auto& R = B->secs[rhs];
      const auto& Lh = B->secs[lhs];
      for (const auto& x : R.subs) {
        for (int sdd = -k; sdd <= k; sdd += SU) {
          if (mode == 2) {  // update_block_ndia_sys/env (code/update.f90:548-958)
            int bid = op->find3(x.bu, x.bd, sdd);
            if (bid < 0) continue;
            const int lu = x.bu + up_dif, ld = x.bd + sdd;
            const hh_bsub* y = nullptr;
            for (const auto& yy : Lh.subs)
              if (yy.bu == lu && yy.bd == ld && yy.sd == x.sd) { y = &yy; break; }
            if (!y) continue;
            double sign = 1.0;
            if (side == 1 && flag == 'F' && (x.su % 2) == 1) sign = -1.0;
            double c = w6j(Lh.down, k, R.down, x.bd, x.sd, ld);
            c *= std::sqrt((1.0 + Lh.down) * (1.0 + R.down)) * psign(ld + x.sd + R.down + k);
            if (c == 0.0) continue;
            const auto& bs = op->subs[bid];
            Place p{};
            p.dst = addr_of(nb, (int)i) + (long long)16 * ((long long)x.spos * s.row + y->spos);
            p.ldd = s.row;
            p.src = addr_of(op, bid);
            p.lds = bs.row;
            p.rows = y->sdim;
            p.cols = x.sdim;
            p.cre = sign * c;
            P.push_back(p);
          } else {  // update_site_ndia_sys/env (code/update.f90:969-1381)
            int sid = op->find3(x.su, x.sd, sdd);
            if (sid < 0) continue;
            const int lu = x.su + up_dif, ld = x.sd + sdd;
            const hh_bsub* y = nullptr;
            for (const auto& yy : Lh.subs)
              if (yy.su == lu && yy.sd == ld && yy.bd == x.bd) { y = &yy; break; }
            if (!y) continue;
            double sign = 1.0;
            if (side == 0 && flag == 'F' && (x.bu % 2) == 1) sign = -1.0;
            double c = w6j(Lh.down, k, R.down, x.sd, x.bd, ld);
            c *= psign(x.bd + x.sd + Lh.down + k) * std::sqrt((1.0 + Lh.down) * (1.0 + R.down));
            if (c == 0.0) continue;
            const cplx v = op->scalar.empty() ? cplx(0, 0) : op->scalar[sid];
            Place p{};
            p.dst = addr_of(nb, (int)i) + (long long)16 * ((long long)x.spos * s.row + y->spos);
            p.ldd = s.row;
            p.src = 0;
            p.lds = 1;
            p.rows = p.cols = x.sdim;
            p.cre = sign * c * v.real();
            p.cim = sign * c * v.imag();
            P.push_back(p);
          }
        }
      }
    }
  }
  nb->build_index();
  if ((st = run_places_safe(ctx, P))) {
    hh_block_free(nb);
    return st;
  }
  *out = nb;
  return HH_OK;
}

// Get_hamiltonian_ndia (code/get_ham.f90:954-1152): ham += coef [O_block . O_site]^0 (+ h.c.)
// flags: 'S' (sys: sign from the block electron parity) or 'E' (env: sign from
// the site parity); site is used through its 1x1 reduced elements.
extern "C" int hh_ham_add_bond(hh_ctx_t* ctx, hh_block_t* ham, const hh_block_t* block, const hh_block_t* site,
                               int site_trans, const hh_basis_t* B, const double* coef, int flag_sign, int flags) {
  if (!ctx || !ham || !block || !site || !B || !coef) return HH_ERR_INVALID;
  const int up_dif = block->up_dif, k = block->down_dif;
  // the site operator, possibly seen through block_transfer_trans
  const int s_up = site_trans ? -site->up_dif : site->up_dif;
  const int s_rank = site->down_dif;
  auto site_find = [&](int up, int down, int dd) -> int {
    if (!site_trans) return site->find3(up, down, dd);
    for (size_t j = 0; j < site->subs.size(); ++j) {
      const auto& s = site->subs[j];
      if (s.up + site->up_dif == up && s.down + s.dd == down && -s.dd == dd) return (int)j;
    }
    return -1;
  };
  auto site_val = [&](int j) {
    cplx v = site->scalar.empty() ? cplx(0, 0) : site->scalar[j];
    return site_trans ? std::conj(v) : v;
  };
  const cplx cf(coef[0], coef[1]);
  std::vector<Place> P;
  for (size_t i = 0; i < ham->subs.size(); ++i) {
    const auto& hs = ham->subs[i];
    int rhs = B->find(hs.up, hs.down), lhs = B->find(hs.up, hs.down + hs.dd);
    if (rhs < 0 || lhs < 0) continue;
    const auto& R = B->secs[rhs];
    const auto& Lh = B->secs[lhs];
    for (const auto& x : R.subs) {
      for (int sdd = -k; sdd <= k; sdd += SU) {
        int bid = block->find3(x.bu, x.bd, sdd);
        if (bid < 0) continue;
        const int lsu = x.bu + up_dif, lsd = x.bd + sdd;
        for (int nsd = std::abs(x.sd - s_rank); nsd <= x.sd + s_rank; nsd += SU) {
          const int st_dd = x.sd - nsd, nsu = x.su - s_up;
          int sid = site_find(nsu, nsd, st_dd);
          const hh_bsub* y = nullptr;
          for (const auto& yy : Lh.subs)
            if (yy.bu == lsu && yy.bd == lsd && yy.sd == nsd) { y = &yy; break; }
          if (!y || sid < 0) continue;
          double c = w6j(lsd, x.bd, k, x.sd, nsd, R.down);
          c *= std::sqrt((1.0 + R.down) / (1.0 + k)) * psign(x.bd + nsd + k + R.down);
          const cplx cv = c * site_val(sid);
          double sign = 1.0;
          if (flags == 'S') {
            if (flag_sign == 'F' && x.bu % 2 == 1) sign = -1.0;
          } else {
            if (flag_sign == 'F' && x.su % 2 == 0) sign = -1.0;
          }
          if (cv == cplx(0, 0)) continue;
          const cplx c1 = cv * cf * sign;
          const auto& bs = block->subs[bid];
          Place p{};
          p.dst = addr_of(ham, (int)i) + (long long)16 * ((long long)x.spos * hs.row + y->spos);
          p.ldd = hs.row;
          p.src = addr_of(block, bid);
          p.lds = bs.row;
          p.rows = y->sdim;
          p.cols = x.sdim;
          p.cre = c1.real();
          p.cim = c1.imag();
          P.push_back(p);
          if (s_up != 0) {  // the h.c. block at the transposed position
            Place q{};
            q.dst = addr_of(ham, (int)i) + (long long)16 * ((long long)y->spos * hs.row + x.spos);
            q.ldd = hs.row;
            q.src = addr_of(block, bid);
            q.lds = bs.row;
            q.rows = x.sdim;
            q.cols = y->sdim;
            q.herm = 1;
            q.cre = c1.real();
            q.cim = -c1.imag();
            P.push_back(q);
          }
        }
      }
    }
  }
  return run_places_safe(ctx, P);
}

// Get_hamiltonian_dia (code/get_ham.f90:852-941) with FlagConjg = false:
// ham += coef / sqrt(2S+1) O1 O2 per sector (products on the FP64 GEMM).
extern "C" int hh_ham_add_product(hh_ctx_t* ctx, hh_block_t* ham, const hh_block_t* o1, const hh_block_t* o2,
                                  const double* coef) {
  if (!ctx || !ham || !o1 || !o2 || !coef) return HH_ERR_INVALID;
  hh_gemm_list L;
  for (size_t i = 0; i < ham->subs.size(); ++i) {
    const auto& hs = ham->subs[i];
    int a = o1->find2(hs.up, hs.down), b = o2->find2(hs.up, hs.down);
    if (a < 0 || b < 0 || hs.row == 0) continue;
    const double f = 1.0 / std::sqrt(1.0 + hs.down);
    hh_seg s{};
    s.poff = addr_of(o1, a);
    s.pbase = HH_BASE_ABS;
    s.ldp = o1->subs[a].row;
    s.opP = HH_OP_N;
    s.qoff = addr_of(o2, b);
    s.qbase = HH_BASE_ABS;
    s.ldq = o2->subs[b].row;
    s.opQ = HH_OP_N;
    s.K = o1->subs[a].sdim;
    s.kind = HH_SEG_GEMM;
    s.cre = coef[0] * f;
    s.cim = coef[1] * f;
    int seg0 = (int)L.segs.size();
    L.segs.push_back(s);
    for (int m0 = 0; m0 < hs.row; m0 += 64)
      for (int n0 = 0; n0 < hs.sdim; n0 += 64) {
        hh_tile t{};
        t.ooff = hs.off;
        t.obase = HH_BASE_OUT;
        t.ldo = hs.row;
        t.M = hs.row;
        t.N = hs.sdim;
        t.m0 = m0;
        t.n0 = n0;
        t.seg0 = seg0;
        t.nseg = 1;
        t.accumulate = 1;
        L.tiles.push_back(t);
      }
  }
  L.upload(ctx);
  cudaError_t e = launch_segment_gemm_fp64(L, nullptr, nullptr, ham->d, ctx->stream);
  L.release();
  return cuda_check(ctx, e, "ham_add_product");
}

// block_mul_block_ndia with flags 'N', 'N' (code/space_info.f90:373-631):
// *out = coef (o1 o2)^K in the basis B, K = down_dif / 2.  Sub-blocks follow
// the basis: for each sector (N, 2S) and each 2S' within down_dif of 2S whose
// sector (N + up_dif, 2S') exists.  The reduced product is the regular matrix
// element at the stretched projections (M' = S', M = S) by the
// Wigner-Eckart theorem, summed over the intermediate projection with the
// Clebsch-Gordan coefficient of the coupling, divided by the product's own
// 3j at those projections; one FP64 segment GEMM per intermediate spin.
extern "C" int hh_block_product(hh_ctx_t* ctx, const hh_block_t* o1, const hh_block_t* o2, int down_dif,
                                const hh_basis_t* B, const double* coef, hh_block_t** out) {
  if (!ctx || !o1 || !o2 || !B || !coef || !out || down_dif < 0) return HH_ERR_INVALID;
  *out = nullptr;
  const int up_dif = o1->up_dif + o2->up_dif, k1 = o1->down_dif, k2 = o2->down_dif, K = down_dif;
  std::vector<int> qn;
  for (const auto& sec : B->secs)
    for (int nnd = std::abs(sec.down - K); nnd <= sec.down + K; nnd += SU) {
      int l = B->find(sec.up + up_dif, nnd);
      if (l >= 0) qn.insert(qn.end(), {sec.up, sec.down, nnd - sec.down, B->secs[l].dim, sec.dim});
    }
  hh_block* nb = nullptr;
  int st = new_block(ctx, B->len, up_dif, K, qn, &nb);
  if (st) return st;
  hh_gemm_list L;
  for (size_t i = 0; i < nb->subs.size(); ++i) {
    const auto& s = nb->subs[i];
    const int nd = s.down, nnd = s.down + s.dd, q = s.dd;
    const double norm = w3j(nnd, K, nd, -nnd, q, nd);
    const int seg0 = (int)L.segs.size();
    for (int md = std::abs(nd - k2); md <= nd + k2; md += SU) {
      const int ib = o2->find3(s.up, nd, md - nd), ia = o1->find3(s.up + o2->up_dif, md, nnd - md);
      if (ia < 0 || ib < 0) continue;
      if (o1->subs[ia].row != s.row || o2->subs[ib].sdim != s.sdim || o1->subs[ia].sdim != o2->subs[ib].row) {
        hh_block_free(nb);
        return fail(ctx, HH_ERR_INVALID, "block product: factor dimensions do not match the basis");
      }
      double c = 0.0;
      for (int mm = -md; mm <= md; mm += SU) {
        const int q1 = nnd - mm, q2 = mm - nd;
        double ea = w3j(nnd, k1, md, -nnd, q1, mm);
        double eb = w3j(md, k2, nd, -mm, q2, nd);
        if (((md - mm) / 2) & 1) eb = -eb;
        double cgk = w3j(k1, k2, K, q1, q2, -q) * std::sqrt(K + 1.0);
        if (((-k1 + k2 + q) / 2) & 1) cgk = -cgk;
        c += ea * eb * cgk;
      }
      if (c == 0.0 || o1->subs[ia].sdim == 0) continue;
      c /= norm;
      hh_seg g{};
      g.poff = addr_of(o1, ia);
      g.pbase = HH_BASE_ABS;
      g.ldp = o1->subs[ia].row;
      g.opP = HH_OP_N;
      g.qoff = addr_of(o2, ib);
      g.qbase = HH_BASE_ABS;
      g.ldq = o2->subs[ib].row;
      g.opQ = HH_OP_N;
      g.K = o1->subs[ia].sdim;
      g.kind = HH_SEG_GEMM;
      g.cre = coef[0] * c;
      g.cim = coef[1] * c;
      L.segs.push_back(g);
    }
    const int nseg = (int)L.segs.size() - seg0;
    if (nseg == 0 || s.row == 0 || s.sdim == 0) continue;
    for (int m0 = 0; m0 < s.row; m0 += 64)
      for (int n0 = 0; n0 < s.sdim; n0 += 64) {
        hh_tile t{};
        t.ooff = s.off;
        t.obase = HH_BASE_OUT;
        t.ldo = s.row;
        t.M = s.row;
        t.N = s.sdim;
        t.m0 = m0;
        t.n0 = n0;
        t.seg0 = seg0;
        t.nseg = nseg;
        t.accumulate = 1;
        L.tiles.push_back(t);
      }
  }
  L.upload(ctx);
  cudaError_t e = launch_segment_gemm_fp64(L, nullptr, nullptr, nb->d, ctx->stream);
  L.release();
  if (e != cudaSuccess) {
    hh_block_free(nb);
    return cuda_check(ctx, e, "block product");
  }
  *out = nb;
  return HH_OK;
}

// block_transfer (code/space_info.f90:100-129): a device copy of a block.
extern "C" int hh_block_copy(hh_ctx_t* ctx, const hh_block_t* src, hh_block_t** out) {
  if (!ctx || !src || !out) return HH_ERR_INVALID;
  std::vector<int> qn;
  for (const auto& s : src->subs) qn.insert(qn.end(), {s.up, s.down, s.dd, s.row, s.sdim});
  hh_block* nb = nullptr;
  int st = new_block(ctx, src->len, src->up_dif, src->down_dif, qn, &nb);
  if (st) return st;
  nb->scalar = src->scalar;
  if (src->nelem > 0) {
    cudaError_t e = cudaMemcpyAsync(nb->d, src->d, src->nelem * sizeof(double2), cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) {
      hh_block_free(nb);
      return cuda_check(ctx, e, "block copy");
    }
  }
  *out = nb;
  return HH_OK;
}
