// Task-list builder of the superblock matvec.
//
// Each model_wave term kernel of the reference (code/mat_vec.f90) is a loop
// nest over wave sectors and sub-blocks that, for every admissible quantum
// number combination, issues one or two ZGEMMs (or a scaled sub-block copy)
// with a coefficient built from 6j symbols, phases and fermion signs.  Here the
// same loop nests run once per superblock on the host and emit "contributions"
//     out_k[rect] += c * opA(A) * X_i[region] * opB(B)
// which are then scheduled as a two-stage grouped GEMM on the device:
//   stage 1: T = opA(A) X_i[region]              (deduplicated: the reference
//            recomputes it for every output spin, code/mat_vec.f90:1617-1749)
//   stage 2: out_k[rect] = sum_s c_s P_s Q_s      (one owner tile per output
//            sub-block: no atomics, deterministic summation order)
#include <cmath>
#include <map>
#include <tuple>
#include <algorithm>
#include <cstring>

#include "hh_internal.h"

namespace hh {

namespace {

constexpr int SU = 2;  // spin steps in doubled units (code/pubdata.f90:11)

inline double psign(int n) { return ((n / 2) & 1) ? -1.0 : 1.0; }
inline double fsign(int flag, int n) {
  if (flag == 'B') return 1.0;
  return (n % 2 == 0) ? 1.0 : -1.0;
}

// A block operand, possibly viewed through block_transfer_trans
// (code/space_info.f90:32-63): keyed by the original bra, down_dif negated,
// matrix = original^H.
struct OpView {
  const hh_block* b = nullptr;
  bool trans = false;
  std::unordered_map<uint64_t, int> t2, t3;
  void init(const hh_block* blk, bool tr) {
    b = blk;
    trans = tr;
    if (trans) {
      for (int j = int(b->subs.size()) - 1; j >= 0; --j) {
        const auto& s = b->subs[j];
        int up = s.up + b->up_dif, down = s.down + s.dd;
        t2[key2(up, down)] = j;
        t3[key3(up, down, -s.dd)] = j;
      }
    }
  }
  int up_dif() const { return trans ? -b->up_dif : b->up_dif; }
  int rank() const { return b->down_dif; }
  int find2(int up, int down) const {
    if (!trans) return b->find2(up, down);
    auto it = t2.find(key2(up, down));
    return it == t2.end() ? -1 : it->second;
  }
  int find3(int up, int down, int dd) const {
    if (!trans) return b->find3(up, down, dd);
    auto it = t3.find(key3(up, down, dd));
    return it == t3.end() ? -1 : it->second;
  }
  int rows(int j) const { return trans ? b->subs[j].sdim : b->subs[j].row; }
  int cols(int j) const { return trans ? b->subs[j].row : b->subs[j].sdim; }
  cplx scalar(int j) const {
    cplx v = b->scalar.empty() ? cplx(0, 0) : b->scalar[j];
    return trans ? std::conj(v) : v;
  }
};

using Mat = hh_mat_ref;

inline Mat op_mat(const OpView& v, int j, bool herm) {
  Mat m;
  const auto& s = v.b->subs[j];
  m.off = (long long)(uintptr_t)(v.b->d + s.off);
  m.base = HH_BASE_ABS;  // operators are absolute addresses
  m.ld = s.row > 0 ? s.row : 1;
  bool c = v.trans ^ herm;
  m.op = c ? HH_OP_C : HH_OP_N;
  return m;
}

using Contrib = hh_contrib;

struct Emitter {
  const hh_basis* sb;
  const hh_basis* eb;
  const hh_wave* w;
  std::vector<Contrib> out;
  double ref_flops = 0.0;
  double ref_first = 0.0;  // first GEMM of the two-GEMM terms
  std::string err;

  const hh_bsec* ssec(int i) const {
    int x = sb->find(w->secs[i].su, w->secs[i].sd);
    return x < 0 ? nullptr : &sb->secs[x];
  }
  const hh_bsec* esec(int i) const {
    int x = eb->find(w->secs[i].eu, w->secs[i].ed);
    return x < 0 ? nullptr : &eb->secs[x];
  }
  const hh_bsec* ssec_qn(int up, int down) const {
    int x = sb->find(up, down);
    return x < 0 ? nullptr : &sb->secs[x];
  }
  const hh_bsec* esec_qn(int up, int down) const {
    int x = eb->find(up, down);
    return x < 0 ? nullptr : &eb->secs[x];
  }
  static const hh_bsub* find_full(const hh_bsec* s, int bu, int bd, int su, int sd) {
    if (!s) return nullptr;
    auto it = s->full.find(key4(bu, bd, su, sd));
    return it == s->full.end() ? nullptr : &s->subs[it->second];
  }

  bool check(const OpView& v, int j, int r, int c) {
    if (v.rows(j) != r || v.cols(j) != c) {
      err = "operator sub-block " + std::to_string(j) + " is " + std::to_string(v.rows(j)) +
            "x" + std::to_string(v.cols(j)) + ", basis expects " + std::to_string(r) + "x" +
            std::to_string(c);
      return false;
    }
    return true;
  }

  void add(int k, int orow, int ocol, int M, int N, int i, int irow, int icol, int Ka, int Kb,
           const Mat* A, const Mat* B, cplx c) {
    Contrib t;
    t.k_out = k; t.orow = orow; t.ocol = ocol; t.M = M; t.N = N;
    t.i_in = i; t.irow = irow; t.icol = icol; t.Ka = Ka; t.Kb = Kb;
    t.hasA = A != nullptr; t.hasB = B != nullptr;
    if (A) t.A = *A;
    if (B) t.B = *B;
    t.cre = c.real();
    t.cim = c.imag();
    out.push_back(t);
  }
  // rows [orow, orow+M) of sector k (all env columns) += c opA(A) X_i rows [irow, +Ka)
  void add_rows(int k, int orow, int M, int i, int irow, int Ka, const Mat& A, cplx c) {
    const hh_bsec* es = esec(k);
    for (const auto& n : es->subs)
      add(k, orow, n.spos, M, n.sdim, i, irow, n.spos, Ka, n.sdim, &A, nullptr, c);
  }
  // cols [ocol, +N) of sector k += c X_i cols [icol, +Kb) opB(B)
  void add_cols(int k, int ocol, int N, int i, int icol, int Kb, const Mat& B, cplx c) {
    const hh_bsec* ss = ssec(k);
    for (const auto& m : ss->subs)
      add(k, m.spos, ocol, m.sdim, N, i, m.spos, icol, m.sdim, Kb, nullptr, &B, c);
  }
};

// ----------------------------------------------------------------- dia terms
bool t_block_vec_dia(Emitter& E, const OpView& A, cplx coef) {  // code/mat_vec.f90:165-215
  for (int i = 0; i < (int)E.w->secs.size(); ++i) {
    const hh_bsec* sec = E.ssec(i);
    if (!sec) continue;
    for (const auto& y : sec->subs) {
      cplx c1 = coef / std::sqrt(1.0 + y.bd);
      int k = A.find2(y.bu, y.bd);
      if (k < 0) continue;
      if (!E.check(A, k, y.sdim, y.sdim)) return false;
      Mat a = op_mat(A, k, false);
      E.add_rows(i, y.spos, y.sdim, i, y.spos, y.sdim, a, c1);
      E.ref_flops += 8.0 * y.sdim * (double)E.w->secs[i].edim * y.sdim;
    }
  }
  return true;
}

bool t_vec_block_dia(Emitter& E, const OpView& B, cplx coef) {  // code/mat_vec.f90:218-267
  for (int i = 0; i < (int)E.w->secs.size(); ++i) {
    const hh_bsec* sec = E.esec(i);
    if (!sec) continue;
    for (const auto& y : sec->subs) {
      cplx c1 = coef / std::sqrt(1.0 + y.bd);
      int k = B.find2(y.bu, y.bd);
      if (k < 0) continue;
      if (!E.check(B, k, y.sdim, y.sdim)) return false;
      Mat b = op_mat(B, k, true);  // psi * B^H
      E.add_cols(i, y.spos, y.sdim, i, y.spos, y.sdim, b, c1);
      E.ref_flops += 8.0 * E.w->secs[i].sdim * (double)y.sdim * y.sdim;
    }
  }
  return true;
}

bool t_site_vec_site_dia(Emitter& E, const OpView& S, const OpView& T, cplx coef) {
  // code/mat_vec.f90:540-636
  for (int i = 0; i < (int)E.w->secs.size(); ++i) {
    const hh_bsec* ss = E.ssec(i);
    const hh_bsec* es = E.esec(i);
    if (!ss || !es) continue;
    for (const auto& x : ss->subs) {
      int a = S.find2(x.su, x.sd);
      for (const auto& y : es->subs) {
        int b = T.find2(y.su, y.sd);
        if (a < 0 || b < 0) continue;
        cplx c = coef * S.scalar(a) * T.scalar(b) / std::sqrt((1.0 + x.sd) * (1.0 + y.sd));
        E.add(i, x.spos, y.spos, x.sdim, y.sdim, i, x.spos, y.spos, x.sdim, y.sdim, nullptr,
              nullptr, c);
        E.ref_flops += 8.0 * x.sdim * (double)y.sdim;
      }
    }
  }
  return true;
}

bool t_block_site_vec_dia(Emitter& E, const OpView& A, const OpView& S, cplx coef) {
  // code/mat_vec.f90:388-460
  for (int i = 0; i < (int)E.w->secs.size(); ++i) {
    const hh_bsec* sec = E.ssec(i);
    if (!sec) continue;
    for (const auto& y : sec->subs) {
      int b = A.find2(y.bu, y.bd), s = S.find2(y.su, y.sd);
      if (b < 0 || s < 0) continue;
      if (!E.check(A, b, y.sdim, y.sdim)) return false;
      cplx c = coef * S.scalar(s) / std::sqrt((1.0 + y.bd) * (1.0 + y.sd));
      E.add_rows(i, y.spos, y.sdim, i, y.spos, y.sdim, op_mat(A, b, false), c);
      E.ref_flops += 8.0 * y.sdim * (double)E.w->secs[i].edim * y.sdim;
    }
  }
  return true;
}

bool t_vec_block_site_dia(Emitter& E, const OpView& B, const OpView& S, cplx coef) {
  // code/mat_vec.f90:463-537
  for (int i = 0; i < (int)E.w->secs.size(); ++i) {
    const hh_bsec* sec = E.esec(i);
    if (!sec) continue;
    for (const auto& y : sec->subs) {
      int b = B.find2(y.bu, y.bd), s = S.find2(y.su, y.sd);
      if (b < 0 || s < 0) continue;
      if (!E.check(B, b, y.sdim, y.sdim)) return false;
      cplx c = coef * S.scalar(s) / std::sqrt((1.0 + y.bd) * (1.0 + y.sd));
      E.add_cols(i, y.spos, y.sdim, i, y.spos, y.sdim, op_mat(B, b, true), c);
      E.ref_flops += 8.0 * E.w->secs[i].sdim * (double)y.sdim * y.sdim;
    }
  }
  return true;
}

bool t_block_vec_site_dia(Emitter& E, const OpView& A, const OpView& S, cplx coef) {
  // code/mat_vec.f90:640-740
  for (int i = 0; i < (int)E.w->secs.size(); ++i) {
    const hh_bsec* ss = E.ssec(i);
    const hh_bsec* es = E.esec(i);
    if (!ss || !es) continue;
    for (const auto& x : ss->subs) {
      int a = A.find2(x.bu, x.bd);
      for (const auto& y : es->subs) {
        int b = S.find2(y.su, y.sd);
        if (a < 0 || b < 0) continue;
        if (!E.check(A, a, x.sdim, x.sdim)) return false;
        cplx c = coef * S.scalar(b) / std::sqrt((1.0 + y.sd) * (1.0 + x.bd));
        Mat am = op_mat(A, a, false);
        E.add(i, x.spos, y.spos, x.sdim, y.sdim, i, x.spos, y.spos, x.sdim, y.sdim, &am, nullptr, c);
        E.ref_flops += 8.0 * x.sdim * (double)y.sdim * x.sdim;
      }
    }
  }
  return true;
}

bool t_site_vec_block_dia(Emitter& E, const OpView& S, const OpView& B, cplx coef) {
  // code/mat_vec.f90:743-843
  for (int i = 0; i < (int)E.w->secs.size(); ++i) {
    const hh_bsec* ss = E.ssec(i);
    const hh_bsec* es = E.esec(i);
    if (!ss || !es) continue;
    for (const auto& x : ss->subs) {
      int a = S.find2(x.su, x.sd);
      for (const auto& y : es->subs) {
        int b = B.find2(y.bu, y.bd);
        if (a < 0 || b < 0) continue;
        if (!E.check(B, b, y.sdim, y.sdim)) return false;
        cplx c = coef * S.scalar(a) / std::sqrt((1.0 + y.bd) * (1.0 + x.sd));
        Mat bm = op_mat(B, b, true);
        E.add(i, x.spos, y.spos, x.sdim, y.sdim, i, x.spos, y.spos, x.sdim, y.sdim, nullptr, &bm, c);
        E.ref_flops += 8.0 * x.sdim * (double)y.sdim * y.sdim;
      }
    }
  }
  return true;
}

bool t_block_vec_block_dia(Emitter& E, const OpView& A, const OpView& B, cplx coef) {
  // code/mat_vec.f90:846-951
  for (int i = 0; i < (int)E.w->secs.size(); ++i) {
    const hh_bsec* ss = E.ssec(i);
    const hh_bsec* es = E.esec(i);
    if (!ss || !es) continue;
    for (const auto& x : ss->subs) {
      int a = A.find2(x.bu, x.bd);
      for (const auto& y : es->subs) {
        int b = B.find2(y.bu, y.bd);
        if (a < 0 || b < 0) continue;
        if (!E.check(A, a, x.sdim, x.sdim) || !E.check(B, b, y.sdim, y.sdim)) return false;
        cplx c = coef / std::sqrt((1.0 + y.bd) * (1.0 + x.bd));
        Mat am = op_mat(A, a, false), bm = op_mat(B, b, true);
        E.add(i, x.spos, y.spos, x.sdim, y.sdim, i, x.spos, y.spos, x.sdim, y.sdim, &am, &bm, c);
        E.ref_flops += 8.0 * x.sdim * (double)y.sdim * x.sdim + 8.0 * x.sdim * (double)y.sdim * y.sdim;
        E.ref_first += 8.0 * x.sdim * (double)y.sdim * x.sdim;
      }
    }
  }
  return true;
}

// ------------------------------------------------------------- ndia terms
bool t_block_site_vec_ndia(Emitter& E, const OpView& A, int flA, const OpView& S, int flS, cplx coef) {
  // code/mat_vec.f90:960-1216
  const int up_dif = A.up_dif(), k = A.rank();
  if (up_dif != S.up_dif() || k != S.rank()) { E.err = "block_site_vec_ndia: quantum number error"; return false; }
  for (int i = 0; i < (int)E.w->secs.size(); ++i) {
    const hh_bsec* sec = E.ssec(i);
    if (!sec) continue;
    const int edim = E.w->secs[i].edim;
    for (const auto& x : sec->subs) {
      for (int dd = -k; dd <= k; dd += SU) {
        for (int sdd = -k; sdd <= k; sdd += SU) {
          int bl = A.find3(x.bu, x.bd, dd);
          int nsu = x.su - up_dif, nsd = x.sd - sdd;
          int st = S.find3(nsu, nsd, sdd);
          int nbu = x.bu + up_dif, nbd = x.bd + dd;
          if (bl < 0 || st < 0) continue;
          const hh_bsub* y = Emitter::find_full(sec, nbu, nbd, nsu, nsd);
          if (!y) continue;
          double sg = fsign(flS, x.bu);
          double c1 = w6j(nbd, x.bd, k, x.sd, nsd, E.w->secs[i].sd);
          if (c1 == 0.0) continue;
          c1 = c1 * psign(x.bd + nsd + k + E.w->secs[i].sd) / std::sqrt(1.0 + k);
          cplx c = sg * c1 * coef * S.scalar(st);
          if (!E.check(A, bl, y->sdim, x.sdim)) return false;
          E.add_rows(i, y->spos, y->sdim, i, x.spos, x.sdim, op_mat(A, bl, false), c);
          E.ref_flops += 8.0 * y->sdim * (double)edim * x.sdim;
          if (up_dif != 0) {
            E.add_rows(i, x.spos, x.sdim, i, y->spos, y->sdim, op_mat(A, bl, true), std::conj(c));
            E.ref_flops += 8.0 * x.sdim * (double)edim * y->sdim;
          }
        }
      }
    }
  }
  return true;
}

bool t_vec_block_site_ndia(Emitter& E, const OpView& B, int flB, const OpView& S, int flS, cplx coef) {
  // code/mat_vec.f90:1219-1503
  const int up_dif = B.up_dif(), k = B.rank();
  if (up_dif != S.up_dif() || k != S.rank()) { E.err = "vec_block_site_ndia: quantum number error"; return false; }
  for (int i = 0; i < (int)E.w->secs.size(); ++i) {
    const hh_bsec* sec = E.esec(i);
    if (!sec) continue;
    const int sdim = E.w->secs[i].sdim;
    const int sys_up = E.w->secs[i].su;
    for (const auto& x : sec->subs) {
      for (int bdd = -k; bdd <= k; bdd += SU) {
        int bl = B.find3(x.bu, x.bd, bdd);
        for (int sdd = -k; sdd <= k; sdd += SU) {
          int nsu = x.su - up_dif, nsd = x.sd - sdd;
          int st = S.find3(nsu, nsd, sdd);
          int nbu = x.bu + up_dif, nbd = x.bd + bdd;
          if (st < 0 || bl < 0) continue;
          const hh_bsub* y = Emitter::find_full(sec, nbu, nbd, nsu, nsd);
          if (!y) continue;
          double sbl = fsign(flB, sys_up + nsu);
          double sst = fsign(flS, sys_up);
          double c1 = w6j(nbd, x.bd, k, x.sd, nsd, E.w->secs[i].ed);
          if (c1 == 0.0) continue;
          c1 = c1 * psign(x.bd + nsd + k + E.w->secs[i].ed) / std::sqrt(1.0 + k);
          cplx c = sbl * sst * c1 * coef * S.scalar(st);
          if (!E.check(B, bl, y->sdim, x.sdim)) return false;
          E.add_cols(i, y->spos, y->sdim, i, x.spos, x.sdim, op_mat(B, bl, true), c);
          E.ref_flops += 8.0 * sdim * (double)y->sdim * x.sdim;
          if (up_dif != 0) {
            E.add_cols(i, x.spos, x.sdim, i, y->spos, y->sdim, op_mat(B, bl, false), std::conj(c));
            E.ref_flops += 8.0 * sdim * (double)x.sdim * y->sdim;
          }
        }
      }
    }
  }
  return true;
}

bool t_block_vec_block_ndia(Emitter& E, const OpView& A, int flA, const OpView& B, int flB, cplx coef) {
  // code/mat_vec.f90:1505-1928
  const int up_dif = A.up_dif(), k = A.rank();
  if (up_dif != B.up_dif() || k != B.rank()) { E.err = "block_vec_block_ndia: quantum number error"; return false; }
  for (int i = 0; i < (int)E.w->secs.size(); ++i) {
    const hh_wsec& wi = E.w->secs[i];
    const hh_bsec* ss = E.ssec(i);
    const hh_bsec* es = E.esec(i);
    if (!ss || !es) continue;
    for (const auto& m : ss->subs) {
      for (const auto& n : es->subs) {
        for (int dd = -k; dd <= k; dd += SU) {
          int sb = A.find3(m.bu, m.bd, dd);
          int nsbu = m.bu + up_dif, nsbd = m.bd + dd;
          for (int edd = -k; edd <= k; edd += SU) {
            int nebu = n.bu - up_dif, nebd = n.bd - edd;
            int ebi = B.find3(nebu, nebd, edd);
            if (sb < 0 || ebi < 0) continue;
            for (int nsd = std::abs(wi.sd - k); nsd <= wi.sd + k; nsd += SU) {
              int nsu = wi.su + up_dif, neu = wi.eu - up_dif, ned = nsd;
              const hh_bsub* ms = Emitter::find_full(E.ssec_qn(nsu, nsd), nsbu, nsbd, m.su, m.sd);
              const hh_bsub* me = Emitter::find_full(E.esec_qn(neu, ned), nebu, nebd, n.su, n.sd);
              if (!ms || !me) continue;
              int kk = E.w->find(nsu, nsd, neu, ned);
              if (kk < 0) continue;
              double sel = fsign(flB, wi.su + n.su);
              double c1 = w6j(nsd, k, wi.sd, m.bd, m.sd, nsbd);
              if (c1 == 0.0) continue;
              double c11 = w6j(ned, k, wi.ed, n.bd, n.sd, nebd);
              if (c11 == 0.0) continue;
              c1 = c1 * c11 * std::sqrt((1.0 + ned) * (1.0 + wi.ed) / (1.0 + k));
              if ((((nsbd + m.sd + wi.sd + k) / 2 + (nebd + n.sd + wi.ed + k) / 2) & 1) == 1) c1 = -c1;
              cplx c = sel * coef * c1;
              if (!E.check(A, sb, ms->sdim, m.sdim) || !E.check(B, ebi, n.sdim, me->sdim)) return false;
              Mat am = op_mat(A, sb, false), bm = op_mat(B, ebi, false);
              E.add(kk, ms->spos, me->spos, ms->sdim, me->sdim, i, m.spos, n.spos, m.sdim, n.sdim,
                    &am, &bm, c);
              E.ref_flops += 8.0 * ms->sdim * (double)n.sdim * m.sdim + 8.0 * ms->sdim * (double)me->sdim * n.sdim;
              E.ref_first += 8.0 * ms->sdim * (double)n.sdim * m.sdim;
              if (up_dif != 0) {
                Mat ah = op_mat(A, sb, true), bh = op_mat(B, ebi, true);
                E.add(i, m.spos, n.spos, m.sdim, n.sdim, kk, ms->spos, me->spos, ms->sdim, me->sdim,
                      &ah, &bh, std::conj(c));
                E.ref_flops += 8.0 * m.sdim * (double)me->sdim * ms->sdim + 8.0 * m.sdim * (double)n.sdim * me->sdim;
                E.ref_first += 8.0 * m.sdim * (double)me->sdim * ms->sdim;
              }
            }
          }
        }
      }
    }
  }
  return true;
}

bool t_block_vec_site_ndia(Emitter& E, const OpView& A, int flA, const OpView& S, int flS, cplx coef) {
  // code/mat_vec.f90:2324-2690
  const int up_dif = A.up_dif(), k = A.rank();
  if (up_dif != S.up_dif() || k != S.rank()) { E.err = "block_vec_site_ndia: quantum number error"; return false; }
  for (int i = 0; i < (int)E.w->secs.size(); ++i) {
    const hh_wsec& wi = E.w->secs[i];
    const hh_bsec* ss = E.ssec(i);
    const hh_bsec* es = E.esec(i);
    if (!ss || !es) continue;
    for (const auto& m : ss->subs) {
      for (const auto& n : es->subs) {
        for (int bdd = -k; bdd <= k; bdd += SU) {
          int nsbu = m.bu + up_dif, nsbd = m.bd + bdd;
          int sb = A.find3(m.bu, m.bd, bdd);
          for (int sdd = -k; sdd <= k; sdd += SU) {
            int nesu = n.su - up_dif, nesd = n.sd - sdd;
            int st = S.find3(nesu, nesd, sdd);
            int nsu = wi.su + up_dif, neu = wi.eu - up_dif;
            if (sb < 0 || st < 0) continue;
            for (int nsd = std::abs(wi.sd - k); nsd <= wi.sd + k; nsd += SU) {
              int ned = nsd;
              const hh_bsec* t1 = E.ssec_qn(nsu, nsd);
              const hh_bsub* ms = nullptr;
              if (t1)
                for (const auto& l : t1->subs)
                  if (l.bu == nsbu && l.bd == nsbd && l.sd == m.sd) { ms = &l; break; }
              const hh_bsec* t2 = E.esec_qn(neu, ned);
              const hh_bsub* me = nullptr;
              if (t2)
                for (const auto& l : t2->subs)
                  if (l.su == nesu && l.sd == nesd && l.bd == n.bd) { me = &l; break; }
              if (!ms || !me) continue;
              int kk = E.w->find(nsu, nsd, neu, ned);
              if (kk < 0) continue;
              double se = fsign(flS, wi.su);
              double c1 = w6j(nsd, k, wi.sd, m.bd, m.sd, nsbd);
              if (c1 == 0.0) continue;
              double c11 = w6j(ned, k, wi.ed, n.sd, n.bd, nesd);
              if (c11 == 0.0) continue;
              c1 = c1 * c11 * std::sqrt((1.0 + ned) * (1.0 + wi.ed) / (1.0 + k));
              if ((((nsbd + m.sd + wi.sd + k) / 2 + (n.bd + n.sd + ned + k) / 2) & 1) != 0) c1 = -c1;
              cplx c = se * c1 * coef * S.scalar(st);
              int edim = n.sdim;
              if (!E.check(A, sb, ms->sdim, m.sdim)) return false;
              Mat am = op_mat(A, sb, false);
              E.add(kk, ms->spos, me->spos, ms->sdim, edim, i, m.spos, n.spos, m.sdim, edim, &am, nullptr, c);
              E.ref_flops += 8.0 * ms->sdim * (double)edim * m.sdim;
              if (up_dif != 0) {
                Mat ah = op_mat(A, sb, true);
                E.add(i, m.spos, n.spos, m.sdim, edim, kk, ms->spos, me->spos, ms->sdim, edim, &ah, nullptr,
                      std::conj(c));
                E.ref_flops += 8.0 * m.sdim * (double)edim * ms->sdim;
              }
            }
          }
        }
      }
    }
  }
  return true;
}

bool t_site_vec_block_ndia(Emitter& E, const OpView& S, int flS, const OpView& B, int flB, cplx coef) {
  // code/mat_vec.f90:2695-3098
  const int up_dif = S.up_dif(), k = S.rank();
  if (up_dif != B.up_dif() || k != B.rank()) { E.err = "site_vec_block_ndia: quantum number error"; return false; }
  for (int i = 0; i < (int)E.w->secs.size(); ++i) {
    const hh_wsec& wi = E.w->secs[i];
    const hh_bsec* ss = E.ssec(i);
    const hh_bsec* es = E.esec(i);
    if (!ss || !es) continue;
    for (const auto& m : ss->subs) {
      for (const auto& n : es->subs) {
        for (int sdd = -k; sdd <= k; sdd += SU) {
          int nssu = m.su + up_dif, nssd = m.sd + sdd;
          int st = S.find3(m.su, m.sd, sdd);
          for (int bdd = -k; bdd <= k; bdd += SU) {
            int nebu = n.bu - up_dif, nebd = n.bd - bdd;
            int eb = B.find3(nebu, nebd, bdd);
            int nsu = wi.su + up_dif, neu = wi.eu - up_dif;
            if (st < 0 || eb < 0) continue;
            for (int nsd = std::abs(wi.sd - k); nsd <= wi.sd + k; nsd += SU) {
              int ned = nsd;
              const hh_bsub* ms = Emitter::find_full(E.ssec_qn(nsu, nsd), m.bu, m.bd, nssu, nssd);
              const hh_bsub* me = Emitter::find_full(E.esec_qn(neu, ned), nebu, nebd, n.su, n.sd);
              if (!ms || !me) continue;
              int kk = E.w->find(nsu, nsd, neu, ned);
              if (kk < 0) continue;
              double c1 = w6j(nsd, k, wi.sd, m.sd, m.bd, nssd);
              if (c1 == 0.0) continue;
              double c11 = w6j(ned, k, wi.ed, n.bd, n.sd, nebd);
              if (c11 == 0.0) continue;
              c1 = c1 * c11 * std::sqrt((1.0 + ned) * (wi.ed + 1.0) / (1.0 + k));
              if ((((nebd + n.sd + wi.ed + k) / 2 + (m.bd + m.sd + nsd + k) / 2) & 1) != 0) c1 = -c1;
              double sst = fsign(flS, m.bu);
              double sel = fsign(flB, wi.su + n.su);
              cplx c = sst * sel * c1 * coef * S.scalar(st);
              int sdim = m.sdim;
              if (!E.check(B, eb, n.sdim, me->sdim)) return false;
              Mat bm = op_mat(B, eb, false);
              E.add(kk, ms->spos, me->spos, sdim, me->sdim, i, m.spos, n.spos, sdim, n.sdim, nullptr, &bm, c);
              E.ref_flops += 8.0 * sdim * (double)me->sdim * n.sdim;
              if (up_dif != 0) {
                Mat bh = op_mat(B, eb, true);
                E.add(i, m.spos, n.spos, sdim, n.sdim, kk, ms->spos, me->spos, sdim, me->sdim, nullptr, &bh,
                      std::conj(c));
                E.ref_flops += 8.0 * sdim * (double)n.sdim * me->sdim;
              }
            }
          }
        }
      }
    }
  }
  return true;
}

bool t_site_vec_site_ndia(Emitter& E, const OpView& S, int flS, const OpView& T, int flT, cplx coef) {
  // code/mat_vec.f90:3101-3470
  const int up_dif = S.up_dif(), k = S.rank();
  if (up_dif != T.up_dif() || k != T.rank()) { E.err = "site_vec_site_ndia: quantum number error"; return false; }
  for (int i = 0; i < (int)E.w->secs.size(); ++i) {
    const hh_wsec& wi = E.w->secs[i];
    const hh_bsec* ss = E.ssec(i);
    const hh_bsec* es = E.esec(i);
    if (!ss || !es) continue;
    for (const auto& m : ss->subs) {
      for (const auto& n : es->subs) {
        for (int d1 = -k; d1 <= k; d1 += SU) {
          int sid = S.find3(m.su, m.sd, d1);
          int nssu = m.su + up_dif, nssd = m.sd + d1;
          for (int d2 = -k; d2 <= k; d2 += SU) {
            int nesu = n.su - up_dif, nesd = n.sd - d2;
            int eid = T.find3(nesu, nesd, d2);
            int nsu = wi.su + up_dif, neu = wi.eu - up_dif;
            if (sid < 0 || eid < 0) continue;
            for (int nsd = std::abs(wi.sd - k); nsd <= wi.sd + k; nsd += SU) {
              int ned = nsd;
              const hh_bsec* t1 = E.ssec_qn(nsu, nsd);
              const hh_bsub* ms = nullptr;
              if (t1)
                for (const auto& l : t1->subs)
                  if (l.su == nssu && l.sd == nssd && l.bd == m.bd) { ms = &l; break; }
              const hh_bsec* t2 = E.esec_qn(neu, ned);
              const hh_bsub* me = nullptr;
              if (t2)
                for (const auto& l : t2->subs)
                  if (l.su == nesu && l.sd == nesd && l.bd == n.bd) { me = &l; break; }
              if (!ms || !me) continue;
              int kk = E.w->find(nsu, nsd, neu, ned);
              if (kk < 0) continue;
              double sst = fsign(flS, m.bu), set = fsign(flT, wi.su);
              double c1 = w6j(nsd, k, wi.sd, m.sd, m.bd, nssd);
              if (c1 == 0.0) continue;
              double c11 = w6j(ned, k, wi.ed, n.sd, n.bd, nesd);
              if (c11 == 0.0) continue;
              c1 = c1 * c11 * std::sqrt((1.0 + ned) * (1.0 + wi.ed) / (1.0 + k));
              if ((((n.bd + n.sd + ned + k) / 2 + (m.bd + m.sd + nsd + k) / 2) & 1) != 0) c1 = -c1;
              cplx c = sst * set * coef * c1 * S.scalar(sid) * T.scalar(eid);
              E.add(kk, ms->spos, me->spos, m.sdim, n.sdim, i, m.spos, n.spos, m.sdim, n.sdim, nullptr, nullptr, c);
              E.ref_flops += 8.0 * m.sdim * (double)n.sdim;
              if (up_dif != 0) {
                E.add(i, m.spos, n.spos, m.sdim, n.sdim, kk, ms->spos, me->spos, m.sdim, n.sdim, nullptr, nullptr,
                      std::conj(c));
                E.ref_flops += 8.0 * m.sdim * (double)n.sdim;
              }
            }
          }
        }
      }
    }
  }
  return true;
}

}  // namespace

// ---------------------------------------------------------------------------
int build_plan(hh_ctx* ctx, const hh_basis* sb, const hh_basis* eb, const hh_wave* layout, int nterm,
               const hh_term_t* terms, hh_plan* plan) {
  Emitter E;
  E.sb = sb;
  E.eb = eb;
  E.w = layout;
  // every wave sector must exist in both bases with matching dimensions
  for (const auto& s : layout->secs) {
    int a = sb->find(s.su, s.sd), b = eb->find(s.eu, s.ed);
    if (a < 0 || b < 0 || sb->secs[a].dim != s.sdim || eb->secs[b].dim != s.edim)
      return fail(ctx, HH_ERR_QN, "wave sector does not match the sys/env bases");
  }
  for (int t = 0; t < nterm; ++t) {
    const hh_term_t& T = terms[t];
    if (!T.op0) return fail(ctx, HH_ERR_INVALID, "term without operator");
    OpView v0, v1;
    v0.init(T.op0, T.trans0 != 0);
    if (T.op1) v1.init(T.op1, T.trans1 != 0);
    cplx c(T.coef_re, T.coef_im);
    bool ok = true;
    auto need1 = [&]() { return T.op1 != nullptr; };
    switch (T.kind) {
      case HH_BLOCK_VEC_DIA: ok = t_block_vec_dia(E, v0, c); break;
      case HH_VEC_BLOCK_DIA: ok = t_vec_block_dia(E, v0, c); break;
      case HH_SITE_VEC_SITE_DIA: ok = need1() && t_site_vec_site_dia(E, v0, v1, c); break;
      case HH_SITE_VEC_SITE_NDIA: ok = need1() && t_site_vec_site_ndia(E, v0, T.flag0, v1, T.flag1, c); break;
      case HH_BLOCK_SITE_VEC_NDIA: ok = need1() && t_block_site_vec_ndia(E, v0, T.flag0, v1, T.flag1, c); break;
      case HH_VEC_BLOCK_SITE_NDIA: ok = need1() && t_vec_block_site_ndia(E, v0, T.flag0, v1, T.flag1, c); break;
      case HH_BLOCK_VEC_SITE_NDIA: ok = need1() && t_block_vec_site_ndia(E, v0, T.flag0, v1, T.flag1, c); break;
      case HH_SITE_VEC_BLOCK_NDIA: ok = need1() && t_site_vec_block_ndia(E, v0, T.flag0, v1, T.flag1, c); break;
      case HH_BLOCK_VEC_BLOCK_NDIA: ok = need1() && t_block_vec_block_ndia(E, v0, T.flag0, v1, T.flag1, c); break;
      case HH_BLOCK_SITE_VEC_DIA: ok = need1() && t_block_site_vec_dia(E, v0, v1, c); break;
      case HH_VEC_BLOCK_SITE_DIA: ok = need1() && t_vec_block_site_dia(E, v0, v1, c); break;
      case HH_BLOCK_VEC_SITE_DIA: ok = need1() && t_block_vec_site_dia(E, v0, v1, c); break;
      case HH_SITE_VEC_BLOCK_DIA: ok = need1() && t_site_vec_block_dia(E, v0, v1, c); break;
      case HH_BLOCK_VEC_BLOCK_DIA: ok = need1() && t_block_vec_block_dia(E, v0, v1, c); break;
      default: return fail(ctx, HH_ERR_INVALID, "unknown term kind " + std::to_string(T.kind));
    }
    if (!ok) return fail(ctx, E.err.empty() ? HH_ERR_INVALID : HH_ERR_QN,
                         "term " + std::to_string(t) + ": " + (E.err.empty() ? "missing operand" : E.err));
    plan->ops.push_back(T.op0);
    if (T.op1) plan->ops.push_back(T.op1);
  }
  plan->ref_flops = E.ref_flops;
  plan->ref_flops_first = E.ref_first;

  // ------------------------------------------------------------ scheduling
  constexpr int TM = 64, TN = 64;
  std::map<std::tuple<long long, int, int, int, int, int, int, int>, long long> t_index;
  long long scr = 0;
  std::map<std::tuple<int, int, int>, std::vector<hh_seg>> rects;  // (k, orow, ocol) -> segs
  std::vector<std::tuple<int, int, int, int, int>> rect_order;     // k, orow, ocol, M, N
  double exec = 0.0, exec1 = 0.0;
  auto xoff = [&](int i, int r, int c) {
    const hh_wsec& s = layout->secs[i];
    return s.off + (long long)c * s.sdim + r;
  };
  // every region must lie inside its wave sector before anything reaches the device
  for (const Contrib& t : E.out) {
    const hh_wsec& wi = layout->secs[t.i_in];
    const hh_wsec& wk = layout->secs[t.k_out];
    if (t.irow < 0 || t.icol < 0 || t.irow + t.Ka > wi.sdim || t.icol + t.Kb > wi.edim || t.orow < 0 ||
        t.ocol < 0 || t.orow + t.M > wk.sdim || t.ocol + t.N > wk.edim)
      return fail(ctx, HH_ERR_QN, "plan region outside its wave sector");
  }
  for (const Contrib& t : E.out) {
    hh_seg s{};
    s.cre = t.cre;
    s.cim = t.cim;
    if (t.hasA && t.hasB) {
      auto key = std::make_tuple(t.A.off, t.A.op, t.A.ld, t.i_in, t.irow, t.icol, t.Ka, t.Kb);
      auto it = t_index.find(key);
      long long toff;
      if (it == t_index.end()) {
        toff = scr;
        t_index.emplace(key, toff);
        scr += (long long)t.M * t.Kb;
        // stage 1 tiles: T (M x Kb) = opA(A) X
        hh_seg s1{};
        s1.poff = t.A.off; s1.pbase = HH_BASE_ABS; s1.ldp = t.A.ld; s1.opP = t.A.op;
        s1.qoff = xoff(t.i_in, t.irow, t.icol); s1.qbase = HH_BASE_IN; s1.ldq = layout->secs[t.i_in].sdim;
        s1.opQ = HH_OP_N; s1.K = t.Ka; s1.kind = HH_SEG_GEMM; s1.cre = 1.0; s1.cim = 0.0;
        int sidx = (int)plan->stage1.segs.size();
        plan->stage1.segs.push_back(s1);
        for (int m0 = 0; m0 < t.M; m0 += TM)
          for (int n0 = 0; n0 < t.Kb; n0 += TN) {
            hh_tile tl{};
            tl.ooff = toff; tl.obase = HH_BASE_SCR; tl.ldo = t.M; tl.M = t.M; tl.N = t.Kb;
            tl.m0 = m0; tl.n0 = n0; tl.seg0 = sidx; tl.nseg = 1; tl.accumulate = 0;
            plan->stage1.tiles.push_back(tl);
          }
        exec += 8.0 * t.M * (double)t.Kb * t.Ka;
        exec1 += 8.0 * t.M * (double)t.Kb * t.Ka;
      } else {
        toff = it->second;
      }
      s.poff = toff; s.pbase = HH_BASE_SCR; s.ldp = t.M; s.opP = HH_OP_N;
      s.qoff = t.B.off; s.qbase = t.B.base; s.ldq = t.B.ld; s.opQ = t.B.op;
      s.K = t.Kb; s.kind = HH_SEG_GEMM;
      exec += 8.0 * t.M * (double)t.N * t.Kb;
    } else if (t.hasA) {
      s.poff = t.A.off; s.pbase = HH_BASE_ABS; s.ldp = t.A.ld; s.opP = t.A.op;
      s.qoff = xoff(t.i_in, t.irow, t.icol); s.qbase = HH_BASE_IN; s.ldq = layout->secs[t.i_in].sdim;
      s.opQ = HH_OP_N; s.K = t.Ka; s.kind = HH_SEG_GEMM;
      exec += 8.0 * t.M * (double)t.N * t.Ka;
    } else if (t.hasB) {
      s.poff = xoff(t.i_in, t.irow, t.icol); s.pbase = HH_BASE_IN; s.ldp = layout->secs[t.i_in].sdim;
      s.opP = HH_OP_N; s.qoff = t.B.off; s.qbase = HH_BASE_ABS; s.ldq = t.B.ld; s.opQ = t.B.op;
      s.K = t.Kb; s.kind = HH_SEG_GEMM;
      exec += 8.0 * t.M * (double)t.N * t.Kb;
    } else {
      s.poff = xoff(t.i_in, t.irow, t.icol); s.pbase = HH_BASE_IN; s.ldp = layout->secs[t.i_in].sdim;
      s.opP = HH_OP_N; s.kind = HH_SEG_COPY; s.K = 0; s.qbase = HH_BASE_ABS; s.qoff = 0; s.ldq = 1;
      exec += 8.0 * t.M * (double)t.N;
    }
    auto rk = std::make_tuple(t.k_out, t.orow, t.ocol);
    auto rit = rects.find(rk);
    if (rit == rects.end()) {
      rect_order.emplace_back(t.k_out, t.orow, t.ocol, t.M, t.N);
      rects[rk].push_back(s);
    } else {
      rit->second.push_back(s);
    }
  }
  for (const auto& r : rect_order) {
    int k, orow, ocol, M, N;
    std::tie(k, orow, ocol, M, N) = r;
    auto& segs = rects[std::make_tuple(k, orow, ocol)];
    int seg0 = (int)plan->stage2.segs.size();
    for (auto& s : segs) plan->stage2.segs.push_back(s);
    const hh_wsec& w = layout->secs[k];
    for (int m0 = 0; m0 < M; m0 += TM)
      for (int n0 = 0; n0 < N; n0 += TN) {
        hh_tile tl{};
        tl.ooff = w.off + (long long)ocol * w.sdim + orow;
        tl.obase = HH_BASE_OUT; tl.ldo = w.sdim; tl.M = M; tl.N = N; tl.m0 = m0; tl.n0 = n0;
        tl.seg0 = seg0; tl.nseg = (int)segs.size(); tl.accumulate = 0;
        plan->stage2.tiles.push_back(tl);
      }
  }
  plan->scratch_elems = scr;
  plan->exec_flops = exec;
  plan->exec_flops_s1 = exec1;
  plan->exec_flops_s2 = exec - exec1;
  double ob = 0.0;
  {
    std::vector<const hh_block*> u = plan->ops;
    std::sort(u.begin(), u.end());
    u.erase(std::unique(u.begin(), u.end()), u.end());
    for (auto* b : u) ob += 16.0 * (double)b->nelem;
  }
  plan->op_bytes = ob;
  plan->contribs = std::move(E.out);
  return HH_OK;
}

}  // namespace hh
