// Schedule of the split-precision tensor-core matvec, built from the plan's
// contribution list on the first split-precision matvec of a plan.
//
//   operator images  built once: one per (operator sub-block, role, op, coef);
//                    the coefficient of a segment is folded into the image of
//                    the operator it multiplies, so every tile accumulates all
//                    of its GEMM segments in TMEM without rescaling;
//   wave images      built every matvec from the FP64 input, one per
//                    (elementary region, role);
//   stage 1          T = opA(A) X for the deduplicated two-operator products,
//                    written as T images (mode 1);
//   stage 2          every output sub-block, 128 x N tiles, GEMM segments
//                    (T B, A X, X B) accumulated in TMEM, copy terms added in
//                    FP64 in the epilogue (mode 0).
#include <map>
#include <tuple>
#include <algorithm>
#include <cstring>

#include "hh_internal.h"
#include "tc.h"

namespace hh {

namespace {

// image rows are padded to 16 so that a B image spanning one tile has planes
// exactly ntile rows high (packed loads, tc_gemm.cu)
inline int rpad(int r) { return (r + 15) & ~15; }
inline int k16(int k) { return (k + 15) & ~15; }
inline long long img_bytes(int rows, int kc) {
  long long b = (long long)rpad(rows) * k16(kc) * 12;  // six bf16 planes
  return (b + 255) & ~255LL;
}

struct ImgRef {
  long long off = 0;  // offset into its arena
  int rows = 0, kc = 0;
};

struct Arena {
  long long size = 0;
  long long take(long long b) {
    long long o = size;
    size += b;
    return o;
  }
};

// Tiles are at most 64 wide (both stages): everything then runs on the
// 64-wide kernels (256 TMEM columns, two CTAs per SM), where one CTA's
// epilogue and pipeline fill overlap the other's MMAs.  A stacked tile costs
// the same MMA cycles cut in two halves (two MMAs of width 128 = one of 256);
// 128-wide tiles ran one CTA per SM with the epilogue exposed (m = 2000:
// stage 1 0.129 -> 0.116 ms, stage 2 + copy terms 0.223 -> 0.205 ms).
constexpr int kTileN = 64;

// MMA cycles of one 16-k chunk of a tile, in units of a plain 128-wide
// chunk: a K = 16 MMA costs about max(45, N/2) cycles whatever its M; plain
// tiles issue four of width ntile per part pair, stacked tiles one of width
// 2 ntile
double chunk_cost(const tc::Tile& x) {
  const double n = x.ntile;
  return x.stack ? std::max(45.0, n) / 256.0 : 4.0 * std::max(45.0, n / 2.0) / 256.0;
}

// MMA work of a tile plus a fixed share for its set-up and epilogue
double tile_cost(const tc::Tile& x) { return x.nchunk * chunk_cost(x) + 4.0; }

void destroy_graph(hh_tc_plan& t) {
  if (t.graph_exec) cudaGraphExecDestroy(t.graph_exec);
  if (t.graph) cudaGraphDestroy(t.graph);
  t.graph_exec = nullptr;
  t.graph = nullptr;
}

}  // namespace

namespace tc {

// A tile is stacked when it has at most 64 rows and every segment copies at
// most 64 rows of A; packed in A when every segment's A copy is its whole
// image (one plane stride for all), packed in B when every B copy is a
// whole image exactly ntile rows high.  The A plane offsets in shared
// memory follow: packed -> the image's plane stride, else 128-row slots
// (64-row halves when stacked).
void finish_tile(Tile& t, const Seg* segs) {
  t.nchunk = 0;
  bool stack = t.mrem <= 64 && t.nseg > 0, pa = t.nseg > 0, pb = t.nseg > 0;
  const long long a_plane = t.nseg > 0 ? segs[t.seg0].a_plane : 0;
  for (int si = 0; si < t.nseg; ++si) {
    const Seg& sg = segs[t.seg0 + si];
    t.nchunk += sg.nkc;
    stack = stack && sg.a_bytes <= 64 * 32;
    pa = pa && sg.a_bytes == sg.a_plane && sg.a_plane == a_plane;
    pb = pb && sg.b_bytes == sg.b_plane && sg.b_plane == (long long)t.ntile * 32;
  }
  t.stack = stack ? 1 : 0;
  t.pack = (pa ? 1 : 0) | (pb ? 2 : 0);
  constexpr int kSlot = 128 * 32;  // one 128-row plane slot
  if (pa) {
    t.a_pair = (int)(2 * a_plane);
    t.a_im = (int)a_plane;
  } else if (stack) {
    t.a_pair = kSlot;
    t.a_im = kSlot / 2;
  } else {
    t.a_pair = 2 * kSlot;
    t.a_im = kSlot;
  }
}

}  // namespace tc

static void release_tc(hh_ctx* ctx, hh_tc_plan& t) {
  destroy_graph(t);
  void* ptrs[] = {t.d_op_img, t.d_x_img, t.d_t_img, t.d_op_tasks, t.d_x_tasks, t.d_tiles1,
                  t.d_tiles2, t.d_tiles2b, t.d_segs, t.d_csegs, t.d_err, t.d_io, t.d_x_blocks,
                  t.d_c_blocks, t.d_pieces};
  for (void* q : ptrs) dev_free(ctx, q);
  t = hh_tc_plan();
}

void release_tc_plan(hh_plan* p) {
  release_tc(p->ctx, p->tc);
  release_tc(p->ctx, p->tcb);
  p->tcb_nb = 0;
}

// The schedule of nb vectors (a wave holding nb vectors one after another):
// nb == 1 is the plan's own (p->tc); nb > 1 replicates every wave image,
// T image and tile once per vector, the copies of a tile adjacent in every
// order, so that ONE launch per stage multiplies the whole batch and the
// copies of a tile, which read the same operator images, run side by side
// and share those loads through L2.
static int build_tc(hh_plan* p, hh_tc_plan& tp, int nb) {
  hh_ctx* ctx = p->ctx;
  const hh_wave* L = p->layout;
  // ---------------------------------------------------------------- images
  std::map<std::tuple<long long, int, int, int, double, double, int, int>, ImgRef> op_imgs;
  std::map<std::tuple<int, int, int, int, int, int>, ImgRef> x_imgs;
  std::vector<tc::ImgTask> op_tasks, x_tasks;
  Arena a_op, a_x, a_t;
  // role 0 = A operand (rows = M, k = K), role 1 = B operand (rows = N, k = K)
  auto op_img = [&](const hh_mat_ref& m, int role, int rows, int kc, double cre, double cim) {
    auto key = std::make_tuple(m.off, m.op, m.ld, role, cre, cim, rows, kc);
    auto it = op_imgs.find(key);
    if (it != op_imgs.end()) return it->second;
    ImgRef r;
    r.rows = rows;
    r.kc = kc;
    r.off = a_op.take(img_bytes(rows, kc));
    tc::ImgTask t{};
    t.src = m.off;
    t.sbase = HH_BASE_ABS;
    t.ld = m.ld;
    t.rows = rows;
    t.kc = kc;
    t.rpad = rpad(rows);
    t.k16 = k16(kc);
    t.row0 = 0;
    t.prow = t.rpad;
    // A, op N: O[r + k ld]; A, op C: conj O[k + r ld]; B, op N: O[k + n ld]; B, op C: conj O[n + k ld]
    t.trans = (role == 0) ? (m.op == HH_OP_C) : (m.op == HH_OP_N);
    t.conj = (m.op == HH_OP_C);
    t.cre = cre;
    t.cim = cim;
    t.dst = r.off;  // fixed up with the arena base below
    op_tasks.push_back(t);
    op_imgs.emplace(key, r);
    return r;
  };
  auto x_img = [&](int i, int irow, int icol, int nrow, int ncol, int role) {
    auto key = std::make_tuple(i, irow, icol, nrow, ncol, role);
    auto it = x_imgs.find(key);
    if (it != x_imgs.end()) return it->second;
    const hh_wsec& w = L->secs[i];
    ImgRef r;
    // role 1 (B): rows = region columns, k = region rows; role 0 (A): rows = region rows
    r.rows = role == 1 ? ncol : nrow;
    r.kc = role == 1 ? nrow : ncol;
    r.off = a_x.take(img_bytes(r.rows, r.kc));
    tc::ImgTask t{};
    t.src = w.off + (long long)icol * w.sdim + irow;
    t.sbase = HH_BASE_IN;
    t.ld = w.sdim;
    t.rows = r.rows;
    t.kc = r.kc;
    t.rpad = rpad(r.rows);
    t.k16 = k16(r.kc);
    t.row0 = 0;
    t.prow = t.rpad;
    t.trans = role == 1 ? 1 : 0;
    t.conj = 0;
    t.cre = 1.0;
    t.cim = 0.0;
    t.dst = r.off;
    x_tasks.push_back(t);
    x_imgs.emplace(key, r);
    return r;
  };

  // --------------------------------------------------------------- stage 1
  std::map<std::tuple<long long, int, int, int, int, int, int, int>, ImgRef> t_imgs;
  std::vector<tc::Seg> segs;
  std::vector<hh_seg> csegs;
  std::vector<tc::Tile> tiles1, tiles2;
  // addresses are arena offsets here; bases are added after allocation
  // (bits 60-61 of an address mark its arena: 0 operators, 1 wave, 2 T)
  auto tag = [](long long off, int arena) { return off | ((long long)arena << 60); };
  double mma1 = 0.0, mma2 = 0.0;
  // A rows [m0, m0 + mrows) (mrows <= 128, m0 a multiple of 8): a tile that
  // reaches the end of its A image copies the image's padding too (a tile
  // spanning the whole image then loads all planes of a chunk at once),
  // others whole 8-row groups
  auto make_seg = [&](long long a, const ImgRef& ai, int m0, long long b, const ImgRef& bi, int n0, int ntile,
                      int mrows = 128) {
    tc::Seg s{};
    const int ar = rpad(ai.rows), br = rpad(bi.rows);
    s.a = a + (long long)(m0 / 8) * 256;
    s.b = b + (long long)(n0 / 8) * 256;
    s.a_plane = (long long)(ar / 8) * 256;
    s.b_plane = (long long)(br / 8) * 256;
    const int arows = m0 + mrows >= ai.rows ? ar - m0 : std::min(((mrows + 7) & ~7), ar - m0);
    s.a_bytes = std::min(128, arows) * 32;
    s.b_bytes = std::min(ntile, br - n0) * 32;
    s.nkc = k16(ai.kc) / 16;
    return s;
  };

  // Unique two-operator products T = opA(A) X (deduplicated), grouped by their
  // X operand.  Products of at most 64 rows that share an X are row-packed:
  // first-fit, largest first, into bins of at most 64 rows; a bin's operators
  // are stacked in one merged operator image (built once per plan) and the
  // bin runs as ONE stacked tile per 64 columns whose pieces route each row
  // to its product's T image.  The epilogue of a stage-1 tile costs about the
  // same for 16 rows as for 64, and most products have few rows, so this cuts
  // the number of epilogues and MMA chunks of stage 1.  Larger products and
  // singletons keep their own tiles.
  std::vector<tc::TPiece> pieces;
  std::vector<ImgRef> contrib_t(p->contribs.size());
  struct Prod {
    ImgRef T;
    size_t ci;
  };
  std::vector<Prod> prods;
  std::map<std::tuple<int, int, int, int, int>, std::vector<int>> by_x;
  for (size_t ci = 0; ci < p->contribs.size(); ++ci) {
    const hh_contrib& c = p->contribs[ci];
    if (!(c.hasA && c.hasB)) continue;
    auto key = std::make_tuple(c.A.off, c.A.op, c.A.ld, c.i_in, c.irow, c.icol, c.Ka, c.Kb);
    auto it = t_imgs.find(key);
    if (it != t_imgs.end()) {
      contrib_t[ci] = it->second;
      continue;
    }
    ImgRef T;
    T.rows = c.M;
    T.kc = c.Kb;
    T.off = a_t.take(img_bytes(c.M, c.Kb));
    t_imgs.emplace(key, T);
    contrib_t[ci] = T;
    by_x[std::make_tuple(c.i_in, c.irow, c.icol, c.Ka, c.Kb)].push_back((int)prods.size());
    prods.push_back(Prod{T, ci});
  }
  auto single_tiles = [&](const Prod& pr) {
    const hh_contrib& c = p->contribs[pr.ci];
    ImgRef ai = op_img(c.A, 0, c.M, c.Ka, 1.0, 0.0);
    ImgRef xi = x_img(c.i_in, c.irow, c.icol, c.Ka, c.Kb, 1);
    for (int m0 = 0; m0 < c.M; m0 += 128)
      for (int n0 = 0; n0 < c.Kb; n0 += kTileN) {
        const int ntile = k16(std::min(kTileN, c.Kb - n0));
        tc::Tile tl{};
        tl.seg0 = (int)segs.size();
        tl.nseg = 1;
        segs.push_back(make_seg(tag(ai.off, 0), ai, m0, tag(xi.off, 1), xi, n0, ntile));
        tl.mode = 1;
        tl.ntile = ntile;
        tl.mrem = std::min(128, c.M - m0);
        tl.nrem = std::min(kTileN, c.Kb - n0);
        tl.out = tag(pr.T.off, 2);
        tl.t_rpad = rpad(c.M);
        tl.m0 = m0;
        tl.n0 = n0;
        tiles1.push_back(tl);
      }
  };
  for (const auto& kv : by_x) {
    std::vector<int> small;
    for (int i : kv.second) {
      if (p->contribs[prods[i].ci].M <= 64)
        small.push_back(i);
      else
        single_tiles(prods[i]);
    }
    std::stable_sort(small.begin(), small.end(), [&](int a, int b) {
      return rpad(p->contribs[prods[a].ci].M) > rpad(p->contribs[prods[b].ci].M);
    });
    std::vector<std::vector<int>> bins;
    std::vector<int> fill;
    for (int i : small) {
      const int r = rpad(p->contribs[prods[i].ci].M);
      size_t b = 0;
      while (b < bins.size() && fill[b] + r > 64) ++b;
      if (b == bins.size()) {
        bins.emplace_back();
        fill.push_back(0);
      }
      bins[b].push_back(i);
      fill[b] += r;
    }
    for (size_t b = 0; b < bins.size(); ++b) {
      if (bins[b].size() == 1) {
        single_tiles(prods[bins[b][0]]);
        continue;
      }
      const hh_contrib& c0 = p->contribs[prods[bins[b][0]].ci];
      const int R = fill[b], Ka = c0.Ka, Kb = c0.Kb;
      ImgRef merged;
      merged.rows = R;
      merged.kc = Ka;
      merged.off = a_op.take(img_bytes(R, Ka));
      const int piece0 = (int)pieces.size();
      int row0 = 0;
      for (int i : bins[b]) {
        const hh_contrib& c = p->contribs[prods[i].ci];
        tc::ImgTask tk{};
        tk.src = c.A.off;
        tk.sbase = HH_BASE_ABS;
        tk.ld = c.A.ld;
        tk.rows = c.M;
        tk.kc = Ka;
        tk.rpad = R;
        tk.k16 = k16(Ka);
        tk.trans = c.A.op == HH_OP_C;  // role A
        tk.conj = c.A.op == HH_OP_C;
        tk.row0 = row0;
        tk.prow = rpad(c.M);
        tk.cre = 1.0;
        tk.cim = 0.0;
        tk.dst = merged.off;
        op_tasks.push_back(tk);
        tc::TPiece pc{};
        pc.out = tag(prods[i].T.off, 2);
        pc.row0 = row0;
        pc.rows = c.M;
        pc.t_rpad = rpad(c.M);
        pieces.push_back(pc);
        row0 += rpad(c.M);
      }
      ImgRef xi = x_img(c0.i_in, c0.irow, c0.icol, Ka, Kb, 1);
      for (int n0 = 0; n0 < Kb; n0 += kTileN) {
        const int ntile = k16(std::min(kTileN, Kb - n0));
        tc::Tile tl{};
        tl.seg0 = (int)segs.size();
        tl.nseg = 1;
        segs.push_back(make_seg(tag(merged.off, 0), merged, 0, tag(xi.off, 1), xi, n0, ntile));
        tl.mode = 1;
        tl.ntile = ntile;
        tl.mrem = R;
        tl.nrem = std::min(kTileN, Kb - n0);
        tl.t_rpad = R;
        tl.m0 = 0;
        tl.n0 = n0;
        tl.piece0 = piece0;
        tl.npiece = (int)bins[b].size();
        tiles1.push_back(tl);
      }
    }
  }

  // --------------------------------------------------------------- stage 2
  std::map<std::tuple<int, int, int>, std::vector<size_t>> rects;
  std::vector<std::tuple<int, int, int>> order;
  for (size_t ci = 0; ci < p->contribs.size(); ++ci) {
    const hh_contrib& c = p->contribs[ci];
    auto k = std::make_tuple(c.k_out, c.orow, c.ocol);
    auto it = rects.find(k);
    if (it == rects.end()) {
      order.push_back(k);
      rects[k].push_back(ci);
    } else {
      it->second.push_back(ci);
    }
  }
  // Tile shape of an output rectangle (hh_plan::tc_shape): 0, tiles of 128
  // rows; 1, every rectangle in near-equal tiles of at most 64 rows (stacked:
  // one MMA of width 2 ntile per part pair, 45-64 cycles for 64 rows, against
  // four of width ntile, 4 x 45 cycles for 128 rows, at the price of one more
  // read of the B panel per 64 rows); 2, tiles of 128 rows whose remainders
  // of 65-127 rows go to two stacked tiles; 3, tiles of 128 rows and up to
  // 128 columns (the 128-wide kernel, one CTA per SM: half the A reads per
  // output, no second CTA to hide an epilogue).  Shapes 0-2 are at most 64
  // wide.  The plan autotuner picks.
  const int shape = p->tc_shape;
  const int tn2 = shape == 3 ? 128 : kTileN;
  auto row_split = [shape](int M) {
    std::vector<std::pair<int, int>> r;  // (m0, rows)
    auto stacked = [&r](int m0, int rows) {
      const int nt = (rows + 63) / 64;
      const int per = ((rows + nt - 1) / nt + 7) & ~7;
      for (int a = 0; a < rows; a += per) r.emplace_back(m0 + a, std::min(per, rows - a));
    };
    if (shape == 1) {
      stacked(0, M);
      return r;
    }
    for (int m0 = 0; m0 < M; m0 += 128) {
      const int rows = std::min(128, M - m0);
      if (shape == 2 && rows > 64 && rows < 128)
        stacked(m0, rows);
      else
        r.emplace_back(m0, rows);
    }
    return r;
  };
  for (const auto& rk : order) {
    const auto& list = rects[rk];
    const hh_contrib& c0 = p->contribs[list[0]];
    const int M = c0.M, N = c0.N;
    const hh_wsec& w = L->secs[c0.k_out];
    for (const auto& [m0, mrows] : row_split(M))
      for (int n0 = 0; n0 < N; n0 += tn2) {
        const int ntile = k16(std::min(tn2, N - n0));
        tc::Tile tl{};
        tl.seg0 = (int)segs.size();
        tl.cseg0 = (int)csegs.size();
        for (size_t ci : list) {
          const hh_contrib& c = p->contribs[ci];
          if (c.hasA && c.hasB) {
            const ImgRef& T = contrib_t[ci];
            ImgRef bi = op_img(c.B, 1, c.N, c.Kb, c.cre, c.cim);
            segs.push_back(make_seg(tag(T.off, 2), T, m0, tag(bi.off, 0), bi, n0, ntile, mrows));
          } else if (c.hasA) {
            ImgRef ai = op_img(c.A, 0, c.M, c.Ka, c.cre, c.cim);
            ImgRef xi = x_img(c.i_in, c.irow, c.icol, c.Ka, c.N, 1);
            segs.push_back(make_seg(tag(ai.off, 0), ai, m0, tag(xi.off, 1), xi, n0, ntile, mrows));
          } else if (c.hasB) {
            ImgRef xi = x_img(c.i_in, c.irow, c.icol, c.M, c.Kb, 0);
            ImgRef bi = op_img(c.B, 1, c.N, c.Kb, c.cre, c.cim);
            segs.push_back(make_seg(tag(xi.off, 1), xi, m0, tag(bi.off, 0), bi, n0, ntile, mrows));
          } else {
            hh_seg cs{};
            const hh_wsec& wi = L->secs[c.i_in];
            cs.poff = wi.off + (long long)c.icol * wi.sdim + c.irow;
            cs.pbase = HH_BASE_IN;
            cs.ldp = wi.sdim;
            cs.kind = HH_SEG_COPY;
            cs.cre = c.cre;
            cs.cim = c.cim;
            // terms copying the same input region (the site-diagonal terms of
            // one sector) add up into one coefficient
            bool merged = false;
            for (size_t q = tl.cseg0; q < csegs.size() && !merged; ++q)
              if (csegs[q].poff == cs.poff && csegs[q].ldp == cs.ldp) {
                csegs[q].cre += cs.cre;
                csegs[q].cim += cs.cim;
                merged = true;
              }
            if (!merged) csegs.push_back(cs);
          }
        }
        tl.nseg = (int)segs.size() - tl.seg0;
        tl.ncseg = (int)csegs.size() - tl.cseg0;
        tl.mode = 0;
        tl.ntile = ntile;
        tl.mrem = mrows;
        tl.nrem = std::min(tn2, N - n0);
        tl.out = w.off + (long long)(c0.ocol + n0) * w.sdim + c0.orow + m0;
        tl.ldo = w.sdim;
        tl.m0 = m0;
        tl.n0 = n0;
        tiles2.push_back(tl);
      }
  }

  // chunk counts and load / MMA forms of every tile; BF16 tensor FLOPs
  // issued per matvec (counted at six split products: four MMAs of width
  // ntile per part pair, or one of 2 ntile when stacked)
  mma1 = mma2 = 0.0;
  for (auto* tl : {&tiles1, &tiles2})
    for (auto& x : *tl) {
      tc::finish_tile(x, segs.data());
      const double f = (double)x.nchunk * 16 * 128 * 2.0 * (x.stack ? 2.0 : 4.0) * x.ntile * 6.0;
      (tl == &tiles1 ? mma1 : mma2) += f;
    }

  // ------------------------------------------------------- batch copies
  if (nb > 1) {
    const long long xs = a_x.size, ts = a_t.size;  // per vector (multiples of 256 bytes)
    constexpr long long kMask = (1LL << 60) - 1;
    auto shift = [&](long long v, int b) {
      const int arena = (int)((unsigned long long)v >> 60);
      const long long o = v & kMask;
      return arena == 1 ? tag(o + b * xs, 1) : arena == 2 ? tag(o + b * ts, 2) : v;
    };
    const int nsegs = (int)segs.size(), npieces = (int)pieces.size(), ncsegs = (int)csegs.size();
    std::vector<tc::Seg> segs_b;
    segs_b.reserve((size_t)nsegs * nb);
    for (int b = 0; b < nb; ++b)
      for (tc::Seg sg : segs) {
        sg.a = shift(sg.a, b);
        sg.b = shift(sg.b, b);
        segs_b.push_back(sg);
      }
    std::vector<tc::TPiece> pieces_b;
    for (int b = 0; b < nb; ++b)
      for (tc::TPiece pc : pieces) {
        pc.out = shift(pc.out, b);
        pieces_b.push_back(pc);
      }
    std::vector<hh_seg> csegs_b;
    for (int b = 0; b < nb; ++b)
      for (hh_seg cs : csegs) {
        cs.poff += (long long)b * p->nelem;
        csegs_b.push_back(cs);
      }
    auto copies = [&](std::vector<tc::Tile>& tl) {
      std::vector<tc::Tile> out;
      out.reserve(tl.size() * nb);
      for (const tc::Tile& x : tl)
        for (int b = 0; b < nb; ++b) {
          tc::Tile y = x;
          y.seg0 += b * nsegs;
          y.piece0 += b * npieces;
          y.cseg0 += b * ncsegs;
          if (y.mode == 0)
            y.out += (long long)b * p->nelem;
          else if (y.npiece == 0)
            y.out = shift(y.out, b);
          out.push_back(y);
        }
      tl.swap(out);
    };
    copies(tiles1);
    copies(tiles2);
    std::vector<tc::ImgTask> x_tasks_b;
    for (int b = 0; b < nb; ++b)
      for (tc::ImgTask tk : x_tasks) {
        tk.src += (long long)b * p->nelem;
        tk.dst += b * xs;
        x_tasks_b.push_back(tk);
      }
    segs.swap(segs_b);
    pieces.swap(pieces_b);
    csegs.swap(csegs_b);
    x_tasks.swap(x_tasks_b);
    a_x.size = xs * nb;
    a_t.size = ts * nb;
    mma1 *= nb;
    mma2 *= nb;
  }

  // ------------------------------------------------------- tile order
  // Stage 1 (thousands of short tiles, at most kTileN wide) runs on the
  // 64-wide kernels (256 TMEM columns, two CTAs per SM; wider tiles, if any,
  // follow on the 128-wide kernel), on the persistent kernel, where CTA c of
  // G resident CTAs takes tiles c, c + G, c + 2G, ...: within each part its
  // tiles go longest first (MMA chunks x N, plus a fixed epilogue share), in
  // a snake over the CTAs, so that every CTA receives a near-equal share.
  // Stage 2 (long, uneven tiles, at most kTileN wide) is kept in two orders:
  // longest first for one CTA per tile (the hardware then hands the next
  // tile to the first free SM: list scheduling; 0.28 against 0.34 ms in plan
  // order at m = 2000), and snake-balanced like stage 1 for the persistent
  // kernel; the launch autotuner picks.
  int sms = 148, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  auto split_narrow = [](std::vector<tc::Tile>& tl) {
    std::stable_partition(tl.begin(), tl.end(), [](const tc::Tile& x) { return x.ntile <= 64; });
    return (int)std::count_if(tl.begin(), tl.end(), [](const tc::Tile& x) { return x.ntile <= 64; });
  };
  auto balance = [](std::vector<tc::Tile>& tl, size_t lo, size_t hi, size_t G) {
    const size_t n = hi - lo;
    if (n <= G) return;
    std::vector<std::pair<double, size_t>> cost(n);
    for (size_t i = 0; i < n; ++i) cost[i] = {8.0 + tl[lo + i].nchunk * chunk_cost(tl[lo + i]), lo + i};
    std::stable_sort(cost.begin(), cost.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
    std::vector<tc::Tile> out(n);
    for (size_t k = 0; k < n; ++k) {
      const size_t round = k / G, c = k % G, base = round * G;
      const size_t cnt = std::min(G, n - base);  // the last round may be partial
      out[base + ((round & 1) ? cnt - 1 - c : c)] = tl[cost[k].second];
    }
    std::copy(out.begin(), out.end(), tl.begin() + lo);
  };
  const int n1n = split_narrow(tiles1);
  const int n2n = split_narrow(tiles2);
  auto longest_first = [](std::vector<tc::Tile>& tl, size_t lo, size_t hi) {
    std::stable_sort(tl.begin() + lo, tl.begin() + hi,
                     [](const tc::Tile& a, const tc::Tile& b) { return tile_cost(a) > tile_cost(b); });
  };
  longest_first(tiles2, 0, n2n);
  longest_first(tiles2, n2n, tiles2.size());
  std::vector<tc::Tile> tiles2b = tiles2;
  balance(tiles1, 0, n1n, 2 * (size_t)sms);
  balance(tiles1, n1n, tiles1.size(), (size_t)sms);
  balance(tiles2b, 0, n2n, 2 * (size_t)sms);
  balance(tiles2b, n2n, tiles2b.size(), (size_t)sms);

  // --------------------------------------------------------------- device
  hh_tc_plan& t = tp;
  auto alloc = [&](void** ptr, size_t bytes) -> int {
    if (bytes == 0) bytes = 256;
    cudaError_t e = dev_alloc(ctx, ptr, bytes);
    return e == cudaSuccess ? HH_OK : cuda_check(ctx, e, "allocate tensor-core plan");
  };
  int st;
  if ((st = alloc(&t.d_op_img, a_op.size)) || (st = alloc(&t.d_x_img, a_x.size)) ||
      (st = alloc(&t.d_t_img, a_t.size))) {
    release_tc(ctx, tp);
    return st;
  }
  const long long base[3] = {(long long)(uintptr_t)t.d_op_img, (long long)(uintptr_t)t.d_x_img,
                             (long long)(uintptr_t)t.d_t_img};
  auto untag = [&](long long v) {
    int arena = (int)((unsigned long long)v >> 60);
    return base[arena] + (v & ((1LL << 60) - 1));
  };
  for (auto& s : segs) {
    s.a = untag(s.a);
    s.b = untag(s.b);
  }
  for (auto& tl : tiles1)
    if (tl.npiece == 0) tl.out = untag(tl.out);
  for (auto& pc : pieces) pc.out = untag(pc.out);
  for (auto& tk : op_tasks) tk.dst += base[0];
  for (auto& tk : x_tasks) tk.dst += base[1];
  std::vector<int2> x_blocks, c_blocks;
  t.n_x_blocks = tc_image_blocks(x_tasks.data(), (int)x_tasks.size(), x_blocks);
  t.n_c_blocks = tc_copy_blocks(tiles2.data(), (int)tiles2.size(), c_blocks);
  // stage-2 tiles partition the output rectangles and store every element;
  // when they cover the whole output wave no zeroing pass is needed
  long long covered = 0;
  for (const auto& x : tiles2) covered += (long long)x.mrem * x.nrem;
  t.zero_out = covered != (long long)nb * p->nelem;
  auto upload = [&](void** dptr, const void* src, size_t bytes) -> int {
    if ((st = alloc(dptr, bytes))) return st;
    if (bytes) {
      cudaError_t e = cudaMemcpyAsync(*dptr, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
      if (e != cudaSuccess) return cuda_check(ctx, e, "upload tensor-core plan");
    }
    return HH_OK;
  };
  if ((st = upload((void**)&t.d_op_tasks, op_tasks.data(), op_tasks.size() * sizeof(tc::ImgTask))) ||
      (st = upload((void**)&t.d_x_tasks, x_tasks.data(), x_tasks.size() * sizeof(tc::ImgTask))) ||
      (st = upload((void**)&t.d_x_blocks, x_blocks.data(), x_blocks.size() * sizeof(int2))) ||
      (st = upload((void**)&t.d_pieces, pieces.data(), pieces.size() * sizeof(tc::TPiece))) ||
      (st = upload((void**)&t.d_c_blocks, c_blocks.data(), c_blocks.size() * sizeof(int2))) ||
      (st = upload((void**)&t.d_tiles1, tiles1.data(), tiles1.size() * sizeof(tc::Tile))) ||
      (st = upload((void**)&t.d_tiles2, tiles2.data(), tiles2.size() * sizeof(tc::Tile))) ||
      (st = upload((void**)&t.d_tiles2b, tiles2b.data(), tiles2b.size() * sizeof(tc::Tile))) ||
      (st = upload((void**)&t.d_segs, segs.data(), segs.size() * sizeof(tc::Seg))) ||
      (st = upload((void**)&t.d_csegs, csegs.data(), csegs.size() * sizeof(hh_seg))) ||
      (st = alloc((void**)&t.d_err, sizeof(int))) || (st = alloc((void**)&t.d_io, sizeof(tc::IoPtrs)))) {
    release_tc(ctx, tp);
    return st;
  }
  cudaMemsetAsync(t.d_err, 0, sizeof(int), ctx->stream);
  t.n_op_tasks = (int)op_tasks.size();
  t.n_x_tasks = (int)x_tasks.size();
  t.n_tiles1 = (int)tiles1.size();
  t.n_tiles2 = (int)tiles2.size();
  t.n_narrow1 = n1n;
  t.n_narrow2 = n2n;
  t.n_cseg = (int)csegs.size();
  t.bytes_op = (double)a_op.size;
  t.bytes_x = (double)a_x.size;
  t.bytes_t = (double)a_t.size;
  t.mma_flops1 = mma1;
  t.mma_flops2 = mma2;
  // stage-2 tile statistics: stacked tiles and the MMA cycles of the whole
  // stage under the per-instruction cost max(45, width / 2) cycles per K = 16
  // MMA (measured), SPLIT = 2 (three part pairs per chunk)
  t.n_stacked2 = 0;
  t.mma_cycles2 = 0.0;
  for (const auto& x : tiles2) {
    t.n_stacked2 += x.stack ? 1 : 0;
    t.mma_cycles2 += 3.0 * x.nchunk * 256.0 * chunk_cost(x);
  }
  // operator images are built once here (block list freed after the build)
  std::vector<int2> op_blocks;
  const int n_op_blocks = tc_image_blocks(op_tasks.data(), (int)op_tasks.size(), op_blocks);
  int2* d_op_blocks = nullptr;
  if ((st = upload((void**)&d_op_blocks, op_blocks.data(), op_blocks.size() * sizeof(int2)))) {
    release_tc(ctx, tp);
    return st;
  }
  cudaError_t e = tc_build_images(t.d_op_tasks, t.n_op_tasks, nullptr, false, ctx->stream, nullptr, 3, d_op_blocks,
                                  n_op_blocks);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  dev_free(ctx, d_op_blocks);
  if (e != cudaSuccess) {
    release_tc(ctx, tp);
    return cuda_check(ctx, e, "build operator images");
  }
  t.ready = true;
  return HH_OK;
}

int build_tc_plan(hh_plan* p) { return build_tc(p, p->tc, 1); }

// The launch sequence of one split-precision matvec: wave images, stage 1,
// zeroed output (only when the stage-2 tiles leave elements uncovered), stage
// 2, copy terms.  Explicit vectors (io == nullptr) or the vectors in t.d_io
// (graph capture).  (Copy terms folded into the stage-2 epilogue measured
// slower, 0.232 against 0.205 ms at m = 2000: their loads sat on every
// tile's critical path.)
static cudaError_t enqueue_tc(hh_plan* p, hh_tc_plan& t, long long nelem, const double2* in, double2* out,
                              const tc::IoPtrs* io, cudaEvent_t* ev, int split) {
  cudaStream_t s = p->ctx->stream;
  if (ev) cudaEventRecord(ev[0], s);
  cudaError_t e = tc_build_images(t.d_x_tasks, t.n_x_tasks, in, true, s, io, split, t.d_x_blocks, t.n_x_blocks);
  if (ev) cudaEventRecord(ev[1], s);
  if (e == cudaSuccess)
    e = tc_run_tiles(t.d_tiles1, t.n_narrow1, t.d_segs, out, t.d_err, t.persistent1, s, io, 64, split, t.d_pieces);
  if (e == cudaSuccess)
    e = tc_run_tiles(t.d_tiles1 + t.n_narrow1, t.n_tiles1 - t.n_narrow1, t.d_segs, out, t.d_err, t.persistent1, s,
                     io, 128, split, t.d_pieces);
  if (ev) cudaEventRecord(ev[2], s);
  if (e == cudaSuccess && t.zero_out) e = tc_zero_out(out, nelem, s, io);
  const tc::Tile* tiles2 = t.persistent2 ? t.d_tiles2b : t.d_tiles2;
  if (e == cudaSuccess)
    e = tc_run_tiles(tiles2, t.n_narrow2, t.d_segs, out, t.d_err, t.persistent2, s, io, 64, split);
  if (e == cudaSuccess)
    e = tc_run_tiles(tiles2 + t.n_narrow2, t.n_tiles2 - t.n_narrow2, t.d_segs, out, t.d_err, t.persistent2, s,
                     io, 128, split);
  if (ev) cudaEventRecord(ev[4], s);
  if (e == cudaSuccess && t.n_c_blocks > 0)
    e = tc_copy_terms(t.d_tiles2, t.d_c_blocks, t.n_c_blocks, t.d_csegs, in, out, s, io);
  if (ev) cudaEventRecord(ev[3], s);
  return e;
}

static int run_tc(hh_plan* p, hh_tc_plan& t, int nb, const double2* in, double2* out, float* ms, bool check,
                  int split) {
  hh_ctx* ctx = p->ctx;
  const long long nelem = (long long)nb * p->nelem;
  cudaError_t e = cudaSuccess;
  if (ms) {
    // eager launches with events between the stages
    cudaEvent_t ev[5];  // start, images done, stage 1 done, end, stage-2 tiles done
    for (int i = 0; i < 5; ++i) cudaEventCreate(&ev[i]);
    e = enqueue_tc(p, t, nelem, in, out, nullptr, ev, split);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[3]);
    if (e == cudaSuccess) {
      cudaEventElapsedTime(&ms[0], ev[0], ev[3]);
      cudaEventElapsedTime(&ms[1], ev[1], ev[2]);
      cudaEventElapsedTime(&ms[2], ev[2], ev[4]);
      cudaEventElapsedTime(&ms[3], ev[0], ev[1]);
    }
    for (int i = 0; i < 5; ++i) cudaEventDestroy(ev[i]);
  } else if (t.calls++ == 0 || split != t.graph_split) {
    // the first call at a split runs eagerly (and initialises the kernels'
    // attributes); the graph is captured again at the new split next time
    destroy_graph(t);
    t.graph_split = split;
    e = enqueue_tc(p, t, nelem, in, out, nullptr, nullptr, split);
  } else {
    if (!t.graph_exec) {
      e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        cudaError_t eq = enqueue_tc(p, t, nelem, nullptr, nullptr, t.d_io, nullptr, split);
        e = cudaStreamEndCapture(ctx->stream, &t.graph);
        if (e == cudaSuccess) e = eq;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&t.graph_exec, t.graph, 0);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_check(ctx, e, "capture the tensor-core matvec graph");
      }
    }
    e = tc_set_io(t.d_io, in, out, ctx->stream);
    if (e == cudaSuccess) e = cudaGraphLaunch(t.graph_exec, ctx->stream);
  }
  if (!check && !ms) return cuda_check(ctx, e, "tensor-core matvec");  // caller reads the flag later
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, t.d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_check(ctx, e, "tensor-core matvec");
  if (herr != 0) {
    cudaMemsetAsync(t.d_err, 0, sizeof(int), ctx->stream);
    return fail(ctx, HH_ERR_TIMEOUT, "tensor-core matvec: a bounded mbarrier wait ran out (code " +
                                         std::to_string(herr) + ")");
  }
  return HH_OK;
}

int matvec_tc(hh_plan* p, const double2* in, double2* out, float* ms, bool check, int split) {
  if (!p->tc.ready) {
    int st = build_tc_plan(p);
    if (st != HH_OK) return st;
  }
  return run_tc(p, p->tc, 1, in, out, ms, check, split);
}

int matvec_tc_batch(hh_plan* p, const double2* in, double2* out, int nb, bool check, int split) {
  if (nb == 1) return matvec_tc(p, in, out, nullptr, check, split);
  if (!p->tcb.ready || p->tcb_nb != nb) {
    release_tc(p->ctx, p->tcb);
    p->tcb_nb = 0;
    int st = build_tc(p, p->tcb, nb);
    if (st != HH_OK) return st;
    p->tcb_nb = nb;
    p->tcb.persistent1 = p->tc.persistent1;  // the launch choices tuned on the single-vector plan
    p->tcb.persistent2 = p->tc.persistent2;
  }
  return run_tc(p, p->tcb, nb, in, out, nullptr, check, split);
}

// Times the stage-2 tile shapes (0 - 3 of build_tc) and, for
// each, the launch variants of the tile GEMM (stage 1 / stage 2 on the
// persistent kernel or one CTA per tile) on this plan's own task lists, reps
// timed runs each after one warm-up, and keeps the fastest; ms[4 s + v]
// receives the mean time of shape s and variant v = 2 * persistent1 +
// persistent2.  A shape is tried by rebuilding the plan's schedule (host
// tiling and the operator images); the batched schedule, if any, is rebuilt
// with the kept shape at its next use.
int tune_tc_plan(hh_plan* p, int reps, double* ms, int split) {
  hh_ctx* ctx = p->ctx;
  const size_t bytes = (size_t)p->nelem * sizeof(double2);
  cudaError_t e = cudaSuccess;
  if (!p->d_host_in) e = dev_alloc(ctx, (void**)&p->d_host_in, bytes);
  if (e == cudaSuccess && !p->d_host_out) e = dev_alloc(ctx, (void**)&p->d_host_out, bytes);
  if (e == cudaSuccess) e = cudaMemsetAsync(p->d_host_in, 0, bytes, ctx->stream);
  if (e != cudaSuccess) return cuda_check(ctx, e, "tune buffers");
  double best = 1e300;
  int best_s = p->tc_shape, best_v = 2 * (int)p->tc.persistent1 + (int)p->tc.persistent2;
  auto rebuild = [&](int shape) {
    release_tc(ctx, p->tc);
    p->tc_shape = shape;
    return build_tc_plan(p);
  };
  for (int shape = 0; shape < HH_TILE_SHAPES; ++shape) {
    if (shape != p->tc_shape || !p->tc.ready) {
      int st = rebuild(shape);
      if (st != HH_OK) return st;
    }
    hh_tc_plan& t = p->tc;
    for (int v = 0; v < 4; ++v) {
      t.persistent1 = (v >> 1) & 1;
      t.persistent2 = v & 1;
      double sum = 0.0;
      for (int r = 0; r <= reps; ++r) {
        float m[4];
        int st = matvec_tc(p, p->d_host_in, p->d_host_out, m, true, split);
        if (st) return st;
        if (r > 0) sum += m[0];
      }
      const double mean = reps > 0 ? sum / reps : 0.0;
      if (ms) ms[4 * shape + v] = mean;
      if (mean < best) {
        best = mean;
        best_s = shape;
        best_v = v;
      }
    }
  }
  if (best_s != p->tc_shape) {
    int st = rebuild(best_s);
    if (st != HH_OK) return st;
  }
  p->tc.persistent1 = (best_v >> 1) & 1;
  p->tc.persistent2 = best_v & 1;
  // the next graph is captured with the chosen kernels
  destroy_graph(p->tc);
  release_tc(ctx, p->tcb);
  p->tcb_nb = 0;
  return HH_OK;
}

}  // namespace hh

// ---------------------------------------------------------------------------
// Self-test of the tensor-core tile path on one dense complex product
// C = A B (column-major, interleaved complex), used by the unit tests.
static int tc_selftest_impl(hh_ctx_t* ctx, int M, int N, int K, const double* A, const double* B, double* C,
                            int precision, bool hold);

extern "C" int hh_tc_selftest(hh_ctx_t* ctx, int M, int N, int K, const double* A, const double* B, double* C,
                              int precision) {
  return tc_selftest_impl(ctx, M, N, K, A, B, C, precision, false);
}

// Failure-detection check: a 16 x 16 x 16 product whose first chunk is
// announced to the copy barrier but never sent, so the kernel's bounded
// waits run out; the call must return HH_ERR_TIMEOUT with the context still
// usable.
extern "C" int hh_tc_selftest_hold(hh_ctx_t* ctx, int precision) {
  std::vector<double> a(2 * 16 * 16, 0.0), c(2 * 16 * 16, 0.0);
  return tc_selftest_impl(ctx, 16, 16, 16, a.data(), a.data(), c.data(), precision, true);
}

static int tc_selftest_impl(hh_ctx_t* ctx, int M, int N, int K, const double* A, const double* B, double* C,
                            int precision, bool hold) {
  using namespace hh;
  if (!ctx || M < 1 || N < 1 || K < 1 || !A || !B || !C || !split_of(precision)) return HH_ERR_INVALID;
  const long long ia = img_bytes(M, K), ib = img_bytes(N, K);
  void *dA = nullptr, *dB = nullptr, *dC = nullptr, *dimg = nullptr, *dtask = nullptr, *dtile = nullptr,
       *dseg = nullptr, *derr = nullptr;
  auto cleanup = [&]() {
    void* q[] = {dA, dB, dC, dimg, dtask, dtile, dseg, derr};
    for (void* x : q)
      if (x) cudaFree(x);
  };
  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaMalloc(&dA, (size_t)M * K * 16);
  if (e == cudaSuccess) e = cudaMalloc(&dB, (size_t)K * N * 16);
  if (e == cudaSuccess) e = cudaMalloc(&dC, (size_t)M * N * 16);
  if (e == cudaSuccess) e = cudaMalloc(&dimg, (size_t)(ia + ib));
  if (e == cudaSuccess) e = cudaMalloc(&derr, sizeof(int));
  if (e != cudaSuccess) {
    cleanup();
    return cuda_check(ctx, e, "selftest alloc");
  }
  cudaMemcpyAsync(dA, A, (size_t)M * K * 16, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dB, B, (size_t)K * N * 16, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(derr, 0, sizeof(int), s);
  tc::ImgTask tk[2] = {};
  tk[0].src = (long long)(uintptr_t)dA; tk[0].sbase = HH_BASE_ABS; tk[0].ld = M; tk[0].rows = M; tk[0].kc = K;
  tk[0].rpad = rpad(M); tk[0].k16 = k16(K); tk[0].trans = 0; tk[0].cre = 1.0; tk[0].dst = (long long)(uintptr_t)dimg;
  tk[0].row0 = 0; tk[0].prow = tk[0].rpad;
  tk[1].src = (long long)(uintptr_t)dB; tk[1].sbase = HH_BASE_ABS; tk[1].ld = K; tk[1].rows = N; tk[1].kc = K;
  tk[1].rpad = rpad(N); tk[1].k16 = k16(K); tk[1].trans = 1; tk[1].cre = 1.0;
  tk[1].row0 = 0; tk[1].prow = tk[1].rpad;
  tk[1].dst = (long long)(uintptr_t)dimg + ia;
  std::vector<tc::Seg> segs;
  std::vector<tc::Tile> tiles;
  ImgRef ai, bi;
  ai.rows = M; ai.kc = K; bi.rows = N; bi.kc = K;
  for (int m0 = 0; m0 < M; m0 += 128)
    for (int n0 = 0; n0 < N; n0 += 128) {
      const int ntile = k16(std::min(128, N - n0));
      tc::Seg sg{};
      const int ar = rpad(M), br = rpad(N);
      sg.a = tk[0].dst + (long long)(m0 / 8) * 256;
      sg.b = tk[1].dst + (long long)(n0 / 8) * 256;
      sg.a_plane = (long long)(ar / 8) * 256;
      sg.b_plane = (long long)(br / 8) * 256;
      sg.a_bytes = std::min(128, ar - m0) * 32;
      sg.b_bytes = std::min(ntile, br - n0) * 32;
      sg.nkc = k16(K) / 16;
      tc::Tile tl{};
      tl.seg0 = (int)segs.size();
      tl.nseg = 1;
      segs.push_back(sg);
      tl.mode = 0;
      tl.ntile = ntile;
      tl.mrem = std::min(128, M - m0);
      tl.nrem = std::min(128, N - n0);
      tl.out = (long long)n0 * M + m0;
      tl.ldo = M;
      tl.m0 = m0;
      tl.n0 = n0;
      tc::finish_tile(tl, segs.data());
      tl.hold = hold ? 1 : 0;
      tiles.push_back(tl);
    }
  e = cudaMalloc(&dtask, sizeof(tk));
  if (e == cudaSuccess) e = cudaMalloc(&dtile, tiles.size() * sizeof(tc::Tile));
  if (e == cudaSuccess) e = cudaMalloc(&dseg, segs.size() * sizeof(tc::Seg));
  if (e == cudaSuccess) e = cudaMemcpyAsync(dtask, tk, sizeof(tk), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dtile, tiles.data(), tiles.size() * sizeof(tc::Tile), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dseg, segs.data(), segs.size() * sizeof(tc::Seg), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = tc_build_images((tc::ImgTask*)dtask, 2, nullptr, false, s);
  if (e == cudaSuccess)
    e = tc_run_tiles((tc::Tile*)dtile, (int)tiles.size(), (tc::Seg*)dseg, (double2*)dC, (int*)derr, true, s,
                     nullptr, 128, split_of(precision));
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(C, dC, (size_t)M * N * 16, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cleanup();
  if (e != cudaSuccess) return cuda_check(ctx, e, "selftest");
  if (herr) return fail(ctx, HH_ERR_TIMEOUT, "selftest: bounded wait ran out, code " + std::to_string(herr));
  return HH_OK;
}
