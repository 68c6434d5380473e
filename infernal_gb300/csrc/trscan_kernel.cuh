// trscan_kernel.cuh -- tiled truncated QDB scanning kernels for sm_103a:
// RefTrCYKScan (ALG 0, max) and RefITrInsideScan (ALG 1, ILogsum),
// src/cm_dpsearch_trunc.c:79-1338.
//
// Same execution model as the standard scan (scan_kernel.cuh): a persistent
// grid pulls sequence windows (W-1 warm-up rows each), end positions advance
// in tiles of T rows, states are swept v = M-1 .. 1 with one CTA barrier per
// state.  Each state now carries three score planes: J (joint), L (left
// marginal: the parse's 3' part is cut off) and R (right marginal: its 5' part
// is cut off); a bifurcation also forms T (both cut).  The pipeline pass
// selects which of L, R, T are filled (cm_TrFillFromPassIdx,
// src/cm_dpsearch_trunc.c:3566).  Inside every cell the scores combine in the
// reference's order (init score first, then children in yoffset order), so
// the integer Inside result is bit-identical; for CYK, whose max is
// order-free, the insert self-loop chains fold their other terms in a
// parallel pass first.
//
// Root.  The truncated scanners leave the root through truncated begins only
// (a penalty into any state), and they never reset the root's cells: a
// (mode, length) cell is only reported at end position j when its score beats
// every earlier score of the same mode and length at the same parity of j
// (src/cm_dpsearch_trunc.c:548-605).  Each state folds its scores plus its
// penalty into per-mode accumulators while its tile is live; the root phase
// walks each (length, parity) chain of the tile in order, keeps the running
// maximum over the window's own rows, and emits every cell that sets a new
// maximum (and passes the score threshold) as a candidate.  The window's
// final maxima go to global memory, so the host can apply the maxima of all
// earlier windows and keep exactly the cells the sequential scan reports.
#pragma once
#include "scan_kernel.cuh"

// Candidate root cell of a truncated scan: (end j, length d, mode) whose best
// truncated-begin score set a new running maximum within its window.
struct TrCand {
  long long j;
  int d;
  float f;      // bit score (Scorify for integer Inside)
  int y;        // state the truncated begin enters (smallest on ties)
  int mode;     // CMGB_TRMODE_*
  int raw;      // bit pattern of the native score (float or int)
  int win;      // window index
};

struct TrKParams {
  const TrStateInfo *st;      // phases in sweep order
  ScanPlan plan;
  const float *oesc, *lmesc, *rmesc;
  const int *ioesc, *ilmesc, *irmesc;
  const int *ilog;            // ILogsum table (integer Inside)
  const unsigned char *dsq;   // device residues, indexed by sequence coordinate
  long long i0, j0;
  long long win_len;
  int nwin;
  int *queue;
  float *carry;               // [grid][2][carry_elems]
  float *ring;                // [grid][ring_elems]
  float *arena;               // [grid][arena_elems] (plans with arena_global)
  TrCand *cand;
  int *ncand;
  int cand_cap;
  float cand_cut;             // emit cells with score >= cand_cut (greedy) ...
  int cand_pos;               // ... or > 0 (optimal resolution) ...
  float env_cut;              // ... or >= env_cut (envelope)
  int fill_L, fill_R, fill_T; // matrices the pass needs
  int pty_idx;                // truncation penalty index of the pass
  unsigned *vsc;              // per-state best score (order-preserving uint), NULL if not wanted
  unsigned long long *winbest;// [nwin] best root cell of each window: score << 32 | ~position
  float *wmax;                // [nwin][4][2][acc_w] root running maxima at window end (native type), or NULL
  int *err;                   // 1: candidate overflow
  // batched scans: window w is the whole scan [win_s[w], win_e[w]] of one sequence (no warm-up rows)
  const long long *win_s, *win_e;
};

// Child loop with a compile-time trip count: the per-child arrays (scores,
// buffer offsets, strides) stay in registers instead of local memory.
#define CMGB_FOR_CHILD(o, first) _Pragma("unroll") for (int o = (first); o < CMGB_MAXC; o++) if (o < cnum)

template <int ALG, bool GL>
CMGB_DEV void tr_scan_body(const TrKParams &p, float *smf, int tid, int nt, int bid)
{
  typedef Sr<ALG> R;
  typedef typename R::T T;
  constexpr bool INS = ALG == 1;
  const ScanPlan &P = p.plan;
  const int W = P.W, TT = P.T, NP = P.nphase, Kp = P.Kp;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  T *sm = GL ? reinterpret_cast<T *>(p.arena) + (size_t) bid * P.arena_elems : reinterpret_cast<T *>(smf);
  T *acc = sm + P.acc_off;                                  // [4][TT][accw]
  int *bestr = reinterpret_cast<int *>(sm) + P.bestr_off;   // [4][TT][accw]
  T *rmax = sm + P.rmax_off;                                // [4][2][accw]
  unsigned char *res = reinterpret_cast<unsigned char *>(smf + P.res_off);
  int *s_win = reinterpret_cast<int *>(smf) + P.smem_elems;
  T *carry0 = reinterpret_cast<T *>(p.carry) + (size_t) bid * 2 * P.carry_elems;
  T *ringb = reinterpret_cast<T *>(p.ring) + (size_t) bid * P.ring_elems;
  const unsigned short *tbl = reinterpret_cast<const unsigned short *>(smf + P.ltbl_off);
  if (INS) {
    unsigned short *t16 = reinterpret_cast<unsigned short *>(smf + P.ltbl_off);
    for (int q = tid; q < CMGB_LTBL; q += nt) t16[q] = (unsigned short) CMGB_LDG(p.ilog + q);
  }
  const float el = P.el_selfsc;
  const int iel = P.iel_selfsc;
  const int accw = P.acc_w, RR = P.ring_rows, rdxW = P.root_dxW;
  const int fL = p.fill_L, fR = p.fill_R, fT = p.fill_T, pidx = p.pty_idx;
  const bool want_vsc = p.vsc != nullptr;
  const int aplane = TT * accw;
  const T imp = R::imp();
  for (int d = tid; d < P.const_row_len; d += nt) { sm[P.const_row + d] = d == 0 ? (T) 0 : imp; sm[P.imp_row + d] = imp; }
  CMGB_SYNC();

  for (;;) {
    CMGB_SYNC();
    if (tid == 0) *s_win = CMGB_ATOMIC_ADD(p.queue, 1);
    CMGB_SYNC();
    const int w = *s_win;
    if (w >= p.nwin) break;
    long long own_s, own_e, s0;
    if (p.win_s) { own_s = s0 = p.win_s[w]; own_e = p.win_e[w]; }
    else {
      own_s = p.i0 + (long long) w * p.win_len;
      own_e = own_s + p.win_len - 1;
      if (own_e > p.j0) own_e = p.j0;
      s0 = own_s - (W - 1);
      if (s0 < p.i0) s0 = p.i0;
    }
    const int own_jp = (int) (own_s - s0 + 1);
    const int last_jp = (int) (own_e - s0 + 1);

    // carry rows of j = s0-1 and ring row 0: d = 0 init in J, IMPOSSIBLE elsewhere
    for (int k = 0; k < NP; k++) {
      const StateInfo &si = p.st[k].s;
      const T i0v = INS ? (T) p.st[k].iinit0 : (T) si.init0;
      const int width = si.hi - si.lo + 1;
      if (si.carry >= 0)
        for (int x = tid; x < 3 * width; x += nt) {
          const int m = x / width, d = si.lo + x - m * width;
          if ((m == 1 && !fL) || (m == 2 && !fR)) continue;   // planes the pass does not fill are never read
          carry0[si.carry + m * si.stride + d - si.lo] = (m == 0 && d == 0) ? i0v : imp;
        }
      if (si.kind == SK_BEGL)
        for (int x = tid; x < 3 * width; x += nt) {
          const int m = x / width, d = si.lo + x - m * width;
          if ((m == 1 && !fL) || (m == 2 && !fR)) continue;
          ringb[si.ring + m * RR * si.stride + d - si.lo] = (m == 0 && d == 0) ? i0v : imp;
        }
    }
    for (int q = tid; q < 8 * accw; q += nt) rmax[q] = imp;
    unsigned long long my_best = 0ULL;

    int par = 0;
    for (int jp0 = 0; jp0 < last_jp; jp0 += TT, par ^= 1) {
      const int nrows = (last_jp - jp0) < TT ? (last_jp - jp0) : TT;
      const T *cin = carry0 + (size_t) par * P.carry_elems;
      T *cout = carry0 + (size_t) (par ^ 1) * P.carry_elems;
      const long long rbase = s0 + jp0 - W;
      const int ringj = jp0 % RR;
      CMGB_SYNC();
      for (int k = tid; k < P.res_len; k += nt) {
        const long long q = rbase + k;
        unsigned char x = (q >= 0 && q <= p.j0 + 1) ? p.dsq[q] : (unsigned char) 0;
        res[k] = x < Kp ? x : (unsigned char) (Kp - 1);
      }
      for (int k = tid; k < 4 * aplane; k += nt) { acc[k] = R::acc_init(); bestr[k] = -1; }
      CMGB_SYNC();

      for (int k = 0; k < NP; k++) {
        const TrStateInfo &ti = p.st[k];
        const StateInfo &si = ti.s;
        const int v = si.v, kind = si.kind, lo = si.lo, hi = si.hi, dxW = si.dxW;
        const int cnum = si.cnum, emit = si.emit, stride = si.stride, buf = si.buf, carry = si.carry;
        const int mst = ti.mstride;
        const bool hasend = INS ? (bool) si.has_iend : (bool) si.has_end;
        const float endsc_f = si.endsc;
        const int iendsc_i = si.iendsc;
        const T pen = INS ? (T) ti.ipty[pidx] : (T) ti.pty[pidx];
        const bool has_pty = INS ? (ti.ipty[pidx] != -CMGB_INF) : CMGB_NOT_IMP(ti.pty[pidx]);
        const T i0v = INS ? (T) ti.iinit0 : (T) si.init0;
        const int wpa = si.wp_all, sra = si.sr_all, sdda = si.sdd_all, wpb = si.wp_band, srb = si.sr_band, sddb = si.sdd_band;
        const float inva = si.inv_all, invb = si.inv_band;
        const int eoff = si.oesc_off;
        float vbest = CMGB_IMP;
        T tv[CMGB_MAXC];
        int cb[CMGB_MAXC], cs[CMGB_MAXC], cmo[CMGB_MAXC];
#pragma unroll
        for (int o = 0; o < CMGB_MAXC; o++) { tv[o] = R::tsc(si, o); cb[o] = si.cbuf[o] - si.clo[o]; cs[o] = si.cstr[o]; cmo[o] = ti.cm[o]; }
#define INIT(dd) R::init_h(hasend, endsc_f, iendsc_i, (dd), el, iel)
#define CHV(o, m, rr, dd) sm[cb[o] + (m) * cmo[o] + (rr) * cs[o] + (dd)]
#define ESC1(x) (INS ? (T) CMGB_LDG(p.ioesc + eoff + (x)) : (T) CMGB_LDG(p.oesc + eoff + (x)))
#define MAXT(a, b) ((a) > (b) ? (a) : (b))
        T *own = sm + buf - lo;   // own[m * mst + r * stride + d]
        // fold this cell's scores into the root's accumulators (truncated begins)
        auto root_fold = [&](int r, int d, int jp, T vJ, T vL, T vR, T vT, bool isB) {
          const int rdx = jp < rdxW ? jp : rdxW;
          if (!has_pty || d > rdx) return;
          const int ai = (r - 1) * accw + d - 1;
          T cc = R::add(vJ, pen);
          if (cc >= acc[ai]) { acc[ai] = cc; bestr[ai] = v; }
          if (fL) { cc = R::add(vL, pen); if (cc >= acc[aplane + ai]) { acc[aplane + ai] = cc; bestr[aplane + ai] = v; } }
          if (fR) { cc = R::add(vR, pen); if (cc >= acc[2 * aplane + ai]) { acc[2 * aplane + ai] = cc; bestr[2 * aplane + ai] = v; } }
          if (fT && isB) { cc = R::add(vT, pen); if (cc >= acc[3 * aplane + ai]) { acc[3 * aplane + ai] = cc; bestr[3 * aplane + ai] = v; } }
        };
        // per-state best score: every owned row for CYK, the final row for integer Inside
        auto vsc_fold = [&](int jp, T vJ, T vL, T vR, T vT, bool isB) {
          if (!want_vsc) return;
          if (INS ? (s0 + jp - 1 != p.j0) : (jp < own_jp)) return;
          T b = vJ;
          if (fL) b = MAXT(b, vL);
          if (fR) b = MAXT(b, vR);
          if (fT && isB) b = MAXT(b, vT);
          const float f = R::score(b);
          vbest = vbest > f ? vbest : f;
        };

        if (kind == SK_ROOT) {
          // ---- root: registration of new running maxima per (length, parity) ----
          for (int q = tid; q < 2 * accw; q += nt) {
            const int d = 1 + (q >> 1), pq = q & 1;
            for (int r = 1; r <= nrows; r++) {
              const int jp = jp0 + r;
              const long long j = s0 + jp - 1;
              if ((int) (j & 1) != pq || jp < own_jp) continue;
              if (d > (jp < rdxW ? jp : rdxW)) continue;
              const int ai = (r - 1) * accw + d - 1;
              float fbest = 0.f; int wm = -1, wy = 0;
              for (int mm = 0; mm < 4; mm++) {
                if ((mm == 1 && !fL) || (mm == 2 && !fR) || (mm == 3 && !fT)) continue;
                const T rv = acc[mm * aplane + ai];
                T &mx = rmax[(mm * 2 + pq) * accw + d - 1];
                if (!(rv > mx)) continue;
                mx = rv;
                const float f = R::score(rv);
                const int y = bestr[mm * aplane + ai];
                if ((p.cand_pos ? (f > 0.0f) : (f >= p.cand_cut)) || f >= p.env_cut) {
                  const int sl = CMGB_ATOMIC_ADD(p.ncand, 1);
                  if (sl < p.cand_cap) {
                    TrCand cc; cc.j = j; cc.d = d; cc.f = f; cc.y = y; cc.mode = 3 - mm; cc.win = w;
                    union { T t; int i; } u; u.t = rv; cc.raw = u.i;
                    p.cand[sl] = cc;
                  } else CMGB_ATOMIC_OR(p.err, 1);
                }
                if (wm < 0 || f > fbest || (f == fbest && y < wy)) { fbest = f; wm = mm; wy = y; }
              }
              if (wm >= 0) {
                const unsigned long long pos = ((unsigned long long) (j - own_s) * (unsigned long long) (W + 1) + (unsigned long long) d) * 4ULL + (unsigned long long) wm;
                const unsigned long long key = ((unsigned long long) cmgb_f2u(fbest) << 32) | (0xFFFFFFFFULL - (pos & 0xFFFFFFFFULL));
                if (key > my_best) my_best = key;
              }
            }
          }
        } else if (kind == SK_IL || kind == SK_IR) {
          for (int x = tid; x < 3 * (hi - lo + 1); x += nt) {
            const int m = x / (hi - lo + 1), xx = x - m * (hi - lo + 1);
            if ((m == 1 && !fL) || (m == 2 && !fR)) continue;
            sm[buf + m * mst + xx] = cin[carry + m * stride + xx];
          }
          const bool il = kind == SK_IL;
          // (1) the mode without a self-loop: R for IL, L for IR (children yoffset >= 1, same row, length d)
          const int pm = il ? 2 : 1;
          if (il ? fR : fL)
            for (CellWalk c(tid, lo, hi, wpa, sra, sdda, inva); c.r <= nrows; c.next()) {
              const int r = c.r, d = c.d, jp = jp0 + r;
              const int dx = jp < dxW ? jp : dxW;
              T val;
              if (d < 1 || d > dx) val = imp;
              else {
                val = INIT(d);
                CMGB_FOR_CHILD(o, 1)
                  val = R::comb(val, R::comb(R::add(CHV(o, 0, r, d), tv[o]), R::add(CHV(o, pm, r, d), tv[o]), tbl), tbl);
              }
              own[pm * mst + r * stride + d] = val;
              if (r == TT) cout[carry + pm * stride + d - lo] = val;
            }
          // (2) the self-loop planes (IL: J and L; IR: J and R)
          if (ALG == 0) {
            // CYK: max is order-free, so every term but the self-loop is folded
            // for all band cells in parallel into the scratch (plane slot 0: J,
            // slot 1: L for IL, R for IR), and the chains fold the self-loop
            // last: x = max(t, x + tself) + e
            T *tmp = reinterpret_cast<T *>(smf) + P.tmp_off;
            const int tstr = P.tmp_stride, tpl = (TT + 1) * tstr;
            const int m1 = il ? 1 : 2;                   // second self-loop plane
            const bool two = il ? (bool) fL : (bool) fR;
            const int crow0 = il ? 0 : 1;                // children at row r (IL) or r-1 (IR), length d-1
            for (CellWalk c(tid, 1, dxW, wpb, srb, sddb, invb); c.r <= nrows; c.next()) {
              const int r = c.r, d = c.d;
              if (d > jp0 + r) continue;
              T sJ = INIT(d - 1), s1 = sJ;
              CMGB_FOR_CHILD(o, 1) {
                sJ = MAXT(sJ, R::add(CHV(o, 0, r - crow0, d - 1), tv[o]));
                if (two) s1 = MAXT(s1, R::add(CHV(o, m1, r - crow0, d - 1), tv[o]));
              }
              tmp[r * tstr + d - lo] = sJ;
              if (two) tmp[tpl + r * tstr + d - lo] = s1;
            }
            CMGB_SYNC();
            const T tself = tv[0];
            if (il) {
              // IL(r,d) <- IL(r,d-1): one thread per (row, plane), serial in d
              const int npl = two ? 2 : 1;
              for (int q = tid; q < npl * nrows; q += nt) {
                const int mi = q % npl, r = 1 + q / npl, m = mi ? 1 : 0;
                const int jp = jp0 + r;
                const int dx = jp < dxW ? jp : dxW;
                T *row = own + m * mst + r * stride;
                const T *trow = tmp + mi * tpl + r * tstr - lo;
                T *crow = r == TT ? cout + carry + m * stride - lo : nullptr;
                for (int d = lo; d <= hi; d++)
                  if (d < 1 || d > dx) { const T pv = d == 0 ? (m == 0 ? i0v : imp) : imp; row[d] = pv; if (crow) crow[d] = pv; }
                T x = m == 0 ? i0v : imp;   // the d = 0 cell
                for (int d0 = 1; d0 <= dx; d0 += CMGB_CHUNK) {
                  const int n = dx - d0 + 1;
                  T tt[CMGB_CHUNK], ee[CMGB_CHUNK];
#pragma unroll
                  for (int u = 0; u < CMGB_CHUNK; u++) {
                    tt[u] = u < n ? trow[d0 + u] : imp;
                    ee[u] = u < n ? ESC1(res[W + r - d0 - u]) : (T) 0;
                  }
#pragma unroll
                  for (int u = 0; u < CMGB_CHUNK; u++) {
                    const T nx = (m == 1 && d0 + u == 1) ? ee[u] : R::add(MAXT(tt[u], R::add(x, tself)), ee[u]);
                    if (u < n) {
                      x = nx;
                      row[d0 + u] = x;
                      if (crow) crow[d0 + u] = x;
                    }
                  }
                }
              }
            } else {
              // IR(r,d) <- IR(r-1,d-1): one thread per (diagonal, plane); a
              // diagonal's band cells are one run b0..b1 (d <= jp holds on a
              // whole diagonal or on none of it)
              const int ndiag = hi - lo + 1 + TT;
              const int npl = two ? 2 : 1;
              const int dstep = stride + 1, tstep = tstr + 1;
              for (int q = tid; q < npl * ndiag; q += nt) {
                const int mi = q % npl, cdg = lo - TT + q / npl, m = mi ? 2 : 0;
                const int ra = lo - cdg > 1 ? lo - cdg : 1, rz = hi - cdg < nrows ? hi - cdg : nrows;
                if (ra > rz) continue;
                const int b0 = 1 - cdg > ra ? 1 - cdg : ra;
                const int b1 = cdg > jp0 ? ra - 1 : (dxW - cdg < rz ? dxW - cdg : rz);
                T *base = own + m * mst;
                const T pad0 = m == 0 ? i0v : imp;   // a d = 0 cell of this plane
                T *out = base + ra * stride + cdg + ra;
                if (b0 > b1) {
                  for (int r = ra; r <= rz; r++, out += dstep) *out = cdg + r == 0 ? pad0 : imp;
                } else {
                  T x = (ra == 1 && cdg >= lo) ? base[cdg] : imp;   // the diagonal's row-0 cell
                  for (int r = ra; r < b0; r++, out += dstep) { x = cdg + r == 0 ? pad0 : imp; *out = x; }
                  for (int r = b0; r <= b1; r += CMGB_CHUNK, out += CMGB_CHUNK * dstep) {
                    const int n = b1 - r + 1;
                    const T *tp = tmp + mi * tpl + r * tstr + cdg + r - lo;
                    T tt[CMGB_CHUNK], ee[CMGB_CHUNK];
#pragma unroll
                    for (int u = 0; u < CMGB_CHUNK; u++) {
                      tt[u] = u < n ? tp[u * tstep] : imp;
                      ee[u] = u < n ? ESC1(res[W + r + u - 1]) : (T) 0;
                    }
#pragma unroll
                    for (int u = 0; u < CMGB_CHUNK; u++) {
                      const T nx = (m == 2 && cdg + r + u == 1) ? ee[u] : R::add(MAXT(tt[u], R::add(x, tself)), ee[u]);
                      if (u < n) { x = nx; out[u * dstep] = x; }
                    }
                  }
                  out = base + (b1 + 1) * stride + cdg + b1 + 1;
                  for (int r = b1 + 1; r <= rz; r++, out += dstep) *out = cdg + r == 0 ? pad0 : imp;
                }
                // the diagonal's row-TT cell is the next tile's carry
                if (TT <= nrows && TT >= ra && TT <= rz) cout[carry + m * stride + cdg + TT - lo] = base[TT * stride + cdg + TT];
              }
            }
          } else {
          CMGB_SYNC();
          // (2) the self-loop chains, children folded in the reference's order
          if (il) {
            // IL(r,d) <- IL(r,d-1): one warp per row, lanes own runs of C cells;
            // carries cross lanes in rounds until none changes (exact)
            for (int r = 1 + warp; r <= nrows; r += nwarp) {
              const int jp = jp0 + r;
              const int dx = jp < dxW ? jp : dxW;
              for (int m = 0; m < 2; m++) {
                if (m == 1 && !fL) break;
                T *row = own + m * mst + r * stride;
                for (int d = lo + lane; d <= hi; d += 32) if (d < 1 || d > dx) row[d] = d == 0 ? (m == 0 ? i0v : imp) : imp;
                const int n = dx;
                if (n > 0) {
                  const int C = (n + 31) >> 5;
                  const int d0 = 1 + lane * C;
                  const int d1 = (d0 + C - 1 < dx) ? d0 + C - 1 : dx;
                  const T start = m == 0 ? i0v : imp;
                  T carry_in = start;
                  for (int round = 0; round < 33; round++) {
                    T x = carry_in;
                    for (int d = d0; d <= d1; d++) {
                      const T e = ESC1(res[W + r - d]);
                      if (m == 1 && d == 1) x = e;
                      else {
                        T s = R::comb(INIT(d - 1), R::add(x, tv[0]), tbl);
                        CMGB_FOR_CHILD(o, 1) s = R::comb(s, R::add(CHV(o, m, r, d - 1), tv[o]), tbl);
                        x = R::add(s, e);
                      }
                      row[d] = x;
                    }
                    const T outv = (d0 <= d1) ? x : carry_in;
                    T nc = cmgb_shfl_up(outv, 1);
                    if (lane == 0) nc = start;
                    const bool changed = (d0 <= d1) && (nc != carry_in);
                    carry_in = nc;
                    if (!cmgb_any(changed)) break;
                  }
                }
                __syncwarp_portable();
                if (r == TT) for (int d = lo + lane; d <= hi; d += 32) cout[carry + m * stride + d - lo] = row[d];
                __syncwarp_portable();
              }
            }
          } else {
            // IR(r,d) <- IR(r-1,d-1): one thread per diagonal, J and R planes
            const int ndiag = hi - lo + 1 + TT;
            for (int q = tid; q < ndiag; q += nt) {
              const int cdg = lo - TT + q;
              T xJ = (cdg >= lo && cdg <= hi) ? own[cdg] : imp;
              T xR = (cdg >= lo && cdg <= hi) ? own[2 * mst + cdg] : imp;
              for (int r = 1; r <= nrows; r++) {
                const int d = cdg + r;
                if (d < lo || d > hi) { xJ = xR = imp; continue; }
                const int jp = jp0 + r;
                const int dx = jp < dxW ? jp : dxW;
                T vJ, vR;
                if (d < 1 || d > dx) { vJ = d == 0 ? i0v : imp; vR = imp; }
                else {
                  const T ej = ESC1(res[W + r - 1]);
                  T s = R::comb(INIT(d - 1), R::add(xJ, tv[0]), tbl);
                  CMGB_FOR_CHILD(o, 1) s = R::comb(s, R::add(CHV(o, 0, r - 1, d - 1), tv[o]), tbl);
                  vJ = R::add(s, ej);
                  if (fR) {
                    if (d == 1) vR = ej;
                    else {
                      T s2 = R::comb(INIT(d - 1), R::add(xR, tv[0]), tbl);
                      CMGB_FOR_CHILD(o, 1) s2 = R::comb(s2, R::add(CHV(o, 2, r - 1, d - 1), tv[o]), tbl);
                      vR = R::add(s2, ej);
                    }
                  } else vR = imp;
                }
                own[r * stride + d] = vJ;
                if (fR) own[2 * mst + r * stride + d] = vR;
                if (r == TT) { cout[carry + d - lo] = vJ; if (fR) cout[carry + 2 * stride + d - lo] = vR; }
                xJ = vJ; xR = vR;
              }
            }
          }
          }
          CMGB_SYNC();
          // (3) root accumulators and per-state best over the finished band cells
          if (has_pty || want_vsc)
            for (CellWalk c(tid, 1, dxW, wpb, srb, sddb, invb); c.r <= nrows; c.next()) {
              const int r = c.r, d = c.d, jp = jp0 + r;
              if (d > jp) continue;
              const T vJ = own[r * stride + d];
              const T vL = fL ? own[mst + r * stride + d] : imp;
              const T vR = fR ? own[2 * mst + r * stride + d] : imp;
              root_fold(r, d, jp, vJ, vL, vR, imp, false);
              vsc_fold(jp, vJ, vL, vR, imp, false);
            }
        } else {
          // ---- generic states, BEGL_S and B: all cells of the phase in parallel ----
          const bool begl = kind == SK_BEGL, isB = kind == SK_B;
          if (!begl)
            for (int x = tid; x < 3 * (hi - lo + 1); x += nt) {
              const int m = x / (hi - lo + 1), xx = x - m * (hi - lo + 1);
              if ((m == 1 && !fL) || (m == 2 && !fR)) continue;
              sm[buf + m * mst + xx] = cin[carry + m * stride + xx];
            }
          for (CellWalk c(tid, lo, hi, wpa, sra, sdda, inva); c.r <= nrows; c.next()) {
            const int r = c.r, d = c.d, jp = jp0 + r;
            const int dx = jp < dxW ? jp : dxW;
            int rrow = ringj + r; if (rrow >= RR) rrow -= RR;
            T vJ, vL = imp, vR = imp, vT = imp;
            const bool band = d >= 1 && d <= dx;
            if (!band) vJ = d == 0 ? i0v : imp;
            else if (isB) {
              // bifurcation: k = length of the right child's part (src/cm_dpsearch_trunc.c:276-320)
              int kmin = 0, kmax = d;
              if (si.banded) { kmin = d - si.dx_w; if (kmin < 0) kmin = 0; kmax = si.dx_y < d ? si.dx_y : d; }
              vJ = INIT(d); vL = vJ; vR = vJ; vT = vJ;
              const T *yJ = sm + cb[1] + r * cs[1], *yL = yJ + cmo[1], *yR = yJ + 2 * cmo[1];
              const T *wJ = ringb + cb[0] + d, *wL = wJ + cmo[0], *wR = wJ + 2 * cmo[0];
              const int wstr = cs[0];
              int rr = rrow - kmin; if (rr < 0) rr += RR;
              for (int kk = kmin; kk <= kmax; kk++) {
                const T a = wJ[rr * wstr - kk];
                vJ = R::comb(vJ, R::add(a, yJ[kk]), tbl);
                if (fL) vL = R::comb(vL, R::add(a, yL[kk]), tbl);
                if (fR) vR = R::comb(vR, R::add(wR[rr * wstr - kk], yJ[kk]), tbl);
                rr = rr == 0 ? RR - 1 : rr - 1;
              }
              if (fT) {
                const int kn = kmin > 1 ? kmin : 1, kx = kmax < d - 1 ? kmax : d - 1;
                rr = rrow - kn; if (rr < 0) rr += RR;
                for (int kk = kn; kk <= kx; kk++) {
                  vT = R::comb(vT, R::add(wR[rr * wstr - kk], yL[kk]), tbl);
                  rr = rr == 0 ? RR - 1 : rr - 1;
                }
              }
              if (fL && kmin == 0) vL = R::comb(vL, MAXT(wJ[rrow * wstr], wL[rrow * wstr]), tbl);
              if (fR && kmax == d) vR = R::comb(vR, MAXT(yJ[d], yR[d]), tbl);
            } else if (emit == 0) {
              // S, D, BEGL_S: every mode from the same mode of the children
              vJ = INIT(d); vL = vJ; vR = vJ;
              CMGB_FOR_CHILD(o, 0) {
                vJ = R::comb(vJ, R::add(CHV(o, 0, r, d), tv[o]), tbl);
                if (fL) vL = R::comb(vL, R::add(CHV(o, 1, r, d), tv[o]), tbl);
                if (fR) vR = R::comb(vR, R::add(CHV(o, 2, r, d), tv[o]), tbl);
              }
            } else if (emit == 1) {
              // ML (src/cm_dpsearch_trunc.c:341-380)
              const T e = ESC1(res[W + r - d]);
              vJ = INIT(d - 1); vL = vJ;
              CMGB_FOR_CHILD(o, 0) {
                vJ = R::comb(vJ, R::add(CHV(o, 0, r, d - 1), tv[o]), tbl);
                if (fL) vL = R::comb(vL, R::add(CHV(o, 1, r, d - 1), tv[o]), tbl);
              }
              vJ = R::add(vJ, e);
              vL = d >= 2 ? R::add(vL, e) : e;
              if (fR) {
                vR = INIT(d);
                CMGB_FOR_CHILD(o, 0)
                  vR = R::comb(vR, R::comb(R::add(CHV(o, 0, r, d), tv[o]), R::add(CHV(o, 2, r, d), tv[o]), tbl), tbl);
              }
            } else if (emit == 2) {
              // MR (src/cm_dpsearch_trunc.c:381-420)
              const T ej = ESC1(res[W + r - 1]);
              vJ = INIT(d - 1); vR = vJ;
              CMGB_FOR_CHILD(o, 0) {
                vJ = R::comb(vJ, R::add(CHV(o, 0, r - 1, d - 1), tv[o]), tbl);
                if (fR) vR = R::comb(vR, R::add(CHV(o, 2, r - 1, d - 1), tv[o]), tbl);
              }
              vJ = R::add(vJ, ej);
              vR = d >= 2 ? R::add(vR, ej) : ej;
              if (fL) {
                vL = INIT(d);
                CMGB_FOR_CHILD(o, 0)
                  vL = R::comb(vL, R::comb(R::add(CHV(o, 0, r, d), tv[o]), R::add(CHV(o, 1, r, d), tv[o]), tbl), tbl);
              }
            } else {
              // MP (src/cm_dpsearch_trunc.c:421-447)
              const int xi = res[W + r - d], xj = res[W + r - 1];
              vJ = d >= 2 ? INIT(d - 2) : imp;
              vL = INIT(d - 1); vR = vL;
              CMGB_FOR_CHILD(o, 0) {
                if (d >= 2) vJ = R::comb(vJ, R::add(CHV(o, 0, r - 1, d - 2), tv[o]), tbl);
                if (fL) vL = R::comb(vL, MAXT(R::add(CHV(o, 0, r, d - 1), tv[o]), R::add(CHV(o, 1, r, d - 1), tv[o])), tbl);
                if (fR) vR = R::comb(vR, MAXT(R::add(CHV(o, 0, r - 1, d - 1), tv[o]), R::add(CHV(o, 2, r - 1, d - 1), tv[o])), tbl);
              }
              vJ = d >= 2 ? R::add(vJ, ESC1(xi * Kp + xj)) : imp;
              const T lm = INS ? (T) CMGB_LDG(p.ilmesc + v * Kp + xi) : (T) CMGB_LDG(p.lmesc + v * Kp + xi);
              const T rm = INS ? (T) CMGB_LDG(p.irmesc + v * Kp + xj) : (T) CMGB_LDG(p.rmesc + v * Kp + xj);
              vL = d >= 2 ? R::add(vL, lm) : lm;
              vR = d >= 2 ? R::add(vR, rm) : rm;
            }
            if (band) {
              root_fold(r, d, jp, vJ, vL, vR, vT, isB);
              vsc_fold(jp, vJ, vL, vR, vT, isB);
            }
            if (begl) {
              T *rg = ringb + si.ring + rrow * stride + d - lo;
              rg[0] = vJ;
              if (fL) rg[mst] = vL;
              if (fR) rg[2 * mst] = vR;
            } else {
              own[r * stride + d] = vJ;
              if (fL) own[mst + r * stride + d] = vL;
              if (fR) own[2 * mst + r * stride + d] = vR;
              if (r == TT) {
                cout[carry + d - lo] = vJ;
                if (fL) cout[carry + stride + d - lo] = vL;
                if (fR) cout[carry + 2 * stride + d - lo] = vR;
              }
            }
          }
        }
#undef INIT
#undef CHV
#undef ESC1
#undef MAXT
        if (want_vsc && vbest > CMGB_IMP) CMGB_ATOMIC_MAXU(p.vsc + v, cmgb_f2u(vbest));
        CMGB_SYNC();
      }
    }
    // window outputs: final running maxima and the best root cell
    if (p.wmax) {
      T *wm = reinterpret_cast<T *>(p.wmax) + (size_t) w * 8 * accw;
      for (int q = tid; q < 8 * accw; q += nt) wm[q] = rmax[q];
    }
    if (my_best) CMGB_ATOMIC_MAXULL(p.winbest + w, my_best);
  }
}

#ifndef CMGB_HOST_EMULATION
template <int ALG, bool GL>
__global__ void __launch_bounds__(512, 2) tr_scan_kernel(TrKParams p)
{
  extern __shared__ __align__(128) float smem_dyn[];
  tr_scan_body<ALG, GL>(p, smem_dyn, threadIdx.x, blockDim.x, blockIdx.x);
}
#endif
