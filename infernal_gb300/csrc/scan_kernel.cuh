// scan_kernel.cuh -- tiled QDB scanning CYK / integer-Inside kernel for sm_103a.
//
// One CTA scans one sequence window at a time (a persistent grid pulls
// windows from a global counter).  A window covers end positions
// [own_start, own_end] plus a warm-up of W-1 residues before own_start; cells
// of the warm-up rows are computed but not reported, and every cell of an
// owned row depends only on residues inside the window, so the result equals
// one sequential scan of [i0, j0] (the reference's scan, src/cm_dpsearch.c:215).
//
// Within a window the end positions advance in tiles of T rows.  For each
// tile the states are swept v = M-1 .. 0 with one CTA barrier per state; the
// state's T x band cells are computed in parallel from its children's tiles
// in shared memory (see scan_plan.h for the layout).  Per state kind:
//   generic states / BEGL_S / B : one warp per row, lanes over d
//   IL (self-loop on the same row, serial in d) : one thread per row
//   IR (self-loop on the previous row, serial along a diagonal) : one thread per diagonal
// BEGL_S rows go to a per-CTA history ring in global memory, which the
// bifurcation's k-loop reads (alpha_begl[(j-k)%(W+1)], src/cm_dpsearch.c:253-277).
// Local begins are folded into a root accumulator while each state's cells
// are live (src/cm_dpsearch.c:567-610), in descending state order with a
// ">=" test, which selects the same (score, root) as the reference's
// ascending-order strict "<" test.
//
// The same source compiles for the GPU and, in the test suite only, for a
// host-thread emulation of one CTA (CMGB_HOST_EMULATION), which is how the
// indexing is checked on machines without a GPU.
#pragma once
#include "scan_plan.h"

#ifndef CMGB_HOST_EMULATION
#define CMGB_DEV __device__ __forceinline__
#define CMGB_SYNC() __syncthreads()
#define CMGB_LDG(p) __ldg(p)
#define CMGB_FADD(a, b) __fadd_rn((a), (b))
#define CMGB_FMUL(a, b) __fmul_rn((a), (b))
#define CMGB_FDIV(a, b) __fdiv_rn((a), (b))
#define CMGB_I2F(x) __int2float_rn(x)
#define CMGB_ATOMIC_ADD(p, v) atomicAdd((p), (v))
#define CMGB_ATOMIC_MAXU(p, v) atomicMax((p), (v))
#define CMGB_ATOMIC_MINLL(p, v) atomicMin((long long *) (p), (long long) (v))
#define CMGB_ATOMIC_MAXLL(p, v) atomicMax((long long *) (p), (long long) (v))
#else
#define CMGB_DEV inline
#define CMGB_SYNC() cmgb_emu_sync()
#define CMGB_LDG(p) (*(p))
#define CMGB_FADD(a, b) ((float) (a) + (float) (b))
#define CMGB_FMUL(a, b) ((float) (a) * (float) (b))
#define CMGB_FDIV(a, b) ((float) (a) / (float) (b))
#define CMGB_I2F(x) ((float) (x))
#define CMGB_ATOMIC_ADD(p, v) __atomic_fetch_add((p), (v), __ATOMIC_SEQ_CST)
#define CMGB_ATOMIC_MAXU(p, v) cmgb_emu_maxu((p), (v))
#define CMGB_ATOMIC_MINLL(p, v) cmgb_emu_minll((long long *) (p), (long long) (v))
#define CMGB_ATOMIC_MAXLL(p, v) cmgb_emu_maxll((long long *) (p), (long long) (v))
#endif

#define CMGB_IMP (-1e36f)
#define CMGB_NOT_IMP(x) ((x) > -9.999e35f)
#define CMGB_INF 987654321
#define CMGB_LTBL 23000

// A candidate cell of the root: end j, length d, score, root state.
struct Cand {
  long long j;
  int d;
  float sc;
  int r;
  int pad;
};

struct KParams {
  const StateInfo *st;
  ScanPlan plan;
  const float *oesc;
  const int *ioesc;
  const int *ilog;            // ILogsum table (integer Inside)
  const unsigned char *dsq;   // device residues, indexed by sequence coordinate
  long long i0, j0;           // scan range
  long long win_len;          // owned end positions per window
  int nwin;
  int *queue;                 // window counter
  float *carry;               // [grid][2][carry_elems]
  float *ring;                // [grid][ring_elems]
  Cand *cand;                 // candidate buffer
  int *ncand;
  int cand_cap;
  float cand_cut;             // report cells with score >= cand_cut (greedy) ...
  int cand_pos;               // ... or with score > 0 (optimal resolution)
  float env_cut;
  long long *env;             // [0] = min i, [1] = max j over cells >= env_cut
  unsigned *vsc;              // per-state best score (order-preserving uint), NULL if not wanted
  unsigned *best;             // best root score (order-preserving uint)
  int *err;                   // error word (candidate overflow)
};

// Order-preserving float <-> uint mapping for atomicMax.
CMGB_DEV unsigned cmgb_f2u(float f)
{
  union { float f; unsigned u; } x; x.f = f;
  return (x.u & 0x80000000u) ? ~x.u : (x.u | 0x80000000u);
}

// Score semiring: CYK is (max, +) over float; integer Inside is
// (ILogsum, +) over int (src/logsum.c:87-92).
template <bool INS> struct Sr;
template <> struct Sr<false> {
  typedef float T;
  static CMGB_DEV T imp() { return CMGB_IMP; }
  static CMGB_DEV T add(T a, T b) { return CMGB_FADD(a, b); }
  static CMGB_DEV T comb(T a, T b, const int *) { return a > b ? a : b; }   // ESL_MAX(a,b)
  static CMGB_DEV T rootfirst(T x) { return CMGB_IMP > x ? CMGB_IMP : x; } // ESL_MAX(IMPOSSIBLE, x)
  static CMGB_DEV float score(T x) { return x; }
  static CMGB_DEV float envval(T x) { return x; }
  static CMGB_DEV T init_sc(const StateInfo &s, int d, float el, int) {
    return s.has_end ? CMGB_FADD(CMGB_FMUL(el, CMGB_I2F(d)), s.endsc) : CMGB_IMP;
  }
  static CMGB_DEV T init0(const StateInfo &s) { return s.init0; }
  static CMGB_DEV T tsc(const StateInfo &s, int o) { return s.tsc[o]; }
  static CMGB_DEV T beginsc(const StateInfo &s) { return s.beginsc; }
  static CMGB_DEV T esc(const KParams &p, int idx) { return CMGB_LDG(p.oesc + idx); }
  static CMGB_DEV T acc_init() { return -3.0e38f; }
};
template <> struct Sr<true> {
  typedef int T;
  static CMGB_DEV T imp() { return -CMGB_INF; }
  static CMGB_DEV T add(T a, T b) { return a + b; }
  static CMGB_DEV T comb(T a, T b, const int *tbl) {
    int mx = a > b ? a : b; mx = mx > -CMGB_INF ? mx : -CMGB_INF;
    int mn = a < b ? a : b;
    return (mn <= -CMGB_INF || (mx - mn) >= CMGB_LTBL) ? mx : mx + CMGB_LDG(tbl + (mx - mn));
  }
  static CMGB_DEV T rootfirst(T x) { return -CMGB_INF > x ? -CMGB_INF : x; }
  static CMGB_DEV float score(T x) { return x == -CMGB_INF ? CMGB_IMP : CMGB_FDIV(CMGB_I2F(x), 1000.0f); }
  static CMGB_DEV float envval(T x) { return CMGB_I2F(x); }
  static CMGB_DEV T init_sc(const StateInfo &s, int d, float, int iel) {
    return s.has_iend ? iel * d + s.iendsc : -CMGB_INF;
  }
  static CMGB_DEV T init0(const StateInfo &s) { return s.iinit0; }
  static CMGB_DEV T tsc(const StateInfo &s, int o) { return s.itsc[o]; }
  static CMGB_DEV T beginsc(const StateInfo &s) { return s.ibeginsc; }
  static CMGB_DEV T esc(const KParams &p, int idx) { return CMGB_LDG(p.ioesc + idx); }
  static CMGB_DEV T acc_init() { return (int) 0x80000000; }
};

// Children fold in the Fast scanners' order per child count
// (src/cm_dpsearch.c:307-519 and 1328-1520): the same sequence of
// max / ILogsum calls, so float and integer results are bit-identical.
template <bool INS>
CMGB_DEV typename Sr<INS>::T fold_children(const StateInfo &s, const typename Sr<INS>::T *sm,
                                           int row, int dp, typename Sr<INS>::T init, const int *tbl)
{
  typedef Sr<INS> R;
  typedef typename R::T T;
#define CH(o) R::add(sm[s.cbuf[o] + row * s.cstr[o] + dp - s.clo[o]], R::tsc(s, o))
  T sc;
  switch (s.cnum) {
  case 2: sc = R::comb(CH(1), init, tbl); sc = R::comb(sc, CH(0), tbl); break;
  case 3: sc = R::comb(CH(2), CH(1), tbl); sc = R::comb(sc, init, tbl); sc = R::comb(sc, CH(0), tbl); break;
  case 4: sc = R::comb(CH(3), CH(2), tbl); sc = R::comb(sc, init, tbl); sc = R::comb(sc, CH(1), tbl);
          sc = R::comb(sc, CH(0), tbl); break;
  case 5: sc = R::comb(CH(4), CH(3), tbl); sc = R::comb(sc, init, tbl); sc = R::comb(sc, CH(1), tbl);
          sc = R::comb(sc, CH(2), tbl); sc = R::comb(sc, CH(0), tbl); break;
  default: sc = R::comb(CH(5), init, tbl); sc = R::comb(sc, CH(4), tbl); sc = R::comb(sc, CH(3), tbl);
           sc = R::comb(sc, CH(2), tbl); sc = R::comb(sc, CH(1), tbl); sc = R::comb(sc, CH(0), tbl); break;
  }
#undef CH
  return sc;
}

template <bool INS>
CMGB_DEV void qdb_scan_body(const KParams &p, float *smf, int tid, int nt, int bid)
{
  typedef Sr<INS> R;
  typedef typename R::T T;
  const ScanPlan &P = p.plan;
  const int M = P.M, W = P.W, TT = P.T;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  T *sm = reinterpret_cast<T *>(smf);
  T *acc = sm + P.acc_off;
  int *bestr = reinterpret_cast<int *>(smf) + P.bestr_off;
  unsigned char *res = reinterpret_cast<unsigned char *>(smf + P.res_off);
  T *carry0 = reinterpret_cast<T *>(p.carry) + (size_t) bid * 2 * P.carry_elems;
  T *ringb = reinterpret_cast<T *>(p.ring) + (size_t) bid * P.ring_elems;
  const int *tbl = p.ilog;
  const float el = P.el_selfsc;
  const int iel = P.iel_selfsc;
  int *s_win = reinterpret_cast<int *>(smf) + P.smem_elems;   // one shared int past the plan's arena

  // constant row of the E states: d = 0 is 0, every other d is impossible
  for (int d = tid; d < P.const_row_len; d += nt) sm[P.const_row + d] = d == 0 ? (T) 0 : R::imp();

  long long envi = 0x7fffffffffffffffLL, envj = -1;
  float best_root = CMGB_IMP;

  for (;;) {
    CMGB_SYNC();
    if (tid == 0) *s_win = CMGB_ATOMIC_ADD(p.queue, 1);
    CMGB_SYNC();
    const int w = *s_win;
    if (w >= p.nwin) break;
    const long long own_s = p.i0 + (long long) w * p.win_len;
    long long own_e = own_s + p.win_len - 1;
    if (own_e > p.j0) own_e = p.j0;
    long long s0 = own_s - (W - 1);
    if (s0 < p.i0) s0 = p.i0;

    // carry rows of j = s0-1 and the ring row jp = 0 hold the initial matrix values
    for (int v = 0; v < M; v++) {
      const StateInfo &si = p.st[v];
      if (si.carry >= 0) {
        T i0v = R::init0(si);
        for (int d = si.lo + tid; d <= si.hi; d += nt) carry0[si.carry + d - si.lo] = d == 0 ? i0v : R::imp();
      }
      if (si.kind == SK_BEGL) {
        T i0v = R::init0(si);
        for (int d = si.lo + tid; d <= si.hi; d += nt) ringb[si.ring + d - si.lo] = d == 0 ? i0v : R::imp();
      }
    }

    int par = 0;
    for (long long t = s0; t <= own_e; t += TT, par ^= 1) {
      const int nrows = (int) ((own_e - t + 1) < TT ? (own_e - t + 1) : TT);
      const long long jp0 = t - s0;          // jp of row r is jp0 + r
      const T *cin = carry0 + (size_t) par * P.carry_elems;
      T *cout = carry0 + (size_t) (par ^ 1) * P.carry_elems;
      const long long rbase = t - W;         // res[k] = dsq[rbase + k]
      CMGB_SYNC();
      for (int k = tid; k < P.res_len; k += nt) {
        long long q = rbase + k;
        res[k] = (q >= 0 && q <= p.j0 + 1) ? p.dsq[q] : (unsigned char) 0;
      }
      for (int k = tid; k < TT * (W + 1); k += nt) { acc[k] = R::acc_init(); bestr[k] = -1; }
      CMGB_SYNC();

      for (int v = M - 1; v >= 0; v--) {
        const StateInfo &si = p.st[v];
        if (si.kind == SK_E) continue;
        const int lo = si.lo, hi = si.hi;
        float vbest = CMGB_IMP;
        if (si.kind == SK_ROOT) {
          // ---- root: children fold, local-begin accumulator, candidates ----
          for (int r = 1 + warp; r <= nrows; r += nwarp) {
            const long long jp = jp0 + r, j = t + r - 1;
            int dx = (int) (jp < si.dxW ? jp : si.dxW);
            for (int d = si.dn + lane; d <= dx; d += 32) {
              T sc = R::rootfirst(R::add(sm[si.cbuf[0] + r * si.cstr[0] + d - si.clo[0]], R::tsc(si, 0)));
              for (int o = 1; o < si.cnum; o++)
                sc = R::comb(sc, R::add(sm[si.cbuf[o] + r * si.cstr[o] + d - si.clo[o]], R::tsc(si, o)), tbl);
              const int ai = (r - 1) * (W + 1) + d;
              int br = 0;
              if (!(sc >= acc[ai])) { sc = acc[ai]; br = bestr[ai]; }
              if (j < own_s) continue;
              float f = R::score(sc);
              best_root = best_root > f ? best_root : f;
              if (R::envval(sc) >= p.env_cut) {
                long long ii = j - d + 1;
                envi = envi < ii ? envi : ii;
                envj = envj > j ? envj : j;
              }
              if (d >= 1 && CMGB_NOT_IMP(f) && (p.cand_pos ? (f > 0.0f) : (f >= p.cand_cut))) {
                int slot = CMGB_ATOMIC_ADD(p.ncand, 1);
                if (slot < p.cand_cap) { Cand c; c.j = j; c.d = d; c.sc = f; c.r = br; c.pad = 0; p.cand[slot] = c; }
                else *p.err = 1;
              }
            }
          }
        } else if (si.kind == SK_IL) {
          // ---- row 0 from the carry, then one thread per row runs the d chain ----
          for (int d = lo + tid; d <= hi; d += nt) sm[si.buf + d - lo] = cin[si.carry + d - lo];
          for (int r = 1 + tid; r <= nrows; r += nt) {
            const long long jp = jp0 + r, j = t + r - 1;
            const int dx = (int) (jp < si.dxW ? jp : si.dxW);
            T *row = sm + si.buf + r * si.stride - lo;
            const int jres = (int) (j - rbase);
            for (int d = lo; d <= hi; d++) {
              T val;
              if (d < si.dn || d > dx) val = d == 0 ? R::init0(si) : R::imp();
              else {
                val = fold_children<INS>(si, sm, r, d - 1, R::init_sc(si, d - 1, el, iel), tbl);
                val = R::add(val, R::esc(p, si.oesc_off + res[jres - d + 1]));
                if (j >= own_s) { float f = R::score(val); vbest = vbest > f ? vbest : f; }
                if (si.has_begin && d >= P.root_dn && d <= (jp < P.root_dxW ? jp : P.root_dxW)) {
                  T c = R::add(val, R::beginsc(si));
                  const int ai = (r - 1) * (W + 1) + d;
                  if (c >= acc[ai]) { acc[ai] = c; bestr[ai] = v; }
                }
              }
              row[d] = val;
              if (r == TT) cout[si.carry + d - lo] = val;
            }
          }
        } else if (si.kind == SK_IR) {
          // ---- one thread per diagonal (r, c + r), r = 0 .. nrows ----
          const int ndiag = hi - lo + 1 + TT;
          for (int q = tid; q < ndiag; q += nt) {
            const int c = lo - TT + q;   // d at r = 0
            for (int r = 0; r <= nrows; r++) {
              const int d = c + r;
              if (d < lo || d > hi) continue;
              T val;
              if (r == 0) val = cin[si.carry + d - lo];
              else {
                const long long jp = jp0 + r, j = t + r - 1;
                const int dx = (int) (jp < si.dxW ? jp : si.dxW);
                if (d < si.dn || d > dx) val = d == 0 ? R::init0(si) : R::imp();
                else {
                  val = fold_children<INS>(si, sm, r - 1, d - 1, R::init_sc(si, d - 1, el, iel), tbl);
                  val = R::add(val, R::esc(p, si.oesc_off + res[(int) (j - rbase)]));
                  if (j >= own_s) { float f = R::score(val); vbest = vbest > f ? vbest : f; }
                  if (si.has_begin && d >= P.root_dn && d <= (jp < P.root_dxW ? jp : P.root_dxW)) {
                    T cc = R::add(val, R::beginsc(si));
                    const int ai = (r - 1) * (W + 1) + d;
                    if (cc >= acc[ai]) { acc[ai] = cc; bestr[ai] = v; }
                  }
                }
                if (r == TT) cout[si.carry + d - lo] = val;
              }
              sm[si.buf + r * si.stride + d - lo] = val;
            }
          }
        } else {
          // ---- generic, BEGL_S and B: one warp per row, lanes over d ----
          const bool begl = si.kind == SK_BEGL;
          for (int r = (begl ? 1 : 0) + warp; r <= nrows; r += nwarp) {
            const long long jp = jp0 + r, j = t + r - 1;
            const int dx = (int) (jp < si.dxW ? jp : si.dxW);
            const int jres = (int) (j - rbase);
            const int crow = si.right ? r - 1 : r;
            T *dst = begl ? ringb + si.ring + (int) (jp % P.ring_rows) * si.stride - lo
                          : sm + si.buf + r * si.stride - lo;
            for (int d = lo + lane; d <= hi; d += 32) {
              if (r == 0) { dst[d] = cin[si.carry + d - lo]; continue; }
              T val;
              if (d < si.dn || d > dx) val = d == 0 ? R::init0(si) : R::imp();
              else {
                if (si.kind == SK_B) {
                  // bifurcation: max/ILogsum over k of BEGL(j-k, d-k) + BEGR(j, k)
                  const int kmin = si.banded ? (0 > (si.dn_y > d - si.dx_w ? si.dn_y : d - si.dx_w) ? 0 : (si.dn_y > d - si.dx_w ? si.dn_y : d - si.dx_w)) : 0;
                  const int kmax = si.banded ? (si.dx_y < d - si.dn_w ? si.dx_y : d - si.dn_w) : d;
                  val = R::init_sc(si, d, el, iel);
                  const T *yrow = sm + si.cbuf[1] + r * si.cstr[1] - si.clo[1];
                  const T *wring = ringb + si.cbuf[0] - si.clo[0];
                  const int wstr = si.cstr[0];
                  long long rr = (jp - kmin) % P.ring_rows;
                  for (int k = kmin; k <= kmax; k++) {
                    T term = R::add(wring[(int) rr * wstr + d - k], yrow[k]);
                    val = R::comb(val, term, tbl);
                    rr = rr == 0 ? P.ring_rows - 1 : rr - 1;
                  }
                } else if (begl) {
                  val = R::init_sc(si, d, el, iel);
                  for (int o = 0; o < si.cnum; o++)
                    val = R::comb(val, R::add(sm[si.cbuf[o] + crow * si.cstr[o] + d - si.clo[o]], R::tsc(si, o)), tbl);
                } else {
                  val = fold_children<INS>(si, sm, crow, d - si.sd, R::init_sc(si, d - si.sd, el, iel), tbl);
                  if (si.emit == 3)      val = R::add(val, R::esc(p, si.oesc_off + res[jres - d + 1] * P.Kp + res[jres]));
                  else if (si.emit == 1) val = R::add(val, R::esc(p, si.oesc_off + res[jres - d + 1]));
                  else if (si.emit == 2) val = R::add(val, R::esc(p, si.oesc_off + res[jres]));
                }
                if (j >= own_s) { float f = R::score(val); vbest = vbest > f ? vbest : f; }
                if (si.has_begin && d >= P.root_dn && d <= (jp < P.root_dxW ? jp : P.root_dxW)) {
                  T cc = R::add(val, R::beginsc(si));
                  const int ai = (r - 1) * (W + 1) + d;
                  if (cc >= acc[ai]) { acc[ai] = cc; bestr[ai] = v; }
                }
              }
              dst[d] = val;
              if (r == TT && !begl) cout[si.carry + d - lo] = val;
            }
          }
        }
        if (p.vsc && vbest > CMGB_IMP) CMGB_ATOMIC_MAXU(p.vsc + v, cmgb_f2u(vbest));
        CMGB_SYNC();
      }
    }
  }
  if (envj >= 0) { CMGB_ATOMIC_MINLL(p.env, envi); CMGB_ATOMIC_MAXLL(p.env + 1, envj); }
  if (best_root > CMGB_IMP) CMGB_ATOMIC_MAXU(p.best, cmgb_f2u(best_root));
}

#ifndef CMGB_HOST_EMULATION
template <bool INS>
__global__ void __launch_bounds__(256) qdb_scan_kernel(KParams p)
{
  extern __shared__ float smem_dyn[];
  qdb_scan_body<INS>(p, smem_dyn, threadIdx.x, blockDim.x, blockIdx.x);
}
#endif
